"""Rasterised primary visibility (TT_PRIMARY_RASTER) against traversed camera rays and the oracle.

With TT_PRIMARY_RASTER the wavefront integrator finds the closest hit of every camera ray of a
flat BVH4 scene by bounding each triangle on the screen and testing the samples inside its
rectangle (primary.cu); the hit must be the traversal's, bit for bit.  The scenes below aim at
the bound's edge cases: triangles crossing the camera plane and behind the camera (camera inside
the Cornell box, on a ground plane, among spheres), mirrored and strongly anisotropic instances,
a degenerate triangle, narrow and wide fields of view, and sample chunks after the first.
Tolerance: zero (bit-exact images).
"""
import ctypes

import numpy as np
import pytest

from conftest import assert_same_bits
from oracle import oracle
from tinytrace_gb300 import native, scenes
from tinytrace_gb300.asset import Material, Model, Node
from tinytrace_gb300.asset import Scene as AssetScene
from tinytrace_gb300.camera import Camera
from tinytrace_gb300.native import check
from tinytrace_gb300.renderer import Config, Renderer, make_constants

pytestmark = pytest.mark.gpu

MODES = {"raster": native.TT_PRIMARY_RASTER, "traverse": native.TT_PRIMARY_TRAVERSE}


def _ground_and_slabs() -> AssetScene:
    """A ground quad far larger than the view (it crosses the camera plane), a thin slab scaled
    (40, 0.05, 40) and rotated (condition number ~800), a mirrored sphere, a degenerate
    triangle and an emissive quad."""
    s = AssetScene()
    grey = s.insert_material(scenes.lambertian((0.6, 0.6, 0.6)))
    blue = s.insert_material(Material(base_color=(0.2, 0.3, 0.8), specular_roughness=0.3))
    light = s.insert_material(Material(emission_luminance=20.0, emission_color=(1.0, 0.9, 0.8)))
    lq = scenes._quad((-2, 6, -2), (-2, 6, 2), (2, 6, 2), (2, 6, -2))
    s.root.children.append(Node(models=[Model(s.insert_mesh(lq[0], lq[3], lq[1], lq[2]), light)]))
    g = scenes._quad((-200, 0, 200), (200, 0, 200), (200, 0, -200), (-200, 0, -200))
    s.root.children.append(Node(models=[Model(s.insert_mesh(g[0], g[3], g[1], g[2]), grey)]))
    pos, idx, nrm, uv = scenes._box((-1, -1, -1), (1, 1, 1), 0.0)
    cube = s.insert_mesh(pos, uv, idx, nrm)
    t = np.eye(4)
    ang = 0.5
    rot = np.array([[np.cos(ang), 0, np.sin(ang)], [0, 1, 0], [-np.sin(ang), 0, np.cos(ang)]])
    t[:3, :3] = rot @ np.diag([40.0, 0.05, 40.0])
    t[:3, 3] = (0.0, 0.3, -10.0)
    s.root.children.append(Node(transform=t, models=[Model(cube, blue)]))
    pts, tris = scenes.geodesic_sphere(6)
    sphere = s.insert_mesh(pts.astype(np.float32), None, tris)
    t = np.eye(4)
    t[:3, :3] = np.diag([-1.5, 1.5, 1.5])  # mirrored
    t[:3, 3] = (3.0, 1.6, -6.0)
    s.root.children.append(Node(transform=t, models=[Model(sphere, grey)]))
    deg = np.array([[0, 1, -4], [1, 2, -4], [2, 3, -4], [0, 2, -5]], np.float32)  # (0,1,2) collinear
    dm = s.insert_mesh(deg, None, np.array([0, 1, 2, 0, 1, 3], np.uint32), np.tile(np.float32([0, 0, 1]), (4, 1)))
    s.root.children.append(Node(models=[Model(dm, grey)]))
    return s


def _workloads():
    cornell = scenes.cornell_box()
    field = scenes.icosphere_field(instances=14, freq=8, lights=30, seed=5, box=40.0)
    slabs = _ground_and_slabs()
    return [
        # inside the Cornell box: floor, ceiling and side walls cross the camera plane; 70 spp = two chunks
        scenes.Workload("cornell_inside", cornell, Camera.looking_at((0.0, 1.0, 0.6), (0.3, 0.8, -1.0)), (48, 36),
                        Config(bounce_count=4, sample_count=70)),
        # among the spheres: records behind the camera and spheres around it
        scenes.Workload("field_inside", field, Camera.looking_at((0.0, 0.0, 0.0), (10.0, 2.0, 3.0)), (80, 45),
                        Config(bounce_count=5, sample_count=3)),
        scenes.Workload("field_narrow", field, Camera.looking_at((0.0, 10.0, 95.0), (0, 0, 0), fov=0.12), (64, 40),
                        Config(bounce_count=3, sample_count=2)),
        scenes.Workload("slabs_wide", slabs, Camera.looking_at((0.0, 1.5, 0.0), (5.0, 0.5, -5.0), fov=2.6), (72, 40),
                        Config(bounce_count=4, sample_count=3)),
        scenes.Workload("slabs_low", slabs, Camera.looking_at((-2.0, 0.35, 2.0), (3.0, 0.2, -12.0)), (64, 36),
                        Config(bounce_count=3, sample_count=2)),
        scenes.Workload("instanced", scenes.instanced_spheres(copies=24), Camera.looking_at((0.0, 8.0, 30.0), (0, 0, 0)),
                        (64, 48), Config(bounce_count=4, sample_count=2)),
    ]


def _render(w, mode, graphs=1, timing=False):
    r = Renderer(w.extent)
    lib, hd = r.context.lib, r.context.handle
    check(lib.tt_set_option(hd, native.TT_OPTION_ACCEL, native.TT_ACCEL_FLAT))
    check(lib.tt_set_option(hd, native.TT_OPTION_PRIMARY_VISIBILITY, MODES[mode]))
    check(lib.tt_set_option(hd, native.TT_OPTION_GRAPHS, graphs))
    check(lib.tt_set_option(hd, native.TT_OPTION_STAGE_TIMING, 1 if timing else 0))
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(w.config)
    c = make_constants(w.camera, w.extent, w.config, r.context.frame_index(), r.accumulated_frame_count)
    img = r.render_to_texture()
    launches = None
    if timing:
        stt = native.StageTimings()
        check(lib.tt_stage_timings_get(hd, ctypes.byref(stt)))
        launches = int(stt.launches[native.TT_STAGE_PRIMARY])
    arrays = r.scene_arrays
    r.close()
    return img, c, arrays, launches


@pytest.mark.parametrize("index", range(6))
def test_primary_raster_equals_traversal_and_oracle(gpu_context, index):
    w = _workloads()[index]
    raster, c, arrays, _ = _render(w, "raster")
    traverse, _, _, _ = _render(w, "traverse")
    assert_same_bits(raster, traverse, f"{w.name}: raster vs traversal")
    assert_same_bits(raster, oracle.OracleScene(arrays).render(c), f"{w.name}: raster vs oracle")
    assert np.isfinite(raster).all() and raster[..., :3].max() > 0.0


def test_primary_stage_runs_only_when_rastering(gpu_context):
    """The host-driven loop with stage timing: one set-up and one key pass per sample chunk
    with TT_PRIMARY_RASTER (so the keys are what the image came from), none with traversal or on
    a two-level scene."""
    w = _workloads()[0]  # 70 spp: two chunks
    img_r, c, arrays, n_r = _render(w, "raster", graphs=0, timing=True)
    img_t, _, _, n_t = _render(w, "traverse", graphs=0, timing=True)
    assert n_r == 3 and n_t == 0
    assert_same_bits(img_r, img_t, "host loop raster vs traversal")
    r = Renderer(w.extent)
    lib, hd = r.context.lib, r.context.handle
    check(lib.tt_set_option(hd, native.TT_OPTION_ACCEL, native.TT_ACCEL_TWO_LEVEL))
    check(lib.tt_set_option(hd, native.TT_OPTION_STAGE_TIMING, 1))
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(w.config)
    r.render_to_texture()
    stt = native.StageTimings()
    check(lib.tt_stage_timings_get(hd, ctypes.byref(stt)))
    assert int(stt.launches[native.TT_STAGE_PRIMARY]) == 0
    r.close()


def test_primary_option_rejects_unknown(gpu_context):
    lib, hd = gpu_context.lib, gpu_context.handle
    assert lib.tt_set_option(hd, native.TT_OPTION_PRIMARY_VISIBILITY, 2) == native.TT_ERR_INVALID_ARGUMENT
    check(lib.tt_set_option(hd, native.TT_OPTION_PRIMARY_VISIBILITY, native.TT_PRIMARY_RASTER))


def test_primary_raster_restir_frames(gpu_context):
    """ReSTIR's G-buffer pass takes its camera-ray hits from one sample of rasterised keys per
    pixel: images and reservoirs equal the traversed frames and the oracle's, with the camera
    moving inside the Cornell box (walls crossing the camera plane)."""
    extent = (48, 36)
    frames = {}
    for mode in ("raster", "traverse"):
        r = Renderer(extent)
        lib, hd = r.context.lib, r.context.handle
        check(lib.tt_set_option(hd, native.TT_OPTION_ACCEL, native.TT_ACCEL_FLAT))
        check(lib.tt_set_option(hd, native.TT_OPTION_PRIMARY_VISIBILITY, MODES[mode]))
        r.set_scene(scenes.cornell_box())
        r.set_config(Config(bounce_count=1, sample_count=1))
        orc = oracle.OracleScene(r.scene_arrays)
        R = oracle.OracleRestir(orc, *extent)
        cpu = np.zeros((extent[1], extent[0], 4), np.float32)
        out = []
        for f in range(4):
            r.camera = Camera.looking_at((0.1 * f, 1.0, 0.6), (0.3, 0.8 - 0.05 * f, -1.0))
            c = make_constants(r.camera, extent, r.config(), r.context.frame_index(), r.accumulated_frame_count)
            r.render_restir_to_target()
            gpu = r.context.download(r.render_target, *extent)
            R.frame(c, cpu)
            assert_same_bits(gpu, cpu, f"restir {mode} frame {f} image")
            assert_same_bits(r.restir_reservoirs(), R.reservoirs(), f"restir {mode} frame {f} reservoirs")
            out.append(gpu.copy())
            r.present()
        frames[mode] = out
        r.close()
    for f, (a, b) in enumerate(zip(frames["raster"], frames["traverse"])):
        assert_same_bits(a, b, f"restir frame {f}: raster vs traversal")
