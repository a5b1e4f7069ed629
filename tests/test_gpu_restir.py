"""ReSTIR DI on the GPU (tt_render_restir) against the CPU oracle, bit for bit: images and the
final reservoirs of every frame, with a moving camera (temporal reprojection), on scenes with
few and with many lights, with textured materials and lights, and with every lobe combination."""
import numpy as np
import pytest

from conftest import assert_same_bits
from materials import material_spheres
from oracle import oracle
from tinytrace_gb300 import scenes
from tinytrace_gb300.camera import Camera
from tinytrace_gb300.renderer import Config, Renderer, SceneArrays, make_constants

pytestmark = pytest.mark.gpu


def _orbit(center, radius, height, frame, step=0.02):
    a = frame * step
    pos = (center[0] + radius * np.sin(a), height, center[2] + radius * np.cos(a))
    return Camera.looking_at(pos, center, fov=0.8)


CASES = {
    "cornell": (lambda: scenes.cornell_box(), (0.0, 1.0, 0.0), 3.4, 1.0, (64, 48)),
    "field": (lambda: scenes.icosphere_field(instances=6, freq=8, lights=300, seed=11), (0.0, 0.0, 0.0), 95.0, 10.0,
              (96, 54)),
    "instanced": (lambda: scenes.instanced_spheres(), (0.0, 0.0, 0.0), 40.0, 6.0, (80, 60)),
    "textured": (lambda: scenes.textured_cornell(), (0.0, 1.0, 0.0), 3.4, 1.0, (64, 48)),
    # every lobe combination of the BSDF suite; the candidate pass runs each bucket's lobe set
    "materials": (material_spheres, (0.0, 0.0, -0.5), 5.0, 3.0, (80, 60)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_restir_frames_match_oracle(gpu_context, name):
    make, center, radius, height, extent = CASES[name]
    r = Renderer(extent)
    r.set_scene(make())
    r.set_config(Config(bounce_count=1, sample_count=1))
    orc = oracle.OracleScene(r.scene_arrays)
    R = oracle.OracleRestir(orc, *extent)
    cpu = np.zeros((extent[1], extent[0], 4), np.float32)
    for f in range(6):
        r.camera = _orbit(center, radius, height, f)
        c = make_constants(r.camera, extent, r.config(), r.context.frame_index(), r.accumulated_frame_count)
        r.render_restir_to_target()
        gpu = r.context.download(r.render_target, *extent)
        R.frame(c, cpu)
        assert_same_bits(gpu, cpu, f"{name} frame {f} image")
        assert_same_bits(r.restir_reservoirs(), R.reservoirs(), f"{name} frame {f} reservoirs")
        r.present()
    assert (R.reservoirs()[..., 5] > 0).mean() > 0.05
    r.close()


@pytest.mark.parametrize("accel", ["two_level", "wide"])
def test_restir_structures_match_oracle(gpu_context, accel):
    """The ReSTIR passes compiled for the two-level and the compressed wide structure (each
    scene's passes use the traversal of its own structure): the field's frames as above."""
    from tinytrace_gb300 import native
    from tinytrace_gb300.native import check

    make, center, radius, height, extent = CASES["field"]
    r = Renderer(extent)
    value = {"two_level": native.TT_ACCEL_TWO_LEVEL, "wide": native.TT_ACCEL_FLAT_WIDE}[accel]
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_ACCEL, value))
    r.set_scene(make())
    assert r.context.scene_stats(r.scene).accel == value
    r.set_config(Config(bounce_count=1, sample_count=1))
    orc = oracle.OracleScene(r.scene_arrays)
    R = oracle.OracleRestir(orc, *extent)
    cpu = np.zeros((extent[1], extent[0], 4), np.float32)
    for f in range(3):
        r.camera = _orbit(center, radius, height, f)
        c = make_constants(r.camera, extent, r.config(), r.context.frame_index(), r.accumulated_frame_count)
        r.render_restir_to_target()
        gpu = r.context.download(r.render_target, *extent)
        R.frame(c, cpu)
        assert_same_bits(gpu, cpu, f"{accel} frame {f} image")
        assert_same_bits(r.restir_reservoirs(), R.reservoirs(), f"{accel} frame {f} reservoirs")
        r.present()
    r.close()


def test_restir_config_and_reset(gpu_context):
    make, center, radius, height, extent = CASES["cornell"]
    r = Renderer(extent)
    r.set_scene(make())
    r.set_config(Config(bounce_count=1, sample_count=1))
    r.restir_configure(candidates=8, temporal_m_cap=4.0, spatial_neighbours=2, spatial_radius=10.0)
    orc = oracle.OracleScene(r.scene_arrays)
    R = oracle.OracleRestir(orc, *extent, candidates=8, m_cap_factor=4.0, neighbours=2, radius=10.0)
    cpu = np.zeros((extent[1], extent[0], 4), np.float32)
    for f in range(3):
        if f == 2:  # forget the history on both sides
            r.restir_reset()
            R = oracle.OracleRestir(orc, *extent, candidates=8, m_cap_factor=4.0, neighbours=2, radius=10.0)
        r.camera = _orbit(center, radius, height, f)
        c = make_constants(r.camera, extent, r.config(), r.context.frame_index(), r.accumulated_frame_count)
        r.render_restir_to_target()
        R.frame(c, cpu)
        assert_same_bits(r.context.download(r.render_target, *extent), cpu, f"frame {f}")
        r.present()
    assert r.restir_reservoirs()[..., 4].max() <= 3 * 8
    r.close()


def test_restir_power_candidates(gpu_context):
    """ReSTIR with candidates drawn by emitted power (TT_LIGHT_SELECTION_POWER), bit for bit."""
    from tinytrace_gb300 import native
    from tinytrace_gb300.native import check

    make, center, radius, height, extent = CASES["field"]
    r = Renderer(extent)
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_LIGHT_SELECTION,
                                      native.TT_LIGHT_SELECTION_POWER))
    r.set_scene(make())
    r.set_config(Config(bounce_count=1, sample_count=1))
    orc = oracle.OracleScene(r.scene_arrays)
    orc.set_light_power(True)
    R = oracle.OracleRestir(orc, *extent)
    cpu = np.zeros((extent[1], extent[0], 4), np.float32)
    for f in range(3):
        r.camera = _orbit(center, radius, height, f)
        c = make_constants(r.camera, extent, r.config(), r.context.frame_index(), r.accumulated_frame_count)
        r.render_restir_to_target()
        gpu = r.context.download(r.render_target, *extent)
        R.frame(c, cpu)
        assert_same_bits(gpu, cpu, f"power candidates frame {f} image")
        assert_same_bits(r.restir_reservoirs(), R.reservoirs(), f"power candidates frame {f} reservoirs")
        r.present()
    r.close()
