"""CUDA path vs the CPU oracle, bit for bit, through the C ABI (GPU required).

Tolerance: zero.  Every kernel on the path is specified operation by operation (IEEE-754
single precision, no implicit contraction, project-owned elementary functions), so the GPU
must reproduce the oracle's bits exactly; only NaN payloads may differ.
"""
import ctypes

import numpy as np
import pytest

from conftest import assert_same_bits
from materials import eval_samples, material_spheres, material_suite, sample_samples
from oracle import oracle
from tinytrace_gb300 import native, scenes
from tinytrace_gb300.native import NODE4_DTYPE, TRI_RECORD_DTYPE, check
from tinytrace_gb300.renderer import SceneArrays, make_constants

pytestmark = pytest.mark.gpu


def gpu_math(ctx, which, x):
    x = np.ascontiguousarray(x, np.float32)
    y = np.zeros_like(x)
    check(ctx.lib.tt_math_batch(ctx.handle, which, native.ptr(x), x.size, native.ptr(y)))
    return y


def test_math_bits(gpu_context):
    rng = np.random.default_rng(0)
    xs = {
        0: np.concatenate([rng.uniform(-20, 20, 100000), rng.uniform(0, 2 * np.pi, 100000), [0.0, -0.0, 1e7, 3e7]]),
        1: np.concatenate([rng.uniform(-20, 20, 100000), rng.uniform(0, 2 * np.pi, 100000)]),
        2: np.concatenate([rng.uniform(-110, 90, 200000), [0.0, -0.0, 88.7, -87.3, -103.0]]),
        3: np.concatenate([np.exp(rng.uniform(-100, 88, 200000)), [1e-42, 1.0, 0.0, 2.0]]),
        4: np.concatenate([rng.uniform(-1, 1, 200000), [-1.0, 1.0, 0.5, -0.5, 0.0]]),
    }
    for which, x in xs.items():
        x = x.astype(np.float32)
        assert_same_bits(gpu_math(gpu_context, which, x), oracle.math(which, x), f"math {which}")


def test_bsdf_eval_bits(gpu_context):
    rng = np.random.default_rng(1)
    for i, m in enumerate(material_suite()):
        s = eval_samples(rng, 4096)
        out = np.zeros((len(s), 8), np.float32)
        m = np.ascontiguousarray(m)
        check(gpu_context.lib.tt_bsdf_eval_batch(gpu_context.handle, native.ptr(m), native.ptr(s), len(s),
                                                 native.ptr(out)))
        assert_same_bits(out, oracle.bsdf_eval(m, s), f"bsdf_evaluate material {i}")


def test_bsdf_sample_bits(gpu_context):
    rng = np.random.default_rng(2)
    for i, m in enumerate(material_suite()):
        s = sample_samples(rng, 4096)
        out = np.zeros((len(s), 12), np.float32)
        m = np.ascontiguousarray(m)
        check(gpu_context.lib.tt_bsdf_sample_batch(gpu_context.handle, native.ptr(m), native.ptr(s), len(s),
                                                   native.ptr(out)))
        assert_same_bits(out, oracle.bsdf_sample(m, s), f"bsdf_sample material {i}")


def _gpu_bvh(ctx, scene):
    st = ctx.scene_stats(scene)
    blas = np.zeros(st.blas_nodes, NODE4_DTYPE)
    tris = np.zeros(st.triangle_count, TRI_RECORD_DTYPE)
    tlas = np.zeros(st.tlas_nodes, native.NODE8_DTYPE if st.accel == native.TT_ACCEL_FLAT_WIDE else NODE4_DTYPE)
    check(ctx.lib.tt_scene_bvh_download(ctx.handle, scene, native.ptr(blas), blas.nbytes, native.ptr(tris),
                                        tris.nbytes, native.ptr(tlas), tlas.nbytes))
    return blas, tris, tlas, st


def _small_field():
    return scenes.icosphere_field(instances=6, freq=8, lights=40, seed=11)


def _duplicate_keys():
    """Equal Morton codes in bulk: 2,100 copies of one small triangle and 400 random ones in one
    mesh, placed three times with the same transform, so the flat build sorts 7,500 keys (four
    2,048-key tiles of the onesweep sort) of which 6,300 are equal and must keep primitive
    order."""
    from tinytrace_gb300.asset import Model, Node, Scene
    rng = np.random.default_rng(7)
    tri = np.array([[0.1, 0.2, 0.3], [0.12, 0.2, 0.3], [0.1, 0.23, 0.31]], np.float32)
    rand = rng.uniform(-1.0, 1.0, (400, 3, 3)).astype(np.float32)
    pos = np.concatenate([np.tile(tri, (2100, 1)), rand.reshape(-1, 3)])
    idx = np.arange(len(pos), dtype=np.uint32)
    s = Scene()
    m = s.insert_mesh(pos, None, idx)
    mat = s.insert_material(scenes.lambertian((0.5, 0.5, 0.5)))
    for _ in range(3):
        s.root.children.append(Node(models=[Model(m, mat)]))
    return s


ACCELS = {"flat": native.TT_ACCEL_FLAT, "two_level": native.TT_ACCEL_TWO_LEVEL, "wide": native.TT_ACCEL_FLAT_WIDE}


def _create_scene(ctx, arrays, accel):
    check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_ACCEL, ACCELS[accel]))
    try:
        return ctx.create_scene(arrays)
    finally:
        check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_ACCEL, native.TT_ACCEL_AUTO))


@pytest.mark.parametrize("accel", ["two_level", "flat", "wide"])
@pytest.mark.parametrize("name", ["cornell", "field", "instanced", "duplicates"])
def test_bvh_topology_bits(gpu_context, name, accel):
    scene = {"cornell": scenes.cornell_box, "field": _small_field, "instanced": scenes.instanced_spheres,
             "duplicates": _duplicate_keys}[name]()
    arrays = SceneArrays(scene)
    h = _create_scene(gpu_context, arrays, accel)
    blas, tris, tlas, st = _gpu_bvh(gpu_context, h)
    orc = oracle.OracleScene(arrays, wide=accel == "wide")
    if accel == "wide":
        assert st.accel == native.TT_ACCEL_FLAT_WIDE
        on, ot, ol = orc.wide_bvh()
        assert st.blas_nodes == 0 and st.tlas_levels == ol
        assert tris.tobytes() == ot.tobytes(), "wide triangle records differ"
        assert tlas.tobytes() == on.tobytes(), "wide nodes differ"
    elif accel == "two_level":
        assert st.accel == native.TT_ACCEL_TWO_LEVEL
        ob, ot, otl, bl, tl = orc.bvh()
        assert (st.blas_levels, st.tlas_levels) == (bl, tl)
        assert blas.tobytes() == ob.tobytes(), "BLAS nodes differ"
        assert tris.tobytes() == ot.tobytes(), "triangle records differ"
        assert tlas.tobytes() == otl.tobytes(), "TLAS nodes differ"
    else:
        assert st.accel == native.TT_ACCEL_FLAT
        on, ot, ol = orc.flat_bvh()
        assert st.blas_nodes == 0 and st.tlas_levels == ol
        assert tris.tobytes() == ot.tobytes(), "flat triangle records differ"
        assert tlas.tobytes() == on.tobytes(), "flat BVH nodes differ"


def test_accel_auto_is_flat(gpu_context):
    h = gpu_context.create_scene(SceneArrays(scenes.cornell_box()))
    assert gpu_context.scene_stats(h).accel == native.TT_ACCEL_FLAT


def _random_rays(rng, n, center, spread):
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = center + rng.uniform(-spread, spread, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 4:7] = d
    rays[:, 3] = 1e-3
    rays[:, 7] = rng.choice([1000.0, 10000.0, 3.0], n)
    return rays


@pytest.mark.parametrize("accel", ["two_level", "flat", "wide"])
@pytest.mark.parametrize("name", ["cornell", "field"])
def test_closest_hit_matches_brute_force(gpu_context, name, accel):
    scene = scenes.cornell_box() if name == "cornell" else _small_field()
    arrays = SceneArrays(scene)
    h = _create_scene(gpu_context, arrays, accel)
    rng = np.random.default_rng(5)
    center, spread = ((0, 1, 0), 1.2) if name == "cornell" else ((0, 0, 0), 60.0)
    rays = _random_rays(rng, 20000, np.array(center), spread)
    if name == "field":  # aim most rays at instance centres so that the field is actually hit
        targets = arrays.instances["transform"][:, 12:15]
        t = targets[rng.integers(0, len(targets), len(rays))] + rng.normal(0, 3.0, (len(rays), 3))
        d = t - rays[:, 0:3]
        rays[:15000, 4:7] = (d / np.linalg.norm(d, axis=1, keepdims=True))[:15000]
    rays[:50, 4:7] = np.nan  # NaN directions never hit
    orc = oracle.OracleScene(arrays)
    for cull in (False, True):
        hits = np.zeros((len(rays), 8), np.uint32)
        check(gpu_context.lib.tt_trace_batch(gpu_context.handle, h, native.ptr(rays), len(rays),
                                             1 if cull else 0, native.ptr(hits)))
        brute = orc.trace(rays, cull=cull, brute=True)
        bvh = orc.trace(rays, cull=cull, brute=False, flat=accel == "flat")
        assert np.array_equal(bvh, brute), "oracle BVH traversal differs from brute force"
        assert np.array_equal(hits, brute), f"GPU closest hits differ (cull={cull}): {np.sum(np.any(hits != brute, 1))}"
        assert hits[:, 0].sum() > len(rays) // 20


INTEGRATORS = {"wavefront": native.TT_INTEGRATOR_WAVEFRONT, "megakernel": native.TT_INTEGRATOR_MEGAKERNEL}


def _render_pair(ctx, w, frames=1, integrator="wavefront", slots=0, accel="flat"):
    from tinytrace_gb300.renderer import Renderer

    r = Renderer(w.extent)
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_INTEGRATOR, INTEGRATORS[integrator]))
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_WAVEFRONT_SLOTS, slots))
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_ACCEL, ACCELS[accel]))
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(w.config)
    orc = oracle.OracleScene(r.scene_arrays)
    cpu = np.zeros((w.extent[1], w.extent[0], 4), np.float32)
    for f in range(frames):
        c = make_constants(w.camera, w.extent, w.config, r.context.frame_index(), r.accumulated_frame_count)
        gpu = r.render_to_texture()
        orc.render(c, cpu)
        assert_same_bits(gpu, cpu, f"{w.name} frame {f}")
        r.present()
    r.close()
    return gpu


@pytest.mark.parametrize("accel", ["flat", "two_level", "wide"])
@pytest.mark.parametrize("integrator", ["wavefront", "megakernel"])
def test_render_cornell_c1(gpu_context, integrator, accel):
    img = _render_pair(gpu_context, scenes.cornell_workload(), integrator=integrator, accel=accel)
    assert img[..., :3].mean() > 0.05


@pytest.mark.parametrize("integrator", ["wavefront", "megakernel"])
def test_render_accumulation(gpu_context, integrator):
    # frames 0 and 1 both overwrite (n = 0 and n = 1), later frames average
    _render_pair(gpu_context, scenes.cornell_workload(extent=(48, 40), spp=1, depth=3), frames=4,
                 integrator=integrator)


@pytest.mark.parametrize("accel", ["flat", "two_level", "wide"])
@pytest.mark.parametrize("integrator", ["wavefront", "megakernel"])
def test_render_field_small(gpu_context, integrator, accel):
    w = scenes.Workload("field_small", _small_field(), scenes.Camera.looking_at((0.0, 10.0, 95.0), (0, 0, 0)),
                        (96, 54), scenes.Config(bounce_count=8, sample_count=3))
    _render_pair(gpu_context, w, integrator=integrator, accel=accel)


@pytest.mark.parametrize("accel", ["flat", "two_level"])
def test_render_material_buckets(gpu_context, accel):
    w = scenes.Workload("material_spheres", material_spheres(),
                        scenes.Camera.looking_at((0.0, 3.0, 4.0), (0.0, -0.4, -0.6)), (96, 64),
                        scenes.Config(bounce_count=6, sample_count=3))
    img = _render_pair(gpu_context, w, integrator="wavefront", accel=accel)
    assert img[..., :3].mean() > 0.01


def test_render_wavefront_small_pool_and_chunks(gpu_context):
    # a pool much smaller than the frame (many refills) and 70 samples (two sample chunks)
    w = scenes.Workload("cornell_pool", scenes.cornell_box(), scenes.cornell_workload().camera, (40, 24),
                        scenes.Config(bounce_count=5, sample_count=70))
    _render_pair(gpu_context, w, integrator="wavefront", slots=256)


@pytest.mark.parametrize("integrator", ["wavefront", "megakernel"])
def test_render_edge_configs(gpu_context, integrator):
    base = scenes.cornell_workload(extent=(21, 13))
    for cfg in (scenes.Config(bounce_count=0, sample_count=2), scenes.Config(bounce_count=1, sample_count=1),
                scenes.Config(bounce_count=3, sample_count=2, light_sampling=scenes.LightSampling.ON_HIT)):
        w = scenes.Workload("edge", base.scene, base.camera, base.extent, cfg)
        _render_pair(gpu_context, w, integrator=integrator)


def test_tonemap_bits(gpu_context):
    rng = np.random.default_rng(9)
    img = rng.exponential(1.0, (32, 40, 4)).astype(np.float32)
    img[0, :4, :3] = [[0, 0, 0], [1e-8, 0, 0], [100, 50, 1], [np.inf, 1, 1]]
    ctx = gpu_context
    h = ctx.create_image(native.TT_LIFETIME_FRAME, 40, 32)
    ctx.write_image(h, img)
    c = np.zeros((), native.CONSTANTS_DTYPE)
    for enabled in (1, 0):
        c["tonemap"] = enabled
        out = np.zeros((32, 40, 4), np.float32)
        check(ctx.lib.tt_tonemap(ctx.handle, h, native.ptr(c), native.TT_FORMAT_RGBA32F, native.ptr(out), out.nbytes))
        assert_same_bits(out, oracle.tonemap(img, bool(enabled)), f"tonemap {enabled}")
    out8 = np.zeros((32, 40, 4), np.uint8)
    c["tonemap"] = 1
    check(ctx.lib.tt_tonemap(ctx.handle, h, native.ptr(c), native.TT_FORMAT_RGBA8_UNORM, native.ptr(out8), out8.nbytes))
    ref = oracle.tonemap(img, True)
    exp8 = (np.clip(np.nan_to_num(ref, nan=0.0), 0, 1) * np.float32(255) + np.float32(0.5)).astype(np.uint8)
    exp8[..., 3] = 255
    assert np.array_equal(out8, exp8)


@pytest.mark.parametrize("graphs", [0, 1])
def test_render_host_and_graph_loops(gpu_context, graphs):
    """The wavefront loop driven from the host and as a device-side while loop inside one CUDA
    graph give the oracle's image; the small pool makes the loop run many iterations and two
    sample chunks exercise two loops in one graph."""
    from tinytrace_gb300.renderer import Renderer

    w = scenes.Workload("cornell_loop", scenes.cornell_box(), scenes.cornell_workload().camera, (40, 24),
                        scenes.Config(bounce_count=5, sample_count=70))
    r = Renderer(w.extent)
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_GRAPHS, graphs))
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_WAVEFRONT_SLOTS, 300))
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(w.config)
    c = make_constants(w.camera, w.extent, w.config, r.context.frame_index(), r.accumulated_frame_count)
    gpu = r.render_to_texture()
    cpu = oracle.OracleScene(r.scene_arrays).render(c)
    assert_same_bits(gpu, cpu, f"loop graphs={graphs}")
    r.close()


def test_autotune_keeps_the_image(gpu_context):
    """tt_autotune leaves valid options on the context and renders stay bit-exact with them."""
    from tinytrace_gb300.renderer import Renderer

    w = scenes.Workload("field_tune", _small_field(), scenes.Camera.looking_at((0.0, 10.0, 95.0), (0, 0, 0)),
                        (96, 54), scenes.Config(bounce_count=6, sample_count=4))
    r = Renderer(w.extent)
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(w.config)
    res = r.autotune(sample_count=2)
    assert res.renders >= 10 and res.best_ms <= res.default_ms and res.best_ms > 0
    assert res.slots >= 128 and 1 <= res.refill_lanes <= 32 and res.trace_blocks_per_sm >= 1
    c = make_constants(w.camera, w.extent, w.config, r.context.frame_index(), r.accumulated_frame_count)
    gpu = r.render_to_texture()
    cpu = oracle.OracleScene(r.scene_arrays).render(c)
    assert_same_bits(gpu, cpu, "after autotune")
    r.close()


@pytest.mark.parametrize("mode", ["hash", "triangle"])
@pytest.mark.parametrize("integrator", ["wavefront", "megakernel"])
def test_light_visibility_modes(gpu_context, integrator, mode):
    """Both visibility tests of next-event estimation on a scene whose lights lie past global
    triangle index 65535 (the reference's hash never matches there), bit for bit."""
    from tinytrace_gb300.renderer import Renderer

    extent = (64, 48)
    cfg = scenes.Config(bounce_count=4, sample_count=3)
    cam = scenes.Camera.looking_at((0.0, 3.0, 4.0), (0.0, 0.0, 0.0), fov=0.8)
    r = Renderer(extent)
    lib, hd = r.context.lib, r.context.handle
    check(lib.tt_set_option(hd, native.TT_OPTION_INTEGRATOR, INTEGRATORS[integrator]))
    value = native.TT_LIGHT_VISIBILITY_TRIANGLE if mode == "triangle" else native.TT_LIGHT_VISIBILITY_HASH
    check(lib.tt_set_option(hd, native.TT_OPTION_LIGHT_VISIBILITY, value))
    assert lib.tt_set_option(hd, native.TT_OPTION_LIGHT_VISIBILITY, 7) == native.TT_ERR_INVALID_ARGUMENT
    r.set_scene(scenes.late_lights())
    r.camera = cam
    r.set_config(cfg)
    orc = oracle.OracleScene(r.scene_arrays)
    orc.set_light_exact(mode == "triangle")
    c = make_constants(cam, extent, cfg, r.context.frame_index(), r.accumulated_frame_count)
    assert_same_bits(r.render_to_texture(), orc.render(c), f"light visibility {mode} {integrator}")
    r.close()


@pytest.mark.parametrize("integrator", ["wavefront", "megakernel"])
def test_power_light_selection(gpu_context, integrator):
    """Power-proportional light selection through the alias table, bit for bit with the
    oracle's restatement, before and after the instances move (the table follows the new
    world-space areas)."""
    from moves import moved_instances
    from tinytrace_gb300.renderer import Renderer

    w = scenes.icosphere_workload(extent=(64, 40), spp=3, depth=4, instances=6, freq=8, lights=300)
    r = Renderer(w.extent)
    lib, hd = r.context.lib, r.context.handle
    check(lib.tt_set_option(hd, native.TT_OPTION_INTEGRATOR, INTEGRATORS[integrator]))
    check(lib.tt_set_option(hd, native.TT_OPTION_LIGHT_SELECTION, native.TT_LIGHT_SELECTION_POWER))
    assert lib.tt_set_option(hd, native.TT_OPTION_LIGHT_SELECTION, 5) == native.TT_ERR_INVALID_ARGUMENT
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(w.config)
    orc = oracle.OracleScene(r.scene_arrays)
    orc.set_light_power(True)
    c = make_constants(w.camera, w.extent, w.config, r.context.frame_index(), r.accumulated_frame_count)
    assert_same_bits(r.render_to_texture(), orc.render(c), f"power selection {integrator}")
    inst = moved_instances(r.scene_arrays.instances, np.random.default_rng(4), scale=0.2)
    check(lib.tt_scene_update_instances(hd, r.scene, native.ptr(inst), len(inst)))
    orc.update_instances(inst)
    r.reset_accumulation()
    c = make_constants(w.camera, w.extent, w.config, r.context.frame_index(), r.accumulated_frame_count)
    assert_same_bits(r.render_to_texture(), orc.render(c), f"power selection after update {integrator}")
    r.close()


def test_render_large_frame_and_many_chunks(gpu_context):
    """A 3840x2160 frame (8.3 M pixels, 32-bit item and pixel arithmetic at scale) and a tiny
    frame at 200 spp (four sample chunks: 64 + 64 + 64 + 8), both bit for bit."""
    big = scenes.Workload("cornell_4k", scenes.cornell_box(), scenes.cornell_workload().camera, (3840, 2160),
                          scenes.Config(bounce_count=2, sample_count=1))
    _render_pair(gpu_context, big, integrator="wavefront")
    many = scenes.Workload("cornell_200spp", scenes.cornell_box(), scenes.cornell_workload().camera, (8, 6),
                           scenes.Config(bounce_count=3, sample_count=200))
    _render_pair(gpu_context, many, integrator="wavefront")
