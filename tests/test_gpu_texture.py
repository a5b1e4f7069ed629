"""Textured materials on the GPU against the oracle, bit for bit: texel decoding and
trilinear filtering of every format (tt_texture_sample_batch), and renders of the textured
Cornell box (BC1 colour, BC5 normal map, R8 roughness / metalness, R16F and BC1 emission) by
the wavefront integrator (graph and host loops), the megakernel and the server (ReSTIR's
textured frames are in test_gpu_restir); scenes with malformed textures are rejected."""
import ctypes

import numpy as np
import pytest

from conftest import assert_same_bits
from oracle import oracle
from tinytrace_gb300 import native, scenes
from tinytrace_gb300.native import TinytraceError, check
from tinytrace_gb300.renderer import Config, LightSampling, Renderer, SceneArrays, make_constants
from tinytrace_gb300.server import RenderServer

pytestmark = pytest.mark.gpu

CAMERA = scenes.Camera.looking_at((0.0, 1.0, 3.4), (0.0, 1.0, 0.0), fov=0.75)


def test_texture_sampling_bits(gpu_context):
    ctx = gpu_context
    arrays = SceneArrays(scenes.textured_cornell())
    h = ctx.create_scene(arrays)
    orc = oracle.OracleScene(SceneArrays.from_arrays(arrays.save(None)), use_bvh=False)
    rng = np.random.default_rng(4)
    n = 20000
    uvl = np.stack([rng.uniform(-3, 3, n), rng.uniform(-3, 3, n), rng.uniform(-1, 10, n)], -1).astype(np.float32)
    uvl[:10, 2] = [np.nan, np.inf, -np.inf, 0.0, 1.0, 2.0, 3.0, 0.5, 1e9, -1e9]
    uvl[10:14, :2] = [[np.nan, 0.5], [np.inf, 0.2], [1e20, -1e20], [0.0, 1.0]]
    for t in range(len(arrays.texture_info)):
        out = np.zeros((n, 4), np.float32)
        check(ctx.lib.tt_texture_sample_batch(ctx.handle, h, t, native.ptr(uvl), n, native.ptr(out)))
        assert_same_bits(out, orc.texture_sample(t, uvl), f"texture {t} format {arrays.texture_info[t, 0]}")


def _workload(extent=(64, 48), spp=4, depth=5, sampling=LightSampling.NEXT_EVENT_ESTIMATION):
    return scenes.Workload("textured_cornell", scenes.textured_cornell(), CAMERA, extent,
                           Config(bounce_count=depth, sample_count=spp, light_sampling=sampling))


@pytest.mark.parametrize("mode", ["graph", "host_loop", "megakernel", "on_hit"])
def test_textured_render_bits(gpu_context, mode):
    w = _workload(sampling=LightSampling.ON_HIT if mode == "on_hit" else LightSampling.NEXT_EVENT_ESTIMATION)
    r = Renderer(w.extent)
    lib, hd = r.context.lib, r.context.handle
    if mode == "megakernel":
        check(lib.tt_set_option(hd, native.TT_OPTION_INTEGRATOR, native.TT_INTEGRATOR_MEGAKERNEL))
    if mode == "host_loop":
        check(lib.tt_set_option(hd, native.TT_OPTION_GRAPHS, 0))
        check(lib.tt_set_option(hd, native.TT_OPTION_WAVEFRONT_SLOTS, 512))
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(w.config)
    orc = oracle.OracleScene(r.scene_arrays)
    cpu = np.zeros((w.extent[1], w.extent[0], 4), np.float32)
    for f in range(2):
        c = make_constants(w.camera, w.extent, w.config, r.context.frame_index(), r.accumulated_frame_count)
        gpu = r.render_to_texture()
        orc.render(c, cpu)
        assert_same_bits(gpu, cpu, f"textured {mode} frame {f}")
        r.present()
    assert gpu[..., :3].mean() > 0.02
    r.close()


def test_textured_server_request(gpu_context):
    """A textured and an untextured request rendered in the same rounds (the batch then shades
    with texture sampling on for both)."""
    ctx = gpu_context
    arrays = SceneArrays(scenes.textured_cornell())
    h = ctx.create_scene(arrays)
    plain = SceneArrays(scenes.cornell_box())
    hp = ctx.create_scene(plain)
    c = make_constants(CAMERA, (40, 32), Config(bounce_count=4, sample_count=3), 3, 0)
    cp = make_constants(scenes.cornell_workload().camera, (48, 24), Config(bounce_count=3, sample_count=5), 1, 0)
    with RenderServer(ctx, max_inflight=2, pool_paths=1 << 12, round_items=2000) as srv:
        ids = [srv.submit(h, c), srv.submit(hp, cp)]
        img, img_plain = (srv.wait(i) for i in ids)
        assert srv.stats().peak_inflight == 2
    assert_same_bits(img, oracle.OracleScene(SceneArrays.from_arrays(arrays.save(None))).render(c), "server")
    assert_same_bits(img_plain, oracle.OracleScene(plain).render(cp), "untextured in the textured batch")


def test_textured_scene_rejects(gpu_context):
    ctx = gpu_context
    good = SceneArrays(scenes.textured_cornell())

    def create(mutate):
        a = SceneArrays.from_arrays(good.save(None))
        a.materials = a.materials.copy()
        a.texture_info = a.texture_info.copy()
        mutate(a)
        with pytest.raises(TinytraceError) as e:
            ctx.create_scene(a)
        return e.value.code

    def bad_index(a):
        a.materials["textures"][1, 0] = 6

    def bad_bytes(a):
        a.texture_info[0, 4] -= 8
        a.texture_data = a.texture_data[:-8].copy()

    def bad_levels(a):
        a.texture_info[3, 3] = 7  # 22 x 38 has 5 levels

    def bad_format(a):
        a.texture_info[2, 0] = 9

    for m in (bad_index, bad_bytes, bad_levels, bad_format):
        assert create(m) == native.TT_ERR_INVALID_ARGUMENT, m.__name__
    ctx.create_scene(good)  # the context still works
