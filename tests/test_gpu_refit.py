"""Instance updates on the GPU (tt_scene_update_instances) against the oracle: after moving the
instances, the refitted world structure (the rebuilt one for the compressed wide format) is
byte-identical to the oracle's, closest hits equal brute force, and renders equal the oracle's."""
import numpy as np
import pytest

from conftest import assert_same_bits
from moves import moved_instances
from oracle import oracle
from test_oracle_bvh import _rays
from tinytrace_gb300 import native, scenes
from tinytrace_gb300.native import NODE4_DTYPE, TRI_RECORD_DTYPE, check
from tinytrace_gb300.renderer import Renderer, SceneArrays, make_constants

pytestmark = pytest.mark.gpu

ACCELS = {"flat": native.TT_ACCEL_FLAT, "two_level": native.TT_ACCEL_TWO_LEVEL, "wide": native.TT_ACCEL_FLAT_WIDE}


def _download(ctx, h):
    st = ctx.scene_stats(h)
    blas = np.zeros(st.blas_nodes, NODE4_DTYPE)
    tris = np.zeros(st.triangle_count, TRI_RECORD_DTYPE)
    tlas = np.zeros(st.tlas_nodes, native.NODE8_DTYPE if st.accel == native.TT_ACCEL_FLAT_WIDE else NODE4_DTYPE)
    check(ctx.lib.tt_scene_bvh_download(ctx.handle, h, native.ptr(blas), blas.nbytes, native.ptr(tris), tris.nbytes,
                                        native.ptr(tlas), tlas.nbytes))
    return tlas


@pytest.mark.parametrize("accel", ["flat", "two_level", "wide"])
def test_update_refits_like_the_oracle(gpu_context, accel):
    ctx = gpu_context
    arrays = SceneArrays(scenes.icosphere_field(instances=6, freq=8, lights=40, seed=11))
    check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_ACCEL, ACCELS[accel]))
    try:
        h = ctx.create_scene(arrays)
    finally:
        check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_ACCEL, native.TT_ACCEL_AUTO))
    orc = oracle.OracleScene(SceneArrays.from_arrays(arrays.save(None)), wide=accel == "wide")
    rng = np.random.default_rng(8)
    for step in range(3):
        moved = moved_instances(arrays.instances, rng)
        check(ctx.lib.tt_scene_update_instances(ctx.handle, h, native.ptr(moved), len(moved)))
        orc.update_instances(moved)
        got = _download(ctx, h)
        want = {"flat": lambda: orc.flat_bvh()[0], "wide": lambda: orc.wide_bvh()[0],
                "two_level": lambda: orc.bvh()[2]}[accel]()
        assert got.tobytes() == want.tobytes(), f"step {step}: refitted nodes differ"
        rays = _rays(rng, orc.arrays, 6000, 30.0)
        hits = np.zeros((len(rays), 8), np.uint32)
        check(ctx.lib.tt_trace_batch(ctx.handle, h, native.ptr(rays), len(rays), 0, native.ptr(hits)))
        assert np.array_equal(hits, orc.trace(rays, cull=False, brute=True)), f"step {step}: hits differ"


def test_update_then_render(gpu_context):
    w = scenes.Workload("field_small", scenes.icosphere_field(instances=6, freq=8, lights=40, seed=11),
                        scenes.Camera.looking_at((0.0, 10.0, 95.0), (0, 0, 0)), (96, 54),
                        scenes.Config(bounce_count=6, sample_count=2))
    r = Renderer(w.extent)
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(w.config)
    moved = moved_instances(r.scene_arrays.instances, np.random.default_rng(5), max_shift=8.0)
    check(r.context.lib.tt_scene_update_instances(r.context.handle, r.scene, native.ptr(moved), len(moved)))
    orc = oracle.OracleScene(SceneArrays.from_arrays(r.scene_arrays.save(None)))
    orc.update_instances(moved)
    c = make_constants(w.camera, w.extent, w.config, r.context.frame_index(), r.accumulated_frame_count)
    assert_same_bits(r.render_to_texture(), orc.render(c), "render after update")
    bad = moved.copy()
    bad["mesh_index"][0] ^= 1
    assert r.context.lib.tt_scene_update_instances(r.context.handle, r.scene, native.ptr(bad), len(bad)) == \
        native.TT_ERR_INVALID_ARGUMENT
    r.close()
