"""The CUDA path against the frozen oracle fixtures (tests/golden/oracle_golden.npz), bit for
bit, through the C ABI (GPU required).  Unlike the live-oracle comparisons these need no
oracle build on the GPU host, and the inputs (scene arrays, rays, constants) come from the
fixture file rather than from the generators."""
import hashlib

import numpy as np
import pytest

from conftest import assert_same_bits, golden_constants, golden_scene
from tinytrace_gb300 import native
from tinytrace_gb300.native import NODE4_DTYPE, TRI_RECORD_DTYPE, check

pytestmark = pytest.mark.gpu

ACCELS = {"flat": native.TT_ACCEL_FLAT, "two_level": native.TT_ACCEL_TWO_LEVEL}


def _scene(ctx, golden, name, accel):
    check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_ACCEL, ACCELS[accel]))
    try:
        return ctx.create_scene(golden_scene(golden, name))
    finally:
        check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_ACCEL, native.TT_ACCEL_AUTO))


@pytest.mark.parametrize("which", range(5))
def test_math(gpu_context, golden, which):
    x = golden[f"math{which}_x"]
    y = np.zeros_like(x)
    check(gpu_context.lib.tt_math_batch(gpu_context.handle, which, native.ptr(x), x.size, native.ptr(y)))
    assert_same_bits(y, golden[f"math{which}_y"], f"math {which}")


def test_bsdf(gpu_context, golden):
    lib, h = gpu_context.lib, gpu_context.handle
    for k, m in enumerate(golden["bsdf_materials"]):
        m = np.ascontiguousarray(m)
        s = np.ascontiguousarray(golden["bsdf_eval_in"][k])
        out = np.zeros((len(s), 8), np.float32)
        check(lib.tt_bsdf_eval_batch(h, native.ptr(m), native.ptr(s), len(s), native.ptr(out)))
        assert_same_bits(out, golden["bsdf_eval_out"][k], f"eval {k}")
        s = np.ascontiguousarray(golden["bsdf_sample_in"][k])
        out = np.zeros((len(s), 12), np.float32)
        check(lib.tt_bsdf_sample_batch(h, native.ptr(m), native.ptr(s), len(s), native.ptr(out)))
        assert_same_bits(out, golden["bsdf_sample_out"][k], f"sample {k}")


@pytest.mark.parametrize("accel", ["flat", "two_level"])
def test_closest_hits(gpu_context, golden, accel):
    h = _scene(gpu_context, golden, "field", accel)
    rays = np.ascontiguousarray(golden["trace_rays"])
    for cull, key in ((0, "trace_hits"), (1, "trace_hits_cull")):
        hits = np.zeros((len(rays), 8), np.uint32)
        check(gpu_context.lib.tt_trace_batch(gpu_context.handle, h, native.ptr(rays), len(rays), cull,
                                             native.ptr(hits)))
        assert np.array_equal(hits, golden[key]), f"cull={cull}"


@pytest.mark.parametrize("accel", ["flat", "two_level"])
@pytest.mark.parametrize("name", ["cornell", "field", "instanced"])
def test_bvh_bytes(gpu_context, golden, name, accel):
    ctx = gpu_context
    h = _scene(ctx, golden, name, accel)
    st = ctx.scene_stats(h)
    blas = np.zeros(st.blas_nodes, NODE4_DTYPE)
    tris = np.zeros(st.triangle_count, TRI_RECORD_DTYPE)
    tlas = np.zeros(st.tlas_nodes, NODE4_DTYPE)
    check(ctx.lib.tt_scene_bvh_download(ctx.handle, h, native.ptr(blas), blas.nbytes, native.ptr(tris),
                                        tris.nbytes, native.ptr(tlas), tlas.nbytes))
    digest = lambda *arrs: hashlib.sha256(b"".join(a.tobytes() for a in arrs)).hexdigest()
    if accel == "flat":
        assert digest(tlas, tris) + f":{st.tlas_levels}" == str(golden[f"bvh_{name}_flat"])
    else:
        got = digest(blas, tris, tlas) + f":{st.blas_levels}:{st.tlas_levels}"
        assert got == str(golden[f"bvh_{name}_two_level"])


@pytest.mark.parametrize("integrator", ["wavefront", "megakernel"])
@pytest.mark.parametrize("name", ["cornell", "field"])
def test_render(gpu_context, golden, name, integrator):
    ctx = gpu_context
    integ = native.TT_INTEGRATOR_WAVEFRONT if integrator == "wavefront" else native.TT_INTEGRATOR_MEGAKERNEL
    check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_INTEGRATOR, integ))
    try:
        scene = _scene(ctx, golden, name, "flat")
        c = golden_constants(golden, name)
        w, hgt = (int(v) for v in c["screen_size"])
        img = ctx.create_image(native.TT_LIFETIME_FRAME, w, hgt)
        check(ctx.lib.tt_render(ctx.handle, scene, native.ptr(c), img))
        assert_same_bits(ctx.download(img, w, hgt), golden[f"render_{name}"], f"render {name}")
    finally:
        check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_INTEGRATOR, native.TT_INTEGRATOR_WAVEFRONT))
