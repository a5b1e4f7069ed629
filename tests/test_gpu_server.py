"""The continuous-batching server (tt_server_*) on the GPU: requests of different scenes,
acceleration structures, resolutions, sample and bounce counts rendered together through the
shared path pool, over many rounds, give each request's image exactly as tt_render gives it
alone (bit for bit); several requests are in flight at once, admission respects the HBM budget,
and bad requests fail cleanly."""
import ctypes

import numpy as np
import pytest

from conftest import assert_same_bits
from oracle import oracle
from tinytrace_gb300 import native, scenes
from tinytrace_gb300.native import check
from tinytrace_gb300.renderer import Config, Context, SceneArrays, make_constants
from tinytrace_gb300.server import RenderServer

pytestmark = pytest.mark.gpu


@pytest.fixture()
def ctx():
    from tinytrace_gb300 import build

    build.build()
    c = Context(0)
    yield c
    c.close()


def _scenes():
    field = SceneArrays(scenes.icosphere_field(instances=6, freq=8, lights=40, seed=11))
    field_cam = scenes.Camera.looking_at((0.0, 10.0, 95.0), (0, 0, 0))
    return {
        "cornell": (SceneArrays(scenes.cornell_box()), scenes.cornell_workload().camera, native.TT_ACCEL_AUTO),
        "field": (field, field_cam, native.TT_ACCEL_AUTO),
        "field_two_level": (field, field_cam, native.TT_ACCEL_TWO_LEVEL),
        "field_wide": (field, field_cam, native.TT_ACCEL_FLAT_WIDE),
        "instanced": (SceneArrays(scenes.instanced_spheres()), scenes.Camera.looking_at((0.0, 6.0, 40.0), (0, 0, 0)),
                      native.TT_ACCEL_AUTO),
    }


def _create(ctx, sc):
    handles = {}
    for name, (arrays, _, accel) in sc.items():
        check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_ACCEL, accel))
        handles[name] = ctx.create_scene(arrays)
    check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_ACCEL, native.TT_ACCEL_AUTO))
    return handles


def _requests(rng, n):
    names = ["cornell", "field", "instanced", "field_two_level", "field_wide"]
    out = []
    for k in range(n):
        w, h = int(rng.choice([40, 64, 96, 128])), int(rng.choice([24, 48, 72]))
        cfg = Config(bounce_count=int(rng.integers(2, 9)), sample_count=int(rng.integers(1, 13)))
        out.append((names[k % len(names)], (w, h), cfg, int(rng.integers(0, 50))))
    return out


def _alone(ctx, handle, constants):
    w, h = (int(v) for v in constants["screen_size"])
    img = ctx.create_image(native.TT_LIFETIME_FRAME, w, h)
    check(ctx.lib.tt_render(ctx.handle, handle, native.ptr(constants), img))
    return ctx.download(img, w, h)


@pytest.mark.parametrize("round_items,policy", [(20_000, native.TT_SERVER_POLICY_FAIR), (0, native.TT_SERVER_POLICY_FAIR),
                                               (20_000, native.TT_SERVER_POLICY_SMALLEST_FIRST)])
def test_requests_in_the_mix_equal_alone(ctx, round_items, policy):
    """round_items 20,000: every request takes several rounds of a few samples per pixel, and the
    requests that finish early are replaced by queued ones between rounds; 0: the default share
    (each request's whole sample count in one round); smallest first: requests are admitted and
    served out of arrival order, some of them left out of some rounds."""
    sc = _scenes()
    handles = _create(ctx, sc)
    rng = np.random.default_rng(21)
    reqs = _requests(rng, 15)
    consts = [make_constants(sc[name][1], ext, cfg, frame, 0) for name, ext, cfg, frame in reqs]
    alone = [_alone(ctx, handles[name], c) for (name, _, _, _), c in zip(reqs, consts)]
    with RenderServer(ctx, max_inflight=4, pool_paths=1 << 14, round_items=round_items, policy=policy) as srv:
        ids = [srv.submit(handles[name], c) for (name, _, _, _), c in zip(reqs, consts)]
        imgs = [srv.wait(i) for i in ids]
        st = srv.stats()
        lat = [srv.status(i)[1] for i in ids]
    assert st.completed == len(reqs) and st.failed == 0 and st.queued == 0 and st.inflight == 0
    assert st.peak_inflight >= 2, "requests never overlapped"
    assert all(x > 0 for x in lat)
    for k, (a, b) in enumerate(zip(alone, imgs)):
        assert_same_bits(b, a, f"request {k} {reqs[k]}")
    # and the alone renders are the oracle's
    for k in (0, 1):
        name = reqs[k][0]
        assert_same_bits(alone[k], oracle.OracleScene(sc[name][0]).render(consts[k]), f"oracle {k}")


@pytest.mark.parametrize("primary", [native.TT_PRIMARY_RASTER, native.TT_PRIMARY_TRAVERSE])
def test_flat_rounds_with_camera_keys(ctx, primary):
    """Rounds whose scenes are all flat BVH4 take camera-ray hits from per-request rasterised
    keys (TT_PRIMARY_RASTER, the context's setting when the server is created) or traverse them;
    the images are tt_render's either way, over rounds that carry several requests' chunks."""
    sc = {k: v for k, v in _scenes().items() if k in ("cornell", "field", "instanced")}
    handles = _create(ctx, sc)
    rng = np.random.default_rng(5)
    reqs = [r for r in _requests(rng, 12) if r[0] in sc]
    consts = [make_constants(sc[name][1], ext, cfg, frame, 0) for name, ext, cfg, frame in reqs]
    alone = [_alone(ctx, handles[name], c) for (name, _, _, _), c in zip(reqs, consts)]
    check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_PRIMARY_VISIBILITY, primary))
    try:
        with RenderServer(ctx, max_inflight=4, pool_paths=1 << 14, round_items=30_000) as srv:
            ids = [srv.submit(handles[name], c) for (name, _, _, _), c in zip(reqs, consts)]
            imgs = [srv.wait(i) for i in ids]
            st = srv.stats()
    finally:
        check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_PRIMARY_VISIBILITY, native.TT_PRIMARY_RASTER))
    assert st.completed == len(reqs) and st.failed == 0 and st.peak_inflight >= 2
    for k, (a, b) in enumerate(zip(alone, imgs)):
        assert_same_bits(b, a, f"request {k} {reqs[k]}")


def _arena_bytes(w, h, spp, round_items=1 << 26):
    """Mirror of the server's per-request arena (server.cu, arena_bytes): the per-sample radiance
    of the largest chunk, running sums, image, error word."""
    wh = w * h
    chunk = max(1, min(round_items // wh, 64, spp))
    return sum((s + 255) // 256 * 256 for s in (16 * chunk * wh, 16 * wh, 16 * wh)) + 256


def test_budget_admits_one_at_a_time(ctx):
    a, cam, _ = _scenes()["cornell"]
    h = ctx.create_scene(a)
    c = make_constants(cam, (64, 48), Config(bounce_count=4, sample_count=4), 0, 0)
    need = _arena_bytes(64, 48, 4)
    with RenderServer(ctx, hbm_budget_bytes=int(need * 1.5), max_inflight=4, pool_paths=4096) as srv:
        ids = [srv.submit(h, c) for _ in range(5)]
        imgs = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st.completed == 5 and st.peak_inflight == 1 and st.peak_bytes_in_flight == need
    for img in imgs[1:]:
        assert_same_bits(img, imgs[0], "same request")


def test_request_larger_than_budget_fails(ctx):
    a, cam, _ = _scenes()["cornell"]
    h = ctx.create_scene(a)
    c = make_constants(cam, (64, 48), Config(bounce_count=4, sample_count=4), 0, 0)
    assert _arena_bytes(64, 48, 4) > 1 << 16
    with RenderServer(ctx, hbm_budget_bytes=1 << 16, max_inflight=2) as srv:
        rid = srv.submit(h, c)
        st = ctypes.c_int32()
        assert ctx.lib.tt_server_wait(srv.handle, rid, 60_000, ctypes.byref(st)) == native.TT_OK
        assert st.value == native.TT_REQUEST_FAILED and b"budget" in ctx.lib.tt_last_error()
        assert srv.stats().failed == 1


def test_bad_requests(ctx):
    a, cam, _ = _scenes()["cornell"]
    h = ctx.create_scene(a)
    c = make_constants(cam, (32, 16), Config(bounce_count=2, sample_count=1), 0, 0)
    with RenderServer(ctx, max_inflight=1) as srv:
        out = np.zeros((16, 32, 4), np.float32)
        rid = ctypes.c_uint64()
        lib = ctx.lib
        assert lib.tt_server_submit(srv.handle, h, native.ptr(c), native.ptr(out), out.nbytes - 16,
                                    ctypes.byref(rid)) == native.TT_ERR_INVALID_ARGUMENT
        assert lib.tt_server_submit(srv.handle, h ^ (1 << 40), native.ptr(c), native.ptr(out), out.nbytes,
                                    ctypes.byref(rid)) == native.TT_ERR_BAD_HANDLE
        st = ctypes.c_int32()
        assert lib.tt_server_wait(srv.handle, 999_999, 10, ctypes.byref(st)) == native.TT_ERR_BAD_HANDLE
        z = c.copy()
        z["sample_count"] = 0
        assert lib.tt_server_submit(srv.handle, h, native.ptr(z), native.ptr(out), out.nbytes,
                                    ctypes.byref(rid)) == native.TT_ERR_INVALID_ARGUMENT
