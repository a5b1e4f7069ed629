"""The learned radiance cache's CUDA kernels against the NumPy reference (GPU required).

The kernels read the hash-grid features as FP16 copies of the FP32 parameters (rounded to
nearest), so the FP16 emulations below encode with the parameters rounded the same way.
Tolerances: queries and training run FP16-in / FP32-accumulate on the tensor cores, so queries
are compared with the reference's FP16 emulation within 2e-3 of the output scale, the reported
loss with the loss of that FP16 forward pass within 1e-3 relative, and the first Adam step
(which moves every parameter with a nonzero gradient by exactly the learning rate, against the
sign of its gradient) must agree in sign with the reference's float64 gradients on 98 % of the
parameters whose gradient is above 1e-4 of the largest.  The gradient values of one step
(tt_cache_gradients) are compared with a NumPy restatement of the kernel's FP16 roundings
within 5e-3 relative L2 and with the float64 gradients within 5e-2 (weights) / 1e-1 (grid)."""
import ctypes

import numpy as np
import pytest

import cache_reference as cr
from tinytrace_gb300 import native
from tinytrace_gb300.native import check

pytestmark = pytest.mark.gpu


def _configure(ctx, seed=3, lr=1e-2):
    cfg = native.CacheConfig(lr, 65536, 2, seed)
    check(ctx.lib.tt_cache_configure(ctx.handle, ctypes.byref(cfg)))


def _f16(grid):
    """The FP16 grid features the kernels read, as float64."""
    return grid.astype(np.float16).astype(np.float64)


def _params(ctx):
    grid = np.zeros(native.TT_CACHE_GRID_FLOATS, np.float32)
    w = np.zeros(native.TT_CACHE_WEIGHTS, np.float32)
    check(ctx.lib.tt_cache_parameters(ctx.handle, native.ptr(grid), native.ptr(w)))
    return grid.reshape(cr.LEVELS, cr.TABLE, 2), w


def _queries(rng, n):
    q = np.zeros((n, 12), np.float32)
    q[:, 0:3] = rng.uniform(0, 1, (n, 3))
    d = rng.normal(size=(n, 3))
    q[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    m = rng.normal(size=(n, 3))
    q[:, 6:9] = m / np.linalg.norm(m, axis=1, keepdims=True)
    q[:, 9] = rng.uniform(0, 1, n)
    return q


def _field(q):
    """A smooth synthetic radiance field to learn."""
    p, d = q[:, 0:3], q[:, 3:6]
    r = 1.0 + 0.8 * np.sin(6.0 * p[:, 0]) * np.cos(5.0 * p[:, 1]) + 0.5 * d[:, 2]
    g = 1.0 + 0.6 * np.cos(4.0 * p[:, 2] + 2.0 * d[:, 0])
    b = 0.5 + 0.4 * p[:, 1] * (1.0 + d[:, 1])
    return np.stack([r, g, b], axis=1).astype(np.float32)


def _train(ctx, q, t):
    loss = ctypes.c_float()
    check(ctx.lib.tt_cache_train(ctx.handle, native.ptr(q), native.ptr(t), len(q), ctypes.byref(loss)))
    return loss.value


def _query(ctx, q):
    out = np.zeros((len(q), 3), np.float32)
    check(ctx.lib.tt_cache_query(ctx.handle, native.ptr(q), len(q), native.ptr(out)))
    return out


def test_first_step_follows_the_reference_gradients(gpu_context):
    ctx = gpu_context
    _configure(ctx, seed=5)
    rng = np.random.default_rng(1)
    q = _queries(rng, 2048)
    t = _field(q)
    grid0, w0 = _params(ctx)
    loss = _train(ctx, q, t)
    grid1, w1 = _params(ctx)
    ref_loss, g_w, g_grid = cr.loss_and_grads(q.astype(np.float64), t.astype(np.float64), grid0.astype(np.float64),
                                              w0.astype(np.float64))
    y16, _ = cr.forward(cr.encode(q.astype(np.float64), _f16(grid0)), w0, fp16=True)
    loss16 = float((((y16 - t) ** 2) / (y16 * y16 + 0.01)).sum())
    assert abs(loss - loss16) <= 1e-3 * loss16, (loss, loss16, ref_loss)
    for before, after, g, name in ((w0, w1, g_w, "weights"), (grid0.ravel(), grid1.ravel(), g_grid.ravel(), "grid")):
        big = np.abs(g) > 1e-4 * np.abs(g).max()
        step = after.astype(np.float64) - before
        agree = np.sign(step[big]) == -np.sign(g[big])
        assert agree.mean() > 0.98, (name, agree.mean(), big.sum())
        assert np.allclose(np.abs(step[big]), 1e-2, rtol=1e-2, atol=1e-5), name


def _gradients(ctx, q, t):
    gw = np.zeros(native.TT_CACHE_WEIGHTS, np.float32)
    gg = np.zeros(native.TT_CACHE_GRID_FLOATS, np.float32)
    loss = ctypes.c_float()
    check(ctx.lib.tt_cache_gradients(ctx.handle, native.ptr(q), native.ptr(t), len(q), native.ptr(gw),
                                     native.ptr(gg), ctypes.byref(loss)))
    return loss.value, gw.astype(np.float64), gg.astype(np.float64).reshape(cr.LEVELS, cr.TABLE, 2)


def _rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("train_steps", [0, 25])
def test_gradient_values_match_the_reference(gpu_context, train_steps):
    """The values (not only the signs) of one step's weight and grid gradients, at the initial
    parameters and after 25 Adam steps, with a batch that ends in a partial tile: within 5e-3
    (relative L2) of the NumPy restatement of the kernel's FP16 roundings, and within 5e-2
    (weights) / 1e-1 (grid, four FP16 deltas deep) of the float64 gradients of the FP32 network;
    99 % of the large weight gradients within 2 % of the FP16 restatement.  The parameters are
    unchanged by the call."""
    ctx = gpu_context
    _configure(ctx, seed=13)
    rng = np.random.default_rng(4)
    for _ in range(train_steps):
        qt = _queries(rng, 4096)
        _train(ctx, qt, _field(qt))
    grid0, w0 = _params(ctx)
    q = _queries(rng, 2000)
    t = _field(q)
    loss, gw, gg = _gradients(ctx, q, t)
    grid1, w1 = _params(ctx)
    assert np.array_equal(w0, w1) and np.array_equal(grid0, grid1)
    q64, t64, grid64, w64 = q.astype(np.float64), t.astype(np.float64), grid0.astype(np.float64), w0.astype(np.float64)
    loss16, gw16, gg16 = cr.grads_fp16(q64, t64, _f16(grid0), w64)
    _, gw64, gg64 = cr.loss_and_grads(q64, t64, grid64, w64)
    assert abs(loss - loss16) <= 1e-3 * loss16, (loss, loss16)
    errs = {"weights_fp16": _rel_l2(gw, gw16), "grid_fp16": _rel_l2(gg, gg16),
            "weights_f64": _rel_l2(gw, gw64), "grid_f64": _rel_l2(gg, gg64)}
    assert errs["weights_fp16"] <= 5e-3 and errs["grid_fp16"] <= 5e-3, errs
    assert errs["weights_f64"] <= 5e-2 and errs["grid_f64"] <= 1e-1, errs
    big = np.abs(gw16) > 1e-2 * np.abs(gw16).max()
    close = np.abs(gw[big] - gw16[big]) <= 2e-2 * np.abs(gw16[big])
    assert close.mean() >= 0.99, (close.mean(), errs)
    # a second call gives the same gradients up to the order of the FP32 atomics
    loss2, gw2, _ = _gradients(ctx, q, t)
    assert _rel_l2(gw2, gw) <= 1e-5 and abs(loss2 - loss) <= 1e-5 * loss


def test_queries_match_the_reference(gpu_context):
    ctx = gpu_context
    _configure(ctx, seed=7)
    rng = np.random.default_rng(2)
    for _ in range(20):  # move the parameters away from their initial values
        qt = _queries(rng, 4096)
        _train(ctx, qt, _field(qt))
    grid, w = _params(ctx)
    q = _queries(rng, 3000)
    got = _query(ctx, q)
    x = cr.encode(q.astype(np.float64), _f16(grid))
    want16, _ = cr.forward(x, w, fp16=True)
    want32, _ = cr.forward(cr.encode(q.astype(np.float64), grid.astype(np.float64)), w, fp16=False)
    scale = np.abs(want32).max()
    assert scale > 0.1
    assert np.abs(got - want16).max() <= 2e-3 * scale + 1e-4, np.abs(got - want16).max() / scale
    assert np.abs(got - want32).max() <= 2e-2 * scale


def test_learns_a_smooth_field(gpu_context):
    ctx = gpu_context
    _configure(ctx, seed=11)
    rng = np.random.default_rng(3)
    first = None
    for step in range(300):
        q = _queries(rng, 8192)
        loss = _train(ctx, q, _field(q)) / (3 * len(q))
        first = loss if first is None else first
    assert loss < first / 10, (first, loss)
    q = _queries(rng, 4096)
    err = np.abs(_query(ctx, q) - _field(q)).mean() / np.abs(_field(q)).mean()
    assert err < 0.1, err


def _cache_renderer(extent=(96, 54), spp=8, depth=6, terminate=2, train_paths=4096, spread=0.0, scene=None,
                    camera=None):
    from tinytrace_gb300 import scenes
    from tinytrace_gb300.renderer import Config, Renderer

    w = scenes.Workload("field_small", scene or scenes.icosphere_field(instances=6, freq=8, lights=40, seed=11),
                        camera or scenes.Camera.looking_at((0.0, 10.0, 95.0), (0, 0, 0)), extent,
                        Config(bounce_count=depth, sample_count=spp))
    r = Renderer(w.extent)
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(w.config)
    cfg = native.CacheConfig(1e-2, train_paths, terminate, 1, spread)
    check(r.context.lib.tt_cache_configure(r.context.handle, ctypes.byref(cfg)))
    return r, w


def test_cache_plumbing_leaves_the_estimator_alone(gpu_context):
    """With the cache vertex beyond the last bounce no path ends in the cache, so the image is
    the plain path tracer's bit for bit (training paths only record their vertices)."""
    from conftest import assert_same_bits
    from oracle import oracle
    from tinytrace_gb300.renderer import make_constants

    r, w = _cache_renderer(terminate=6)
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_RADIANCE_CACHE, 1))
    c = make_constants(w.camera, w.extent, w.config, r.context.frame_index(), r.accumulated_frame_count)
    img = r.render_to_texture()
    assert_same_bits(img, oracle.OracleScene(r.scene_arrays).render(c), "cache beyond the last bounce")
    st = native.CacheStatus()
    check(r.context.lib.tt_cache_status_get(r.context.handle, ctypes.byref(st)))
    assert st.pairs > 0 and st.steps >= 1
    r.close()


def test_cached_render_trains_and_stays_close(gpu_context):
    """Paths ending in the cache at the third vertex: after online training the frame mean is
    within 15 % of the plain path tracer's and the training loss has dropped."""
    r, w = _cache_renderer(spp=16, train_paths=16384)
    plain = r.render_to_texture()
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_RADIANCE_CACHE, 1))
    losses = []
    for f in range(24):
        r.reset_accumulation()
        img = r.render_to_texture()
        st = native.CacheStatus()
        check(r.context.lib.tt_cache_status_get(r.context.handle, ctypes.byref(st)))
        losses.append(st.last_loss)
        r.present()
    assert np.isfinite(img).all() and st.pairs > 200
    assert np.mean(losses[-4:]) < np.mean(losses[:4])
    a, b = img[..., :3].mean(), plain[..., :3].mean()
    assert abs(a - b) <= 0.15 * b, (a, b)
    r.close()


def test_spread_rule_without_termination_is_the_plain_tracer(gpu_context):
    """With the path-spread rule and a threshold no path reaches, no path ends in the cache:
    the image is the plain path tracer's bit for bit."""
    from conftest import assert_same_bits
    from oracle import oracle
    from tinytrace_gb300.renderer import make_constants

    r, w = _cache_renderer(terminate=1, spread=1e30)
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_RADIANCE_CACHE, 1))
    c = make_constants(w.camera, w.extent, w.config, r.context.frame_index(), r.accumulated_frame_count)
    assert_same_bits(r.render_to_texture(), oracle.OracleScene(r.scene_arrays).render(c), "spread rule, no ending")
    r.close()


def test_spread_rule_in_a_closed_room(gpu_context):
    """The path-spread rule in the textured Cornell box (every path bounces to full depth):
    after online training the frame mean is within 10 % of the plain tracer's and the cached
    frames are faster."""
    import time

    from tinytrace_gb300 import scenes

    cam = scenes.Camera.looking_at((0.0, 1.0, 3.4), (0.0, 1.0, 0.0), fov=0.75)
    r, w = _cache_renderer(extent=(256, 192), spp=16, depth=8, terminate=1, train_paths=16384, spread=0.01,
                           scene=scenes.textured_cornell(), camera=cam)
    plain = np.zeros((192, 256, 3))
    for f in range(4):
        r.reset_accumulation()
        plain += r.render_to_texture()[..., :3] / 4
        r.present()
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_RADIANCE_CACHE, 1))
    for f in range(32):
        r.reset_accumulation()
        img = r.render_to_texture()
        r.present()
    st = native.CacheStatus()
    check(r.context.lib.tt_cache_status_get(r.context.handle, ctypes.byref(st)))
    assert np.isfinite(img).all() and st.pairs > 1000 and st.steps >= 32
    a, b = img[..., :3].mean(), plain.mean()
    assert abs(a - b) <= 0.10 * b, (a, b)
    r.close()


def test_large_query_batch(gpu_context):
    """2^20 queries (8,192 tiles of 128 over many CTAs per SM): a sample of rows matches the
    reference's FP16 emulation as in test_queries_match_the_reference."""
    ctx = gpu_context
    _configure(ctx, seed=13)
    rng = np.random.default_rng(5)
    for _ in range(5):
        qt = _queries(rng, 4096)
        _train(ctx, qt, _field(qt))
    grid, w = _params(ctx)
    q = _queries(rng, 1 << 20)
    got = _query(ctx, q)
    assert np.isfinite(got).all()
    pick = rng.choice(len(q), 2000, replace=False)
    x = cr.encode(q[pick].astype(np.float64), _f16(grid))
    want16, _ = cr.forward(x, w, fp16=True)
    scale = np.abs(want16).max()
    assert np.abs(got[pick] - want16).max() <= 2e-3 * scale + 1e-4
