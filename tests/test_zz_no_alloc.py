"""Allocation-free ray queries: tt_trace_batch_noalloc against tt_trace_batch (GPU required).

Some callers cannot allocate device memory at the moment they query rays: an application
that owns the whole device-memory budget through its own pool, or a real-time frame loop in
which an allocation's implicit device synchronisation would stall the frame.  For them the
library stages rays, hits and the traversal error word in one static device array (at most
TT_TRACE_NOALLOC_MAX_RAYS rays per call).  This file checks, through the C ABI, that the
allocation-free entry point returns exactly the hits of the allocating one (tolerance zero,
as in the other ray-query tests) on calls in a row — the shared array keeps the previous
call's contents, and a smaller call after a larger one must return only its own hits — and
that a batch above the maximum is refused before any GPU work.
"""
import numpy as np
import pytest

from tinytrace_gb300 import native, scenes
from tinytrace_gb300.native import TinytraceError, check
from tinytrace_gb300.renderer import SceneArrays

pytestmark = pytest.mark.gpu


def _rays(rng, n, targets):
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-60.0, 60.0, (n, 3))
    t = targets[rng.integers(0, len(targets), n)] + rng.normal(0.0, 3.0, (n, 3))
    d = t - rays[:, 0:3]
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 3] = 1e-3
    rays[:, 7] = 1000.0
    return rays


def _trace(ctx, fn, scene, rays, flags):
    hits = np.zeros((len(rays), 8), np.uint32)
    check(fn(ctx.handle, scene, native.ptr(rays), len(rays), flags, native.ptr(hits)))
    return hits


def test_noalloc_matches_allocating_entry_point(gpu_context):
    ctx = gpu_context
    arrays = SceneArrays(scenes.icosphere_field(instances=6, freq=8, lights=40, seed=11))
    scene = ctx.create_scene(arrays)
    targets = arrays.instances["transform"][:, 12:15]
    rng = np.random.default_rng(21)
    # calls in a row: a small batch, the largest accepted batch, then a smaller one again (the
    # shared array still holds the larger call's rays and hits beyond its n)
    for n, flags in ((5000, native.TT_TRACE_CULL_BACK_FACES), (native.TT_TRACE_NOALLOC_MAX_RAYS, 0),
                     (3001, native.TT_TRACE_CULL_BACK_FACES)):
        rays = _rays(rng, n, targets)
        expected = _trace(ctx, ctx.lib.tt_trace_batch, scene, rays, flags)
        got = _trace(ctx, ctx.lib.tt_trace_batch_noalloc, scene, rays, flags)
        assert np.array_equal(got, expected)
        assert expected[:, 0].sum() > n // 20


def test_noalloc_rejects_batches_above_the_maximum(gpu_context):
    ctx = gpu_context
    arrays = SceneArrays(scenes.cornell_box())
    scene = ctx.create_scene(arrays)
    n = native.TT_TRACE_NOALLOC_MAX_RAYS + 1
    rays = np.zeros((n, 8), np.float32)
    hits = np.zeros((n, 8), np.uint32)
    status = ctx.lib.tt_trace_batch_noalloc(ctx.handle, scene, native.ptr(rays), n, 0, native.ptr(hits))
    assert status == native.TT_ERR_INVALID_ARGUMENT
    assert b"TT_TRACE_NOALLOC_MAX_RAYS" in ctx.lib.tt_last_error()
    # the context stays usable
    ok = _trace(ctx, ctx.lib.tt_trace_batch_noalloc, scene, np.ascontiguousarray(rays[:16]), 0)
    assert ok.shape == (16, 8)
    with pytest.raises(TinytraceError):
        check(status)
