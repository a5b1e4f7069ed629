"""Continuous-batching render server over the C ABI (tt_server_*).

Scenes are created on the server's Context first and stay resident; `submit` queues a
request (scene, Constants, a host RGBA32F buffer the image lands in) and returns its id; the
library's scheduler thread admits requests in arrival order as room in the batch and HBM budget
free up, and renders the admitted requests together, round by round, through one shared
wavefront path pool.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native
from .native import check
from .renderer import Context, SceneArrays


class RenderServer:
    def __init__(self, context: Context, hbm_budget_bytes: int = 0, max_inflight: int = 0,
                 pool_paths: int = 0, round_items: int = 0, policy: int = native.TT_SERVER_POLICY_FAIR):
        self.context = context
        self.lib = context.lib
        cfg = native.ServerConfig(hbm_budget_bytes, max_inflight, pool_paths, round_items, policy, 0)
        h = ctypes.c_void_p()
        check(self.lib.tt_server_create(context.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        self._outputs: dict[int, np.ndarray] = {}  # keeps each request's host buffer alive

    def add_scene(self, arrays: SceneArrays) -> int:
        return self.context.create_scene(arrays)

    def submit(self, scene: int, constants: np.ndarray, out: np.ndarray | None = None) -> int:
        w, h = (int(v) for v in constants["screen_size"])
        if out is None:
            out = np.empty((h, w, 4), np.float32)
        assert out.shape == (h, w, 4) and out.dtype == np.float32 and out.flags["C_CONTIGUOUS"]
        c = np.ascontiguousarray(constants)
        rid = ctypes.c_uint64()
        check(self.lib.tt_server_submit(self.handle, scene, native.ptr(c), native.ptr(out), out.nbytes,
                                        ctypes.byref(rid)))
        self._outputs[rid.value] = out
        return rid.value

    def status(self, request: int) -> tuple[int, float]:
        st, lat = ctypes.c_int32(), ctypes.c_double()
        check(self.lib.tt_server_status(self.handle, request, ctypes.byref(st), ctypes.byref(lat)))
        return st.value, lat.value

    def wait(self, request: int, timeout_ms: int = 600_000) -> np.ndarray:
        """Blocks until the request is done; returns its image, or None once `release` dropped it
        (raises if it failed)."""
        st = ctypes.c_int32()
        check(self.lib.tt_server_wait(self.handle, request, timeout_ms, ctypes.byref(st)))
        if st.value != native.TT_REQUEST_DONE:
            raise native.TinytraceError(native.TT_ERR_DEVICE, self.lib.tt_last_error().decode())
        return self._outputs.get(request)

    def release(self, request: int) -> np.ndarray | None:
        """Drops the server's reference to a finished request's image buffer (returned)."""
        st, _ = self.status(request)
        if st < native.TT_REQUEST_DONE:
            raise native.TinytraceError(native.TT_ERR_INVALID_ARGUMENT, "the request is still queued or running")
        return self._outputs.pop(request, None)

    def stats(self) -> native.ServerStats:
        s = native.ServerStats()
        check(self.lib.tt_server_stats_get(self.handle, ctypes.byref(s)))
        return s

    def close(self) -> None:
        if self.handle:
            check(self.lib.tt_server_destroy(self.handle))
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
