"""The CUDA path's converged image against the float64 render of the Cornell box (see
test_fp64_reference.py): 64 accumulated frames of 64 spp on the GPU, no per-channel bias
beyond 0.5 %, RMSE at the noise level; and the RMSE of a single 16-spp frame (C1's sample
count) is reported in the assertion message."""
import numpy as np
import pytest

from test_fp64_reference import _fixture, accumulated_fp32
from tinytrace_gb300 import native, scenes
from tinytrace_gb300.native import check
from tinytrace_gb300.renderer import make_constants

pytestmark = pytest.mark.gpu


def test_gpu_converges_to_the_fp64_render(gpu_context):
    ref = _fixture()
    ctx = gpu_context
    state = {}

    def frame(w, c, img):
        if "scene" not in state:
            from tinytrace_gb300.renderer import SceneArrays

            state["scene"] = ctx.create_scene(SceneArrays(w.scene))
            state["target"] = ctx.create_image(native.TT_LIFETIME_FRAME, 64, 64)
        check(ctx.lib.tt_render(ctx.handle, state["scene"], native.ptr(c), state["target"]))
        return ctx.download(state["target"], 64, 64)

    acc = accumulated_fp32(frame)
    bias = np.abs(acc.mean(axis=(0, 1)) - ref.mean(axis=(0, 1))) / ref.mean(axis=(0, 1))
    rmse = float(np.sqrt(np.mean((acc - ref) ** 2)))
    assert bias.max() < 0.005 and rmse < 0.03, (bias, rmse)
    w = scenes.cornell_workload(extent=(64, 64), spp=16, depth=4)
    one = frame(w, make_constants(w.camera, w.extent, w.config, 0, 0), None)[..., :3].astype(np.float64)
    rmse16 = float(np.sqrt(np.mean((one - ref) ** 2)))
    assert rmse16 < 0.3, rmse16
