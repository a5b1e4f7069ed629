"""Converged-image error against a float64 render (oracle/fp64_cornell.py, an independent
sampler of the same estimator) for the Cornell box at 64x64, depth 4: the fixture is the
float64 render at 4096 spp (tests/golden/make_fp64_cornell.py).  The FP32 path (the oracle on
the CPU here; the CUDA path is bit-identical to it, test_gpu_fp64_reference.py) converges to it:
its 4032-spp accumulation has no per-channel bias beyond 0.5 % and an RMSE at the noise level
of the two estimates, and its 16-spp frame's RMSE is stated."""
from pathlib import Path

import numpy as np
import pytest

from oracle import fp64_cornell, oracle
from tinytrace_gb300 import scenes
from tinytrace_gb300.renderer import SceneArrays, make_constants

FIXTURE = Path(__file__).resolve().parent / "golden" / "cornell_fp64_64x64.npz"


def _fixture():
    if not FIXTURE.exists():
        pytest.skip("float64 fixture not generated")
    return np.load(FIXTURE)["image"]


def accumulated_fp32(render_frame, frames=64, spp=64):
    """Frames 0..frames-1 accumulated as the reference does (frames 0 and 1 both overwrite)."""
    w = scenes.cornell_workload(extent=(64, 64), spp=spp, depth=4)
    img = None
    for f in range(frames):
        img = render_frame(w, make_constants(w.camera, w.extent, w.config, f, f), img)
    return img[..., :3].astype(np.float64)


def test_fp64_tracer_agrees_with_the_fp32_oracle_in_the_mean():
    w = scenes.cornell_workload(extent=(16, 16), spp=128, depth=4)
    a = SceneArrays(w.scene)
    c = make_constants(w.camera, w.extent, w.config, 0, 0)
    f64 = fp64_cornell.render(a, c, 512, seed=3)
    f32 = oracle.OracleScene(a).render(c)[..., :3].astype(np.float64)
    assert np.all(np.abs(f64.mean(axis=(0, 1)) - f32.mean(axis=(0, 1))) < 0.02 * f32.mean(axis=(0, 1)))


def test_fp32_converges_to_the_fp64_render():
    ref = _fixture()
    o = None

    def frame(w, c, img):
        nonlocal o
        if o is None:
            o = oracle.OracleScene(SceneArrays(w.scene))
        img = np.zeros((64, 64, 4), np.float32) if img is None else img
        o.render(c, img)
        return img

    acc = accumulated_fp32(frame)
    bias = np.abs(acc.mean(axis=(0, 1)) - ref.mean(axis=(0, 1))) / ref.mean(axis=(0, 1))
    rmse = float(np.sqrt(np.mean((acc - ref) ** 2)))
    assert bias.max() < 0.005, bias
    assert rmse < 0.03, rmse
