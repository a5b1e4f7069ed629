"""Accuracy of the oracle's elementary functions against float64 numpy (CPU only).

The path tracer uses its own sin/cos/exp/log/acos (Cody-Waite reduction plus polynomials)
on both the CPU oracle and the GPU, so that the two agree bit for bit.  These tests pin the
functions themselves to the mathematics: at most 2 ulp from the correctly rounded value on
the ranges the shaders use, and exact special values.
"""
import numpy as np
import pytest

from oracle import oracle

FUNCS = {
    0: ("sin", np.sin, (-100.0, 100.0)),
    1: ("cos", np.cos, (-100.0, 100.0)),
    2: ("exp", np.exp, (-87.0, 88.0)),
    4: ("acos", np.arccos, (-1.0, 1.0)),
}


def ulp_error(y: np.ndarray, ref: np.ndarray) -> np.ndarray:
    spacing = np.spacing(np.abs(ref.astype(np.float32))).astype(np.float64)
    return np.abs(y.astype(np.float64) - ref) / spacing


@pytest.mark.parametrize("which", sorted(FUNCS))
def test_ulp_bound(which):
    name, f, (lo, hi) = FUNCS[which]
    rng = np.random.default_rng(which)
    x = rng.uniform(lo, hi, 300000).astype(np.float32)
    err = ulp_error(oracle.math(which, x), f(x.astype(np.float64)))
    assert err.max() <= 2.0, f"{name}: {err.max():.3f} ulp"


def test_log_ulp_bound():
    rng = np.random.default_rng(7)
    x = np.exp(rng.uniform(-80, 80, 300000)).astype(np.float32)
    x = np.concatenate([x, np.float32(1.0) + rng.uniform(-1e-3, 1e-3, 10000).astype(np.float32)])
    y = oracle.math(3, x)
    ref = np.log(x.astype(np.float64))
    # near x = 1 the result is tiny: bound the absolute error by one ulp of the argument instead
    far = np.abs(x - 1) > 1e-2
    assert ulp_error(y[far], ref[far]).max() <= 2.0
    assert np.abs(y[~far] - ref[~far]).max() <= 2.0 * np.spacing(np.float32(1.0))


def test_special_values():
    s = oracle.math(0, np.array([0.0, -0.0], np.float32))
    assert s[0] == 0.0 and s[1] == 0.0  # the sign of sin(-0) is not specified (GLSL gives no guarantee)
    assert oracle.math(1, np.array([0.0], np.float32))[0] == 1.0
    assert oracle.math(2, np.array([0.0], np.float32))[0] == 1.0
    assert oracle.math(3, np.array([1.0], np.float32))[0] == 0.0
    a = oracle.math(4, np.array([1.0, -1.0, 0.0], np.float32))
    assert a[0] == 0.0
    assert abs(a[1] - np.pi) <= np.spacing(np.float32(np.pi))
    assert abs(a[2] - np.pi / 2) <= np.spacing(np.float32(np.pi / 2))
    e = oracle.math(2, np.array([-200.0, 200.0], np.float32))
    assert e[0] == 0.0 and np.isinf(e[1])


def test_periodicity():
    # sin(x) and sin(x + 2 pi k) agree to the accuracy of the reduced argument
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 1, 10000).astype(np.float32)
    for k in (1, 5, 12):
        shifted = (x.astype(np.float64) + 2 * np.pi * k).astype(np.float32)
        a = oracle.math(0, shifted)
        b = np.sin(shifted.astype(np.float64))
        assert np.abs(a - b).max() < 2e-7
