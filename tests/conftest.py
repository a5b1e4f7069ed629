import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on GB300)")


def assert_same_bits(a, b, what=""):
    """Exact equality of float arrays bit for bit, except that any NaN equals any NaN
    (x86-64 and CUDA produce different NaN payloads)."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    assert a.shape == b.shape, (a.shape, b.shape)
    both_nan = np.isnan(a) & np.isnan(b)
    same = (a.view(np.uint32) == b.view(np.uint32)) | both_nan
    if not same.all():
        idx = np.argwhere(~same)
        first = tuple(idx[0])
        raise AssertionError(f"{what}: {len(idx)} of {a.size} values differ; first at {first}: "
                             f"{a[first]!r} vs {b[first]!r}")


@pytest.fixture(scope="session")
def gpu_context():
    from tinytrace_gb300 import build as cuda_build

    cuda_build.build()
    from tinytrace_gb300.renderer import Context

    ctx = Context(0)
    yield ctx
    ctx.close()


GOLDEN = ROOT / "tests" / "golden" / "oracle_golden.npz"


@pytest.fixture(scope="session")
def golden():
    """Frozen oracle inputs and outputs (tests/golden/make_golden.py)."""
    with np.load(GOLDEN, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def golden_scene(golden, name):
    from tinytrace_gb300.renderer import SceneArrays

    return SceneArrays.from_arrays(golden, prefix=f"scene_{name}_")


def golden_constants(golden, name):
    from tinytrace_gb300 import native

    return np.frombuffer(golden[f"render_{name}_constants"].tobytes(), native.CONSTANTS_DTYPE).reshape(()).copy()
