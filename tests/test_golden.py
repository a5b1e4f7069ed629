"""The oracle against its frozen outputs (tests/golden/oracle_golden.npz), bit for bit.

The fixtures were produced by tests/golden/make_golden.py from the same seeded inputs; a
difference means the restatement changed or the compiler/CPU changed its float results.
The reference's tests hold no known-answer vectors for this path, so these fixtures pin the
oracle itself; the GPU tests compare the CUDA path to the same files.
"""
import hashlib

import numpy as np
import pytest

from conftest import assert_same_bits, golden_constants, golden_scene
from oracle import oracle


@pytest.mark.parametrize("which", range(5))
def test_math(golden, which):
    assert_same_bits(oracle.math(which, golden[f"math{which}_x"]), golden[f"math{which}_y"], f"math {which}")


def test_bsdf(golden):
    for k, m in enumerate(golden["bsdf_materials"]):
        assert_same_bits(oracle.bsdf_eval(m, golden["bsdf_eval_in"][k]), golden["bsdf_eval_out"][k], f"eval {k}")
        assert_same_bits(oracle.bsdf_sample(m, golden["bsdf_sample_in"][k]), golden["bsdf_sample_out"][k],
                         f"sample {k}")


def test_closest_hits(golden):
    orc = oracle.OracleScene(golden_scene(golden, "field"))
    rays = golden["trace_rays"]
    for flat in (False, True):
        assert np.array_equal(orc.trace(rays, cull=False, flat=flat), golden["trace_hits"])
        assert np.array_equal(orc.trace(rays, cull=True, flat=flat), golden["trace_hits_cull"])
    assert np.array_equal(orc.trace(rays, cull=False, brute=True), golden["trace_hits"])


@pytest.mark.parametrize("name", ["cornell", "field", "instanced"])
def test_bvh_bytes(golden, name):
    orc = oracle.OracleScene(golden_scene(golden, name))
    blas, tris, tlas, bl, tl = orc.bvh()
    nodes, ftris, fl = orc.flat_bvh()
    h = lambda *arrs: hashlib.sha256(b"".join(a.tobytes() for a in arrs)).hexdigest()
    assert h(blas, tris, tlas) + f":{bl}:{tl}" == str(golden[f"bvh_{name}_two_level"])
    assert h(nodes, ftris) + f":{fl}" == str(golden[f"bvh_{name}_flat"])


@pytest.mark.parametrize("name", ["cornell", "field"])
def test_render(golden, name):
    c = golden_constants(golden, name)
    img = oracle.OracleScene(golden_scene(golden, name)).render(c)
    assert_same_bits(img, golden[f"render_{name}"], f"render {name}")
