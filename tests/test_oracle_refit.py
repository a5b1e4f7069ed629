"""Instance updates on the oracle: after moving every instance and refitting (topology kept),
both world structures still find exactly the brute-force closest hits, and every child box
still lies inside its parent's slot."""
import numpy as np
import pytest

from moves import moved_instances
from oracle import oracle
from test_oracle_bvh import _rays, _scene, _walk
from tinytrace_gb300.renderer import SceneArrays


@pytest.mark.parametrize("name", ["field", "instanced", "cornell"])
def test_refit_keeps_hits_exact(name):
    arrays = SceneArrays(_scene(name))
    orc = oracle.OracleScene(arrays)
    rng = np.random.default_rng(31)
    for step in range(3):
        orc.update_instances(moved_instances(arrays.instances, rng))
        rays = _rays(rng, arrays, 4000, 1.0 if name == "cornell" else 30.0)
        for cull in (False, True):
            brute = orc.trace(rays, cull=cull, brute=True)
            assert brute[:, 0].sum() > 0
            for flat in (False, True):
                assert np.array_equal(orc.trace(rays, cull=cull, flat=flat), brute), (step, cull, flat)


def test_refit_boxes_nest():
    arrays = SceneArrays(_scene("field"))
    orc = oracle.OracleScene(arrays)
    orc.update_instances(moved_instances(arrays.instances, np.random.default_rng(4)))
    nodes, tris, levels = orc.flat_bvh()
    _walk(nodes, 0, lambda ref, box: None)
    _, _, tlas, _, _ = orc.bvh()
    _walk(tlas, 0, lambda ref, box: None)
