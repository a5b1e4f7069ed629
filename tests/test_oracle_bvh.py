"""The oracle's LBVH restatement: structure invariants and closest hits (CPU only).

The closed driver BVH of the reference's ray queries has no source, so the oracle carries
a brute-force closest hit (every instance, every triangle, in object space) as ground truth
and the project's own BVH4 construction, which the GPU build must reproduce byte for byte.
These tests check that both oracle structures (two-level and flat) and the flat structure's
compressed 8-wide format find exactly the brute force's hits, and that their node arrays are
well-formed bounding hierarchies.
"""
import numpy as np
import pytest

from oracle import oracle
from tinytrace_gb300 import scenes
from tinytrace_gb300.renderer import SceneArrays

CHILD_LEAF = 0x80000000


def leaf_range(ref):
    return ref & 0x07FFFFFF, ((ref >> 27) & 0xF) + 1


def _scene(name):
    if name == "cornell":
        return scenes.cornell_box()
    if name == "field":
        return scenes.icosphere_field(instances=6, freq=8, lights=40, seed=11)
    return scenes.instanced_spheres()


def _instance_matrix(inst):
    return np.asarray(inst["transform"], np.float64).reshape(4, 4).T  # column-major storage


def _walk(nodes, root, visit_leaf, box_of_root=None):
    """Depth-first walk; checks that every child box lies inside its parent's slot."""
    stack = [(root, box_of_root, 0)]
    depth = 0
    while stack:
        i, parent_box, d = stack.pop()
        depth = max(depth, d + 1)
        nd = nodes[i]
        cnt = int(nd["count"])
        assert 1 <= cnt <= 4
        lo = nd["box"][[0, 2, 4]].T  # (4, 3)
        hi = nd["box"][[1, 3, 5]].T
        for c in range(4):
            if c >= cnt:  # empty slots never pass the slab test
                assert np.all(np.isposinf(lo[c])) and np.all(np.isneginf(hi[c]))
                continue
            assert np.all(lo[c] <= hi[c])
            if parent_box is not None:
                assert np.all(lo[c] >= parent_box[0]) and np.all(hi[c] <= parent_box[1])
            ref = int(nd["child"][c])
            if ref & CHILD_LEAF:
                visit_leaf(ref, (lo[c], hi[c]))
            else:
                stack.append((ref, (lo[c], hi[c]), d + 1))
    return depth


def _object_triangle(arrays, mesh_index, prim):
    me = arrays.meshes[mesh_index]
    idx = arrays.indices[int(me["index_offset"]) + 3 * prim: int(me["index_offset"]) + 3 * prim + 3]
    p = arrays.positions[idx.astype(np.int64) + int(me["vertex_offset"])].astype(np.float32)
    return p / np.float32(32767.0)


@pytest.mark.parametrize("name", ["cornell", "field", "instanced"])
def test_flat_bvh_structure(name):
    arrays = SceneArrays(_scene(name))
    nodes, tris, levels = oracle.OracleScene(arrays).flat_bvh()
    seen = np.zeros(len(tris), np.int32)

    def leaf(ref, box):
        first, count = leaf_range(ref)
        assert count <= 2
        seen[first:first + count] += 1
        for r in tris[first:first + count]:
            inst = arrays.instances[int(r["mesh"])]
            q = _object_triangle(arrays, int(inst["mesh_index"]), int(r["prim"]))
            assert np.array_equal(q, np.stack([r["v0"], r["v1"], r["v2"]]))
            m = _instance_matrix(inst)
            w = (m[:3, :3] @ q.astype(np.float64).T).T + m[:3, 3]
            # the world box was computed in float32; allow its rounding
            slack = 1e-5 * (1.0 + np.abs(w))
            assert np.all(w >= box[0] - slack) and np.all(w <= box[1] + slack)

    depth = _walk(nodes, 0, leaf)
    assert np.all(seen == 1), "every (instance, triangle) record sits in exactly one leaf"
    pairs = {(int(r["mesh"]), int(r["prim"])) for r in tris}
    expect = sum(int(arrays.meshes[int(i["mesh_index"])]["index_count"]) // 3 for i in arrays.instances)
    assert len(pairs) == len(tris) == expect
    assert depth <= levels


@pytest.mark.parametrize("name", ["cornell", "field", "instanced"])
def test_two_level_bvh_structure(name):
    arrays = SceneArrays(_scene(name))
    blas, tris, tlas, blas_levels, tlas_levels = oracle.OracleScene(arrays).bvh()
    # BLAS root of mesh m is node m; each mesh's triangles appear once in its own leaves
    for m, me in enumerate(arrays.meshes):
        n = int(me["index_count"]) // 3
        if n == 0:
            continue
        prims = []

        def leaf(ref, box, m=m, prims=prims):
            first, count = leaf_range(ref)
            assert count <= 2
            for r in tris[first:first + count]:
                assert int(r["mesh"]) == m
                prims.append(int(r["prim"]))
                q = np.stack([r["v0"], r["v1"], r["v2"]])
                assert np.all(q >= box[0]) and np.all(q <= box[1])

        _walk(blas, m, leaf)
        assert sorted(prims) == list(range(n))
    insts = []

    def tleaf(ref, box):
        first, count = leaf_range(ref)
        assert count == 1
        insts.append(first)

    _walk(tlas, 0, tleaf)
    assert sorted(insts) == list(range(len(arrays.instances)))


def _rays(rng, arrays, n, spread):
    centres = np.array([_instance_matrix(i)[:3, 3] for i in arrays.instances])
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = centres.mean(0) + rng.uniform(-spread, spread, (n, 3))
    target = centres[rng.integers(0, len(centres), n)] + rng.normal(0, 1.0, (n, 3))
    d = target - rays[:, 0:3]
    d[: n // 4] = rng.normal(size=(n // 4, 3))
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 3] = 1e-3
    rays[:, 7] = rng.choice([1000.0, 10000.0, 2.0], n)
    rays[:8, 4:7] = np.nan  # non-finite directions miss
    rays[8:12, 4:7] = 0.0
    return rays


@pytest.mark.parametrize("name", ["cornell", "field", "instanced"])
@pytest.mark.parametrize("cull", [False, True])
def test_closest_hit_equals_brute_force(name, cull):
    arrays = SceneArrays(_scene(name))
    orc = oracle.OracleScene(arrays)
    rng = np.random.default_rng(17)
    spread = 1.0 if name == "cornell" else 30.0
    rays = _rays(rng, arrays, 6000, spread)
    brute = orc.trace(rays, cull=cull, brute=True)
    assert brute[:, 0].sum() > len(rays) // 10
    assert not brute[:12, 0].any()
    for flat in (False, True):
        got = orc.trace(rays, cull=cull, brute=False, flat=flat)
        diff = np.any(got != brute, axis=1)
        assert not diff.any(), f"flat={flat}: {diff.sum()} rays differ"
    wide = oracle.OracleScene(arrays, wide=True).trace(rays, cull=cull, wide=True)
    assert np.array_equal(wide, brute), f"wide format: {np.any(wide != brute, axis=1).sum()} rays differ"


def _decoded(node):
    """(8, 3) low and high planes of a wide node's child slots, decoded in float64."""
    scale = np.ldexp(1.0, node["exponent"].astype(np.int64) - 127)
    org = node["origin"].astype(np.float64)
    lo = np.stack([node["qlo_x"], node["qlo_y"], node["qlo_z"]], 1).astype(np.float64) * scale + org
    hi = np.stack([node["qhi_x"], node["qhi_y"], node["qhi_z"]], 1).astype(np.float64) * scale + org
    return lo, hi


@pytest.mark.parametrize("name", ["cornell", "field", "instanced"])
def test_wide_bvh_structure(name):
    """The compressed 8-wide format of the flat BVH: every (instance, triangle) record sits in
    exactly one leaf slot (1..3 records, offsets within the node's record run), internal slots
    address nodes of the next level, decoded child boxes contain their subtrees' triangles (the
    quantisation rounds outwards) and empty slots carry inverted boxes."""
    arrays = SceneArrays(_scene(name))
    orc = oracle.OracleScene(arrays, wide=True)
    nodes, tris, levels = orc.wide_bvh()
    assert len(tris) == len(orc.flat_bvh()[1])
    seen = np.zeros(len(tris), np.int32)
    world = {}
    for k, r in enumerate(tris):
        inst = arrays.instances[int(r["mesh"])]
        m = _instance_matrix(inst)
        q = np.stack([r["v0"], r["v1"], r["v2"]]).astype(np.float64)
        world[k] = (m[:3, :3] @ q.T).T + m[:3, 3]

    def subtree_points(i):
        nd = nodes[i]
        pts = []
        rank = 0
        for s in range(8):
            internal = (int(nd["imask"]) >> s) & 1
            if internal:
                pts.append(subtree_points(int(nd["child_base"]) + rank))
                rank += 1
            elif nd["meta"][s]:
                off, units = int(nd["meta"][s]) & 31, int(nd["meta"][s]) >> 5
                for j in range(bin(units).count("1")):
                    pts.append(world[int(nd["tri_base"]) + off + j])
        return np.concatenate(pts)

    def visit(i, depth):
        nd = nodes[i]
        lo, hi = _decoded(nd)
        rank = 0
        deepest = depth
        for s in range(8):
            internal = (int(nd["imask"]) >> s) & 1
            meta = int(nd["meta"][s])
            if not internal and meta == 0:
                assert np.all(lo[s] > hi[s]), "empty slots are inverted boxes"
                continue
            if internal:
                child = int(nd["child_base"]) + rank
                rank += 1
                assert 0 < child < len(nodes)
                pts = subtree_points(child)
                deepest = max(deepest, visit(child, depth + 1))
            else:
                off, units = meta & 31, meta >> 5
                assert units in (1, 3, 7) and off + bin(units).count("1") <= 24
                pts = []
                for j in range(bin(units).count("1")):
                    seen[int(nd["tri_base"]) + off + j] += 1
                    pts.append(world[int(nd["tri_base"]) + off + j])
                pts = np.concatenate(pts)
            slack = 1e-5 * (1.0 + np.abs(pts))
            assert np.all(pts >= lo[s] - slack) and np.all(pts <= hi[s] + slack)
        return deepest

    depth = visit(0, 1)
    assert np.all(seen == 1), "every record sits in exactly one leaf slot"
    assert depth <= levels


def test_empty_interval_misses():
    """A ray interval with tmin > tmax never hits."""
    arrays = SceneArrays(scenes.cornell_box())
    orc = oracle.OracleScene(arrays)
    rays = _rays(np.random.default_rng(2), arrays, 2000, 1.0)
    rays[:, 3], rays[:, 7] = 5.0, 4.0
    assert not orc.trace(rays, cull=False, brute=True)[:, 0].any()
    assert not orc.trace(rays, cull=False, flat=True)[:, 0].any()
