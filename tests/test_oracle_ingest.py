"""The oracle's restatement of Scene::insert_mesh (src/asset/mod.rs:89-161) and
emissive_triangles_in_model (src/asset/mod.rs:163-193), pinned on the CPU:

* tatan2 (the atan2 of the tangent-frame angle) against numpy's float64 atan2;
* the f32 -> f16 rounding against numpy's float16 cast over normal, subnormal, overflowing
  and tie values;
* a hand-derived TangentFrame and the running-mean bounding sphere;
* generated normals against a sequential float32 restatement of generate_normals;
* agreement with the package's host-side asset path (which uses a float64 mean, so positions
  may differ by one snorm16 step) and with its emissive triangles, bit for bit;
* the cases on which the reference panics are rejected.
"""
import numpy as np
import pytest

from oracle import oracle
from tinytrace_gb300 import asset, scenes
from tinytrace_gb300.asset import Material, Model, Node


def test_atan2_accuracy():
    rng = np.random.default_rng(1)
    y = (rng.standard_normal(200000) * np.exp(rng.uniform(-8, 8, 200000))).astype(np.float32)
    x = (rng.standard_normal(200000) * np.exp(rng.uniform(-8, 8, 200000))).astype(np.float32)
    got = oracle.atan2(y, x).astype(np.float64)
    want = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert np.abs(got - want).max() < 4e-7  # a few float ulps of pi


def test_atan2_special_values():
    v = np.array([0.0, -0.0, 1.0, -1.0, 3.5, np.inf, -np.inf], np.float32)
    y, x = (a.ravel() for a in np.meshgrid(v, v))
    got = oracle.atan2(y, x)
    want = np.arctan2(y, x)
    assert np.array_equal(np.signbit(got), np.signbit(want))
    assert np.abs(got.astype(np.float64) - want).max() < 3e-7
    assert np.isnan(oracle.atan2(np.float32([np.nan, 1.0]), np.float32([1.0, np.nan]))).all()


def test_half_rounding_matches_numpy():
    rng = np.random.default_rng(2)
    vals = np.concatenate([
        rng.uniform(-1, 1, 5000), rng.uniform(-70000, 70000, 5000),
        rng.uniform(-1e-4, 1e-4, 5000),  # subnormal halves
        np.float32([65504, 65519.99, 65520, 1e9, -1e9, 2.0 ** -25, 2.0 ** -24, 3 * 2.0 ** -26, 0.0, -0.0]),
        # exact ties between two halves: 1 + (2k + 1) 2^-11
        1.0 + (2 * np.arange(64) + 1) * 2.0 ** -11,
    ]).astype(np.float32)
    n = len(vals) // 2 * 2
    uv = vals[:n].reshape(-1, 2)
    p = np.random.default_rng(3).standard_normal((len(uv), 3)).astype(np.float32)
    _, v, _ = oracle.mesh_ingest(p, uv, normals=np.tile([0, 0, 1], (len(uv), 1)))
    with np.errstate(over="ignore"):
        want = uv.astype(np.float16).view(np.uint16)
    assert np.array_equal(v["texture_coordinates"].view(np.uint16), want)


def test_tangent_frame_known_answer():
    # n = +z, t = +x: octahedral (0.5, 0.5) -> 512, 512; the decoded normal picks
    # orthonormal (0, -z, y), so the tangent sits a quarter turn around n: 0.25 * 2047 -> 512.
    p = np.float32([[1, 0, 0], [0, 1, 0], [0, 0, 1]])
    _, v, _ = oracle.mesh_ingest(p, normals=np.tile([0, 0, 1], (3, 1)), tangents=np.tile([1, 0, 0, 1], (3, 1)))
    assert (v["tangent_frame"] == np.uint32(1 << 31 | 512 << 20 | 512 << 10 | 512)).all()
    _, v, _ = oracle.mesh_ingest(p, normals=np.tile([0, 0, 1], (3, 1)), tangents=np.tile([1, 0, 0, -1], (3, 1)))
    assert (v["tangent_frame"] >> 31 == 0).all()


def test_running_mean_sphere():
    rng = np.random.default_rng(4)
    p = (rng.standard_normal((3000, 3)) * 5 + 7).astype(np.float32)
    _, _, s = oracle.mesh_ingest(p)
    mean = np.zeros(3, np.float32)
    for i, x in enumerate(p):  # src/asset/mod.rs:308-317, f32 throughout
        mean = (mean + (x - mean) / np.float32(i + 1)).astype(np.float32)
    assert np.array_equal(s[:3], mean)
    r = np.sqrt(((p - mean) ** 2).sum(axis=1, dtype=np.float32)).max()
    assert s[3] == r


def _sequential_normals(p, idx):
    n = np.zeros_like(p)
    for t in idx.reshape(-1, 3):
        f = np.cross(p[t[1]] - p[t[0]], p[t[2]] - p[t[0]]).astype(np.float32)
        for i in t:
            n[i] = (n[i] + f).astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):  # unreferenced vertices: NaN, as in the reference
        inv = (np.float32(1) / np.sqrt((n * n).sum(axis=1, dtype=np.float32))).astype(np.float32)
        return (n * inv[:, None]).astype(np.float32)


def test_generated_normals_follow_triangle_order():
    rng = np.random.default_rng(5)
    p = rng.standard_normal((60, 3)).astype(np.float32)
    idx = rng.integers(0, 60, 600).astype(np.uint32)
    idx[3:6] = [7, 7, 9]  # a degenerate triangle repeats a vertex
    seq = _sequential_normals(p, idx)
    # the oracle's frames from generated normals equal its frames from these normals given
    _, v_gen, _ = oracle.mesh_ingest(p, indices=idx)
    _, v_giv, _ = oracle.mesh_ingest(p, indices=idx, normals=seq)
    assert np.array_equal(v_gen["tangent_frame"], v_giv["tangent_frame"])


@pytest.mark.parametrize("with_normals", [False, True])
def test_agrees_with_host_asset_path(with_normals):
    rng = np.random.default_rng(6)
    p = (rng.standard_normal((2000, 3)) * 3 + 1).astype(np.float32)
    idx = rng.integers(0, 2000, 6000).astype(np.uint32)
    uv = rng.random((2000, 2)).astype(np.float32)
    nrm = None
    if with_normals:
        nrm = rng.standard_normal((2000, 3)).astype(np.float32)
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    q, v, s = oracle.mesh_ingest(p, uv, idx, nrm)
    sc = asset.Scene()
    with np.errstate(invalid="ignore", divide="ignore"):
        sc.insert_mesh(p, uv, idx, nrm)
    assert np.abs(q.astype(np.int32) - sc.positions).max() <= 1  # float64 vs running mean centre
    assert np.allclose(s[:3], sc.meshes[0]["center"], atol=1e-5) and np.isclose(s[3], sc.meshes[0]["radius"])
    assert np.array_equal(v["texture_coordinates"].view(np.uint16), sc.vertices["texture_coordinates"].view(np.uint16))
    f1, f2 = v["tangent_frame"], sc.vertices["tangent_frame"]
    live = np.isfinite(_sequential_normals(p, idx)).all(axis=1) if nrm is None else np.ones(2000, bool)
    assert np.array_equal(f1[live] & 0x800FFFFF, f2[live] & 0x800FFFFF)
    da = np.abs(((f1 >> 20) & 0x7FF).astype(np.int32) - ((f2 >> 20) & 0x7FF))
    assert np.minimum(da, 2047 - da)[live].max() <= 1


def test_rejects_what_the_reference_panics_on():
    p = np.float32([[0, 0, 0], [1, 0, 0], [0, 1, 0]])
    with pytest.raises(ValueError):
        oracle.mesh_ingest(p, indices=np.uint32([0, 1, 3]))  # index out of range
    with pytest.raises(ValueError):
        oracle.mesh_ingest(p, indices=np.uint32([0, 1]))  # not triangles, normals generated
    with pytest.raises(ValueError):
        oracle.mesh_ingest(p[:1])  # zero radius
    oracle.mesh_ingest(p, indices=np.uint32([0, 1]), normals=np.tile([0, 0, 1], (3, 1)))  # normals given: fine
    q, v, s = oracle.mesh_ingest(np.zeros((0, 3), np.float32))
    assert len(q) == 0 and len(v) == 0 and (s == 0).all()


def test_emissive_triangles_match_host_path():
    sc = scenes.cornell_box()
    models = []

    def visit(_i, node, parent):
        for m in node.models:
            models.append(m)
        return parent

    asset.depth_first_node_tree(sc.root, None, visit)
    pairs = [(m.mesh_index, k) for k, m in enumerate(models) if m.material_index in sc.emissive_materials]
    got = oracle.emissive_triangles(sc.positions, sc.vertices, sc.indices, sc.mesh_array, pairs)
    want = np.concatenate([sc.emissive_triangles_in_model(models[k], k) for _, k in pairs])
    assert got.tobytes() == want.tobytes()


def test_emissive_hash_wraps_like_the_reference():
    sc = asset.Scene()
    p = np.random.default_rng(7).standard_normal((3 * 70000, 3)).astype(np.float32)
    mesh = sc.insert_mesh(p, normals=np.tile([0, 0, 1], (len(p), 1)))
    mat = sc.insert_material(Material(emission_luminance=1.0, emission_color=(1, 1, 1)))
    sc.root.children.append(Node(models=[Model(mesh, mat)]))
    got = oracle.emissive_triangles(sc.positions, sc.vertices, sc.indices, sc.mesh_array, [(mesh, 3)])
    assert len(got) == 70000
    offset = np.arange(70000)
    assert np.array_equal(got["hash"], ((offset % 65535) & 0xFFFF).astype(np.uint16))
    assert (got["instance_index"] == 3).all()
