"""Mesh ingest on the GPU (tt_mesh_ingest, tt_emissive_extract) against the oracle's
restatement of Scene::insert_mesh and emissive_triangles_in_model: snorm16 positions, packed
vertices and bounding spheres bit for bit, for indexed and non-indexed meshes, with and
without normals and tangents, from a few vertices up to a 2.5M-vertex mesh; the errors the
reference panics on come back as TT_ERR_INVALID_ARGUMENT; scene arrays built with the device
extraction equal the host path's."""
import numpy as np
import pytest

from oracle import oracle
from tinytrace_gb300 import asset, native, scenes
from tinytrace_gb300.ingest import DeviceIngest
from tinytrace_gb300.native import TinytraceError
from tinytrace_gb300.renderer import SceneArrays

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ingest(gpu_context):
    return DeviceIngest(gpu_context)


def _check(ingest, *args):
    q, v, rec = ingest.process_mesh(*args)
    oq, ov, os_ = oracle.mesh_ingest(*args)
    assert q.tobytes() == oq.tobytes(), "positions"
    assert v.tobytes() == ov.tobytes(), "vertices"
    assert np.array_equal(np.append(rec["center"], rec["radius"]).view(np.uint32), os_.view(np.uint32)), "sphere"
    return q, v, rec


def _unit(a):
    return (a / np.linalg.norm(a, axis=-1, keepdims=True)).astype(np.float32)


@pytest.mark.parametrize("case", ["generated", "normals", "normals_tangents", "non_indexed"])
def test_random_mesh_matches_oracle(ingest, case):
    rng = np.random.default_rng(["generated", "normals", "normals_tangents", "non_indexed"].index(case))
    n = 5000
    p = (rng.standard_normal((n, 3)) * 4 - 2).astype(np.float32)
    uv = (rng.standard_normal((n, 2)) * 3).astype(np.float32)
    idx = rng.integers(0, n, 3 * 9000).astype(np.uint32)
    nrm = _unit(rng.standard_normal((n, 3))) if case.startswith("normals") else None
    tan = None
    if case == "normals_tangents":
        tan = np.concatenate([_unit(rng.standard_normal((n, 3))), rng.choice([-1.0, 1.0], (n, 1))], 1)
        tan = tan.astype(np.float32)
    if case == "non_indexed":
        idx = None
        p = p[: n // 3 * 3]
        uv = uv[: len(p)]
    _check(ingest, p, uv, idx, nrm, tan)


def test_icosphere_and_axis_normals(ingest):
    p, idx = scenes.geodesic_sphere(24)
    _check(ingest, p, None, idx)
    # normals on the axes and octahedron seams (+-0 components, the z < 0 fold)
    axes = np.float32([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
                       [0.0, -0.0, -1.0], [-0.0, 0.6, -0.8], [0.6, -0.0, -0.8], [0.7071068, 0.7071068, 0]])
    pts = np.random.default_rng(9).standard_normal((len(axes), 3)).astype(np.float32)
    _check(ingest, pts, None, None, axes)


def test_large_mesh(ingest):
    """2.5M vertices / 5M triangles, the size of the large scenes the host loop is slow on."""
    rng = np.random.default_rng(10)
    n = 2_500_000
    p = rng.standard_normal((n, 3)).astype(np.float32)
    idx = rng.integers(0, n, 3 * 5_000_000).astype(np.uint32)
    uv = rng.random((n, 2)).astype(np.float32)
    _check(ingest, p, uv, idx)


def test_errors(ingest):
    p = np.float32([[0, 0, 0], [1, 0, 0], [0, 1, 0]])
    for args in [(p, None, np.uint32([0, 1, 3])), (p, None, np.uint32([0, 1])), (p[:1],)]:
        with pytest.raises(TinytraceError) as e:
            ingest.process_mesh(*args)
        assert e.value.code == native.TT_ERR_INVALID_ARGUMENT
    q, v, rec = ingest.process_mesh(np.zeros((0, 3), np.float32))
    assert len(q) == 0 and rec["radius"] == 0
    ingest.process_mesh(p)  # the context still works after the errors


def test_emissive_extraction(ingest):
    sc = scenes.icosphere_field(instances=8, freq=8, lights=300, seed=5)
    host = SceneArrays(sc)
    dev = ingest.scene_arrays(sc)
    assert len(host.emissive) > 0
    for f in SceneArrays.FIELDS:
        assert getattr(dev, f).tobytes() == getattr(host, f).tobytes(), f


def test_emissive_errors(ingest):
    sc = scenes.cornell_box()
    pos, ver, idx, meshes = sc.positions, sc.vertices, sc.indices, sc.mesh_array
    with pytest.raises(TinytraceError) as e:
        ingest.emissive_triangles(pos, ver, idx, meshes, [(len(meshes), 0)])
    assert e.value.code == native.TT_ERR_INVALID_ARGUMENT
    bad = idx.copy()
    bad[meshes[0]["index_offset"]] = 10 ** 6
    with pytest.raises(TinytraceError):
        ingest.emissive_triangles(pos, ver, bad, meshes, [(0, 0)])
    got = ingest.emissive_triangles(pos, ver, idx, meshes, [(0, 2), (1, 5)])
    want = oracle.emissive_triangles(pos, ver, idx, meshes, [(0, 2), (1, 5)])
    assert got.tobytes() == want.tobytes()


def test_insert_mesh_into_scene(ingest):
    rng = np.random.default_rng(11)
    sc = asset.Scene()
    sc.insert_mesh(rng.standard_normal((30, 3)).astype(np.float32))
    p = rng.standard_normal((300, 3)).astype(np.float32)
    idx = rng.integers(0, 300, 900).astype(np.uint32)
    k = ingest.insert_mesh(sc, p, None, idx)
    me = sc.meshes[k]
    assert me["vertex_offset"] == 30 and me["index_offset"] == 30 and me["index_count"] == 900
    oq, ov, _ = oracle.mesh_ingest(p, None, idx)
    assert sc.positions[30:].tobytes() == oq.tobytes() and sc.vertices[30:].tobytes() == ov.tobytes()
    assert np.array_equal(sc.indices[30:], idx)
