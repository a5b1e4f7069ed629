"""Scene ingest on the GPU: Scene::insert_mesh (src/asset/mod.rs:89-161) and the
emissive-triangle extraction of Scene::new (src/asset/mod.rs:163-193, src/scene.rs:29-64)
through tt_mesh_ingest / tt_emissive_extract, for meshes and scenes too large for the
host loops.

Results are the reference's: the bounding-sphere centre is its f32 running mean, normals are
summed in triangle order, and the tangent frames, snorm16 positions and f16 texture
coordinates follow its quantisation bit for bit.  Generated tangents are cross(up, n)
normalised (the reference runs mikktspace, which is not available).  Errors the reference
panics on (an index out of range, a degenerate bounding sphere) raise TinytraceError.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native
from .asset import Scene
from .native import EMISSIVE_DTYPE, MESH_DTYPE, VERTEX_DTYPE, check
from .renderer import Context, SceneArrays


def _arr(a, dtype, width: int):
    if a is None:
        return None
    a = np.asarray(a, dtype)
    return np.ascontiguousarray(a.reshape(-1, width) if width else a.reshape(-1))


class DeviceIngest:
    """Mesh processing and emissive-triangle extraction on one GPU context."""

    def __init__(self, context: Context | None = None, device: int = 0):
        self._own = context is None
        self.ctx = context if context is not None else Context(device)

    def close(self) -> None:
        if self._own and self.ctx is not None:
            self.ctx.close()
        self.ctx = None

    def process_mesh(self, positions, texture_coordinates=None, indices=None, normals=None, tangents=None,
                     vertex_offset: int = 0, index_offset: int = 0):
        """Returns (snorm16 positions (n, 3), vertices (n,), mesh record of MESH_DTYPE)."""
        p = _arr(positions, np.float32, 3)
        uv = _arr(texture_coordinates, np.float32, 2)
        nrm = _arr(normals, np.float32, 3)
        tan = _arr(tangents, np.float32, 4)
        idx = _arr(indices, np.uint32, 0)
        n = len(p)
        for name, a in (("texture_coordinates", uv), ("normals", nrm), ("tangents", tan)):
            if a is not None and len(a) != n:
                raise ValueError(f"{name} has {len(a)} entries for {n} vertices")
        d = native.MeshData()
        d.positions, d.texture_coordinates = native.ptr(p), native.ptr(uv)
        d.indices, d.normals, d.tangents = native.ptr(idx), native.ptr(nrm), native.ptr(tan)
        d.vertex_count = n
        d.index_count = 0 if idx is None else len(idx)
        out_p = np.zeros((n, 3), np.int16)
        out_v = np.zeros(n, VERTEX_DTYPE)
        rec = np.zeros((), MESH_DTYPE)
        check(self.ctx.lib.tt_mesh_ingest(self.ctx.handle, ctypes.byref(d), vertex_offset, index_offset,
                                          native.ptr(out_p), native.ptr(out_v), rec.ctypes.data))
        return out_p, out_v, rec

    def insert_mesh(self, scene: Scene, positions, texture_coordinates=None, indices=None, normals=None,
                    tangents=None) -> int:
        """Scene::insert_mesh with the per-vertex work on the GPU; returns the mesh index."""
        n = len(np.asarray(positions).reshape(-1, 3))
        idx = np.arange(n, dtype=np.uint32) if indices is None else _arr(indices, np.uint32, 0)
        q, v, rec = self.process_mesh(positions, texture_coordinates, idx, normals, tangents,
                                      scene.vertex_total, scene.index_total)
        return scene.append_processed_mesh(q, idx, v, rec["center"], float(rec["radius"]))

    def emissive_triangles(self, positions, vertices, indices, meshes, models) -> np.ndarray:
        """The emissive triangles of the (mesh index, instance index) pairs `models`, in order."""
        positions = np.ascontiguousarray(positions, np.int16).reshape(-1, 3)
        vertices = np.ascontiguousarray(vertices, VERTEX_DTYPE).reshape(-1)
        indices = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        meshes = np.ascontiguousarray(meshes, MESH_DTYPE).reshape(-1)
        models = np.asarray(models, np.uint32).reshape(-1, 2)
        model_mesh = np.ascontiguousarray(models[:, 0])
        model_instance = np.ascontiguousarray(models[:, 1])
        s = native.EmissiveSource()
        s.positions, s.vertices, s.vertex_count = native.ptr(positions), native.ptr(vertices), len(positions)
        s.indices, s.index_count = native.ptr(indices), len(indices)
        s.meshes, s.mesh_count, s.model_count = native.ptr(meshes), len(meshes), len(models)
        s.model_mesh, s.model_instance = native.ptr(model_mesh), native.ptr(model_instance)
        count = ctypes.c_uint64()
        total = sum(int(meshes[m]["index_count"]) // 3 for m in model_mesh if m < len(meshes))
        out = np.zeros(total, EMISSIVE_DTYPE)
        check(self.ctx.lib.tt_emissive_extract(self.ctx.handle, ctypes.byref(s), native.ptr(out) if total else None,
                                               total, ctypes.byref(count)))
        return out[: count.value]

    def scene_arrays(self, scene: Scene) -> SceneArrays:
        """SceneArrays of `scene` with the emissive triangles extracted on the GPU."""
        positions = np.ascontiguousarray(scene.positions, np.int16).reshape(-1, 3)
        vertices = np.ascontiguousarray(scene.vertices)
        indices = np.ascontiguousarray(scene.indices, np.uint32)
        meshes = np.ascontiguousarray(scene.mesh_array)
        return SceneArrays(scene, emissive_fn=lambda models: self.emissive_triangles(positions, vertices, indices,
                                                                                     meshes, models))
