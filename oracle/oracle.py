"""TEST INFRASTRUCTURE — ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg may import this module;
it is the checker for the CUDA path, never the thing measured or shipped.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build as _build

_lib = None
_P = ctypes.c_void_p


class OracleSceneDesc(ctypes.Structure):
    _fields_ = [("positions", _P), ("position_count", ctypes.c_uint64), ("indices", _P),
                ("index_count", ctypes.c_uint64), ("vertices", _P), ("vertex_count", ctypes.c_uint64),
                ("materials", _P), ("material_count", ctypes.c_uint32), ("mesh_count", ctypes.c_uint32),
                ("meshes", _P), ("instances", _P), ("instance_count", ctypes.c_uint32),
                ("emissive_count", ctypes.c_uint32), ("emissive", _P), ("textures", _P),
                ("texture_count", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class OracleTexture(ctypes.Structure):  # tt_texture
    _fields_ = [("format", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("level_count", ctypes.c_uint32), ("data", _P), ("bytes", ctypes.c_uint64)]


def _textures(arrays):
    info = np.asarray(getattr(arrays, "texture_info", np.zeros((0, 5), np.uint64)), np.uint64).reshape(-1, 5)
    data = getattr(arrays, "texture_data", np.zeros(0, np.uint8))
    out = (OracleTexture * max(len(info), 1))()
    at = 0
    for i, (fmt, w, h, levels, nbytes) in enumerate(info.tolist()):
        out[i] = OracleTexture(fmt, w, h, levels, (data.ctypes.data + at) if nbytes else None, nbytes)
        at += nbytes
    return out, len(info)


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        lib = ctypes.CDLL(str(path))
        lib.oracle_scene_create.restype = _P
        lib.oracle_scene_create.argtypes = [ctypes.POINTER(OracleSceneDesc), ctypes.c_int, ctypes.c_int]
        lib.oracle_scene_destroy.argtypes = [_P]
        lib.oracle_scene_bvh_info.argtypes = [_P, _P]
        lib.oracle_scene_bvh_copy.argtypes = [_P, _P, _P, _P]
        lib.oracle_scene_flat_copy.argtypes = [_P, _P, _P]
        lib.oracle_scene_wide_copy.argtypes = [_P, _P, _P]
        lib.oracle_trace_batch.argtypes = [_P, _P, ctypes.c_uint32, ctypes.c_uint32, _P, ctypes.c_int]
        lib.oracle_render.argtypes = [_P, _P, _P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.c_uint32, ctypes.c_int]
        lib.oracle_tonemap.argtypes = [_P, ctypes.c_uint64, ctypes.c_int, _P]
        lib.oracle_bsdf_eval_batch.argtypes = [_P, _P, ctypes.c_uint32, _P]
        lib.oracle_bsdf_sample_batch.argtypes = [_P, _P, ctypes.c_uint32, _P]
        lib.oracle_math.argtypes = [ctypes.c_int, _P, ctypes.c_uint64, _P]
        lib.oracle_scene_update_instances.argtypes = [_P, _P, ctypes.c_uint32]
        lib.oracle_restir_create.restype = _P
        lib.oracle_restir_create.argtypes = [_P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float,
                                             ctypes.c_uint32, ctypes.c_float]
        lib.oracle_restir_destroy.argtypes = [_P]
        lib.oracle_restir_frame.argtypes = [_P, _P, _P, ctypes.c_int]
        lib.oracle_restir_reservoirs.argtypes = [_P, _P]
        lib.oracle_atan2.argtypes = [_P, _P, ctypes.c_uint64, _P]
        lib.oracle_scene_set_light_exact.argtypes = [_P, ctypes.c_int]
        lib.oracle_scene_set_light_power.argtypes = [_P, ctypes.c_int]
        lib.oracle_texture_sample.argtypes = [_P, ctypes.c_uint32, _P, ctypes.c_uint32, _P]
        lib.oracle_mesh_ingest.restype = ctypes.c_int
        lib.oracle_mesh_ingest.argtypes = [_P, _P, _P, _P, _P, ctypes.c_uint32, ctypes.c_uint32, _P, _P, _P]
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


class OracleScene:
    """CPU restatement of the scene (brute-force or LBVH ray queries)."""

    def __init__(self, arrays, use_bvh: bool = True, leaf_max: int = 2, flat: bool = False, wide: bool = False):
        """use_bvh=False traces by brute force; otherwise render() traces through the
        two-level BVH, or the flat one when `flat` (the hits are the same).  `wide` also builds
        the compressed 8-wide format of the flat BVH (wide_bvh(), trace(..., wide=True))."""
        self.arrays = arrays  # keeps the borrowed arrays alive
        self._tex, ntex = _textures(arrays)
        d = OracleSceneDesc(_p(arrays.positions), len(arrays.positions), _p(arrays.indices), len(arrays.indices),
                            _p(arrays.vertices), len(arrays.vertices), _p(arrays.materials), len(arrays.materials),
                            len(arrays.meshes), _p(arrays.meshes), _p(arrays.instances), len(arrays.instances),
                            len(arrays.emissive), _p(arrays.emissive), ctypes.addressof(self._tex), ntex, 0)
        self.lib = load()
        accel = (3 if wide else (2 if flat else 1)) if use_bvh else 0
        self.handle = self.lib.oracle_scene_create(ctypes.byref(d), accel, leaf_max)

    def __del__(self):
        try:
            self.lib.oracle_scene_destroy(self.handle)
        except Exception:
            pass

    def set_light_exact(self, exact: bool) -> None:
        """Visibility of next-event estimation: the reference's hash test (False) or the sampled
        triangle itself (True)."""
        self.lib.oracle_scene_set_light_exact(self.handle, 1 if exact else 0)

    def set_light_power(self, power: bool) -> None:
        """Light selection of next-event estimation: uniform (False, the reference's) or by
        emitted power through the alias table (True)."""
        self.lib.oracle_scene_set_light_power(self.handle, 1 if power else 0)

    def texture_sample(self, index: int, uvl: np.ndarray) -> np.ndarray:
        """textureLod of texture `index` at (n, 3) (u, v, lod) -> (n, 4) RGBA."""
        uvl = np.ascontiguousarray(uvl, np.float32).reshape(-1, 3)
        out = np.zeros((len(uvl), 4), np.float32)
        self.lib.oracle_texture_sample(self.handle, index, _p(uvl), len(uvl), _p(out))
        return out

    def bvh(self):
        from tinytrace_gb300.native import NODE4_DTYPE, TRI_RECORD_DTYPE

        info = np.zeros(12, np.uint64)
        self.lib.oracle_scene_bvh_info(self.handle, _p(info))
        blas = np.zeros(int(info[0]), NODE4_DTYPE)
        tris = np.zeros(int(info[1]), TRI_RECORD_DTYPE)
        tlas = np.zeros(int(info[2]), NODE4_DTYPE)
        self.lib.oracle_scene_bvh_copy(self.handle, _p(blas), _p(tris), _p(tlas))
        return blas, tris, tlas, int(info[3]), int(info[4])

    def flat_bvh(self):
        from tinytrace_gb300.native import NODE4_DTYPE, TRI_RECORD_DTYPE

        info = np.zeros(12, np.uint64)
        self.lib.oracle_scene_bvh_info(self.handle, _p(info))
        nodes = np.zeros(int(info[5]), NODE4_DTYPE)
        tris = np.zeros(int(info[6]), TRI_RECORD_DTYPE)
        self.lib.oracle_scene_flat_copy(self.handle, _p(nodes), _p(tris))
        return nodes, tris, int(info[7])

    def wide_bvh(self):
        """(80-byte wide nodes, triangle records in wide order, levels) of the flat structure."""
        from tinytrace_gb300.native import NODE8_DTYPE, TRI_RECORD_DTYPE

        info = np.zeros(12, np.uint64)
        self.lib.oracle_scene_bvh_info(self.handle, _p(info))
        nodes = np.zeros(int(info[8]), NODE8_DTYPE)
        tris = np.zeros(int(info[9]), TRI_RECORD_DTYPE)
        self.lib.oracle_scene_wide_copy(self.handle, _p(nodes), _p(tris))
        return nodes, tris, int(info[10])

    def update_instances(self, instances: np.ndarray) -> None:
        """New instance transforms (the TLAS update); refits both world structures."""
        inst = np.ascontiguousarray(instances)
        self.arrays.instances = inst
        self.lib.oracle_scene_update_instances(self.handle, _p(inst), len(inst))

    def trace(self, rays: np.ndarray, cull: bool, brute: bool = False, threads: int = 0, flat: bool = False,
              wide: bool = False) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.zeros((len(rays), 8), np.uint32)
        flags = (1 if cull else 0) | (2 if brute else 0) | (4 if flat else 0) | (8 if wide else 0)
        self.lib.oracle_trace_batch(self.handle, _p(rays), len(rays), flags, _p(hits), threads)
        return hits

    def render(self, constants: np.ndarray, target: np.ndarray | None = None, rows=None, cols=None,
               threads: int = 0) -> np.ndarray:
        w, h = (int(x) for x in constants["screen_size"])
        if target is None:
            target = np.zeros((h, w, 4), np.float32)
        y0, y1 = rows if rows is not None else (0, h)
        x0, x1 = cols if cols is not None else (0, w)
        c = np.ascontiguousarray(constants)
        self.lib.oracle_render(self.handle, _p(c), _p(target), y0, y1, x0, x1, threads)
        return target


class OracleRestir:
    """ReSTIR DI frames on the CPU (the checker of tt_render_restir), keeping the previous
    frame's G-buffer, reservoirs and camera like the device context does."""

    def __init__(self, scene: "OracleScene", width: int, height: int, candidates: int = 32,
                 m_cap_factor: float = 20.0, neighbours: int = 5, radius: float = 30.0):
        self.scene = scene  # keeps the scene alive
        self.lib = scene.lib
        self.width, self.height = width, height
        self.handle = self.lib.oracle_restir_create(scene.handle, width, height, candidates, m_cap_factor,
                                                    neighbours, radius)

    def __del__(self):
        try:
            self.lib.oracle_restir_destroy(self.handle)
        except Exception:
            pass

    def frame(self, constants: np.ndarray, target: np.ndarray, threads: int = 0) -> np.ndarray:
        c = np.ascontiguousarray(constants)
        self.lib.oracle_restir_frame(self.handle, _p(c), _p(target), threads)
        return target

    def reservoirs(self) -> np.ndarray:
        out = np.zeros((self.height, self.width, 8), np.float32)
        self.lib.oracle_restir_reservoirs(self.handle, _p(out))
        return out


def tonemap(image: np.ndarray, enabled: bool = True) -> np.ndarray:
    img = np.ascontiguousarray(image, np.float32)
    out = np.zeros_like(img)
    load().oracle_tonemap(_p(img), img.size // 4, 1 if enabled else 0, _p(out))
    return out


def bsdf_eval(material_constants: np.ndarray, samples: np.ndarray) -> np.ndarray:
    s = np.ascontiguousarray(samples, np.float32).reshape(-1, 8)
    out = np.zeros((len(s), 8), np.float32)
    m = np.ascontiguousarray(material_constants)
    load().oracle_bsdf_eval_batch(_p(m), _p(s), len(s), _p(out))
    return out


def bsdf_sample(material_constants: np.ndarray, samples: np.ndarray) -> np.ndarray:
    s = np.ascontiguousarray(samples, np.float32).reshape(-1, 4)
    out = np.zeros((len(s), 12), np.float32)
    m = np.ascontiguousarray(material_constants)
    load().oracle_bsdf_sample_batch(_p(m), _p(s), len(s), _p(out))
    return out


def math(which: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    y = np.zeros_like(x)
    load().oracle_math(which, _p(x), x.size, _p(y))
    return y


def atan2(y: np.ndarray, x: np.ndarray) -> np.ndarray:
    """tatan2, the atan2 of the tangent-frame encoding."""
    y = np.ascontiguousarray(y, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(y)
    load().oracle_atan2(_p(y), _p(x), y.size, _p(out))
    return out


VERTEX_DTYPE = np.dtype([("texture_coordinates", "<f2", (2,)), ("tangent_frame", "<u4")])
EMISSIVE_DTYPE = np.dtype([("positions", "<i2", (3, 3)), ("hash", "<u2"),
                           ("texture_coordinates", "<f2", (3, 2)), ("instance_index", "<u4")])


def mesh_ingest(positions, texture_coordinates=None, indices=None, normals=None, tangents=None):
    """Scene::insert_mesh (src/asset/mod.rs:89-161) restated: (snorm16 positions (n, 3),
    vertices (n,) of VERTEX_DTYPE, (centre x, y, z, radius)); ValueError where the reference
    panics (index out of range, index count not a multiple of 3, degenerate sphere)."""
    def arr(a, dtype, width):
        return None if a is None else np.ascontiguousarray(np.asarray(a, dtype).reshape(-1, width) if width
                                                            else np.asarray(a, dtype).reshape(-1))
    p = arr(positions, np.float32, 3)
    uv, nrm, tan = arr(texture_coordinates, np.float32, 2), arr(normals, np.float32, 3), arr(tangents, np.float32, 4)
    idx = arr(indices, np.uint32, 0)
    n = len(p)
    out_p = np.zeros((n, 3), np.int16)
    out_v = np.zeros(n, VERTEX_DTYPE)
    sphere = np.zeros(4, np.float32)
    rc = load().oracle_mesh_ingest(_p(p), _p(uv), _p(idx), _p(nrm), _p(tan), n, 0 if idx is None else len(idx),
                                   _p(out_p), _p(out_v), _p(sphere))
    if rc != 0:
        raise ValueError("mesh rejected (the reference panics on it)")
    return out_p, out_v, sphere


def emissive_triangles(positions, vertices, indices, meshes, models):
    """Scene::emissive_triangles_in_model (src/asset/mod.rs:163-193) for the (mesh index,
    instance index) pairs `models` in order; `meshes` is a structured array with the
    vertex_offset / index_offset / index_count fields of ProcessedMesh."""
    positions = np.asarray(positions).reshape(-1, 3)
    uv = np.asarray(vertices)["texture_coordinates"]
    indices = np.asarray(indices).reshape(-1)
    out = []
    for mesh_index, instance_index in models:
        me = meshes[mesh_index]
        vo, io, ic = int(me["vertex_offset"]), int(me["index_offset"]), int(me["index_count"])
        tri = indices[io:io + ic // 3 * 3].reshape(-1, 3).astype(np.int64) + vo
        e = np.zeros(len(tri), EMISSIVE_DTYPE)
        e["positions"] = positions[tri]
        e["texture_coordinates"] = uv[tri]
        offset = np.arange(len(tri), dtype=np.int64)
        e["hash"] = ((io // 3 + offset % 65535) & 0xFFFF).astype(np.uint16)
        e["instance_index"] = instance_index
        out.append(e)
    return np.concatenate(out) if out else np.zeros(0, EMISSIVE_DTYPE)
