"""Host-side scene model: the reference's `asset::Scene` (src/asset/mod.rs), `Material`
(src/asset/material.rs), `TangentFrame` (src/asset/normal.rs) and the quantisation helpers
(src/math/mod.rs), producing the byte layouts that tt_scene_create consumes.

Differences from the reference, all on the host side of the boundary:
  * arithmetic is numpy float32/float64 instead of glam, so bounding-sphere centres and
    matrix inverses may differ from the Rust results in the last bits (they are inputs to
    the renderer, not part of the parity-checked path);
  * tangents are not generated with mikktspace (the crate is unavailable): when a mesh has
    no tangents, `default_tangents` builds a deterministic tangent orthogonal to the normal.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .native import EMISSIVE_DTYPE, MATERIAL_DTYPE, MESH_DTYPE, VERTEX_DTYPE

INVALID_INDEX = 0xFFFFFFFF


# ---------------------------------------------------------------- src/math/mod.rs
def quantize_unorm(v: np.ndarray, n: int) -> np.ndarray:
    """src/math/mod.rs:24-29"""
    scale = np.float32((1 << n) - 1)
    v = np.asarray(v, np.float32)
    v = np.where(v >= 0, v, np.float32(0.0))  # NaN -> 0, as the comparisons of the reference
    v = np.where(v <= 1, v, np.float32(1.0)).astype(np.float32)
    return (v * scale + np.float32(0.5)).astype(np.int32)


def quantize_snorm(v: np.ndarray, n: int) -> np.ndarray:
    """src/math/mod.rs:31-37: round half away from zero, then truncate."""
    scale = np.float32((1 << (n - 1)) - 1)
    v = np.asarray(v, np.float32)
    rnd = np.where(v >= 0, np.float32(0.5), np.float32(-0.5)).astype(np.float32)
    v = np.clip(v, np.float32(-1.0), np.float32(1.0))
    return np.trunc(v * scale + rnd).astype(np.int32)


def dequantize_unorm(value: np.ndarray, n: int) -> np.ndarray:
    return np.asarray(value, np.float32) / np.float32((1 << n) - 1)


def encode_octahedron(normal: np.ndarray) -> np.ndarray:
    """src/math/mod.rs:3-13"""
    n = np.asarray(normal, np.float32)
    n = n / np.abs(n).sum(axis=-1, keepdims=True).astype(np.float32)
    xy = n[..., :2]
    wrapped = (np.float32(1.0) - np.abs(xy[..., ::-1])) * np.sign(xy).astype(np.float32)
    # glam signum returns 1 for +0.0
    wrapped = np.where(xy == 0, (np.float32(1.0) - np.abs(xy[..., ::-1])) * np.where(np.signbit(xy), -1, 1),
                       wrapped).astype(np.float32)
    out = np.where((n[..., 2] < 0)[..., None], wrapped, xy)
    return (out * np.float32(0.5) + np.float32(0.5)).astype(np.float32)


def decode_octahedron(o: np.ndarray) -> np.ndarray:
    """src/math/mod.rs:15-22"""
    o = np.asarray(o, np.float32) * np.float32(2.0) - np.float32(1.0)
    z = np.float32(1.0) - np.abs(o[..., 0]) - np.abs(o[..., 1])
    n = np.stack([o[..., 0], o[..., 1], z], axis=-1).astype(np.float32)
    t = np.clip(-n[..., 2], 0.0, 1.0).astype(np.float32)
    n[..., 0] += np.where(n[..., 0] >= 0, -t, t)
    n[..., 1] += np.where(n[..., 1] >= 0, -t, t)
    return (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)


def _orthonormal(n: np.ndarray) -> np.ndarray:
    """src/asset/normal.rs:55-62"""
    a = np.stack([-n[..., 1], n[..., 0], np.zeros_like(n[..., 0])], axis=-1)
    b = np.stack([np.zeros_like(n[..., 0]), -n[..., 2], n[..., 1]], axis=-1)
    v = np.where((np.abs(n[..., 0]) > np.abs(n[..., 2]))[..., None], a, b).astype(np.float32)
    return (v / np.linalg.norm(v, axis=-1, keepdims=True)).astype(np.float32)


def encode_tangent_frames(normals: np.ndarray, tangents: np.ndarray) -> np.ndarray:
    """TangentFrame::new (src/asset/normal.rs:17-36): 10+10 bit octahedral normal, 11-bit
    tangent angle around the normal, 1 bitangent-sign bit."""
    normals = np.asarray(normals, np.float32)
    tangents = np.asarray(tangents, np.float32)
    octa = encode_octahedron(normals)
    u = quantize_unorm(octa[..., 0], 10).astype(np.uint32)
    v = quantize_unorm(octa[..., 1], 10).astype(np.uint32)
    decoded = decode_octahedron(np.stack([dequantize_unorm(u, 10), dequantize_unorm(v, 10)], axis=-1))
    ortho = _orthonormal(decoded)
    t = tangents[..., :3]
    dot = (ortho * t).sum(-1)
    det = (normals * np.cross(ortho, t)).sum(-1)
    angle = np.arctan2(det, dot).astype(np.float32)
    angle = np.where(angle < 0, angle + np.float32(2.0 * np.pi), angle).astype(np.float32)
    a = quantize_unorm(angle / np.float32(2.0 * np.pi), 11).astype(np.uint32)
    sign = (tangents[..., 3] >= 0).astype(np.uint32)
    return (sign << 31) | (a << 20) | (v << 10) | u


def generate_normals(positions: np.ndarray, indices: np.ndarray) -> np.ndarray:
    """src/asset/mod.rs:226-242: area-weighted face normals accumulated per vertex."""
    p = np.asarray(positions, np.float32)
    tri = np.asarray(indices, np.int64).reshape(-1, 3)
    fn = np.cross(p[tri[:, 1]] - p[tri[:, 0]], p[tri[:, 2]] - p[tri[:, 0]]).astype(np.float32)
    n = np.zeros_like(p)
    for k in range(3):
        np.add.at(n, tri[:, k], fn)
    return (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)


def default_tangents(normals: np.ndarray) -> np.ndarray:
    """Deterministic unit tangent orthogonal to each normal (w = +1); stands in for the
    mikktspace tangents of src/asset/mod.rs:244-265."""
    n = np.asarray(normals, np.float32)
    up = np.where((np.abs(n[..., 1]) < 0.999)[..., None], np.array([0, 1, 0], np.float32),
                  np.array([1, 0, 0], np.float32))
    t = np.cross(up, n)
    t = t / np.linalg.norm(t, axis=-1, keepdims=True)
    return np.concatenate([t, np.ones_like(t[..., :1])], axis=-1).astype(np.float32)


def bounding_sphere(positions: np.ndarray) -> tuple[np.ndarray, float]:
    """src/asset/mod.rs:308-321 (mean centre, max distance radius)."""
    p = np.asarray(positions, np.float64)
    if len(p) == 0:
        return np.zeros(3, np.float32), 0.0
    center = p.mean(axis=0).astype(np.float32)
    radius = float(np.max(np.linalg.norm(p.astype(np.float32) - center, axis=-1)))
    return center, radius


# ---------------------------------------------------------------- src/asset/material.rs
@dataclass
class Material:
    """OpenPBR parameters (src/asset/material.rs:35-175) with their reference defaults.
    Only constant parameters are supported (textured parameters are not)."""

    base_weight: float = 1.0
    base_color: tuple = (0.8, 0.8, 0.8)
    base_metalness: float = 0.0
    base_diffuse_roughness: float = 0.0
    specular_weight: float = 1.0
    specular_color: tuple = (1.0, 1.0, 1.0)
    specular_roughness: float = 0.3
    specular_roughness_anisotropy: float = 0.0
    specular_ior: float = 1.5
    specular_rotation: float = 0.0
    transmission_weight: float = 0.0
    transmission_color: tuple = (1.0, 1.0, 1.0)
    transmission_depth: float = 0.0
    coat_weight: float = 0.0
    coat_color: tuple = (1.0, 1.0, 1.0)
    coat_roughness: float = 0.0
    coat_roughness_anisotropy: float = 0.0
    coat_ior: float = 1.6
    coat_darkening: float = 1.0
    coat_rotation: float = 0.0
    fuzz_weight: float = 0.0
    fuzz_color: tuple = (1.0, 1.0, 1.0)
    fuzz_roughness: float = 0.5
    emission_luminance: float = 0.0
    emission_color: tuple = (1.0, 1.0, 1.0)
    geometry_opacity: float = 1.0
    geometry_normal: tuple = (0.0, 0.0, 1.0)
    # Param::Texture: parameter name -> texture, (h, w, 3) floats for colours and normals,
    # (h, w) floats for scalars; the parameter's constant is then the type's default (zero)
    textures: dict = field(default_factory=dict)

    def is_emissive(self) -> bool:
        """src/asset/material.rs:177-183"""
        if "emission_luminance" in self.textures:
            return bool(np.any(np.asarray(self.textures["emission_luminance"]) > 0.0))
        return self.emission_luminance > 0.0

    def constants(self) -> np.ndarray:
        """Material::constants (src/asset/material.rs:233-265); vec3s extended with 0, textured
        parameters zero (Param::constant_or_default, material.rs:20-25)."""
        from .native import MATERIAL_CONSTANTS_DTYPE

        c = np.zeros((), MATERIAL_CONSTANTS_DTYPE)
        for name in MATERIAL_CONSTANTS_DTYPE.names:
            if name in self.textures:
                continue
            v = getattr(self, name)
            if isinstance(v, tuple):
                c[name] = (*v, 0.0)
            else:
                c[name] = v
        return c


# ---------------------------------------------------------------- src/asset/mod.rs
@dataclass
class Model:
    mesh_index: int
    material_index: int


@dataclass
class Node:
    transform: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float64))
    models: list = field(default_factory=list)
    children: list = field(default_factory=list)


def depth_first_node_tree(node: Node, value, visitor, index: int = 0) -> int:
    """src/asset/mod.rs:207-224"""
    v = visitor(index, node, value)
    for child in node.children:
        index = depth_first_node_tree(child, v, visitor, index + 1)
    return index


class Scene:
    """asset::Scene (src/asset/mod.rs:75-194)."""

    def __init__(self) -> None:
        self._positions: list[np.ndarray] = []
        self._indices: list[np.ndarray] = []
        self._vertices: list[np.ndarray] = []
        self.meshes: list[np.ndarray] = []
        self.materials: list[np.ndarray] = []
        self.emissive_materials: set[int] = set()
        self.textures: list = []  # texture.ProcessedTexture
        self.root = Node()
        self._vertex_total = 0
        self._index_total = 0
        self._cache = None

    # arrays in the reference's layout
    @property
    def positions(self) -> np.ndarray:
        self._pack()
        return self._cache[0]

    @property
    def indices(self) -> np.ndarray:
        self._pack()
        return self._cache[1]

    @property
    def vertices(self) -> np.ndarray:
        self._pack()
        return self._cache[2]

    @property
    def mesh_array(self) -> np.ndarray:
        return np.array(self.meshes, MESH_DTYPE).reshape(-1) if self.meshes else np.zeros(0, MESH_DTYPE)

    @property
    def material_array(self) -> np.ndarray:
        return np.array(self.materials, MATERIAL_DTYPE).reshape(-1) if self.materials else np.zeros(0, MATERIAL_DTYPE)

    def _pack(self) -> None:
        if self._cache is None:
            pos = np.concatenate(self._positions) if self._positions else np.zeros((0, 3), np.int16)
            idx = np.concatenate(self._indices) if self._indices else np.zeros(0, np.uint32)
            ver = np.concatenate(self._vertices) if self._vertices else np.zeros(0, VERTEX_DTYPE)
            self._cache = (np.ascontiguousarray(pos, np.int16), np.ascontiguousarray(idx, np.uint32),
                           np.ascontiguousarray(ver))

    def insert_mesh(self, positions: np.ndarray, texture_coordinates: np.ndarray | None = None,
                    indices: np.ndarray | None = None, normals: np.ndarray | None = None,
                    tangents: np.ndarray | None = None) -> int:
        """Scene::insert_mesh (src/asset/mod.rs:89-161): snorm16 positions relative to the
        bounding sphere, packed tangent frames and f16 texture coordinates."""
        self._cache = None
        positions = np.asarray(positions, np.float32).reshape(-1, 3)
        n = len(positions)
        mesh_index = len(self.meshes)
        center, radius = bounding_sphere(positions)
        rel = (positions - center) / np.float32(radius if radius > 0 else 1.0)
        q = quantize_snorm(np.clip(rel, -1.0, 1.0), 16).astype(np.int16)
        self._positions.append(q)
        if indices is None:
            indices = np.arange(n, dtype=np.uint32)
        indices = np.asarray(indices, np.uint32).reshape(-1)
        self._indices.append(indices)
        if normals is None:
            normals = generate_normals(positions, indices)
        if tangents is None:
            tangents = default_tangents(normals)
        if texture_coordinates is None:
            texture_coordinates = np.zeros((n, 2), np.float32)
        v = np.zeros(n, VERTEX_DTYPE)
        v["texture_coordinates"] = np.asarray(texture_coordinates, np.float32).astype(np.float16)
        v["tangent_frame"] = encode_tangent_frames(normals, tangents)
        self._vertices.append(v)
        self.meshes.append(np.array((center, radius, self._vertex_total, n, self._index_total, len(indices)),
                                    MESH_DTYPE))
        self._vertex_total += n
        self._index_total += len(indices)
        return mesh_index

    def append_processed_mesh(self, positions: np.ndarray, indices: np.ndarray, vertices: np.ndarray,
                              center, radius: float) -> int:
        """Appends a mesh whose positions (snorm16), vertices (packed) and bounding sphere were
        produced elsewhere (tt_mesh_ingest); returns its index."""
        self._cache = None
        positions = np.ascontiguousarray(positions, np.int16).reshape(-1, 3)
        indices = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        vertices = np.ascontiguousarray(vertices, VERTEX_DTYPE).reshape(-1)
        if len(vertices) != len(positions):
            raise ValueError("positions and vertices differ in length")
        mesh_index = len(self.meshes)
        self._positions.append(positions)
        self._indices.append(indices)
        self._vertices.append(vertices)
        self.meshes.append(np.array((np.asarray(center, np.float32), np.float32(radius), self._vertex_total,
                                     len(positions), self._index_total, len(indices)), MESH_DTYPE))
        self._vertex_total += len(positions)
        self._index_total += len(indices)
        return mesh_index

    @property
    def vertex_total(self) -> int:
        return self._vertex_total

    @property
    def index_total(self) -> int:
        return self._index_total

    def insert_material(self, material: Material) -> int:
        """Scene::insert_material (src/asset/material.rs:305-357): textured parameters are
        processed (texture.process) and referenced by their index in `textures`."""
        from . import texture

        index = len(self.materials)
        if material.is_emissive():
            self.emissive_materials.add(index)
        m = np.zeros((), MATERIAL_DTYPE)
        m["constants"] = material.constants()
        m["textures"] = INVALID_INDEX
        for name, tex in material.textures.items():
            if name not in texture.SLOTS:
                raise ValueError(f"{name} is not a material parameter")
            m["textures"][texture.SLOTS.index(name)] = len(self.textures)
            self.textures.append(texture.process(name, np.asarray(tex, np.float32)))
        self.materials.append(m)
        return index

    def emissive_triangles_in_model(self, model: Model, instance_index: int) -> np.ndarray | None:
        """src/asset/mod.rs:163-193, including the hash
        (mesh.index_offset / 3 + offset % u16::MAX) as u16."""
        if model.material_index not in self.emissive_materials:
            return None
        me = self.meshes[model.mesh_index]
        io, ic, vo = int(me["index_offset"]), int(me["index_count"]), int(me["vertex_offset"])
        tri = self.indices[io:io + ic // 3 * 3].reshape(-1, 3).astype(np.int64) + vo
        out = np.zeros(len(tri), EMISSIVE_DTYPE)
        out["positions"] = self.positions[tri]
        out["texture_coordinates"] = self.vertices["texture_coordinates"][tri]
        offset = np.arange(len(tri), dtype=np.uint64)
        out["hash"] = ((np.uint64(io // 3) + offset % np.uint64(65535)) & np.uint64(0xFFFF)).astype(np.uint16)
        out["instance_index"] = instance_index
        return out
