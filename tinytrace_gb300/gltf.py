"""glTF 2.0 importer: `.gltf` (JSON with external or base64 `data:` buffers) and `.glb` files
into an `asset.Scene`, following the reference importer (src/asset/gltf.rs):

* one model per mesh primitive (triangle lists), cached per (mesh, primitive); attributes
  POSITION (f32 vec3), TEXCOORD_0 (f32 vec2, zeros when absent), NORMAL (f32 vec3),
  TANGENT (f32 vec4); indices u16 or u32 (gltf.rs:140-166; other types are errors);
* materials cached per glTF material (the default material too), mapped as gltf.rs:242-381:
  base colour, metallic -> base metalness, roughness -> specular roughness, emissive factor ->
  emission colour, KHR_materials_emissive_strength -> emission luminance,
  KHR_materials_specular -> specular weight / colour, KHR_materials_ior -> specular IOR,
  KHR_materials_transmission -> transmission weight with transmission colour 1 - base colour;
* the node tree of the default scene (or the first scene), node matrices or TRS composed as
  T * R * S.

* textures (gltf.rs:86-137, 259-366): PNG images (from files, data URIs or buffer views)
  decoded to 8-bit RGBA, scaled to [0, 1] and multiplied by their factors: base colour
  (x baseColorFactor), metallic (blue) and roughness (green) x their factors, normals
  (rgb * 2 - 1), emission (x emissiveFactor), specular weight (alpha x specularFactor),
  specular colour (x specularColorFactor); a transmission texture sets the specular weight
  (transmission x red), as the reference does; the transmission colour follows a textured
  base colour as 1 - colour.

Differences from the reference: tangents missing from the file come from
`asset.default_tangents` instead of mikktspace; `.glb` containers are read (the reference
rejects them); images that are not PNG are skipped and counted in
`Import.ignored_textures` (the reference panics); grey PNGs become RGB (the reference
reinterprets their bytes as RGBA).
"""
from __future__ import annotations

import base64
import json
import struct
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import png
from .asset import Material, Model, Node, Scene

COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
WIDTH = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}
F32, U16, U32 = 5126, 5123, 5125


class GltfError(ValueError):
    pass


@dataclass
class Import:
    scene: Scene
    meshes: int
    materials: int
    ignored_textures: int


class _Reader:
    def __init__(self, doc: dict, buffers: list[bytes]):
        self.doc = doc
        self.buffers = buffers

    def accessor(self, index: int, name: str, component: int | tuple, kind: str) -> np.ndarray:
        acc = self.doc["accessors"][index]
        comps = component if isinstance(component, tuple) else (component,)
        if acc["componentType"] not in comps or acc["type"] != kind:
            raise GltfError(f"unsupported format {acc['componentType']} {acc['type']} for {name}: expected "
                            f"{comps} {kind}")
        dtype = np.dtype(COMPONENT[acc["componentType"]])
        width = WIDTH[kind]
        count = acc["count"]
        if "bufferView" not in acc:
            return np.zeros((count, width), dtype)
        view = self.doc["bufferViews"][acc["bufferView"]]
        data = self.buffers[view["buffer"]]
        start = view.get("byteOffset", 0) + acc.get("byteOffset", 0)
        elem = dtype.itemsize * width
        stride = view.get("byteStride", elem)
        if stride == elem:
            out = np.frombuffer(data, dtype, count * width, start).reshape(count, width)
        else:
            raw = np.frombuffer(data, np.uint8, (count - 1) * stride + elem, start)
            rows = np.lib.stride_tricks.as_strided(raw, (count, elem), (stride, 1))
            out = np.ascontiguousarray(rows).view(dtype).reshape(count, width)
        return out.copy()


def _load_buffers(doc: dict, base: Path, glb_bin: bytes | None) -> list[bytes]:
    out = []
    for b in doc.get("buffers", []):
        uri = b.get("uri")
        if uri is None:
            if glb_bin is None:
                raise GltfError("buffer without uri outside a .glb container")
            out.append(glb_bin)
        elif uri.startswith("data:"):
            out.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            out.append((base / uri).read_bytes())
    return out


def _read(path: Path) -> tuple[dict, bytes | None]:
    raw = path.read_bytes()
    if raw[:4] != b"glTF":
        return json.loads(raw.decode("utf-8")), None
    _, _, length = struct.unpack_from("<III", raw, 0)
    at, doc, binary = 12, None, None
    while at < length:
        chunk_len, chunk_type = struct.unpack_from("<II", raw, at)
        body = raw[at + 8: at + 8 + chunk_len]
        if chunk_type == 0x4E4F534A:  # JSON
            doc = json.loads(body.decode("utf-8"))
        elif chunk_type == 0x004E4942:  # BIN
            binary = body
        at += 8 + chunk_len
    if doc is None:
        raise GltfError("glb without a JSON chunk")
    return doc, binary


def _node_matrix(node: dict) -> np.ndarray:
    if "matrix" in node:
        return np.asarray(node["matrix"], np.float64).reshape(4, 4).T  # column-major in the file
    t = np.eye(4)
    t[:3, 3] = node.get("translation", [0.0, 0.0, 0.0])
    x, y, z, w = node.get("rotation", [0.0, 0.0, 0.0, 1.0])
    r = np.eye(4)
    r[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                 [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                 [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
    s = np.diag(list(node.get("scale", [1.0, 1.0, 1.0])) + [1.0])
    return t @ r @ s


def _image_rgba(doc: dict, reader: _Reader, base: Path, texture_index: int, cache: dict) -> np.ndarray | None:
    """(h, w, 4) float32 RGBA in [0, 1] of a glTF texture (dequantize_unorm of its 8-bit
    samples), or None for an image that is not PNG."""
    source = doc["textures"][texture_index]["source"]
    if source in cache:
        return cache[source]
    img = doc["images"][source]
    if "bufferView" in img:
        view = doc["bufferViews"][img["bufferView"]]
        start = view.get("byteOffset", 0)
        data = bytes(reader.buffers[view["buffer"]][start:start + view["byteLength"]])
    elif img.get("uri", "").startswith("data:"):
        data = base64.b64decode(img["uri"].split(",", 1)[1])
    else:
        data = (base / img["uri"]).read_bytes()
    try:
        rgba = png.decode(data).astype(np.float32) / np.float32(255.0)
    except png.PngError:
        rgba = None
    cache[source] = rgba
    return rgba


def load(path: str | Path, scene: Scene | None = None) -> Import:
    """Imports the file's default scene into `scene` (a new one by default)."""
    path = Path(path)
    doc, glb_bin = _read(path)
    reader = _Reader(doc, _load_buffers(doc, path.parent, glb_bin))
    scene = scene if scene is not None else Scene()
    mesh_cache: dict[tuple[int, int], int] = {}
    material_cache: dict[int, int] = {}
    image_cache: dict[int, np.ndarray | None] = {}
    ignored = 0

    def image(info: dict | None) -> np.ndarray | None:
        nonlocal ignored
        if info is None:
            return None
        rgba = _image_rgba(doc, reader, path.parent, info["index"], image_cache)
        if rgba is None:
            ignored += 1
        return rgba

    def material(index: int | None) -> int:
        nonlocal ignored
        key = -1 if index is None else index
        if key in material_cache:
            return material_cache[key]
        src = doc["materials"][index] if index is not None else {}
        pbr = src.get("pbrMetallicRoughness", {})
        ext = src.get("extensions", {})
        m = Material()
        f32 = np.float32
        base = np.asarray(pbr.get("baseColorFactor", [1.0, 1.0, 1.0, 1.0]), f32)
        m.base_color = tuple(float(v) for v in base[:3])
        tex = image(pbr.get("baseColorTexture"))
        if tex is not None:
            m.textures["base_color"] = (base * tex)[..., :3]
        metalness = f32(pbr.get("metallicFactor", 1.0))
        roughness = f32(pbr.get("roughnessFactor", 1.0))
        m.base_metalness, m.specular_roughness = float(metalness), float(roughness)
        tex = image(pbr.get("metallicRoughnessTexture"))
        if tex is not None:
            m.textures["base_metalness"] = tex[..., 2] * metalness
            m.textures["specular_roughness"] = tex[..., 1] * roughness
        tex = image(src.get("normalTexture"))
        if tex is not None:
            m.textures["geometry_normal"] = tex[..., :3] * f32(2.0) - f32(1.0)
        emissive = np.asarray(src.get("emissiveFactor", [0.0, 0.0, 0.0]), f32)
        m.emission_color = tuple(float(v) for v in emissive)
        tex = image(src.get("emissiveTexture"))
        if tex is not None:
            m.textures["emission_color"] = emissive * tex[..., :3]
        if "KHR_materials_emissive_strength" in ext:
            m.emission_luminance = float(ext["KHR_materials_emissive_strength"].get("emissiveStrength", 1.0))
        if "KHR_materials_specular" in ext:
            spec = ext["KHR_materials_specular"]
            factor = f32(spec.get("specularFactor", 1.0))
            color = np.asarray(spec.get("specularColorFactor", [1.0, 1.0, 1.0]), f32)
            m.specular_weight = float(factor)
            m.specular_color = tuple(float(v) for v in color)
            tex = image(spec.get("specularTexture"))
            if tex is not None:
                m.textures["specular_weight"] = tex[..., 3] * factor
            tex = image(spec.get("specularColorTexture"))
            if tex is not None:
                m.textures["specular_color"] = color * tex[..., :3]
        if "KHR_materials_ior" in ext:
            m.specular_ior = float(ext["KHR_materials_ior"].get("ior", 1.5))
        if "KHR_materials_transmission" in ext:
            tr = ext["KHR_materials_transmission"]
            factor = f32(tr.get("transmissionFactor", 0.0))
            tex = image(tr.get("transmissionTexture"))
            if tex is not None:  # gltf.rs:358-365 assigns it to the specular weight
                m.textures["specular_weight"] = factor * tex[..., 0]
            else:
                m.transmission_weight = float(factor)
            m.transmission_color = tuple(1.0 - c for c in m.base_color)
            if "base_color" in m.textures:
                m.textures["transmission_color"] = f32(1.0) - m.textures["base_color"]
        material_cache[key] = scene.insert_material(m)
        return material_cache[key]

    def mesh(mi: int, pi: int) -> int:
        if (mi, pi) in mesh_cache:
            return mesh_cache[(mi, pi)]
        prim = doc["meshes"][mi]["primitives"][pi]
        if prim.get("mode", 4) != 4:
            raise GltfError("only triangle lists are supported")
        attr = prim["attributes"]
        pos = reader.accessor(attr["POSITION"], "positions", F32, "VEC3")
        uv = (reader.accessor(attr["TEXCOORD_0"], "texture coordinates", F32, "VEC2") if "TEXCOORD_0" in attr
              else np.zeros((len(pos), 2), np.float32))
        nrm = reader.accessor(attr["NORMAL"], "normals", F32, "VEC3") if "NORMAL" in attr else None
        tan = reader.accessor(attr["TANGENT"], "tangents", F32, "VEC4") if "TANGENT" in attr else None
        idx = (reader.accessor(prim["indices"], "index", (U16, U32), "SCALAR").reshape(-1).astype(np.uint32)
               if "indices" in prim else None)
        mesh_cache[(mi, pi)] = scene.insert_mesh(pos, uv, idx, nrm, tan)
        return mesh_cache[(mi, pi)]

    def node(ni: int) -> Node:
        src = doc["nodes"][ni]
        models = []
        if "mesh" in src:
            for pi, prim in enumerate(doc["meshes"][src["mesh"]]["primitives"]):
                models.append(Model(mesh(src["mesh"], pi), material(prim.get("material"))))
        return Node(transform=_node_matrix(src), models=models, children=[node(c) for c in src.get("children", [])])

    scenes = doc.get("scenes", [])
    if scenes:
        chosen = scenes[doc.get("scene", 0)]
        for ni in chosen.get("nodes", []):
            scene.root.children.append(node(ni))
    return Import(scene, len(mesh_cache), len(material_cache), ignored)
