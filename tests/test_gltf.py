"""The glTF importer (tinytrace_gb300/gltf.py) on files written by the test: external .bin,
base64 data URIs and .glb containers give the same scene; materials, node transforms and
attribute formats follow the reference importer's mapping (src/asset/gltf.rs); the imported
scene renders in the oracle."""
import base64
import json
import struct
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from tinytrace_gb300 import asset, gltf
from tinytrace_gb300.camera import Camera
from tinytrace_gb300.renderer import Config, SceneArrays, flatten_scene, make_constants

def _png_rgba(img: np.ndarray) -> bytes:
    """A minimal RGBA8 PNG (filter 0) of an (h, w, 4) uint8 image."""
    import zlib

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)

    h, w = img.shape[:2]
    raw = b"".join(b"\0" + img[y].tobytes() for y in range(h))
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))


IMAGE = np.random.default_rng(3).integers(0, 256, (8, 8, 4)).astype(np.uint8)

QUAD_POS = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], np.float32)
QUAD_IDX = np.array([0, 2, 1, 0, 3, 2], np.uint16)
TRI_POS = np.array([[0, 0, 0], [0.5, 0, 0], [0, 0, 0.5]], np.float32)


def _doc(uri):
    """Two meshes: a floor quad (u16 indices, normals) and a light triangle (no indices);
    nodes: floor at the origin, light under a parent with TRS."""
    binary = QUAD_POS.tobytes() + QUAD_IDX.tobytes() + TRI_POS.tobytes()
    normals = np.tile(np.array([[0, 1, 0]], np.float32), (4, 1)).tobytes()
    binary += normals
    doc = {
        "asset": {"version": "2.0"},
        "buffers": [{"byteLength": len(binary)} | ({"uri": uri} if uri else {})],
        "bufferViews": [
            {"buffer": 0, "byteOffset": 0, "byteLength": 48},
            {"buffer": 0, "byteOffset": 48, "byteLength": 12},
            {"buffer": 0, "byteOffset": 60, "byteLength": 36},
            {"buffer": 0, "byteOffset": 96, "byteLength": 48},
        ],
        "accessors": [
            {"bufferView": 0, "componentType": 5126, "count": 4, "type": "VEC3"},
            {"bufferView": 1, "componentType": 5123, "count": 6, "type": "SCALAR"},
            {"bufferView": 2, "componentType": 5126, "count": 3, "type": "VEC3"},
            {"bufferView": 3, "componentType": 5126, "count": 4, "type": "VEC3"},
        ],
        "materials": [
            {"pbrMetallicRoughness": {"baseColorFactor": [0.6, 0.5, 0.4, 1.0], "metallicFactor": 0.0,
                                      "roughnessFactor": 0.7},
             "extensions": {"KHR_materials_ior": {"ior": 1.33},
                            "KHR_materials_specular": {"specularFactor": 0.5, "specularColorFactor": [1, 0.9, 0.8]}}},
            {"emissiveFactor": [1.0, 0.9, 0.8], "pbrMetallicRoughness": {"metallicFactor": 0.0},
             "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 30.0}}},
            {"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.4, 0.6, 1.0],
                                      "baseColorTexture": {"index": 0},
                                      "metallicRoughnessTexture": {"index": 0}, "roughnessFactor": 0.5},
             "normalTexture": {"index": 0},
             "extensions": {"KHR_materials_transmission": {"transmissionFactor": 0.5}}},
        ],
        "images": [{"uri": "data:image/png;base64," + base64.b64encode(_png_rgba(IMAGE)).decode()}],
        "textures": [{"source": 0}],
        "meshes": [
            {"primitives": [{"attributes": {"POSITION": 0, "NORMAL": 3}, "indices": 1, "material": 0}]},
            {"primitives": [{"attributes": {"POSITION": 2}, "material": 1},
                            {"attributes": {"POSITION": 2}, "material": 2}]},
        ],
        "nodes": [
            {"mesh": 0},
            {"translation": [0.0, 1.5, 0.0], "children": [2]},
            {"mesh": 1, "rotation": [1.0, 0.0, 0.0, 0.0], "scale": [2.0, 2.0, 2.0]},
        ],
        "scenes": [{"nodes": [0, 1]}],
        "scene": 0,
    }
    return doc, binary


def _write(tmp_path: Path, kind: str) -> Path:
    if kind == "bin":
        doc, binary = _doc("scene.bin")
        (tmp_path / "scene.bin").write_bytes(binary)
        p = tmp_path / "scene.gltf"
        p.write_text(json.dumps(doc))
    elif kind == "data":
        doc, binary = _doc(None)
        doc["buffers"][0]["uri"] = "data:application/octet-stream;base64," + base64.b64encode(binary).decode()
        p = tmp_path / "scene_data.gltf"
        p.write_text(json.dumps(doc))
    else:
        doc, binary = _doc(None)
        js = json.dumps(doc).encode()
        js += b" " * (-len(js) % 4)
        binary += b"\0" * (-len(binary) % 4)
        body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(binary), 0x004E4942) + binary
        p = tmp_path / "scene.glb"
        p.write_bytes(b"glTF" + struct.pack("<II", 2, 12 + len(body)) + body)
    return p


@pytest.mark.parametrize("kind", ["bin", "data", "glb"])
def test_import(tmp_path, kind):
    imp = gltf.load(_write(tmp_path, kind))
    s = imp.scene
    assert imp.meshes == 3 and imp.materials == 3 and imp.ignored_textures == 0  # (mesh, primitive) pairs
    mats = s.material_array["constants"]
    assert np.allclose(mats[0]["base_color"][:3], [0.6, 0.5, 0.4]) and np.isclose(mats[0]["specular_roughness"], 0.7)
    assert np.isclose(mats[0]["specular_ior"], 1.33) and np.isclose(mats[0]["specular_weight"], 0.5)
    assert np.isclose(mats[1]["emission_luminance"], 30.0) and np.allclose(mats[1]["emission_color"][:3], [1, 0.9, 0.8])
    assert np.isclose(mats[1]["specular_roughness"], 1.0)  # glTF default roughness
    assert np.isclose(mats[2]["transmission_weight"], 0.5)
    # textured parameters: constants zero, textures processed (gltf.rs:259-305)
    assert np.array_equal(mats[2]["base_color"], [0, 0, 0, 0]) and mats[2]["base_metalness"] == 0.0
    slots = s.material_array["textures"][2]
    from tinytrace_gb300 import texture
    used = {texture.SLOTS[k] for k in range(27) if slots[k] != 0xFFFFFFFF}
    assert used == {"base_color", "base_metalness", "specular_roughness", "geometry_normal", "transmission_color"}
    assert len(s.textures) == 5
    t = s.textures[slots[texture.SLOTS.index("specular_roughness")]]
    assert t.format == texture.TT_TEXTURE_R8_UNORM and (t.width, t.height) == (8, 8)
    g = IMAGE[..., 1].astype(np.float32) / np.float32(255) * np.float32(0.5)
    assert t.levels[0] == asset.quantize_unorm(g, 8).astype(np.uint8).tobytes()
    instances, emissive = flatten_scene(s)
    assert len(instances) == 3 and len(emissive) == 1
    # the light triangle: parent translation (0, 1.5, 0) * rotation of 180 degrees about x * scale 2
    t = np.asarray(instances[1]["transform"], np.float64).reshape(4, 4).T
    me = s.mesh_array[1]
    p = (TRI_POS[1] - me["center"]) / me["radius"]
    world = t @ np.append(p, 1.0)
    assert np.allclose(world[:3], [1.0, 1.5, 0.0], atol=1e-3)


def test_all_containers_give_the_same_arrays(tmp_path):
    arrs = [SceneArrays(gltf.load(_write(tmp_path, k)).scene) for k in ("bin", "data", "glb")]
    for a in arrs[1:]:
        for f in SceneArrays.FIELDS:
            assert getattr(a, f).tobytes() == getattr(arrs[0], f).tobytes(), f


def test_bad_formats(tmp_path):
    doc, binary = _doc("scene.bin")
    (tmp_path / "scene.bin").write_bytes(binary)
    doc["accessors"][1]["componentType"] = 5121  # u8 indices: rejected like the reference
    (tmp_path / "bad.gltf").write_text(json.dumps(doc))
    with pytest.raises(gltf.GltfError):
        gltf.load(tmp_path / "bad.gltf")


def test_imported_scene_renders(tmp_path):
    s = gltf.load(_write(tmp_path, "bin")).scene
    arrays = SceneArrays(s)
    cam = Camera.looking_at((0.0, 3.0, 4.0), (0.0, 0.0, 0.0), fov=0.9)
    img = oracle.OracleScene(arrays).render(make_constants(cam, (32, 24), Config(bounce_count=3, sample_count=4), 0, 0))
    assert np.isfinite(img).all() and img[..., :3].max() > 0.0


REFERENCE_CORNELL = Path(__file__).resolve().parent / "golden" / "cornell_box.gltf"
FIXTURE_SHA256 = {"cornell_box.gltf": "a15d11edadb3ff1c975bf22da50fa01b49075e48ae2507c1d8053abebe509012",
                  "cornell_box.bin": "4bd62cf514d12da6801612a5b4b126967488715f634872c45a0c22f45f9cc5f1"}


def test_reference_cornell_fixture():
    """The reference's own Cornell box (scenes/cornell_box.gltf + .bin, committed unchanged by
    tests/golden/copy_reference_gltf.py) imports with its 32 triangles, its two emissive
    triangles of strength 40 and its metal material (src/asset/gltf.rs:50-122, 242-383)."""
    import hashlib

    for name, digest in FIXTURE_SHA256.items():
        assert hashlib.sha256((REFERENCE_CORNELL.parent / name).read_bytes()).hexdigest() == digest, name
    imp = gltf.load(REFERENCE_CORNELL)
    arrays = SceneArrays(imp.scene)
    assert arrays.triangle_count == 32 and len(arrays.emissive) == 2
    mats = arrays.materials["constants"]
    assert np.isclose(mats["emission_luminance"].max(), 40.0) and mats["base_metalness"].max() == 1.0
