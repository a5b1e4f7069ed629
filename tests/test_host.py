"""Host side of the boundary (CPU only): the encoders of src/asset, src/math and
src/scene.rs that produce the byte arrays tt_scene_create borrows, the camera matrices of
src/camera.rs and the Constants of Renderer::render_to_target.
"""
import numpy as np
import pytest

from tinytrace_gb300 import asset, scenes
from tinytrace_gb300.asset import Material, Model, Node, Scene
from tinytrace_gb300.camera import Camera, look_at_rh, perspective_infinite_reverse_rh
from tinytrace_gb300.renderer import Config, LightSampling, SceneArrays, flatten_scene, make_constants


def col_major(a):
    return np.asarray(a, np.float64).reshape(4, 4).T


def test_quantize_snorm_rounding():
    v = np.array([-1.0, -0.5, 0.0, 0.5, 1.0, 2.0, -2.0, 1.0 / 32767 * 0.5], np.float32)
    q = asset.quantize_snorm(v, 16)
    assert list(q[:7]) == [-32767, -16384, 0, 16384, 32767, 32767, -32767]
    assert q[7] == 1  # half away from zero


def test_quantize_unorm():
    q = asset.quantize_unorm(np.array([0.0, 1.0, 0.5, -1.0, 3.0], np.float32), 10)
    assert list(q) == [0, 1023, 512, 0, 1023]


def test_octahedron_roundtrip():
    rng = np.random.default_rng(0)
    n = rng.normal(size=(20000, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    n[:6] = [[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, -1, 0], [-1, 0, 0], [0, 1, 0]]
    d = asset.decode_octahedron(asset.encode_octahedron(n))
    assert np.max(np.linalg.norm(d - n, axis=1)) < 1e-5


def _decode_frames(frames):
    u = (frames & 1023).astype(np.float32) / 1023
    v = ((frames >> 10) & 1023).astype(np.float32) / 1023
    a = ((frames >> 20) & 2047).astype(np.float32) / 2047 * np.float32(2 * np.pi)
    sign = np.where(frames >> 31, 1.0, -1.0)
    normal = asset.decode_octahedron(np.stack([u, v], axis=1))
    ortho = asset._orthonormal(normal)
    b = np.cross(normal, ortho)
    tangent = ortho * np.cos(a)[:, None] + b * np.sin(a)[:, None]
    return normal, tangent, sign


def test_tangent_frame_encoding():
    """TangentFrame::new packs a 10+10-bit octahedral normal, an 11-bit tangent angle and a
    bitangent sign (src/asset/normal.rs:17-36); decoding recovers the frame."""
    rng = np.random.default_rng(1)
    n = rng.normal(size=(5000, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    t = np.cross(n, rng.normal(size=(5000, 3))).astype(np.float32)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    w = np.where(rng.uniform(size=5000) < 0.5, -1.0, 1.0).astype(np.float32)
    frames = asset.encode_tangent_frames(n, np.concatenate([t, w[:, None]], axis=1))
    dn, dt, ds = _decode_frames(frames.astype(np.uint64))
    assert np.max(np.degrees(np.arccos(np.clip((dn * n).sum(1), -1, 1)))) < 0.25
    assert np.max(np.degrees(np.arccos(np.clip((dt * t).sum(1), -1, 1)))) < 0.5
    assert np.array_equal(ds, w)


def test_generated_normals_of_a_sphere_are_radial():
    pts, tris = scenes.geodesic_sphere(6)
    nrm = asset.generate_normals(pts, tris)
    radial = pts / np.linalg.norm(pts, axis=1, keepdims=True)
    assert np.min((nrm * radial).sum(1)) > 0.99


def test_bounding_sphere_contains_points():
    rng = np.random.default_rng(2)
    p = rng.normal(size=(1000, 3)).astype(np.float32) * 3 + 5
    c, r = asset.bounding_sphere(p)
    assert np.all(np.linalg.norm(p - c, axis=1) <= r * (1 + 1e-6))


def test_insert_mesh_quantises_relative_to_bounding_sphere():
    s = Scene()
    pts, tris = scenes.geodesic_sphere(4)
    pts = pts * 7.0 + np.array([1.0, -2.0, 3.0])
    m = s.insert_mesh(pts.astype(np.float32), None, tris)
    me = s.mesh_array[m]
    q = s.positions[int(me["vertex_offset"]):int(me["vertex_offset"]) + len(pts)].astype(np.float64) / 32767
    back = q * float(me["radius"]) + np.asarray(me["center"], np.float64)
    assert np.max(np.abs(back - pts)) < 7.0 * 2 / 32767
    assert np.all(np.abs(s.positions) <= 32767)


def test_material_defaults_and_layout():
    c = Material().constants()
    # OpenPBR defaults (src/asset/material.rs)
    assert c["base_weight"] == 1.0 and np.allclose(c["base_color"][:3], 0.8)
    assert c["specular_weight"] == 1.0 and np.isclose(c["specular_roughness"], 0.3)
    assert np.isclose(c["specular_ior"], 1.5) and np.isclose(c["coat_ior"], 1.6)
    assert c["base_color"][3] == 0.0
    assert not Material().is_emissive() and Material(emission_luminance=1.0).is_emissive()


def test_flatten_scene_instances_and_light_hash():
    s = Scene()
    light = s.insert_material(Material(emission_luminance=5.0))
    plain = s.insert_material(Material())
    pts, tris = scenes.geodesic_sphere(2)
    m = s.insert_mesh(pts.astype(np.float32), None, tris)
    t = np.eye(4)
    t[:3, :3] *= 2.0
    t[:3, 3] = (1, 2, 3)
    s.root.children.append(Node(transform=t, models=[Model(m, light), Model(m, plain)]))
    inst, em = flatten_scene(s)
    assert len(inst) == 2 and len(em) == len(tris)
    for i in inst:
        T, Ti = col_major(i["transform"]), col_major(i["inverse_transform"])
        assert np.allclose(T @ Ti, np.eye(4), atol=1e-5)
        assert np.allclose(col_major(i["normal_transform"])[:3, :3], np.linalg.inv(t[:3, :3]).T, atol=1e-6)
    assert np.all(em["instance_index"] == 0)
    # src/asset/mod.rs:186: (index_offset / 3 + offset % u16::MAX) as u16
    io = int(s.mesh_array[m]["index_offset"])
    assert np.array_equal(em["hash"], (io // 3 + np.arange(len(tris)) % 65535) & 0xFFFF)


def test_light_hash_wraps_past_65535():
    """The host hash and the shader's `% 0xffff` disagree past 65535 triangles
    (src/asset/mod.rs:186 vs src/integrate/integrate.glsl:184); the encoder keeps the host side."""
    s = Scene()
    big = np.zeros((3 * 70000, 3), np.float32)
    big[1::3, 0] = 1.0
    big[2::3, 1] = 1.0
    s.insert_mesh(big, None, np.arange(3 * 70000, dtype=np.uint32))
    light = s.insert_material(Material(emission_luminance=1.0))
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    lm = s.insert_mesh(tri, None, np.array([0, 1, 2], np.uint32))
    s.root.children.append(Node(models=[Model(lm, light)]))
    _, em = flatten_scene(s)
    global_index = int(s.mesh_array[lm]["index_offset"]) // 3
    assert global_index == 70000
    assert int(em["hash"][0]) == global_index & 0xFFFF
    assert int(em["hash"][0]) != global_index % 0xFFFF


def test_look_at_and_projection():
    eye, center = np.array([1.0, 2.0, 3.0]), np.array([0.0, 0.0, 0.0])
    v = look_at_rh(eye, center, np.array([0.0, 1.0, 0.0]))
    assert np.allclose(v[:3, :3] @ v[:3, :3].T, np.eye(3))
    assert np.allclose(v @ np.append(eye, 1), [0, 0, 0, 1])
    d = np.linalg.norm(center - eye)
    assert np.allclose(v @ np.append(center, 1), [0, 0, -d, 1])
    p = perspective_infinite_reverse_rh(np.pi / 2, 2.0, 0.1)
    assert np.isclose(p[0, 0], 0.5) and np.isclose(p[1, 1], 1.0) and p[3, 2] == -1 and np.isclose(p[2, 3], 0.1)
    cam = Camera()
    assert cam.proj(1.0)[3, 2] == 1.0  # src/camera.rs:41-45 override


@pytest.mark.parametrize("target", [(0.0, 1.0, 0.0), (5.0, -2.0, 1.0)])
def test_camera_looking_at_centres_the_target(target):
    cam = Camera.looking_at((0.0, 1.0, 3.4), target, fov=0.75)
    d = cam.ray_direction(0.0, 0.0, 1.0)
    want = np.asarray(target) - np.asarray(cam.position)
    assert np.allclose(d, want / np.linalg.norm(want), atol=1e-6)


def test_make_constants():
    w = scenes.cornell_workload()
    c = make_constants(w.camera, (320, 200), Config(bounce_count=5, sample_count=7,
                                                    light_sampling=LightSampling.ON_HIT), 11, 3)
    assert c.nbytes == 368
    assert tuple(c["screen_size"]) == (320, 200)
    assert c["sample_count"] == 7 and c["bounce_count"] == 5 and c["frame_index"] == 11
    assert c["accumulated_frame_count"] == 3 and c["light_sampling"] == int(LightSampling.ON_HIT)
    assert np.allclose(col_major(c["inverse_view"]) @ col_major(c["view"]), np.eye(4), atol=1e-5)
    assert np.allclose(col_major(c["proj"]) @ col_major(c["view"]), col_major(c["proj_view"]), atol=1e-5)


def test_generators_are_seeded():
    a = SceneArrays(scenes.icosphere_field(instances=3, freq=4, lights=5, seed=1))
    b = SceneArrays(scenes.icosphere_field(instances=3, freq=4, lights=5, seed=1))
    c = SceneArrays(scenes.icosphere_field(instances=3, freq=4, lights=5, seed=2))
    assert a.positions.tobytes() == b.positions.tobytes()
    assert a.instances.tobytes() == b.instances.tobytes()
    assert a.instances.tobytes() != c.instances.tobytes()


def test_benchmark_scene_shape():
    """The 1M-triangle scene: 64 displaced icospheres of 15,680 triangles and 1000 lights."""
    pts, tris = scenes.geodesic_sphere(28)
    assert len(tris) == 20 * 28 * 28
    assert 64 * len(tris) + 1000 == 1_004_520
