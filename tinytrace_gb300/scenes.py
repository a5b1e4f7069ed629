"""Seeded synthetic scenes for tests and benchmarks, built through the asset pipeline
(`asset.Scene.insert_mesh` / `insert_material`, i.e. snorm16 positions and packed tangent
frames as the reference stores them).

* `cornell_box()` — the procedural Cornell box: five axis-aligned wall quads and two boxes
  (34 triangles) plus one ceiling light quad (2 triangles) of radiance 15; Lambertian
  OpenPBR base colours red/green/white 0.7 (specular weight 0).
* `textured_cornell()` — the Cornell box with every texture format in use (see below).
* `icosphere_field()` — 64 instances of a geodesic sphere (frequency 28: 15,680 triangles)
  with seeded fractal (sum-of-sinusoids) radial displacement of amplitude 0.1, uniform random
  rotations, translations in a 100^3 box and scales in [4, 12]; OpenPBR metalness U{0,1} and
  specular roughness U[0.05, 1]; 1000 emissive triangles whose power P ~ LogNormal(0, 1)
  gives luminance 100 P / (pi A).  Light meshes come first in the index buffer so that the
  reference's 16-bit light hash identifies them exactly.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .asset import Material, Model, Node
from .asset import Scene as AssetScene
from .camera import Camera
from .renderer import Config, LightSampling


@dataclass
class Workload:
    name: str
    scene: AssetScene
    camera: Camera
    extent: tuple
    config: Config


def _quad(a, b, c, d):
    """Two triangles (a,b,c), (a,c,d); counter-clockwise seen from the front side."""
    pos = np.array([a, b, c, d], np.float32)
    n = np.cross(pos[1] - pos[0], pos[2] - pos[0])
    n = n / np.linalg.norm(n)
    normals = np.repeat(n[None], 4, 0).astype(np.float32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    return pos, np.array([0, 1, 2, 0, 2, 3], np.uint32), normals, uv


def _box(lo, hi, angle):
    """Axis-aligned box rotated about +y by `angle`, outward faces, 12 triangles."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    c = (lo + hi) / 2
    corners = np.array([[x, y, z] for z in (lo[2], hi[2]) for y in (lo[1], hi[1]) for x in (lo[0], hi[0])])
    ca, sa = np.cos(angle), np.sin(angle)
    rot = np.array([[ca, 0, sa], [0, 1, 0], [-sa, 0, ca]])
    corners = (corners - c) @ rot.T + c
    faces = [(0, 2, 3, 1), (4, 5, 7, 6), (0, 1, 5, 4), (2, 6, 7, 3), (0, 4, 6, 2), (1, 3, 7, 5)]
    pos, idx, nrm, uv = [], [], [], []
    for f in faces:
        p, i, n, u = _quad(*corners[list(f)])
        # make the quad face outward
        if np.dot(n[0], p.mean(0) - c) < 0:
            p, i, n, u = _quad(*corners[list(f)][::-1])
        idx.append(i + 4 * len(pos))
        pos.append(p)
        nrm.append(n)
        uv.append(u)
    return np.concatenate(pos), np.concatenate(idx), np.concatenate(nrm), np.concatenate(uv)


def lambertian(color) -> Material:
    return Material(base_color=tuple(float(c) for c in color), specular_weight=0.0)


def cornell_box(light_radiance: float = 15.0) -> AssetScene:
    s = AssetScene()
    white = s.insert_material(lambertian((0.7, 0.7, 0.7)))
    red = s.insert_material(lambertian((0.7, 0.05, 0.05)))
    green = s.insert_material(lambertian((0.05, 0.7, 0.05)))
    light = s.insert_material(Material(base_color=(0.7, 0.7, 0.7), specular_weight=0.0,
                                       emission_luminance=light_radiance, emission_color=(1.0, 1.0, 1.0)))
    items = []
    # light first: its triangles get the smallest global indices
    items.append((_quad((-0.25, 1.98, -0.25), (0.25, 1.98, -0.25), (0.25, 1.98, 0.25), (-0.25, 1.98, 0.25)), light))  # -y
    items.append((_quad((-1, 0, 1), (1, 0, 1), (1, 0, -1), (-1, 0, -1)), white))       # floor, +y
    items.append((_quad((-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1)), white))       # ceiling, -y
    items.append((_quad((-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1)), white))     # back, +z
    items.append((_quad((-1, 0, 1), (-1, 0, -1), (-1, 2, -1), (-1, 2, 1)), red))       # left, +x
    items.append((_quad((1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1)), green))         # right, -x
    items.append((_box((-0.65, 0.0, -0.6), (-0.05, 1.2, 0.0), 0.3), white))            # tall box
    items.append((_box((0.1, 0.0, 0.0), (0.7, 0.6, 0.6), -0.3), white))                # short box
    for (pos, idx, nrm, uv), mat in items:
        m = s.insert_mesh(pos, uv, idx, nrm)
        s.root.children.append(Node(models=[Model(m, mat)]))
    return s


def _checker(h: int, w: int, cells: int, a, b) -> np.ndarray:
    y, x = np.mgrid[0:h, 0:w]
    m = ((x * cells // w + y * cells // h) % 2).astype(bool)
    return np.where(m[..., None], np.asarray(a, np.float32), np.asarray(b, np.float32)).astype(np.float32)


def textured_cornell(seed: int = 5) -> AssetScene:
    """The Cornell box with textured materials covering every texture format and the slots
    the renderer samples: a BC1 checker base colour and an R8 roughness ramp on the floor
    (texture coordinates repeating 4 x), a BC5 normal map (seeded bumps) on the back wall, an
    R8 metalness stripe texture of odd extent (22 x 38, partial blocks) on the tall box, and an
    emissive light with BC1 colour and R16F luminance textures."""
    rng = np.random.default_rng(seed)
    s = AssetScene()
    white = s.insert_material(lambertian((0.7, 0.7, 0.7)))
    red = s.insert_material(lambertian((0.7, 0.05, 0.05)))
    green = s.insert_material(lambertian((0.05, 0.7, 0.05)))
    floor = s.insert_material(Material(specular_weight=1.0, textures={
        "base_color": _checker(256, 256, 8, (0.8, 0.75, 0.7), (0.15, 0.2, 0.3)),
        "specular_roughness": np.tile(np.linspace(0.1, 0.9, 64, dtype=np.float32), (64, 1)),
    }))
    yy, xx = np.mgrid[0:64, 0:64] / 64.0
    bumps = np.stack([0.3 * np.sin(2 * np.pi * 4 * xx + rng.uniform(0, 6)),
                      0.3 * np.cos(2 * np.pi * 3 * yy + rng.uniform(0, 6)), np.ones_like(xx)], -1)
    bumps /= np.linalg.norm(bumps, axis=-1, keepdims=True)
    back = s.insert_material(Material(base_color=(0.6, 0.6, 0.6), specular_weight=0.5,
                                       textures={"geometry_normal": bumps.astype(np.float32)}))
    stripes = ((np.arange(22)[None, :] // 3 + np.arange(38)[:, None] // 5) % 2).astype(np.float32)
    metal = s.insert_material(Material(base_color=(0.9, 0.6, 0.3), specular_roughness=0.35,
                                       textures={"base_metalness": stripes}))
    lum = (10.0 + 20.0 * rng.random((16, 16))).astype(np.float32)
    light = s.insert_material(Material(base_color=(0.7, 0.7, 0.7), specular_weight=0.0, textures={
        "emission_color": _checker(32, 32, 4, (1.0, 0.9, 0.7), (0.7, 0.8, 1.0)),
        "emission_luminance": lum,
    }))
    items = []
    items.append((_quad((-0.25, 1.98, -0.25), (0.25, 1.98, -0.25), (0.25, 1.98, 0.25), (-0.25, 1.98, 0.25)), light))
    items.append((_quad((-1, 0, 1), (1, 0, 1), (1, 0, -1), (-1, 0, -1)), floor, 4.0))
    items.append((_quad((-1, 2, -1), (1, 2, -1), (1, 2, 1), (-1, 2, 1)), white))
    items.append((_quad((-1, 0, -1), (1, 0, -1), (1, 2, -1), (-1, 2, -1)), back))
    items.append((_quad((-1, 0, 1), (-1, 0, -1), (-1, 2, -1), (-1, 2, 1)), red))
    items.append((_quad((1, 0, -1), (1, 0, 1), (1, 2, 1), (1, 2, -1)), green))
    items.append((_box((-0.65, 0.0, -0.6), (-0.05, 1.2, 0.0), 0.3), metal))
    items.append((_box((0.1, 0.0, 0.0), (0.7, 0.6, 0.6), -0.3), white))
    for item in items:
        (pos, idx, nrm, uv), mat = item[0], item[1]
        scale = item[2] if len(item) > 2 else 1.0
        tangents = None
        if mat == back:  # tangent along +x for the normal map
            tangents = np.tile(np.array([1.0, 0.0, 0.0, 1.0], np.float32), (len(pos), 1))
        m = s.insert_mesh(pos, uv * np.float32(scale), idx, nrm, tangents)
        s.root.children.append(Node(models=[Model(m, mat)]))
    return s


def late_lights(freq: int = 60, lights: int = 6) -> AssetScene:
    """A sphere of 20 freq^2 triangles (72,000 at freq 60) inserted before `lights` emissive
    triangles, so that every light triangle has a global index >= 65535: the reference's 16-bit
    light hash (src/asset/mod.rs:186 against src/integrate/integrate.glsl:184) then never
    matches and next-event estimation sees no light, unless visibility tests the sampled
    triangle itself (TT_LIGHT_VISIBILITY_TRIANGLE)."""
    s = AssetScene()
    pts, tris = geodesic_sphere(freq)
    body = s.insert_material(Material(base_color=(0.7, 0.7, 0.7), specular_roughness=0.6))
    m = s.insert_mesh(pts.astype(np.float32), None, tris)
    s.root.children.append(Node(models=[Model(m, body)]))
    for k in range(lights):
        a = 2.0 * np.pi * k / lights
        c = np.array([2.5 * np.cos(a), 2.5, 2.5 * np.sin(a)])
        tri = np.array([c + [-0.4, 0.0, -0.4], c + [0.4, 0.0, -0.4], c + [0.4, 0.0, 0.4]], np.float32)  # faces -y
        mat = s.insert_material(Material(emission_luminance=20.0, emission_color=(1.0, 0.9, 0.8)))
        lm = s.insert_mesh(tri, None, np.array([0, 1, 2], np.uint32), np.tile([0.0, -1.0, 0.0], (3, 1)))
        s.root.children.append(Node(models=[Model(lm, mat)]))
    return s


def cornell_workload(extent=(256, 256), spp: int = 16, depth: int = 4) -> Workload:
    cam = Camera.looking_at((0.0, 1.0, 3.4), (0.0, 1.0, 0.0), fov=0.75)
    cfg = Config(bounce_count=depth, sample_count=spp, tonemap=True,
                 light_sampling=LightSampling.NEXT_EVENT_ESTIMATION)
    return Workload("cornell_box_256x256_16spp_d4", cornell_box(), cam, tuple(extent), cfg)


# ---------------------------------------------------------------- icosphere field
def geodesic_sphere(freq: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit geodesic sphere: each icosahedron face split into freq^2 triangles."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                  [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    pts, tris = [], []
    for a, b, c in faces:
        A, B, C = v[a], v[b], v[c]
        base = len(pts)
        ids = {}
        for i in range(freq + 1):
            for j in range(freq + 1 - i):
                p = A + (B - A) * (i / freq) + (C - A) * (j / freq)
                ids[(i, j)] = len(pts)
                pts.append(p)
        for i in range(freq):
            for j in range(freq - i):
                tris.append((ids[(i, j)], ids[(i + 1, j)], ids[(i, j + 1)]))
                if j < freq - i - 1:
                    tris.append((ids[(i + 1, j)], ids[(i + 1, j + 1)], ids[(i, j + 1)]))
        del base
    pts = np.array(pts)
    pts /= np.linalg.norm(pts, axis=1, keepdims=True)
    # weld shared edge vertices
    key = np.round(pts * 1e6).astype(np.int64)
    _, first, inverse = np.unique(key, axis=0, return_index=True, return_inverse=True)
    tris = inverse.reshape(-1)[np.array(tris)]
    pts = pts[first]
    # outward winding
    p0, p1, p2 = pts[tris[:, 0]], pts[tris[:, 1]], pts[tris[:, 2]]
    flip = np.einsum("ij,ij->i", np.cross(p1 - p0, p2 - p0), p0) < 0
    tris[flip] = tris[flip][:, ::-1]
    return pts, tris.astype(np.uint32)


def _fbm(p: np.ndarray, rng: np.random.Generator, octaves: int = 5) -> np.ndarray:
    out = np.zeros(len(p))
    amp, freq, norm = 1.0, 2.0, 0.0
    for _ in range(octaves):
        for _ in range(3):
            k = rng.normal(size=3)
            k /= np.linalg.norm(k)
            out += amp * np.sin(freq * (p @ k) + rng.uniform(0, 2 * np.pi))
            norm += amp
        amp *= 0.5
        freq *= 2.0
    return out / norm


def _random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _sphere_textures(rng: np.random.Generator, base_color, size: int = 256) -> dict:
    """Procedural textures of one textured sphere material: a BC1 base colour (stripes of the
    material's colour and a random second colour), an R8 roughness noise and, for half of the
    materials, a BC5 bump normal map."""
    y, x = np.mgrid[0:size, 0:size] / size
    k = rng.integers(2, 9, 2)
    stripes = (np.sin(2 * np.pi * (k[0] * x + k[1] * y)) > 0)[..., None]
    other = rng.uniform(0.1, 0.9, 3)
    tex = {"base_color": np.where(stripes, np.asarray(base_color), other).astype(np.float32)}
    rough = 0.5 + 0.45 * np.sin(2 * np.pi * (rng.integers(1, 6) * x)) * np.cos(2 * np.pi * rng.integers(1, 6) * y)
    tex["specular_roughness"] = rough[::2, ::2].astype(np.float32)
    if rng.random() < 0.5:
        n = np.stack([0.3 * np.sin(2 * np.pi * 6 * x), 0.3 * np.sin(2 * np.pi * 6 * y), np.ones_like(x)], -1)
        tex["geometry_normal"] = (n / np.linalg.norm(n, axis=-1, keepdims=True))[::2, ::2].astype(np.float32)
    return tex


def icosphere_field(instances: int = 64, freq: int = 28, lights: int = 1000, seed: int = 7,
                    box: float = 100.0, displacement: float = 0.1, textured: bool = False) -> AssetScene:
    """`textured`: every sphere's material also samples textures (_sphere_textures, from a
    separate generator, so the geometry and constants are those of the untextured field)."""
    rng = np.random.default_rng(seed)
    tex_rng = np.random.default_rng(seed + 1000)
    s = AssetScene()
    half = box / 2.0
    # emissive triangles first (global triangle index < 65535)
    for _ in range(lights):
        power = float(rng.lognormal(0.0, 1.0))
        size = rng.uniform(1.0, 3.0)
        tri = rng.normal(size=(3, 3))
        tri = tri / np.linalg.norm(tri, axis=1, keepdims=True) * size
        area = 0.5 * np.linalg.norm(np.cross(tri[1] - tri[0], tri[2] - tri[0]))
        lum = 100.0 * power / (np.pi * max(area, 1e-3))
        mat = s.insert_material(Material(base_color=(0.8, 0.8, 0.8), emission_luminance=lum,
                                         emission_color=tuple(rng.uniform(0.6, 1.0, 3))))
        m = s.insert_mesh(tri.astype(np.float32), np.zeros((3, 2), np.float32), np.array([0, 1, 2], np.uint32))
        t = np.eye(4)
        t[:3, 3] = rng.uniform(-half, half, 3)
        s.root.children.append(Node(transform=t, models=[Model(m, mat)]))
    base_pts, tris = geodesic_sphere(freq)
    for _ in range(instances):
        disp = 1.0 + displacement * _fbm(base_pts, rng)
        pts = (base_pts * disp[:, None]).astype(np.float32)
        uv = np.stack([np.arctan2(base_pts[:, 2], base_pts[:, 0]) / (2 * np.pi) + 0.5,
                       np.arccos(np.clip(base_pts[:, 1], -1, 1)) / np.pi], axis=1).astype(np.float32)
        m = s.insert_mesh(pts, uv, tris)
        material = Material(base_color=tuple(rng.uniform(0.2, 0.9, 3)), base_metalness=float(rng.integers(0, 2)),
                            specular_roughness=float(rng.uniform(0.05, 1.0)))
        if textured:
            material.textures = _sphere_textures(tex_rng, material.base_color)
        mat = s.insert_material(material)
        t = np.eye(4)
        t[:3, :3] = _random_rotation(rng) * rng.uniform(4.0, 12.0)
        t[:3, 3] = rng.uniform(-half, half, 3)
        s.root.children.append(Node(transform=t, models=[Model(m, mat)]))
    return s


def instanced_spheres(copies: int = 40, freq: int = 6, seed: int = 3, box: float = 20.0) -> AssetScene:
    """One displaced sphere mesh placed `copies` times with overlapping world boxes (rotated,
    scaled and mirrored transforms) and one emissive triangle: the instancing case."""
    rng = np.random.default_rng(seed)
    s = AssetScene()
    light = s.insert_material(Material(emission_luminance=50.0))
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    lm = s.insert_mesh(tri, np.zeros((3, 2), np.float32), np.array([0, 1, 2], np.uint32))  # faces -y
    t = np.eye(4)
    t[:3, :3] *= 3.0
    t[:3, 3] = (0.0, box, 0.0)
    s.root.children.append(Node(transform=t, models=[Model(lm, light)]))
    base_pts, tris = geodesic_sphere(freq)
    pts = (base_pts * (1.0 + 0.1 * _fbm(base_pts, rng))[:, None]).astype(np.float32)
    m = s.insert_mesh(pts, None, tris)
    mat = s.insert_material(Material(base_color=(0.7, 0.6, 0.5), specular_roughness=0.4))
    for k in range(copies):
        t = np.eye(4)
        t[:3, :3] = _random_rotation(rng) * rng.uniform(1.0, 4.0)
        if k % 7 == 3:
            t[:3, 0] *= -1.0  # mirrored instance: flips the triangle winding
        t[:3, 3] = rng.uniform(-box / 2, box / 2, 3)
        s.root.children.append(Node(transform=t, models=[Model(m, mat)]))
    return s


def restir_field(instances: int = 128, freq: int = 28, light_meshes: int = 100, triangles_per_light: int = 1000,
                 seed: int = 9, box: float = 100.0, displacement: float = 0.1) -> AssetScene:
    """The many-light scene of the ReSTIR workload: `instances` displaced icospheres (128 x
    15,680 = 2.0 M triangles at the defaults) and light_meshes x triangles_per_light emissive
    triangles scattered through the box (100 k at the defaults), one emissive material per light
    mesh with power ~ LogNormal(0, 1)."""
    rng = np.random.default_rng(seed)
    s = AssetScene()
    half = box / 2.0
    for _ in range(light_meshes):
        n = triangles_per_light
        centers = rng.uniform(-half, half, (n, 1, 3))
        tri = rng.normal(size=(n, 3, 3))
        tri = tri / np.linalg.norm(tri, axis=2, keepdims=True) * rng.uniform(0.3, 1.0, (n, 1, 1))
        pts = (centers + tri).reshape(-1, 3).astype(np.float32)
        area = 0.5 * np.linalg.norm(np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]), axis=1).mean()
        lum = 100.0 * float(rng.lognormal(0.0, 1.0)) / (np.pi * max(area, 1e-3) * n) * 50.0
        mat = s.insert_material(Material(base_color=(0.8, 0.8, 0.8), emission_luminance=lum,
                                         emission_color=tuple(rng.uniform(0.6, 1.0, 3))))
        m = s.insert_mesh(pts, np.zeros((len(pts), 2), np.float32), np.arange(len(pts), dtype=np.uint32))
        s.root.children.append(Node(models=[Model(m, mat)]))
    base_pts, tris = geodesic_sphere(freq)
    for _ in range(instances):
        disp = 1.0 + displacement * _fbm(base_pts, rng)
        pts = (base_pts * disp[:, None]).astype(np.float32)
        m = s.insert_mesh(pts, None, tris)
        mat = s.insert_material(Material(base_color=tuple(rng.uniform(0.2, 0.9, 3)),
                                         base_metalness=float(rng.integers(0, 2)),
                                         specular_roughness=float(rng.uniform(0.05, 1.0))))
        t = np.eye(4)
        t[:3, :3] = _random_rotation(rng) * rng.uniform(4.0, 12.0)
        t[:3, 3] = rng.uniform(-half, half, 3)
        s.root.children.append(Node(transform=t, models=[Model(m, mat)]))
    return s


def icosphere_workload(extent=(1920, 1080), spp: int = 64, depth: int = 8, **kw) -> Workload:
    cam = Camera.looking_at((0.0, 10.0, 95.0), (0.0, 0.0, 0.0), fov=np.pi / 2.0)
    cfg = Config(bounce_count=depth, sample_count=spp, tonemap=True,
                 light_sampling=LightSampling.NEXT_EVENT_ESTIMATION)
    name = f"icosphere_field_{kw.get('instances', 64)}x{20 * kw.get('freq', 28) ** 2}tri_{extent[0]}x{extent[1]}_{spp}spp_d{depth}"
    return Workload(name, icosphere_field(**kw), cam, tuple(extent), cfg)
