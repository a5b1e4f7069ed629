"""Seeded OpenPBR material constants covering every lobe, for the BSDF parity tests, and a scene
of spheres in those materials for the render parity tests."""
import numpy as np

from tinytrace_gb300.asset import Material


def material_suite(seed: int = 3, count: int = 24) -> list:
    return [m.constants() for m in material_objects(seed, count)]


def material_objects(seed: int = 3, count: int = 24) -> list:
    rng = np.random.default_rng(seed)
    mats = [
        Material(),  # reference defaults: dielectric base + specular
        Material(specular_weight=0.0),  # Lambertian
        Material(base_metalness=1.0, specular_roughness=0.2),  # metal (Cornell fixture's metal)
        Material(base_diffuse_roughness=0.7, specular_roughness=0.6),
        Material(transmission_weight=1.0, specular_roughness=0.1),
        Material(coat_weight=1.0, coat_roughness=0.2, specular_roughness=0.5),
        Material(fuzz_weight=1.0, fuzz_roughness=0.4),
        Material(specular_ior=1.0, transmission_weight=0.5),  # IOR == 1 transmission branch
        Material(specular_roughness_anisotropy=0.8, specular_rotation=0.3, specular_roughness=0.4),
    ]
    for _ in range(count):
        mats.append(Material(
            base_weight=float(rng.uniform(0.2, 1.0)),
            base_color=tuple(rng.uniform(0.0, 1.0, 3)),
            base_metalness=float(rng.choice([0.0, 1.0, rng.uniform()])),
            base_diffuse_roughness=float(rng.uniform()),
            specular_weight=float(rng.uniform(0.0, 1.0)),
            specular_color=tuple(rng.uniform(0.5, 1.0, 3)),
            specular_roughness=float(rng.uniform(0.02, 1.0)),
            specular_roughness_anisotropy=float(rng.choice([0.0, rng.uniform()])),
            specular_ior=float(rng.uniform(1.1, 2.5)),
            specular_rotation=float(rng.choice([0.0, rng.uniform()])),
            transmission_weight=float(rng.choice([0.0, rng.uniform()])),
            transmission_color=tuple(rng.uniform(0.5, 1.0, 3)),
            transmission_depth=float(rng.choice([0.0, 1.0])),
            coat_weight=float(rng.choice([0.0, rng.uniform()])),
            coat_color=tuple(rng.uniform(0.5, 1.0, 3)),
            coat_roughness=float(rng.uniform(0.0, 0.7)),
            coat_roughness_anisotropy=float(rng.choice([0.0, rng.uniform()])),
            coat_ior=float(rng.uniform(1.2, 2.0)),
            coat_darkening=float(rng.uniform()),
            coat_rotation=float(rng.choice([0.0, rng.uniform()])),
            fuzz_weight=float(rng.choice([0.0, rng.uniform()])),
            fuzz_color=tuple(rng.uniform(0.5, 1.0, 3)),
            fuzz_roughness=float(rng.uniform()),
        ))
    return mats


def random_directions(rng, n: int) -> np.ndarray:
    v = rng.normal(size=(n, 3)).astype(np.float32)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v.astype(np.float32)


def eval_samples(rng, n: int) -> np.ndarray:
    """n x 8 floats: wi xyz, generator state bits, wo xyz, 0 (tt_bsdf_eval_batch layout)."""
    s = np.zeros((n, 8), np.float32)
    wi = random_directions(rng, n)
    wi[: n // 2, 2] = np.abs(wi[: n // 2, 2])  # half of the incident directions above the surface
    s[:, 0:3] = wi
    seeds = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    seeds[: n // 8] = 0  # the reference harness uses Generator(0)
    s[:, 3] = seeds.view(np.float32)
    s[:, 4:7] = random_directions(rng, n)
    return s


def sample_samples(rng, n: int) -> np.ndarray:
    s = np.zeros((n, 4), np.float32)
    wi = random_directions(rng, n)
    wi[: 3 * n // 4, 2] = np.abs(wi[: 3 * n // 4, 2])
    s[:, 0:3] = wi
    s[:, 3] = rng.integers(1, 2**32, n, dtype=np.uint64).astype(np.uint32).view(np.float32)
    return s


def material_spheres():
    """Spheres in every material of the BSDF suite (coat, fuzz, glass, partly transmissive,
    anisotropic, random mixtures) plus, carrying the most triangles, fully metallic, opaque
    dielectric and half-metallic spheres: the three largest hit buckets (the wavefront shade
    kernel's, ReSTIR's candidate pass's) then run the metal, dielectric and metal + dielectric
    lobe sets, and the bucket that takes all other materials runs all six lobes."""
    from tinytrace_gb300 import scenes
    from tinytrace_gb300.asset import Model, Node
    from tinytrace_gb300.asset import Scene as AssetScene

    s = AssetScene()
    light = s.insert_material(Material(emission_luminance=12.0, emission_color=(1.0, 0.95, 0.9)))
    lq = scenes._quad((-3, 5, -3), (3, 5, -3), (3, 5, 3), (-3, 5, 3))  # facing -y, onto the spheres
    s.root.children.append(Node(models=[Model(s.insert_mesh(lq[0], lq[3], lq[1], lq[2]), light)]))
    floor = s.insert_material(Material(base_color=(0.6, 0.6, 0.55), specular_roughness=0.5))
    g = scenes._quad((-8, -0.5, 8), (8, -0.5, 8), (8, -0.5, -8), (-8, -0.5, -8))
    s.root.children.append(Node(models=[Model(s.insert_mesh(g[0], g[3], g[1], g[2]), floor)]))
    big_pts, big_tris = scenes.geodesic_sphere(8)
    small_pts, small_tris = scenes.geodesic_sphere(3)
    big = s.insert_mesh(big_pts.astype(np.float32), None, big_tris)
    small = s.insert_mesh(small_pts.astype(np.float32), None, small_tris)
    mats = [(Material(base_metalness=1.0, specular_roughness=0.4, base_color=(0.9, 0.7, 0.4)), 4),
            (Material(base_color=(0.3, 0.5, 0.8), specular_roughness=0.5), 3),
            (Material(base_metalness=0.5, specular_roughness=0.45), 2)]
    mats += [(m, 1) for m in material_objects()]
    spheres = [(s.insert_material(m), big if n > 1 else small) for m, n in mats for _ in range(n)]
    for i, (mat, mesh) in enumerate(spheres):
        t = np.eye(4)
        t[:3, :3] *= 0.42
        t[:3, 3] = (-3.0 + (i % 7), 0.0, -3.0 + (i // 7))
        s.root.children.append(Node(transform=t, models=[Model(mesh, mat)]))
    return s
