"""The oracle's integrator (src/integrate/integrate.glsl restated) on the CPU.

* White furnace: a convex white Lambertian object under the white sky of
  integrate.glsl:273 reflects exactly the light that arrives, so every pixel is 1 for any
  sample count (each path's throughput f cos / pdf is exactly the albedo, 1).
* Accumulation (integrate.glsl:340-346): n = accumulated_frame_count; frames 0 and 1 both
  overwrite, later frames blend (prev (n-1) + new) / n.
* Determinism and trace equivalence: brute-force, two-level and flat tracing give the
  same image bit for bit.
* Light sampling modes: NEE and on-hit rendering agree in the mean on the Cornell box.
"""
import numpy as np
import pytest

from oracle import oracle
from tinytrace_gb300 import scenes
from tinytrace_gb300.asset import Material, Model, Node, Scene
from tinytrace_gb300.camera import Camera
from tinytrace_gb300.renderer import Config, LightSampling, SceneArrays, make_constants


def furnace_scene():
    s = Scene()
    white = s.insert_material(Material(specular_weight=0.0, base_color=(1.0, 1.0, 1.0), base_weight=1.0))
    pts, tris = scenes.geodesic_sphere(6)
    m = s.insert_mesh(pts.astype(np.float32), None, tris)
    s.root.children.append(Node(models=[Model(m, white)]))
    return s


@pytest.mark.parametrize("light_sampling", [LightSampling.NEXT_EVENT_ESTIMATION, LightSampling.ON_HIT])
def test_white_furnace(light_sampling):
    arrays = SceneArrays(furnace_scene())
    cam = Camera.looking_at((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), fov=0.9)
    cfg = Config(bounce_count=4, sample_count=4, light_sampling=light_sampling)
    c = make_constants(cam, (24, 24), cfg, 0, 0)
    img = oracle.OracleScene(arrays).render(c)
    assert np.all(np.abs(img[..., :3] - 1.0) < 1e-4), np.abs(img[..., :3] - 1.0).max()
    # the centre pixels hit the sphere (so the test exercises a bounce, not only the sky)
    hits = oracle.OracleScene(arrays).trace(_centre_rays(cam), cull=True)
    assert hits[:, 0].all()


def _centre_rays(cam):
    r = np.zeros((1, 8), np.float32)
    r[0, 0:3] = cam.position
    r[0, 4:7] = cam.ray_direction(0.0, 0.0, 1.0)
    r[0, 3], r[0, 7] = 1e-3, 1000.0
    return r


def test_accumulation_rule():
    w = scenes.cornell_workload(extent=(20, 16), spp=1, depth=3)
    orc = oracle.OracleScene(SceneArrays(w.scene))
    fresh = [orc.render(make_constants(w.camera, w.extent, w.config, f, 0)) for f in range(3)]
    acc = np.zeros((16, 20, 4), np.float32)
    for f, n in enumerate([0, 1, 2]):
        orc.render(make_constants(w.camera, w.extent, w.config, f, n), acc)
        if f < 2:  # n = 0 and n = 1 overwrite
            assert np.array_equal(acc[..., :3], fresh[f][..., :3])
    blend = (fresh[1][..., :3] * np.float32(1.0) + fresh[2][..., :3]) / np.float32(2.0)
    assert np.array_equal(acc[..., :3], blend.astype(np.float32))


def test_tracing_structures_render_the_same_image():
    w = scenes.cornell_workload(extent=(24, 16), spp=2, depth=4)
    arrays = SceneArrays(w.scene)
    c = make_constants(w.camera, w.extent, w.config, 3, 0)
    a = oracle.OracleScene(arrays, use_bvh=False).render(c)
    b = oracle.OracleScene(arrays).render(c)
    f = oracle.OracleScene(arrays, flat=True).render(c)
    assert a.tobytes() == b.tobytes() == f.tobytes()


def test_render_is_deterministic_and_threads_do_not_matter():
    w = scenes.cornell_workload(extent=(24, 16), spp=2, depth=4)
    orc = oracle.OracleScene(SceneArrays(w.scene))
    c = make_constants(w.camera, w.extent, w.config, 5, 0)
    assert orc.render(c, threads=1).tobytes() == orc.render(c, threads=4).tobytes()


def test_nee_and_on_hit_agree_in_the_mean():
    """Both estimators of integrate.glsl converge to the same image; compare the frame means
    of a few hundred samples per pixel on a coarse Cornell box."""
    base = scenes.cornell_workload(extent=(16, 16), spp=256, depth=4)
    arrays = SceneArrays(base.scene)
    orc = oracle.OracleScene(arrays, flat=True)
    means = []
    for ls in (LightSampling.NEXT_EVENT_ESTIMATION, LightSampling.ON_HIT):
        cfg = Config(bounce_count=4, sample_count=256, light_sampling=ls)
        img = orc.render(make_constants(base.camera, base.extent, cfg, 0, 0))
        means.append(img[..., :3].astype(np.float64).mean(axis=(0, 1)))
    assert np.allclose(means[0], means[1], rtol=0.06), means


def test_cornell_image_is_lit_and_finite():
    w = scenes.cornell_workload(extent=(32, 32), spp=4, depth=4)
    img = oracle.OracleScene(SceneArrays(w.scene)).render(make_constants(w.camera, w.extent, w.config, 0, 0))
    assert np.isfinite(img).all()
    assert img[..., :3].mean() > 0.05
    # the red wall on the left and the green wall on the right (integrate.glsl shading of the fixture)
    left, right = img[12:20, 1:4, :3].mean(axis=(0, 1)), img[12:20, -4:-1, :3].mean(axis=(0, 1))
    assert left[0] > left[1] and right[1] > right[0]


def test_tonemap_curve():
    """neutral_tonemap (src/post_process/tonemap.glsl:17-26): monotone up to float rounding,
    saturating at the 0.97 scale; disabled = pass-through."""
    x = np.linspace(0, 50, 2001, dtype=np.float32)
    img = np.stack([x, x, x, np.ones_like(x)], axis=1).reshape(1, -1, 4)
    y = oracle.tonemap(img, True)[0, :, 0]
    assert np.all(np.diff(y) >= -2.5e-7) and y.max() <= 0.97 + 1e-6
    assert np.array_equal(oracle.tonemap(img, False), img)


def test_light_visibility_modes():
    """The reference's 16-bit light hash fails for lights at global triangle index >= 65535
    (next-event estimation sees nothing); the exact mode tests the sampled triangle and sees
    them.  Where every light lies below index 65535 the two modes give the same image."""
    from tinytrace_gb300 import scenes
    from tinytrace_gb300.camera import Camera
    from tinytrace_gb300.renderer import Config, SceneArrays, make_constants

    cam = Camera.looking_at((0.0, 3.0, 4.0), (0.0, 0.0, 0.0), fov=0.8)
    c = make_constants(cam, (40, 30), Config(bounce_count=3, sample_count=2), 0, 0)
    o = oracle.OracleScene(SceneArrays(scenes.late_lights()))
    hashed = o.render(c)
    o.set_light_exact(True)
    exact = o.render(c)
    assert exact[..., :3].mean() > hashed[..., :3].mean() * 1.01
    w = scenes.cornell_workload(extent=(32, 32), spp=2, depth=3)
    cc = make_constants(w.camera, w.extent, w.config, 0, 0)
    o = oracle.OracleScene(SceneArrays(w.scene))
    a = o.render(cc)
    o.set_light_exact(True)
    assert np.array_equal(a, o.render(cc))


def test_power_light_selection_is_unbiased_and_less_noisy():
    """Power-proportional light selection (alias table) is an unbiased estimator of the same
    image as the reference's uniform pick, with lower error on a field of log-normal lights."""
    from tinytrace_gb300 import scenes
    from tinytrace_gb300.renderer import SceneArrays, make_constants

    w = scenes.icosphere_workload(extent=(24, 16), spp=8, depth=2, instances=3, freq=5, lights=300)
    o = oracle.OracleScene(SceneArrays(w.scene))
    ref_cfg = scenes.Config(bounce_count=2, sample_count=2048)
    ref = o.render(make_constants(w.camera, w.extent, ref_cfg, 99, 0))[..., :3].astype(np.float64)
    errs = {}
    for power in (False, True):
        o.set_light_power(power)
        imgs = [o.render(make_constants(w.camera, w.extent, w.config, f, 0))[..., :3] for f in range(6)]
        errs[power] = np.mean([np.mean((i - ref) ** 2) for i in imgs])
        mean = np.mean(imgs, axis=0)
        assert abs(mean.mean() - ref.mean()) < 0.05 * ref.mean()
    assert errs[True] < errs[False]
