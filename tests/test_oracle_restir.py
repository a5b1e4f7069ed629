"""ReSTIR DI on the CPU oracle (the checker of tt_render_restir): its converged image agrees with
plain next-event estimation of direct light, reservoirs stay well-formed, frames are
deterministic and independent of the thread count."""
import numpy as np

from oracle import oracle
from tinytrace_gb300 import scenes
from tinytrace_gb300.renderer import Config, SceneArrays, make_constants

NO_LIGHT = 0xFFFFFFFF


def _cornell(extent=(48, 48)):
    w = scenes.cornell_workload(extent=extent, spp=1, depth=1)
    return w, oracle.OracleScene(SceneArrays(w.scene), flat=True)


def _frames(w, orc, frames, **cfg):
    R = oracle.OracleRestir(orc, *w.extent, **cfg)
    img = np.zeros((w.extent[1], w.extent[0], 4), np.float32)
    for f in range(frames):
        R.frame(make_constants(w.camera, w.extent, Config(bounce_count=1, sample_count=1), f, f), img)
    return img, R


def test_converges_to_next_event_estimation():
    """The mean of 64 accumulated ReSTIR frames is within 6 % of a 1024-spp direct-light render
    (one bounce with NEE; every Cornell material has roughness > 0.15).  ReSTIR's biased
    reuse (no 1/Z correction, visibility in the initial reservoirs) lands slightly low."""
    w, orc = _cornell()
    img, _ = _frames(w, orc, 64)
    nee = orc.render(make_constants(w.camera, w.extent, Config(bounce_count=1, sample_count=1024), 0, 0))
    a, b = img[..., :3].mean(axis=(0, 1)), nee[..., :3].mean(axis=(0, 1))
    assert np.all(np.abs(a - b) <= 0.06 * b), (a, b)
    assert np.isfinite(img).all()


def test_reservoirs_are_well_formed():
    w, orc = _cornell()
    _, R = _frames(w, orc, 5)
    res = R.reservoirs()
    light = res[..., 0].view(np.uint32)
    M, W = res[..., 4], res[..., 5]
    n_lights = len(orc.arrays.emissive)
    assert np.all((light == NO_LIGHT) | (light < n_lights))
    assert np.all(W >= 0) and np.all(np.isfinite(W))
    # initial 32 + temporal history capped at 20 x 32, then at most 5 neighbours of that size
    assert M.max() <= 6 * (32 + 20 * 32)
    assert (W > 0).mean() > 0.3


def test_first_frame_has_no_history():
    w, orc = _cornell()
    _, R = _frames(w, orc, 1)
    assert R.reservoirs()[..., 4].max() <= 6 * 32


def test_deterministic_and_thread_independent():
    w, orc = _cornell((40, 24))
    a, Ra = _frames(w, orc, 3)
    R = oracle.OracleRestir(orc, *w.extent)
    img = np.zeros((24, 40, 4), np.float32)
    for f in range(3):
        R.frame(make_constants(w.camera, w.extent, Config(bounce_count=1, sample_count=1), f, f), img, threads=1)
    assert a.tobytes() == img.tobytes()
    assert Ra.reservoirs().tobytes() == R.reservoirs().tobytes()


def test_textured_restir_frames_are_deterministic():
    from tinytrace_gb300 import scenes
    from tinytrace_gb300.camera import Camera
    from tinytrace_gb300.renderer import Config, SceneArrays, make_constants

    a = SceneArrays(scenes.textured_cornell())
    cam = Camera.looking_at((0.0, 1.0, 3.4), (0.0, 1.0, 0.0), fov=0.8)
    imgs = []
    for _ in range(2):
        R = oracle.OracleRestir(oracle.OracleScene(a), 40, 30)
        img = np.zeros((30, 40, 4), np.float32)
        for f in range(2):
            R.frame(make_constants(cam, (40, 30), Config(bounce_count=1, sample_count=1), f, 0), img)
        imgs.append(img.copy())
    assert np.isfinite(imgs[0]).all() and imgs[0][..., :3].max() > 0
    assert np.array_equal(imgs[0], imgs[1])
