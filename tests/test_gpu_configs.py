"""The benchmarked configurations against the oracle, bit for bit (tolerance zero, NaN payloads
aside), on the full scenes:

* the plain path tracer on the 1,004,520-triangle icosphere field of the headline benchmark at
  1920x1080, depth 8: a 128x64 crop around the frame centre at 64 spp with the benchmark's
  pool of 2^24 path slots, and stratified rows across the whole frame at 4 spp with the
  default pool (src/integrate/integrate.glsl:323-347 is the path the oracle restates);
* ReSTIR DI on the 2.1 M-triangle, 100 k-light field at 128x72 over 8 frames of the
  benchmark's camera orbit, images and reservoirs.

The GPU renders the whole frame; the oracle renders the compared pixels only.
"""
import numpy as np
import pytest

from conftest import assert_same_bits
from oracle import oracle
from tinytrace_gb300 import native, scenes
from tinytrace_gb300.native import check
from tinytrace_gb300.renderer import Config, Renderer, make_constants

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def field():
    w = scenes.icosphere_workload(extent=(1920, 1080), spp=64, depth=8)
    r = Renderer(w.extent)
    r.set_scene(w.scene)
    r.camera = w.camera
    orc = oracle.OracleScene(r.scene_arrays, flat=True)
    yield w, r, orc
    r.close()


def _gpu_frame(r, c):
    check(r.context.lib.tt_render(r.context.handle, r.scene, native.ptr(c), r.render_target))
    return r.context.download(r.render_target, *r.extent)


def test_field_crop_64spp(field):
    w, r, orc = field
    assert r.scene_arrays.triangle_count == 1004520
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_WAVEFRONT_SLOTS, 1 << 24))
    try:
        c = make_constants(w.camera, w.extent, w.config, 0, 0)
        gpu = _gpu_frame(r, c)
        W, H = w.extent
        x0, y0 = W // 2 - 64, H // 2 - 32
        cpu = np.zeros_like(gpu)
        orc.render(c, cpu, rows=(y0, y0 + 64), cols=(x0, x0 + 128))
        crop = (slice(y0, y0 + 64), slice(x0, x0 + 128))
        assert_same_bits(gpu[crop], cpu[crop], "1080p field, 64 spp, centre crop")
        assert np.isfinite(gpu).all()
        assert (cpu[crop][..., :3] > 0).mean() > 0.5  # the crop sees geometry, not only sky
    finally:
        check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_WAVEFRONT_SLOTS, 0))


def test_field_stratified_rows_4spp(field):
    w, r, orc = field
    cfg = Config(bounce_count=8, sample_count=4)
    c = make_constants(w.camera, w.extent, cfg, 3, 0)
    gpu = _gpu_frame(r, c)
    rows = list(range(18, w.extent[1], 36))
    cpu = np.zeros_like(gpu)
    for y in rows:
        orc.render(c, cpu, rows=(y, y + 1))
    assert_same_bits(gpu[rows], cpu[rows], "1080p field, 4 spp, every 36th row")


def test_restir_field_8_frames():
    extent, frames = (128, 72), 8
    r = Renderer(extent)
    r.set_scene(scenes.restir_field())
    assert r.scene_arrays.triangle_count > 2_000_000 and len(r.scene_arrays.emissive) == 100_000
    r.set_config(Config(bounce_count=1, sample_count=1))
    orc = oracle.OracleScene(r.scene_arrays)
    R = oracle.OracleRestir(orc, *extent)
    cpu = np.zeros((extent[1], extent[0], 4), np.float32)
    for f in range(frames):
        ang = 2.0 * np.pi * f / 60
        r.camera = scenes.Camera.looking_at((95.0 * np.sin(ang), 10.0, 95.0 * np.cos(ang)), (0.0, 0.0, 0.0))
        c = make_constants(r.camera, extent, r.config(), r.context.frame_index(), r.accumulated_frame_count)
        r.render_restir_to_target()
        R.frame(c, cpu)
        assert_same_bits(r.context.download(r.render_target, *extent), cpu, f"ReSTIR field frame {f} image")
        assert_same_bits(r.restir_reservoirs(), R.reservoirs(), f"ReSTIR field frame {f} reservoirs")
        r.present()
    assert (R.reservoirs()[..., 5] > 0).mean() > 0.05
    r.close()
