"""A glTF scene on the GPU: the reference's own Cornell box (tests/golden/cornell_box.gltf,
imported by gltf.load with the reference importer's material mapping, src/asset/gltf.rs:50-122,
242-383) rendered through the C ABI by both integrators and by ReSTIR, against the oracle, bit
for bit."""
from pathlib import Path

import numpy as np
import pytest

from conftest import assert_same_bits
from oracle import oracle
from tinytrace_gb300 import gltf, native
from tinytrace_gb300.camera import Camera
from tinytrace_gb300.native import check
from tinytrace_gb300.renderer import Config, Renderer, make_constants

pytestmark = pytest.mark.gpu

FIXTURE = Path(__file__).resolve().parent / "golden" / "cornell_box.gltf"


@pytest.mark.parametrize("integrator", [native.TT_INTEGRATOR_WAVEFRONT, native.TT_INTEGRATOR_MEGAKERNEL])
def test_imported_cornell_renders_like_the_oracle(gpu_context, integrator):
    extent = (96, 72)
    r = Renderer(extent)
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_INTEGRATOR, integrator))
    r.set_scene(gltf.load(FIXTURE).scene)
    assert r.scene_arrays.triangle_count == 32
    r.camera = Camera.looking_at((0.0, 1.0, 3.6), (0.0, 1.0, 0.0), fov=0.8)
    cfg = Config(bounce_count=6, sample_count=16)
    r.set_config(cfg)
    orc = oracle.OracleScene(r.scene_arrays)
    cpu = np.zeros((extent[1], extent[0], 4), np.float32)
    for f in range(3):  # frames 0 and 1 overwrite, frame 2 accumulates
        c = make_constants(r.camera, extent, cfg, r.context.frame_index(), r.accumulated_frame_count)
        gpu = r.render_to_texture()
        orc.render(c, cpu)
        assert_same_bits(gpu, cpu, f"imported Cornell box frame {f}")
        r.present()
    assert np.isfinite(cpu).all() and cpu[..., :3].mean() > 0.05
    r.close()


def test_imported_cornell_restir(gpu_context):
    extent = (64, 48)
    r = Renderer(extent)
    r.set_scene(gltf.load(FIXTURE).scene)
    r.set_config(Config(bounce_count=1, sample_count=1))
    orc = oracle.OracleScene(r.scene_arrays)
    R = oracle.OracleRestir(orc, *extent)
    cpu = np.zeros((extent[1], extent[0], 4), np.float32)
    for f in range(4):
        a = 0.03 * f
        r.camera = Camera.looking_at((3.6 * np.sin(a), 1.0, 3.6 * np.cos(a)), (0.0, 1.0, 0.0), fov=0.8)
        c = make_constants(r.camera, extent, r.config(), r.context.frame_index(), r.accumulated_frame_count)
        r.render_restir_to_target()
        R.frame(c, cpu)
        assert_same_bits(r.context.download(r.render_target, *extent), cpu, f"imported Cornell ReSTIR frame {f}")
        assert_same_bits(r.restir_reservoirs(), R.reservoirs(), f"imported Cornell ReSTIR frame {f} reservoirs")
        r.present()
    r.close()
