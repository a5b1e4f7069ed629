"""Error behaviour of the C ABI on a device (GPU required): every entry returns a status and
tt_last_error explains it; no call aborts.  The reference panics on these conditions
(src/lib.rs, backend handle.rs); the boundary turns them into TT_ERR_* codes.  None of these
cases launches a kernel with bad inputs: each is rejected on the host first."""
import ctypes

import numpy as np
import pytest

from tinytrace_gb300 import native, scenes
from tinytrace_gb300.renderer import Context, SceneArrays

pytestmark = pytest.mark.gpu


@pytest.fixture()
def ctx():
    from tinytrace_gb300 import build

    build.build()
    c = Context(0)
    yield c
    c.close()


def _create(ctx, arrays):
    h = ctypes.c_uint64()
    d = arrays.desc()
    return ctx.lib.tt_scene_create(ctx.handle, ctypes.byref(d), ctypes.byref(h)), h.value


def _cornell():
    return SceneArrays(scenes.cornell_box())


def test_index_out_of_range(ctx):
    a = _cornell()
    a.indices = a.indices.copy()
    a.indices[5] = 10_000_000
    rc, _ = _create(ctx, a)
    assert rc == native.TT_ERR_INVALID_ARGUMENT and b"outside the vertex arrays" in ctx.lib.tt_last_error()


def test_non_finite_instance_matrix(ctx):
    a = _cornell()
    a.instances = a.instances.copy()
    a.instances["transform"][0, 0] = np.nan
    rc, _ = _create(ctx, a)
    assert rc == native.TT_ERR_INVALID_ARGUMENT and b"finite" in ctx.lib.tt_last_error()


def test_texture_index_without_textures(ctx):
    a = _cornell()
    a.materials = a.materials.copy()
    a.materials["textures"][0, 3] = 0  # the scene holds no textures
    rc, _ = _create(ctx, a)
    assert rc == native.TT_ERR_INVALID_ARGUMENT


def test_bad_mesh_and_material_indices(ctx):
    a = _cornell()
    a.instances = a.instances.copy()
    a.instances["material_index"][0] = 999
    assert _create(ctx, a)[0] == native.TT_ERR_INVALID_ARGUMENT
    b = _cornell()
    b.emissive = b.emissive.copy()
    b.emissive["instance_index"][0] = 999
    assert _create(ctx, b)[0] == native.TT_ERR_INVALID_ARGUMENT


def test_stale_handles_after_clear_lifetime(ctx):
    rc, scene = _create(ctx, _cornell())
    assert rc == native.TT_OK
    img = ctx.create_image(native.TT_LIFETIME_FRAME, 8, 8)
    ctx.clear_lifetime(native.TT_LIFETIME_FRAME)
    out = np.zeros((8, 8, 4), np.float32)
    assert ctx.lib.tt_image_download(ctx.handle, img, native.ptr(out), out.nbytes) == native.TT_ERR_BAD_HANDLE
    assert b"stale" in ctx.lib.tt_last_error()
    st = native.SceneStats()
    assert ctx.lib.tt_scene_stats_get(ctx.handle, scene, ctypes.byref(st)) == native.TT_OK
    # an image handle used as a scene handle
    assert ctx.lib.tt_scene_stats_get(ctx.handle, img, ctypes.byref(st)) == native.TT_ERR_BAD_HANDLE


def test_wrong_byte_counts(ctx):
    img = ctx.create_image(native.TT_LIFETIME_FRAME, 8, 8)
    out = np.zeros((8, 8, 4), np.float32)
    assert ctx.lib.tt_image_download(ctx.handle, img, native.ptr(out), out.nbytes - 16) == \
        native.TT_ERR_INVALID_ARGUMENT
    c = np.zeros((), native.CONSTANTS_DTYPE)
    assert ctx.lib.tt_tonemap(ctx.handle, img, native.ptr(c), 7, native.ptr(out), out.nbytes) == \
        native.TT_ERR_INVALID_ARGUMENT


def test_unknown_options(ctx):
    assert ctx.lib.tt_set_option(ctx.handle, 999, 0) == native.TT_ERR_INVALID_ARGUMENT
    assert ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_ACCEL, 9) == native.TT_ERR_INVALID_ARGUMENT
    assert ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_INTEGRATOR, 9) == native.TT_ERR_INVALID_ARGUMENT


def test_empty_scene_renders_sky(ctx):
    """A scene without instances: every camera ray misses and sees the white sky."""
    a = _cornell()
    a.instances = a.instances[:0].copy()
    a.emissive = a.emissive[:0].copy()
    rc, scene = _create(ctx, a)
    assert rc == native.TT_OK
    w = scenes.cornell_workload(extent=(16, 8), spp=2, depth=3)
    from tinytrace_gb300.renderer import make_constants

    c = make_constants(w.camera, w.extent, w.config, 0, 0)
    img = ctx.create_image(native.TT_LIFETIME_FRAME, 16, 8)
    native.check(ctx.lib.tt_render(ctx.handle, scene, native.ptr(c), img))
    out = ctx.download(img, 16, 8)
    assert np.all(out[..., :3] == 1.0)


def test_stage_timings(ctx):
    """TT_OPTION_STAGE_TIMING records every wavefront launch; without it the call reports an error."""
    from tinytrace_gb300.renderer import make_constants

    rc, scene = _create(ctx, _cornell())
    assert rc == native.TT_OK
    w = scenes.cornell_workload(extent=(32, 16), spp=3, depth=4)
    c = make_constants(w.camera, w.extent, w.config, 0, 0)
    img = ctx.create_image(native.TT_LIFETIME_FRAME, 32, 16)
    native.check(ctx.lib.tt_render(ctx.handle, scene, native.ptr(c), img))
    st = native.StageTimings()
    assert ctx.lib.tt_stage_timings_get(ctx.handle, ctypes.byref(st)) == native.TT_ERR_INVALID_ARGUMENT
    native.check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_STAGE_TIMING, 1))
    native.check(ctx.lib.tt_render(ctx.handle, scene, native.ptr(c), img))
    native.check(ctx.lib.tt_stage_timings_get(ctx.handle, ctypes.byref(st)))
    launches = list(st.launches)
    for s in (native.TT_STAGE_REGEN, native.TT_STAGE_EXTEND, native.TT_STAGE_SHADE, native.TT_STAGE_SHADOW):
        assert launches[s] >= 4 and st.ns[s] > 0, (s, launches)
    assert launches[native.TT_STAGE_EXTEND] == launches[native.TT_STAGE_SHADOW]
    assert launches[native.TT_STAGE_REDUCE] == 1 and launches[native.TT_STAGE_MEGAKERNEL] == 0
    assert st.overflow == 0
    native.check(ctx.lib.tt_set_option(ctx.handle, native.TT_OPTION_INTEGRATOR, native.TT_INTEGRATOR_MEGAKERNEL))
    native.check(ctx.lib.tt_render(ctx.handle, scene, native.ptr(c), img))
    native.check(ctx.lib.tt_stage_timings_get(ctx.handle, ctypes.byref(st)))
    assert list(st.launches)[native.TT_STAGE_MEGAKERNEL] == 1 and sum(st.launches) == 1
