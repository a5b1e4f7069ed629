"""Texture decoding and sampling of the oracle (oracle/ref_texture.h) and the host texture
processing (tinytrace_gb300/texture.py), on the CPU:

* BC1 (both palette modes), BC5 (both BC4 modes), R8 and R16F texels against values worked
  out by hand from the block layouts of src/asset/texture.rs's formats;
* the filter: texel centres return texels, bilinear weights between them, repeat addressing,
  LOD clamping and blending between levels;
* mip chains (texture.rs:121-143) and the encoders' round trip through the decoder;
* material constants of textured parameters (Param::constant_or_default) and scene arrays
  that carry textures through save / from_arrays;
* a textured scene renders deterministically and differs from its untextured constants.
"""
import struct

import numpy as np
import pytest

from oracle import oracle
from tinytrace_gb300 import asset, scenes, texture
from tinytrace_gb300.asset import Material, Model, Node
from tinytrace_gb300.camera import Camera
from tinytrace_gb300.renderer import Config, SceneArrays, make_constants

SRGB = np.array([c / 12.92 if c <= 0.04045 else ((c + 0.055) / 1.055) ** 2.4 for c in np.arange(256) / 255.0],
                np.float64).astype(np.float32)


def _scene_with(textures):
    """A one-triangle scene whose arrays carry the given ProcessedTextures."""
    s = asset.Scene()
    s.insert_mesh(np.float32([[0, 0, 0], [1, 0, 0], [0, 1, 0]]), normals=np.tile([0, 0, 1], (3, 1)))
    s.insert_material(Material())
    s.root.children.append(Node(models=[Model(0, 0)]))
    s.textures.extend(textures)
    return oracle.OracleScene(SceneArrays(s), use_bvh=False)


def _centres(w, h, lod=0.0):
    y, x = np.mgrid[0:h, 0:w]
    return np.stack([(x.ravel() + 0.5) / w, (y.ravel() + 0.5) / h, np.full(w * h, lod)], -1).astype(np.float32)


def test_bc1_four_colour_block():
    c0, c1 = 0xF800, 0x001F  # pure red > pure blue: four-colour mode
    idx = sum((t % 4) << (2 * t) for t in range(16))
    block = struct.pack("<HHI", c0, c1, idx)
    o = _scene_with([texture.ProcessedTexture(texture.TT_TEXTURE_BC1_SRGB, 4, 4, [block])])
    got = o.texture_sample(0, _centres(4, 4))
    pal = [(255, 0, 0), (0, 0, 255), ((2 * 255 + 1) // 3, 0, (255 + 1) // 3), ((255 + 1) // 3, 0, (2 * 255 + 1) // 3)]
    want = np.array([[*SRGB[list(pal[t % 4])], 1.0] for t in range(16)], np.float32)
    assert np.array_equal(got, want)


def test_bc1_three_colour_block_has_transparent_black():
    c0, c1 = 0x001F, 0xF800  # c0 <= c1: three colours and transparent black
    idx = sum((t % 4) << (2 * t) for t in range(16))
    o = _scene_with([texture.ProcessedTexture(texture.TT_TEXTURE_BC1_SRGB, 4, 4, [struct.pack("<HHI", c0, c1, idx)])])
    got = o.texture_sample(0, _centres(4, 4))
    mid = SRGB[[(255 + 1) // 2, 0, (255 + 1) // 2]]
    assert np.array_equal(got[2], [*mid, 1.0])
    assert np.array_equal(got[3], [0.0, 0.0, 0.0, 0.0])


def _bc4(e0, e1, idx):
    bits = sum(k << (3 * t) for t, k in enumerate(idx))
    return bytes([e0, e1]) + bits.to_bytes(6, "little")


def test_bc5_both_modes():
    idx = [t % 8 for t in range(16)]
    block = _bc4(200, 100, idx) + _bc4(50, 150, idx)  # red eight-value, green six-value
    o = _scene_with([texture.ProcessedTexture(texture.TT_TEXTURE_BC5_UNORM, 4, 4, [block])])
    got = o.texture_sample(0, _centres(4, 4))

    def value(e0, e1, k):
        if k < 2:
            return np.float32(np.float32([e0, e1][k]) / np.float32(255))
        if e0 > e1:
            return np.float32(np.float32((8 - k) * e0 + (k - 1) * e1) / np.float32(1785))
        return {6: np.float32(0), 7: np.float32(1)}.get(k, np.float32(np.float32((6 - k) * e0 + (k - 1) * e1)
                                                                      / np.float32(1275)))

    for t in range(16):
        assert got[t, 0] == value(200, 100, idx[t]) and got[t, 1] == value(50, 150, idx[t])
        assert got[t, 2] == 0.0 and got[t, 3] == 1.0


def test_scalar_formats_and_filter():
    r8 = np.arange(16, dtype=np.uint8).reshape(4, 4) * 17
    h16 = (np.arange(8, dtype=np.float32).reshape(2, 4) - 3.5).astype(np.float16)
    o = _scene_with([texture.ProcessedTexture(texture.TT_TEXTURE_R8_UNORM, 4, 4, [r8.tobytes()]),
                     texture.ProcessedTexture(texture.TT_TEXTURE_R16_FLOAT, 4, 2, [h16.tobytes()])])
    got = o.texture_sample(0, _centres(4, 4))
    assert np.array_equal(got[:, 0], (r8.ravel().astype(np.float32) / np.float32(255)))
    assert np.array_equal(got[:, 1:], np.tile([0, 0, 1], (16, 1)).astype(np.float32))
    assert np.array_equal(o.texture_sample(1, _centres(4, 2))[:, 0], h16.ravel().astype(np.float32))
    # halfway between the centres of texels (0, 0) and (1, 0): the mean; at u = 0 the repeat
    # neighbour (3, 0) takes half the weight
    t = r8.astype(np.float32) / np.float32(255)
    mid = o.texture_sample(0, np.float32([[0.25, 0.125, 0.0], [0.0, 0.125, 0.0], [1.0, 0.125, 0.0]]))[:, 0]
    assert np.isclose(mid[0], (t[0, 0] + t[0, 1]) / 2, atol=1e-7)
    assert np.isclose(mid[1], (t[0, 0] + t[0, 3]) / 2, atol=1e-7) and mid[1] == mid[2]
    # texture coordinates repeat
    a = o.texture_sample(0, np.float32([[0.3, 0.6, 0], [1.3, -0.4, 0], [-2.7, 5.6, 0]]))
    assert np.allclose(a, a[0], atol=1e-6)


def test_lod_clamp_and_blend():
    tex = texture.from_scalar_unorm_texture(np.random.default_rng(1).random((16, 16)).astype(np.float32))
    assert len(tex.levels) == 5
    o = _scene_with([tex])
    uv = np.float32([[0.37, 0.61]])
    s = {lod: o.texture_sample(0, np.c_[uv, [[lod]]].astype(np.float32))[0, 0]
         for lod in (-3.0, 0.0, 1.0, 2.0, 0.25, 4.0, 9.0, np.inf, -np.inf, np.nan)}
    assert s[-3.0] == s[0.0] == s[-np.inf] == s[np.nan]
    assert s[4.0] == s[9.0] == s[np.inf]
    l0, l1 = s[0.0], s[1.0]
    assert s[0.25] == np.float32(np.float32(l0 * np.float32(0.75)) + np.float32(l1 * np.float32(0.25)))


def test_mip_chain():
    rng = np.random.default_rng(2)
    img = rng.random((10, 6, 3)).astype(np.float32)
    chain = texture.mip_chain(img)
    assert [c.shape[:2] for c in chain] == [(10, 6), (5, 3), (2, 1)]
    for a, b in zip(chain, chain[1:]):
        for y in range(b.shape[0]):
            for x in range(b.shape[1]):
                s = np.zeros(3, np.float32)
                for dx, dy in ((0, 0), (0, 1), (1, 0), (1, 1)):
                    s = (s + a[2 * y + dy, 2 * x + dx]).astype(np.float32)
                assert np.array_equal(b[y, x], (s / np.float32(4)).astype(np.float32))
    assert len(texture.mip_chain(np.ones((1, 64), np.float32))) == 1


def test_encoders_round_trip():
    rng = np.random.default_rng(3)
    y, x = np.mgrid[0:32, 0:32] / 31.0
    # colours on a line in RGB: BC1's palette holds them to within the 5:6:5 steps
    line = np.stack([x, 0.5 * x, 1.0 - x], -1).astype(np.float32)
    o = _scene_with([texture.from_color_texture(line)])
    got = o.texture_sample(0, _centres(32, 32))[:, :3].reshape(32, 32, 3)
    assert np.abs(got - SRGB[asset.quantize_unorm(line, 8)]).max() < 0.02
    # colours spread over a plane: a four-entry palette per block can only approximate them
    plane = np.stack([x, y, 0.5 * (x + y)], -1).astype(np.float32)
    o = _scene_with([texture.from_color_texture(plane)])
    got = o.texture_sample(0, _centres(32, 32))[:, :3].reshape(32, 32, 3)
    assert np.abs(got - SRGB[asset.quantize_unorm(plane, 8)]).mean() < 0.03
    nrm = np.stack([0.4 * np.sin(6 * x), 0.4 * np.cos(5 * y), np.ones_like(x)], -1).astype(np.float32)
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    o = _scene_with([texture.from_normal_map(nrm)])
    rg = o.texture_sample(0, _centres(32, 32))[:, :2].reshape(32, 32, 2)
    octa = asset.quantize_unorm(asset.encode_octahedron(nrm), 8) / 255.0
    assert np.abs(rg - octa).max() < 0.02  # BC4 of a 4x4 block's range in 8 steps
    noise = rng.random((8, 8, 3)).astype(np.float32)
    o = _scene_with([texture.from_color_texture(noise)])
    assert np.isfinite(o.texture_sample(0, _centres(8, 8))).all()


def test_textured_material_constants_and_arrays(tmp_path):
    m = Material(base_color=(0.3, 0.4, 0.5), emission_luminance=0.0,
                 textures={"base_color": np.ones((4, 4, 3), np.float32),
                           "emission_luminance": np.full((4, 4), 2.0, np.float32)})
    c = m.constants()
    assert np.array_equal(c["base_color"], [0, 0, 0, 0]) and c["emission_luminance"] == 0.0
    assert m.is_emissive()
    sc = scenes.textured_cornell()
    a = SceneArrays(sc)
    assert len(a.texture_info) == 6 and a.texture_data.nbytes == int(a.texture_info[:, 4].sum())
    mats = a.materials["textures"]
    assert (mats[mats != 0xFFFFFFFF] < 6).all()
    b = SceneArrays.from_arrays(a.save(tmp_path / "s.npz"))
    for f in SceneArrays.FIELDS:
        assert getattr(a, f).tobytes() == getattr(b, f).tobytes()


def test_textured_render():
    sc = scenes.textured_cornell()
    a = SceneArrays(sc)
    cam = Camera.looking_at((0.0, 1.0, 3.4), (0.0, 1.0, 0.0), fov=0.75)
    c = make_constants(cam, (48, 48), Config(bounce_count=4, sample_count=2), 0, 0)
    img = oracle.OracleScene(a).render(c)
    assert np.isfinite(img).all() and img[..., :3].max() > 0
    assert np.array_equal(img, oracle.OracleScene(SceneArrays(scenes.textured_cornell())).render(c))
    plain = SceneArrays.from_arrays(a.save(None))
    plain.materials = plain.materials.copy()
    plain.materials["textures"] = 0xFFFFFFFF
    assert not np.array_equal(img, oracle.OracleScene(plain).render(c))
