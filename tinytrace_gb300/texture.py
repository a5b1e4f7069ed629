"""Host-side texture processing: ProcessedTexture of the reference (src/asset/texture.rs) in
numpy, producing the level data tt_texture carries.

* mip chains as generate_mip_chain (texture.rs:121-143): each level averages 2 x 2 texels of
  the previous one, summed in the order (0,0), (0,1), (1,0), (1,1) from zero and divided by 4,
  until a side is below 2 (a level k then has (width >> k) x (height >> k) texels);
* colour textures (texture.rs:88-104): RGB quantised to 8-bit unorm with alpha 1, BC1 blocks
  read as sRGB;
* normal maps (texture.rs:106-118): octahedral encoding of each texel's normal, 8-bit unorm
  (x, y), BC5 blocks;
* scalar unorm (texture.rs:79-86): 8-bit unorm; scalar float (texture.rs:71-77): f16.

The reference compresses with texpresso's cluster fit, which is not available here; the BC1
and BC5 encoders below are this project's own (endpoints from the extent of the block along
its principal colour axis, or the channel's range, then the nearest palette entry per texel,
with the palette the renderer decodes).  Any valid BC1 / BC5 data renders the same way, so
textures compressed by the reference's encoder can be passed in unchanged.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .asset import encode_octahedron, quantize_unorm

TT_TEXTURE_BC1_SRGB, TT_TEXTURE_BC5_UNORM, TT_TEXTURE_R8_UNORM, TT_TEXTURE_R16_FLOAT = 1, 2, 3, 4


@dataclass
class ProcessedTexture:
    format: int
    width: int
    height: int
    levels: list  # bytes of each mip level, level 0 first

    @property
    def data(self) -> bytes:
        return b"".join(self.levels)


def mip_chain(texture: np.ndarray) -> list[np.ndarray]:
    """generate_mip_chain (src/asset/texture.rs:121-143) in float32; `texture` is (h, w) or
    (h, w, c)."""
    chain = [np.ascontiguousarray(texture, np.float32)]
    while True:
        last = chain[-1]
        h, w = last.shape[:2]
        if w < 2 or h < 2:
            return chain
        oh, ow = h >> 1, w >> 1
        a = last[0:2 * oh:2, 0:2 * ow:2]
        b = last[1:2 * oh:2, 0:2 * ow:2]  # (x, y + 1)
        c = last[0:2 * oh:2, 1:2 * ow:2]  # (x + 1, y)
        d = last[1:2 * oh:2, 1:2 * ow:2]
        s = np.float32(0.0) + a
        s = (s + b).astype(np.float32)
        s = (s + c).astype(np.float32)
        s = (s + d).astype(np.float32)
        chain.append((s / np.float32(4.0)).astype(np.float32))


def _blocks(img: np.ndarray) -> np.ndarray:
    """(h, w, c) -> (by, bx, 16, c) 4 x 4 blocks in row-major texel order; edges replicated."""
    h, w, c = img.shape
    ph, pw = (h + 3) // 4 * 4, (w + 3) // 4 * 4
    img = np.pad(img, ((0, ph - h), (0, pw - w), (0, 0)), mode="edge")
    return img.reshape(ph // 4, 4, pw // 4, 4, c).transpose(0, 2, 1, 3, 4).reshape(ph // 4, pw // 4, 16, c)


def _expand565(c: np.ndarray) -> np.ndarray:
    r, g, b = (c >> 11) & 31, (c >> 5) & 63, c & 31
    return np.stack([(r << 3) | (r >> 2), (g << 2) | (g >> 4), (b << 3) | (b >> 2)], -1).astype(np.int32)


def bc1_palette(c0: np.ndarray, c1: np.ndarray) -> np.ndarray:
    """(..., 4, 3) 8-bit palette the renderer decodes for endpoints c0, c1 (u16 arrays)."""
    a, e = _expand565(c0), _expand565(c1)
    four = (c0 > c1)[..., None]
    p2 = np.where(four, (2 * a + e + 1) // 3, (a + e + 1) // 2)
    p3 = np.where(four, (a + 2 * e + 1) // 3, 0)
    return np.stack([a, e, p2, p3], -2)


def encode_bc1(rgb8: np.ndarray) -> bytes:
    """BC1 blocks of an (h, w, 3) uint8 image, 4-colour mode."""
    blk = _blocks(rgb8.astype(np.float32)).astype(np.float64)  # (by, bx, 16, 3)
    mean = blk.mean(axis=2, keepdims=True)
    d = blk - mean
    cov = np.einsum("...ki,...kj->...ij", d, d)
    axis = np.ones(blk.shape[:2] + (3,))
    for _ in range(8):  # power iteration for the principal axis
        axis = np.einsum("...ij,...j->...i", cov, axis)
        axis /= np.maximum(np.linalg.norm(axis, axis=-1, keepdims=True), 1e-12)
    t = np.einsum("...ki,...i->...k", d, axis)
    lo = mean[..., 0, :] + t.min(axis=-1)[..., None] * axis
    hi = mean[..., 0, :] + t.max(axis=-1)[..., None] * axis

    def to565(c):
        c = np.clip(np.rint(c), 0, 255).astype(np.int32)
        return ((np.rint(c[..., 0] * 31 / 255).astype(np.int32) << 11)
                | (np.rint(c[..., 1] * 63 / 255).astype(np.int32) << 5)
                | np.rint(c[..., 2] * 31 / 255).astype(np.int32)).astype(np.uint16)

    c0, c1 = to565(hi), to565(lo)
    swap = c0 < c1
    c0, c1 = np.where(swap, c1, c0), np.where(swap, c0, c1)
    pal = bc1_palette(c0, c1).astype(np.float64)  # (by, bx, 4, 3)
    dist = ((blk[..., :, None, :] - pal[..., None, :, :]) ** 2).sum(-1)  # (by, bx, 16, 4)
    if np.any(c0 == c1):  # one colour: 3-colour mode; index 0 only
        dist[c0 == c1] = np.array([0.0, 1.0, 1.0, 1.0])
    idx = dist.argmin(-1).astype(np.uint32)
    bits = (idx << (2 * np.arange(16, dtype=np.uint32))).sum(-1).astype(np.uint32)
    out = np.zeros(blk.shape[:2] + (4,), np.uint16)
    out[..., 0] = c0
    out[..., 1] = c1
    out[..., 2] = (bits & 0xFFFF).astype(np.uint16)
    out[..., 3] = (bits >> 16).astype(np.uint16)
    return out.astype("<u2").tobytes()


def bc4_palette(e0: np.ndarray, e1: np.ndarray) -> np.ndarray:
    """(..., 8) float values the renderer decodes for endpoints e0, e1."""
    e0 = e0.astype(np.int64)
    e1 = e1.astype(np.int64)
    k = np.arange(2, 8)
    eight = (((8 - k) * e0[..., None] + (k - 1) * e1[..., None]) / 1785.0).astype(np.float32)
    six = (((6 - k[:4]) * e0[..., None] + (k[:4] - 1) * e1[..., None]) / 1275.0).astype(np.float32)
    six = np.concatenate([six, np.zeros(e0.shape + (1,), np.float32), np.ones(e0.shape + (1,), np.float32)], -1)
    rest = np.where((e0 > e1)[..., None], eight, six)
    return np.concatenate([(e0[..., None] / 255.0).astype(np.float32), (e1[..., None] / 255.0).astype(np.float32),
                           rest], -1)


def _encode_bc4(ch: np.ndarray) -> np.ndarray:
    """(by, bx, 16) uint8 channel -> (by, bx, 8) uint8 BC4 blocks (8-value mode)."""
    e0 = ch.max(-1).astype(np.int64)
    e1 = ch.min(-1).astype(np.int64)
    pal = bc4_palette(e0, e1)  # (by, bx, 8)
    v = ch.astype(np.float32) / np.float32(255.0)
    idx = np.abs(v[..., :, None] - pal[..., None, :]).argmin(-1).astype(np.uint64)
    idx = np.where((e0 == e1)[..., None], 0, idx).astype(np.uint64)
    bits = (idx << (3 * np.arange(16, dtype=np.uint64))).sum(-1).astype(np.uint64)
    out = np.zeros(ch.shape[:2] + (8,), np.uint8)
    out[..., 0] = e0
    out[..., 1] = e1
    for k in range(6):
        out[..., 2 + k] = ((bits >> np.uint64(8 * k)) & np.uint64(0xFF)).astype(np.uint8)
    return out


def encode_bc5(rg8: np.ndarray) -> bytes:
    """BC5 blocks of an (h, w, 2) uint8 image."""
    blk = _blocks(rg8)  # (by, bx, 16, 2)
    return np.concatenate([_encode_bc4(blk[..., 0]), _encode_bc4(blk[..., 1])], -1).tobytes()


def from_color_texture(texture: np.ndarray) -> ProcessedTexture:
    """ProcessedTexture::from_color_texture: (h, w, 3) float colours (in [0, 1], sRGB encoded)."""
    levels = [encode_bc1(quantize_unorm(level[..., :3], 8).astype(np.uint8)) for level in mip_chain(texture)]
    h, w = texture.shape[:2]
    return ProcessedTexture(TT_TEXTURE_BC1_SRGB, w, h, levels)


def from_normal_map(texture: np.ndarray) -> ProcessedTexture:
    """ProcessedTexture::from_normal_map: (h, w, 3) normals."""
    levels = []
    for level in mip_chain(texture):
        o = encode_octahedron(level)
        levels.append(encode_bc5(quantize_unorm(o, 8).astype(np.uint8)))
    h, w = texture.shape[:2]
    return ProcessedTexture(TT_TEXTURE_BC5_UNORM, w, h, levels)


def from_scalar_unorm_texture(texture: np.ndarray) -> ProcessedTexture:
    levels = [quantize_unorm(level, 8).astype(np.uint8).tobytes() for level in mip_chain(texture)]
    h, w = texture.shape[:2]
    return ProcessedTexture(TT_TEXTURE_R8_UNORM, w, h, levels)


def from_scalar_float_texture(texture: np.ndarray) -> ProcessedTexture:
    levels = [level.astype(np.float16).astype("<f2").tobytes() for level in mip_chain(texture)]
    h, w = texture.shape[:2]
    return ProcessedTexture(TT_TEXTURE_R16_FLOAT, w, h, levels)


# MaterialTextures slot order (src/material/material.glsl:40-68) and the processing each
# parameter's texture gets (src/asset/material.rs:312-350).
SLOTS = ("base_color", "specular_color", "transmission_color", "coat_color", "fuzz_color", "emission_color",
         "geometry_normal", "base_weight", "base_metalness", "base_diffuse_roughness", "specular_weight",
         "specular_roughness", "specular_roughness_anisotropy", "specular_ior", "specular_rotation",
         "transmission_weight", "transmission_depth", "coat_weight", "coat_roughness", "coat_roughness_anisotropy",
         "coat_ior", "coat_darkening", "coat_rotation", "fuzz_weight", "fuzz_roughness", "emission_luminance",
         "geometry_opacity")
COLOR = {"base_color", "specular_color", "transmission_color", "coat_color", "fuzz_color", "emission_color"}
FLOAT = {"emission_luminance", "coat_ior", "specular_ior", "transmission_depth", "specular_rotation", "coat_rotation"}


def process(slot: str, texture: np.ndarray) -> ProcessedTexture:
    if slot in COLOR:
        return from_color_texture(texture)
    if slot == "geometry_normal":
        return from_normal_map(texture)
    if slot in FLOAT:
        return from_scalar_float_texture(texture)
    return from_scalar_unorm_texture(texture)
