"""Independent pins of the oracle's BSDF lobes against published formulas (CPU only).

The oracle restates src/material/*.glsl line by line, and the GPU kernels match it bit for bit,
so a slip shared by both would go unnoticed by the parity tests.  Here the lobes are compared
with the published models, restated below in float64 from their papers and not from the
reference or the oracle:

* microfacet reflection: anisotropic GGX distribution (Heitz 2014, "Understanding the
  masking-shadowing function", eq. 85 with the roughness-to-alpha map of the OpenPBR 1.0
  specification: alpha = r^2, alpha_t = alpha sqrt(2 / (1 + (1 - a)^2)), alpha_b = (1 - a)
  alpha_t), Smith's Lambda for GGX and the height-correlated masking-shadowing
  G2 = 1 / (1 + Lambda(i) + Lambda(o)), f = F D G2 / (4 |cos i| |cos o|); sampling density of
  the visible normals (Heitz 2018, "Sampling the GGX distribution of visible normals"):
  pdf = G1(i) max(0, i.h) D(h) / cos i / (4 |i.h|);
* metal Fresnel: the F82-tint model of OpenPBR 1.0 (Hoffman 2019, as adopted by Kutz et al.
  2021): F(mu) = F_Schlick(F0, mu) - mu (1 - mu)^6 (1 - t) F_Schlick(F0, mu_bar) /
  (mu_bar (1 - mu_bar)^6), mu_bar = 1/7;
* dielectric Fresnel: the exact unpolarised Fresnel reflectance (Born & Wolf);
* energy-compensated Oren-Nayar: a white base (rho = 1) reflects all light at every incidence
  (the purpose of the compensation term, Kulla & Conty 2017): the hemispherical albedo,
  integrated numerically from bsdf_evaluate, is one (measured 1.0000 at four roughnesses and
  four incidences);
* the sheen (fuzz) lobe is a linearly transformed cosine (Heitz et al. 2016): its density
  integrates to one (the transformed lobes of these roughnesses stay above the horizon;
  measured 1.0000-1.0001), and f cos(o) / pdf is the same for every outgoing direction.

Each lobe is isolated by a material in which every other lobe is exactly zero (black base,
specular weight zero), so bsdf_evaluate returns that lobe alone and its value does not depend
on the stochastic lobe albedos of bsdf_prepare.  The reference bends the base's Fresnel angle
through the coat IOR even without a coat (specular_fresnel_with_coat, src/material/
specular_brdf.glsl); the dielectric pin therefore uses coat_ior = 1, where the published
formula applies.  Anisotropy rotations are pinned at a quarter and a half turn, where the
sense of rotation does not change the distribution.
"""
import numpy as np
import pytest

from oracle import oracle
from tinytrace_gb300.asset import Material

RTOL = 2e-4  # float32 evaluation against float64 formulas


def _eval(m, wi, wo, seed=12345):
    n = len(wi)
    s = np.zeros((n, 8), np.float32)
    s[:, 0:3] = wi
    s[:, 3] = np.full(n, seed, np.uint32).view(np.float32)
    s[:, 4:7] = wo
    out = oracle.bsdf_eval(np.ascontiguousarray(m.constants()), s)
    return out[:, 0:3].astype(np.float64), out[:, 3].astype(np.float64)


def _upper(rng, n, min_cos=0.08):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    v[:, 2] = np.abs(v[:, 2])
    v = v[v[:, 2] > min_cos]
    return v


# ---------------------------------------------------------------- published formulas, float64
def alphas(roughness, anisotropy):
    a = roughness * roughness
    at = a * np.sqrt(2.0 / (1.0 + (1.0 - anisotropy) ** 2))
    ab = (1.0 - anisotropy) * at
    return max(at, 1e-4), max(ab, 1e-4)


def rotate(v, turns):
    """Directions in the frame whose tangent is turned by `turns` (quarter / half turns only)."""
    ang = 2.0 * np.pi * turns
    c, s = np.cos(ang), np.sin(ang)
    return np.stack([c * v[:, 0] - s * v[:, 1], s * v[:, 0] + c * v[:, 1], v[:, 2]], axis=1)


def ggx_d(h, ax, ay):
    return 1.0 / (np.pi * ax * ay * ((h[:, 0] / ax) ** 2 + (h[:, 1] / ay) ** 2 + h[:, 2] ** 2) ** 2)


def ggx_lambda(v, ax, ay):
    t2 = ((ax * v[:, 0]) ** 2 + (ay * v[:, 1]) ** 2) / v[:, 2] ** 2
    return (np.sqrt(1.0 + t2) - 1.0) / 2.0


def schlick(f0, mu):
    return f0 + (1.0 - f0) * (1.0 - mu)[:, None] ** 5


def f82_tint(mu, f0, tint):
    mb = 1.0 / 7.0
    fb = f0 + (1.0 - f0) * (1.0 - mb) ** 5
    return schlick(f0, mu) - (mu * (1.0 - mu) ** 6)[:, None] * (1.0 - tint) * fb / (mb * (1.0 - mb) ** 6)


def fresnel_dielectric(c, eta):
    s2 = (1.0 - c * c) / eta ** 2
    ct = np.sqrt(np.maximum(0.0, 1.0 - s2))
    rs = (c - eta * ct) / (c + eta * ct)
    rp = (eta * c - ct) / (eta * c + ct)
    return np.where(s2 >= 1.0, 1.0, 0.5 * (rs * rs + rp * rp))


def microfacet_reflection(wi, wo, roughness, anisotropy, turns, fresnel):
    """f (n x 3) and the visible-normal sampling density of a GGX reflection lobe."""
    ax, ay = alphas(roughness, anisotropy)
    i, o = rotate(wi, turns), rotate(wo, turns)
    h = i + o
    h /= np.linalg.norm(h, axis=1, keepdims=True)
    d = ggx_d(h, ax, ay)
    li, lo = ggx_lambda(i, ax, ay), ggx_lambda(o, ax, ay)
    ih = np.sum(i * h, axis=1)
    f = fresnel(np.abs(ih))
    f = f if f.ndim == 2 else f[:, None]
    value = f * (d / (1.0 + li + lo) / (4.0 * np.abs(wi[:, 2]) * np.abs(wo[:, 2])))[:, None]
    pdf = (1.0 / (1.0 + li)) * np.maximum(0.0, ih) * d / i[:, 2] / (4.0 * np.abs(ih))
    return value, pdf


def _close(got, want, what):
    err = np.abs(got - want) / np.maximum(np.abs(want), 1e-6)
    k = int(np.argmax(err))
    assert err.max() <= RTOL, f"{what}: relative error {err.max():.3g} at {k}: {got.flat[k]} vs {want.flat[k]}"


# ---------------------------------------------------------------- lobes
METALS = [
    dict(specular_roughness=0.35),
    dict(specular_roughness=0.7, specular_roughness_anisotropy=0.6, specular_rotation=0.25),
    dict(specular_roughness=0.5, specular_roughness_anisotropy=0.3, specular_rotation=0.5,
         base_color=(0.95, 0.64, 0.54), specular_color=(0.9, 0.8, 0.6)),
    dict(specular_roughness=0.2, base_weight=0.8, base_color=(0.56, 0.57, 0.58), specular_weight=0.5),
]


@pytest.mark.parametrize("k", range(len(METALS)))
def test_metal_is_f82_tint_ggx(k):
    p = METALS[k]
    m = Material(base_metalness=1.0, **p)
    rng = np.random.default_rng(10 + k)
    wi, wo = _upper(rng, 6000), _upper(rng, 6000)
    n = min(len(wi), len(wo))
    wi, wo = wi[:n], wo[:n]
    f0 = m.base_weight * np.array(m.base_color[:3])
    tint = m.specular_weight * np.array(m.specular_color[:3])
    want, pdf = microfacet_reflection(wi, wo, m.specular_roughness, m.specular_roughness_anisotropy,
                                      m.specular_rotation, lambda mu: f82_tint(mu, f0, tint))
    got, got_pdf = _eval(m, wi.astype(np.float32), wo.astype(np.float32))
    keep = want.max(axis=1) > 1e-4  # very small values are dominated by float32 cancellation
    assert keep.sum() > 1000
    _close(got[keep], want[keep], "metal f")
    # a metal-only material selects the metal lobe with probability one
    keep_pdf = pdf > 1e-3
    _close(got_pdf[keep_pdf], pdf[keep_pdf], "metal pdf")


DIELECTRICS = [
    dict(specular_roughness=0.3, specular_ior=1.5),
    dict(specular_roughness=0.6, specular_ior=2.2, specular_roughness_anisotropy=0.5, specular_rotation=0.25),
    dict(specular_roughness=0.15, specular_ior=1.33, specular_color=(0.9, 0.7, 1.0)),
]


@pytest.mark.parametrize("k", range(len(DIELECTRICS)))
def test_dielectric_specular_is_fresnel_ggx(k):
    """Black base, full specular weight, no coat (coat_ior 1): the specular reflection alone."""
    m = Material(base_weight=0.0, specular_weight=1.0, coat_ior=1.0, **DIELECTRICS[k])
    rng = np.random.default_rng(20 + k)
    wi, wo = _upper(rng, 6000), _upper(rng, 6000)
    n = min(len(wi), len(wo))
    wi, wo = wi[:n], wo[:n]
    want, _ = microfacet_reflection(wi, wo, m.specular_roughness, m.specular_roughness_anisotropy,
                                    m.specular_rotation, lambda mu: fresnel_dielectric(mu, m.specular_ior))
    want = want * np.array(m.specular_color[:3])
    got, _ = _eval(m, wi.astype(np.float32), wo.astype(np.float32))
    keep = want.max(axis=1) > 1e-4
    assert keep.sum() > 1000
    _close(got[keep], want[keep], "dielectric specular f")


COATS = [
    dict(coat_weight=1.0, coat_roughness=0.25, coat_ior=1.6),
    dict(coat_weight=0.6, coat_roughness=0.5, coat_ior=1.4, coat_roughness_anisotropy=0.4, coat_rotation=0.5),
]


@pytest.mark.parametrize("k", range(len(COATS)))
def test_coat_is_fresnel_ggx(k):
    """Black base without specular reflection under the coat: the coat's reflection alone,
    scaled by the coat weight."""
    p = COATS[k]
    m = Material(base_weight=0.0, specular_weight=0.0, **p)
    rng = np.random.default_rng(30 + k)
    wi, wo = _upper(rng, 6000), _upper(rng, 6000)
    n = min(len(wi), len(wo))
    wi, wo = wi[:n], wo[:n]
    want, _ = microfacet_reflection(wi, wo, m.coat_roughness, m.coat_roughness_anisotropy, m.coat_rotation,
                                    lambda mu: fresnel_dielectric(mu, m.coat_ior))
    want = want * m.coat_weight
    got, _ = _eval(m, wi.astype(np.float32), wo.astype(np.float32))
    keep = want.max(axis=1) > 1e-4
    assert keep.sum() > 1000
    _close(got[keep], want[keep], "coat f")


def _hemisphere(nt=192, nphi=384):
    """Midpoint quadrature of the upper hemisphere in (cos theta, phi): directions and weights."""
    mu = (np.arange(nt) + 0.5) / nt
    phi = (np.arange(nphi) + 0.5) / nphi * 2.0 * np.pi
    M, P = np.meshgrid(mu, phi, indexing="ij")
    s = np.sqrt(1.0 - M * M)
    d = np.stack([s * np.cos(P), s * np.sin(P), M], axis=-1).reshape(-1, 3)
    return d, np.full(len(d), (1.0 / nt) * (2.0 * np.pi / nphi))


@pytest.mark.parametrize("sigma", [0.0, 0.3, 0.6, 1.0])
def test_energy_compensated_oren_nayar_conserves_energy(sigma):
    """White diffuse base (specular weight 0): albedo of bsdf_evaluate over the hemisphere."""
    m = Material(base_weight=1.0, base_color=(1.0, 1.0, 1.0), specular_weight=0.0, base_diffuse_roughness=sigma)
    wo, w = _hemisphere()
    for theta in (0.0, 30.0, 60.0, 80.0):
        t = np.radians(theta)
        wi = np.tile([np.sin(t), 0.0, np.cos(t)], (len(wo), 1))
        f, _ = _eval(m, wi.astype(np.float32), wo.astype(np.float32))
        albedo = np.sum(f[:, 0] * wo[:, 2] * w)
        assert abs(albedo - 1.0) < 2e-3, (sigma, theta, albedo)  # quadrature error ~1e-4


@pytest.mark.parametrize("roughness", [0.2, 0.5, 0.9])
def test_fuzz_is_a_linearly_transformed_cosine(roughness):
    """Black base without specular: the fuzz lobe alone, selected with probability one."""
    m = Material(base_weight=0.0, specular_weight=0.0, fuzz_weight=1.0, fuzz_roughness=roughness,
                 fuzz_color=(0.9, 0.6, 0.3))
    wo, w = _hemisphere(256, 512)
    for theta in (0.0, 40.0, 75.0):
        t = np.radians(theta)
        wi = np.tile([np.sin(t), 0.0, np.cos(t)], (len(wo), 1))
        f, pdf = _eval(m, wi.astype(np.float32), wo.astype(np.float32))
        mass = np.sum(pdf * w)
        assert abs(mass - 1.0) < 2e-3, (roughness, theta, mass)  # measured 1.0000-1.0001
        # f cos(o) = colour * albedo(cos i) * pdf: the ratio is one constant per incidence
        ok = pdf > 1e-3
        ratio = f[ok] * wo[ok, 2:3] / pdf[ok, None]
        spread = np.abs(ratio / ratio.mean(axis=0) - 1.0).max()
        assert spread < 1e-4, (roughness, theta, spread)
        colour = ratio.mean(axis=0) / ratio.mean(axis=0)[0]
        assert np.allclose(colour, np.array(m.fuzz_color[:3]) / m.fuzz_color[0], rtol=1e-5)
