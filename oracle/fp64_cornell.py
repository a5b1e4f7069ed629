"""TEST INFRASTRUCTURE — an independent float64 path tracer for Lambertian scenes, the source
of the converged reference images against which the GPU renders' RMSE is stated.

Only tests/ and the fixture generator beside them use it; it is the checker, never the product.
It estimates the same image as the reference integrator (src/integrate/integrate.glsl) for
scenes whose materials are purely Lambertian (OpenPBR with specular, coat, fuzz, transmission
and metalness at zero, diffuse roughness 0, specular roughness above 0.15 so that every
vertex does next-event estimation), by a different sampler:

* camera rays: the pixel jitter U[-0.5, 0.5)^2 and the camera_ray_direction of the reference
  (integrate.glsl:17-20, 129-132), in float64 from the float32 constants;
* closest hits: Moller-Trumbore against every triangle in float64 (world-space vertices from
  the snorm16 positions and the instance transforms), back faces culled for extension rays,
  t in [1e-3, 1000]; shadow rays not culled, t in [1e-3, 1e4];
* per vertex (integrate.glsl:270-321): next-event estimation with a uniformly chosen emissive
  triangle and a uniform point on it (visible when the shadow ray's first hit is that
  triangle), emission only at the primary hit, a miss adds the white sky, continuation by
  cosine-weighted sampling (throughput *= albedo), `bounce_count` segments.

Geometric normals stand in for the interpolated shading normals (the scenes used have flat
quads whose vertex normals are the face normals).
"""
from __future__ import annotations

import numpy as np


def world_triangles(arrays):
    """(n, 3, 3) float64 world vertices, (n,) instance index, (n,) emissive-triangle flag."""
    tris, inst, emis = [], [], []
    emissive_materials = set()
    mats = arrays.materials["constants"]
    for m in range(len(mats)):
        if float(mats[m]["emission_luminance"]) > 0.0:
            emissive_materials.add(m)
    for i, ins in enumerate(arrays.instances):
        me = arrays.meshes[int(ins["mesh_index"])]
        t = np.asarray(ins["transform"], np.float64).reshape(4, 4).T
        idx = arrays.indices[int(me["index_offset"]):int(me["index_offset"]) + int(me["index_count"]) // 3 * 3]
        p = arrays.positions[idx.astype(np.int64) + int(me["vertex_offset"])].astype(np.float64) / 32767.0
        w = p @ t[:3, :3].T + t[:3, 3]
        tris.append(w.reshape(-1, 3, 3))
        inst.append(np.full(len(idx) // 3, i))
        emis.append(np.full(len(idx) // 3, int(ins["material_index"]) in emissive_materials))
    return np.concatenate(tris), np.concatenate(inst), np.concatenate(emis)


def _intersect(o, d, tri, tmin, tmax, cull):
    """Closest hit of rays (o, d) (m, 3) against triangles (n, 3, 3): (t, triangle), triangle -1
    for a miss."""
    p0, e1, e2 = tri[:, 0], tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]
    pv = np.cross(d[:, None, :], e2[None, :, :])                  # (m, n, 3)
    det = np.einsum("mnk,nk->mn", pv, e1)
    inv = 1.0 / np.where(det == 0.0, np.inf, det)
    tv = o[:, None, :] - p0[None, :, :]
    u = np.einsum("mnk,mnk->mn", tv, pv) * inv
    qv = np.cross(tv, e1[None, :, :])
    v = np.einsum("mnk,mk->mn", qv, d) * inv
    t = np.einsum("mnk,nk->mn", qv, e2) * inv
    ok = (u >= 0) & (v >= 0) & (u + v <= 1) & (t >= tmin) & (t <= tmax) & (det != 0.0)
    if cull:  # front faces: counter-clockwise seen from the ray origin, dot(d, cross(e1, e2)) < 0
        ok &= det > 0.0
    t = np.where(ok, t, np.inf)
    k = np.argmin(t, axis=1)
    tk = t[np.arange(len(o)), k]
    return tk, np.where(np.isfinite(tk), k, -1)


def _frame(n):
    a = np.where(np.abs(n[:, 0:1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t = np.cross(a, n)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    return t, np.cross(n, t)


def render(arrays, constants, spp: int, seed: int = 0, batch_pixels: int = 512) -> np.ndarray:
    """(H, W, 3) float64 mean radiance over `spp` samples per pixel."""
    c = constants
    W, H = (int(v) for v in c["screen_size"])
    depth = int(c["bounce_count"])
    inv_view = np.asarray(c["inverse_view"], np.float64).reshape(4, 4).T
    inv_proj = np.asarray(c["inverse_proj"], np.float64).reshape(4, 4).T
    cam = np.asarray(c["camera_position"], np.float64)[:3]
    tri, inst, emis = world_triangles(arrays)
    n_geo = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    area = 0.5 * np.linalg.norm(n_geo, axis=1)
    n_geo = n_geo / np.linalg.norm(n_geo, axis=1, keepdims=True)
    mats = arrays.materials["constants"]
    mat_of = np.array([int(arrays.instances[i]["material_index"]) for i in inst])
    albedo = np.array([np.asarray(mats[m]["base_color"][:3], np.float64) * float(mats[m]["base_weight"])
                       for m in mat_of])
    emission = np.array([np.asarray(mats[m]["emission_color"][:3], np.float64) * float(mats[m]["emission_luminance"])
                         for m in mat_of])
    lights = np.nonzero(emis)[0]
    rng = np.random.default_rng(seed)
    out = np.zeros((H * W, 3))
    pix = np.arange(H * W)
    for start in range(0, H * W, batch_pixels):
        px = pix[start:start + batch_pixels]
        m = len(px) * spp
        x = np.repeat(px % W, spp).astype(np.float64)
        y = np.repeat(px // W, spp).astype(np.float64)
        jitter = rng.random((m, 2)) - 0.5
        ndc = np.stack([((x + jitter[:, 0]) / W) * 2 - 1, ((y + jitter[:, 1]) / H) * 2 - 1], 1)
        vs = np.stack([-ndc[:, 0], -ndc[:, 1], np.ones(m), np.ones(m)], 1) @ inv_proj.T
        wd = np.concatenate([vs[:, :3], np.zeros((m, 1))], 1) @ inv_view.T
        d = wd[:, :3] / np.linalg.norm(wd[:, :3], axis=1, keepdims=True)
        o = np.repeat(cam[None], m, 0)
        thr = np.ones((m, 3))
        acc = np.zeros((m, 3))
        alive = np.ones(m, bool)
        for bounce in range(depth):
            idx = np.nonzero(alive)[0]
            if len(idx) == 0:
                break
            t, k = _intersect(o[idx], d[idx], tri, 1e-3, 1000.0, True)
            miss = k < 0
            acc[idx[miss]] += thr[idx[miss]]
            alive[idx[miss]] = False
            idx, t, k = idx[~miss], t[~miss], k[~miss]
            if len(idx) == 0:
                break
            pos = o[idx] + t[:, None] * d[idx]
            n = n_geo[k]
            rho = albedo[k]
            if bounce == 0:
                acc[idx] += thr[idx] * emission[k]
            if len(lights):  # next-event estimation
                li = lights[rng.integers(0, len(lights), len(idx))]
                r = rng.random((len(idx), 2))
                su = np.sqrt(r[:, 0])
                b1, b2 = 1 - su, r[:, 1] * su
                lp = tri[li, 0] * b1[:, None] + tri[li, 1] * b2[:, None] + tri[li, 2] * (1 - b1 - b2)[:, None]
                to = lp - pos
                d2 = np.einsum("ij,ij->i", to, to)
                dist = np.sqrt(d2)
                ldir = to / dist[:, None]
                cos_s = np.einsum("ij,ij->i", n, ldir)
                cos_l = -np.einsum("ij,ij->i", n_geo[li], ldir)
                ts, ks = _intersect(pos, ldir, tri, 1e-3, 1e4, False)
                vis = (ks == li) & (cos_s > 0) & (cos_l > 0)
                pdf = d2 / (np.maximum(cos_l, 1e-300) * area[li]) / len(lights)
                contrib = rho / np.pi * emission[li] * cos_s[:, None] / pdf[:, None]
                acc[idx] += np.where(vis[:, None], thr[idx] * contrib, 0.0)
            # continuation: cosine-weighted, throughput *= albedo
            r = rng.random((len(idx), 2))
            rr, ph = np.sqrt(r[:, 0]), 2 * np.pi * r[:, 1]
            lx, ly = rr * np.cos(ph), rr * np.sin(ph)
            lz = np.sqrt(np.maximum(0.0, 1 - lx * lx - ly * ly))
            tb, bb = _frame(n)
            d[idx] = lx[:, None] * tb + ly[:, None] * bb + lz[:, None] * n
            o[idx] = pos
            thr[idx] *= rho
        out[px] = acc.reshape(len(px), spp, 3).mean(axis=1)
    return out.reshape(H, W, 3)
