"""The margin of the rasterised camera-ray bound (tinytrace_gb300/csrc/primary.cu), checked on the
CPU against the float arithmetic of the camera rays and of the ray/triangle test.

The key pass tests a (record, sample) pair only when the sample's pixel position lies inside the
record's projected triangle widened by a margin; the hits must then be exactly the traversal's.
That holds if every hit the float ray/triangle test reports lies within the margin of the exact
projection.  Here the device's operations are restated in numpy float32, operation by operation
(IEEE single precision, no contraction: camera_ray_direction, pixel_ndc, instance_ray,
ray_precompute and the watertight intersect_triangle with its double-precision edge fallback),
and the exact projection of the triangle is computed in float64 through C^-1 = (X B)^-1 as the
kernel does.  Over random cameras (fields of view from 3 to 160 degrees), instances (rotations,
mirrors, scale ratios up to 1000) and triangles, with samples spread over the triangle's pixels
and placed on and just off its projected edges, the largest distance of a hit outside the
projected triangle must stay within the kernel's margin without its float-projection term
(BASE_MARGIN_PX + COND_MARGIN x cond(X) x pixels per radian).  Tolerance: that margin; the
distances measured are around 1e-4 pixel.
"""
import numpy as np

from tinytrace_gb300 import scenes
from tinytrace_gb300.renderer import Config, make_constants

F = np.float32
BASE_MARGIN_PX = 0.05  # primary.cu
COND_MARGIN = 2.0e-6   # primary.cu
TMIN, TMAX = F(1.0e-3), F(1000.0)


def mat4_mul(m, v):
    """tt_common.cuh mat4_mul: column-major m, each row summed left to right in float32."""
    rows = []
    for r in range(4):
        acc = m[r] * v[..., 0]
        acc = acc + m[4 + r] * v[..., 1]
        acc = acc + m[8 + r] * v[..., 2]
        acc = acc + m[12 + r] * v[..., 3]
        rows.append(acc)
    return np.stack(rows, -1)


def camera_ray_direction(c, ndc):
    ip = c["inverse_proj"].astype(F)
    iv = c["inverse_view"].astype(F)
    one = np.ones(ndc.shape[:-1], F)
    vsp = mat4_mul(ip, np.stack([-ndc[..., 0], -ndc[..., 1], one, one], -1))
    wd = mat4_mul(iv, np.stack([vsp[..., 0], vsp[..., 1], vsp[..., 2], np.zeros_like(one)], -1))
    d = wd[..., :3]
    dd = d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2]
    inv = F(1.0) / np.sqrt(dd)
    return d * inv[..., None]


def pixel_ndc_from_draws(px, py, W, H, ox, oy):
    offx, offy = ox - F(0.5), oy - F(0.5)
    nx = ((px.astype(F) + offx) / F(W)) * F(2.0) - F(1.0)
    ny = ((py.astype(F) + offy) / F(H)) * F(2.0) - F(1.0)
    return np.stack([nx, ny], -1)


def instance_ray(rows, o, d):
    r0, r1, r2 = rows
    oo = np.stack([r[0] * o[0] + r[1] * o[1] + r[2] * o[2] + r[3] * F(1.0) for r in (r0, r1, r2)], -1)
    od = np.stack([r[0] * d[..., 0] + r[1] * d[..., 1] + r[2] * d[..., 2] for r in (r0, r1, r2)], -1)
    return oo, od


def intersect(oo, od, p0, p1, p2):
    """ray_precompute + intersect_triangle (tt_bvh.cuh), cull back faces, tmin/tmax of extension rays."""
    ad = np.abs(od)
    kz = np.zeros(od.shape[0], np.int64)
    kz = np.where(ad[:, 1] > ad[:, 0], 1, kz)
    kz = np.where(ad[:, 2] > ad[np.arange(len(kz)), kz], 2, kz)
    kx = np.where(kz + 1 == 3, 0, kz + 1)
    ky = np.where(kx + 1 == 3, 0, kx + 1)
    idx = np.arange(len(kz))
    dz = od[idx, kz]
    swap = dz < 0
    kx, ky = np.where(swap, ky, kx), np.where(swap, kx, ky)
    sx = od[idx, kx] / dz
    sy = od[idx, ky] / dz
    sz = F(1.0) / dz
    A, B, C = p0 - oo, p1 - oo, p2 - oo
    Akz, Bkz, Ckz = A[idx, kz], B[idx, kz], C[idx, kz]
    Ax, Ay = A[idx, kx] - sx * Akz, A[idx, ky] - sy * Akz
    Bx, By = B[idx, kx] - sx * Bkz, B[idx, ky] - sy * Bkz
    Cx, Cy = C[idx, kx] - sx * Ckz, C[idx, ky] - sy * Ckz
    U = Cx * By - Cy * Bx
    V = Ax * Cy - Ay * Cx
    W = Bx * Ay - By * Ax
    fix = (U == 0) | (V == 0) | (W == 0)
    if fix.any():
        d = lambda v: v.astype(np.float64)
        U = np.where(fix, (d(Cx) * d(By) - d(Cy) * d(Bx)).astype(F), U)
        V = np.where(fix, (d(Ax) * d(Cy) - d(Ay) * d(Cx)).astype(F), V)
        W = np.where(fix, (d(Bx) * d(Ay) - d(By) * d(Ax)).astype(F), W)
    neg = (U < 0) | (V < 0) | (W < 0)
    det = U + V + W
    T = U * (sz * Akz) + V * (sz * Bkz) + W * (sz * Ckz)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = T * (F(1.0) / det)
    return ~neg & (det != 0) & (t >= TMIN) & (t <= TMAX)


def random_rotation(rng):
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    return q * np.sign(np.diag(r))


def check_config(rng):
    W, H = int(rng.integers(16, 2000)), int(rng.integers(16, 1200))
    fov = float(rng.uniform(0.05, 2.8))
    # instance: rotation x scales (ratios up to 1000, sometimes mirrored), somewhere in front
    s = np.exp(rng.uniform(np.log(0.05), np.log(50.0), 3))
    if rng.random() < 0.3:
        s[int(rng.integers(3))] *= -1.0
    xform = np.eye(4)
    xform[:3, :3] = random_rotation(rng) @ np.diag(s)
    xform[:3, 3] = rng.uniform(-20, 20, 3)
    inv = np.linalg.inv(xform).astype(F)
    rows = [np.array([inv[r, 0], inv[r, 1], inv[r, 2], inv[r, 3]], F) for r in range(3)]
    tri = rng.uniform(-1, 1, (3, 3)).astype(F) * F(rng.uniform(0.001, 1.0))
    tri += rng.uniform(-1, 1, 3).astype(F) * F(0.5)
    world = (xform[:3, :3] @ tri.astype(np.float64).T).T + xform[:3, 3]
    target = world.mean(0)
    dist = float(np.exp(rng.uniform(np.log(0.5), np.log(200.0))))
    pos = target + random_rotation(rng)[0] * dist
    cam = scenes.Camera.looking_at(pos, target + rng.normal(size=3) * 0.1 * dist, fov=fov)
    c = make_constants(cam, (W, H), Config(), 0, 0)
    O = c["camera_position"][:3].astype(F)
    oo, _ = instance_ray(rows, O, np.zeros((1, 3), F))
    oo = oo[0]
    # front face towards the camera (extension rays cull back faces)
    n = np.cross((tri[1] - tri[0]).astype(np.float64), (tri[2] - tri[0]).astype(np.float64))
    if np.dot(n, oo.astype(np.float64) - tri[0]) < 0:
        tri = tri[[0, 2, 1]]
    # exact projection (float64): B maps (ndc, 1) to the world direction, C = X B
    ip = c["inverse_proj"].astype(np.float64)
    iv = c["inverse_view"].astype(np.float64)
    A = np.array([[-ip[r], -ip[4 + r], ip[8 + r] + ip[12 + r]] for r in range(3)])
    V = np.array([[iv[j * 4 + r] for j in range(3)] for r in range(3)])
    Bm = V @ A
    X = np.array([[float(rows[r][j]) for j in range(3)] for r in range(3)])
    Ci = np.linalg.inv(X @ Bm)
    q = (tri.astype(np.float64) - oo.astype(np.float64)) @ Ci.T
    if (q[:, 2] <= 0).any():
        return None  # crosses or lies behind the camera plane: not this check's case
    P = np.stack([(q[:, 0] / q[:, 2] + 1.0) * 0.5 * W, (q[:, 1] / q[:, 2] + 1.0) * 0.5 * H], -1)
    area = (P[1, 0] - P[0, 0]) * (P[2, 1] - P[0, 1]) - (P[1, 1] - P[0, 1]) * (P[2, 0] - P[0, 0])
    if abs(area) < 1e-3 or np.abs(P).max() > 1e5:
        return None
    # samples: random draws over the triangle's pixels, and positions on and just off its edges
    lo, hi = np.floor(P.min(0)) - 1, np.ceil(P.max(0)) + 1
    npix = 3000
    pts = rng.uniform(lo, hi, (npix, 2))
    k = rng.integers(0, 3, 3000)
    f = rng.random(3000)[:, None]
    e0, e1 = P[k], P[(k + 1) % 3]
    edge = e0 + (e1 - e0) * f
    nrm = np.stack([-(e1 - e0)[:, 1], (e1 - e0)[:, 0]], -1)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    off = rng.choice([0.0, 1e-6, -1e-6, 1e-4, -1e-4, 1e-3, -1e-3, 1e-2, -1e-2], 3000)[:, None]
    pts = np.concatenate([pts, edge + nrm * off])
    pix = np.floor(pts + 0.5)
    inside = (pix[:, 0] >= 0) & (pix[:, 0] < W) & (pix[:, 1] >= 0) & (pix[:, 1] < H)
    pts, pix = pts[inside], pix[inside]
    if len(pts) == 0:
        return None
    # the draws: float32 values of the 23-bit mantissa grid, as random_float gives them
    m = np.clip(np.round((pts - pix + 0.5) * 2.0 ** 23), 0, 2 ** 23 - 1)
    ox, oy = (m[:, 0] / 2.0 ** 23).astype(F), (m[:, 1] / 2.0 ** 23).astype(F)
    px, py = pix[:, 0].astype(np.int64), pix[:, 1].astype(np.int64)
    d = camera_ray_direction(c, pixel_ndc_from_draws(px, py, W, H, ox, oy))
    _, od = instance_ray(rows, O, d)
    ooo = np.broadcast_to(oo, od.shape).astype(F)
    hit = intersect(ooo, od, tri[0], tri[1], tri[2]) & np.isfinite(od).all(1)
    if not hit.any():
        return None
    # distance of each hit's sample position outside the exact projected triangle
    sp = np.stack([px + (ox.astype(np.float64) - 0.5), py + (oy.astype(np.float64) - 0.5)], -1)[hit]
    sgn = 1.0 if area > 0 else -1.0
    out = np.zeros(len(sp))
    for j in range(3):
        a, b = P[j], P[(j + 1) % 3]
        nn = sgn * np.array([-(b - a)[1], (b - a)[0]]) / np.linalg.norm(b - a)
        out = np.maximum(out, -((sp - a) @ nn))
    # the kernel's margin without its float-projection term
    Bi = np.linalg.inv(Bm)
    ex, ey = 1.0 + 1.0 / W + 0.01, 1.0 + 1.0 / H + 0.01
    maxb = max(np.linalg.norm(Bm @ np.array([sx * ex, sy * ey, 1.0])) for sx in (-1, 1) for sy in (-1, 1))
    scale = 0.5 * max(W, H) * np.linalg.norm(Bi) * (1.0 + np.hypot(ex, ey)) * maxb
    cond = np.linalg.norm(X) * np.linalg.norm(np.linalg.inv(X))
    margin = BASE_MARGIN_PX + COND_MARGIN * cond * scale
    return float(out.max()), margin, int(hit.sum())


def test_hits_stay_within_the_margin():
    rng = np.random.default_rng(1234)
    checked = hits = 0
    worst = 0.0
    for _ in range(1000):
        r = check_config(rng)
        if r is None:
            continue
        out, margin, n = r
        checked += 1
        hits += n
        worst = max(worst, out)
        assert out <= margin, f"a hit lies {out} pixels outside the projected triangle (margin {margin})"
    assert checked >= 150 and hits >= 100000
    assert worst < 0.01, worst  # the rounding the base margin covers is far below it
