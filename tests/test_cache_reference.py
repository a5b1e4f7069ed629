"""The NumPy reference of the radiance cache pinned by finite differences (CPU only): its
weight and grid gradients are the derivatives of its loss."""
import numpy as np

import cache_reference as cr


def _setup(seed=0, n=6):
    rng = np.random.default_rng(seed)
    grid = rng.uniform(-0.5, 0.5, (cr.LEVELS, cr.TABLE, 2))
    weights = rng.uniform(-0.3, 0.3, cr.WEIGHTS)
    weights[cr.HIDDEN * cr.WIDTH * cr.WIDTH + 3 * cr.WIDTH:] = 0.0
    q = np.zeros((n, 12))
    q[:, 0:3] = rng.uniform(0.05, 0.95, (n, 3))
    d = rng.normal(size=(n, 3))
    q[:, 3:6] = d / np.linalg.norm(d, axis=1, keepdims=True)
    q[:, 6:9] = q[:, 3:6]
    q[:, 9] = rng.uniform(0, 1, n)
    target = rng.uniform(0, 2, (n, 3))
    return rng, grid, weights, q, target


def test_weight_gradients():
    rng, grid, weights, q, target = _setup()
    _, g_w, _ = cr.loss_and_grads(q, target, grid, weights)
    for k in list(rng.integers(0, cr.HIDDEN * cr.WIDTH * cr.WIDTH, 6)) + [cr.HIDDEN * cr.WIDTH * cr.WIDTH + 5]:
        e = 1e-6
        wp, wm = weights.copy(), weights.copy()
        wp[k] += e
        wm[k] -= e
        lp = cr.loss_and_grads(q, target, grid, wp)[0] / (3 * len(q))
        lm = cr.loss_and_grads(q, target, grid, wm)[0] / (3 * len(q))
        # the denominator y^2 + 0.01 is not differentiated: compare with that convention
        fd = _fd_fixed_den(q, target, grid, weights, k, e)
        assert abs(fd - g_w[k]) <= 1e-6 + 1e-4 * abs(fd), (k, fd, g_w[k], (lp - lm) / (2 * e))


def _fd_fixed_den(q, target, grid, weights, k, e):
    x = cr.encode(q, grid)
    y0, _ = cr.forward(x, weights)
    den = y0 * y0 + 0.01
    out = []
    for s in (+e, -e):
        w = weights.copy()
        w[k] += s
        y, _ = cr.forward(x, w)
        out.append(((y - target) ** 2 / den).sum() / (3 * len(q)))
    return (out[0] - out[1]) / (2 * e)


def test_grid_gradients():
    rng, grid, weights, q, target = _setup(1, n=3)
    _, _, g_grid = cr.loss_and_grads(q, target, grid, weights)
    x = cr.encode(q, grid)
    y0, _ = cr.forward(x, weights)
    den = y0 * y0 + 0.01
    nz = np.argwhere(g_grid != 0)
    for l, i, f in nz[rng.choice(len(nz), 5, replace=False)]:
        vals = []
        for s in (1e-6, -1e-6):
            g = grid.copy()
            g[l, i, f] += s
            y, _ = cr.forward(cr.encode(q, g), weights)
            vals.append(((y - target) ** 2 / den).sum() / (3 * len(q)))
        fd = (vals[0] - vals[1]) / 2e-6
        assert abs(fd - g_grid[l, i, f]) <= 1e-7 + 1e-4 * abs(fd)


def test_corners_cover_the_cell():
    p = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [0.3, 0.7, 0.5]])
    for l in (0, 7, 15):
        idx, w = cr.corners(p, l)
        assert np.allclose(w.sum(axis=1), 1.0, atol=1e-6) and (idx >= 0).all() and (idx < cr.TABLE).all()
