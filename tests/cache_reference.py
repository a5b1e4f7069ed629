"""NumPy reference of the learned radiance cache (tinytrace_gb300/csrc/cache.cu): the hash-grid
encoding, the MLP forward pass in FP32 and in the FP16 arithmetic of the tensor-core queries,
the relative L2 loss and its gradients (float64), and Adam.  The CUDA kernels are checked
against it with the tolerances stated in the tests."""
import numpy as np

LEVELS, TABLE, WIDTH, HIDDEN, OUT_ROWS = 16, 1 << 19, 64, 4, 8
WEIGHTS = HIDDEN * WIDTH * WIDTH + OUT_ROWS * WIDTH
SCALES = np.array([16.0 * 128.0 ** (l / 15.0) for l in range(LEVELS)]).astype(np.float32)


def corners(p: np.ndarray, level: int):
    """(n, 8) table indices and (n, 8) trilinear weights of positions p (n, 3) in [0,1]^3."""
    s = SCALES[level]
    f = (np.clip(p, 0, 1).astype(np.float32) * s).astype(np.float32)
    f0 = np.floor(f)
    t = (f - f0).astype(np.float32)
    i = f0.astype(np.uint64)
    r = np.uint64(int(s) + 2)
    dense = int(r) ** 3 <= TABLE
    idx = np.zeros((len(p), 8), np.uint64)
    w = np.ones((len(p), 8), np.float32)
    for c in range(8):
        cx, cy, cz = i[:, 0] + (c & 1), i[:, 1] + ((c >> 1) & 1), i[:, 2] + ((c >> 2) & 1)
        if dense:
            h = cx + r * (cy + r * cz)
        else:
            h = (cx * np.uint64(1)) ^ ((cy * np.uint64(2654435761)) & np.uint64(0xFFFFFFFF)) ^ \
                ((cz * np.uint64(805459861)) & np.uint64(0xFFFFFFFF))
        idx[:, c] = (h & np.uint64(0xFFFFFFFF)) & np.uint64(TABLE - 1)
        wx = t[:, 0] if c & 1 else 1 - t[:, 0]
        wy = t[:, 1] if c & 2 else 1 - t[:, 1]
        wz = t[:, 2] if c & 4 else 1 - t[:, 2]
        w[:, c] = (wx * wy * wz).astype(np.float32)
    return idx.astype(np.int64), w


def encode(q: np.ndarray, grid: np.ndarray) -> np.ndarray:
    """q: (n, 12) queries; grid: (16, 2^19, 2).  Returns (n, 64) float64 inputs."""
    n = len(q)
    x = np.zeros((n, WIDTH))
    for l in range(LEVELS):
        idx, w = corners(q[:, 0:3], l)
        feats = grid[l][idx]  # (n, 8, 2)
        x[:, 2 * l:2 * l + 2] = (w[:, :, None].astype(np.float64) * feats).sum(axis=1)
    x[:, 32:35] = q[:, 3:6] * 0.5 + 0.5
    x[:, 35:38] = q[:, 6:9] * 0.5 + 0.5
    x[:, 38] = q[:, 9]
    return x


def split(weights: np.ndarray):
    ws = [weights[l * WIDTH * WIDTH:(l + 1) * WIDTH * WIDTH].reshape(WIDTH, WIDTH) for l in range(HIDDEN)]
    wo = weights[HIDDEN * WIDTH * WIDTH:].reshape(OUT_ROWS, WIDTH)[:3]
    return ws, wo


def forward(x: np.ndarray, weights: np.ndarray, fp16: bool = False):
    """Outputs (n, 3) and the hidden activations.  fp16: inputs, weights and hidden
    activations rounded to half precision between layers, as in the tensor-core queries."""
    ws, wo = split(weights.astype(np.float64))
    r = (lambda a: a.astype(np.float16).astype(np.float64)) if fp16 else (lambda a: a)
    h = [r(x)]
    for w in ws:
        h.append(r(np.maximum(h[-1] @ r(w).T, 0.0)))
    return h[-1] @ r(wo).T, h


def loss_and_grads(q, target, grid, weights):
    """Mean relative L2 loss over n * 3 outputs and its gradients (float64)."""
    x = encode(q, grid)
    y, h = forward(x, weights)
    n = len(q)
    d = y - target
    den = y * y + 0.01
    loss = (d * d / den).sum()
    dy = 2.0 * d / den / (3.0 * n)
    ws, wo = split(weights.astype(np.float64))
    g_wo = dy.T @ h[-1]
    delta = (dy @ wo) * (h[-1] > 0)
    g_ws = [None] * HIDDEN
    for l in range(HIDDEN - 1, -1, -1):
        g_ws[l] = delta.T @ h[l]
        delta = delta @ ws[l]
        if l > 0:
            delta = delta * (h[l] > 0)
    g_w = np.concatenate([g.ravel() for g in g_ws] + [np.vstack([g_wo, np.zeros((OUT_ROWS - 3, WIDTH))]).ravel()])
    g_grid = np.zeros(grid.shape)
    for l in range(LEVELS):
        idx, w = corners(q[:, 0:3], l)
        for c in range(8):
            np.add.at(g_grid[l], idx[:, c], w[:, c, None] * delta[:, 2 * l:2 * l + 2])
    return loss, g_w, g_grid


def adam(p, g, m, v, step, lr):
    m = 0.9 * m + 0.1 * g
    v = 0.99 * v + 0.01 * g * g
    c1, c2 = 1 - 0.9 ** step, 1 - 0.99 ** step
    return p - lr * (m / c1) / (np.sqrt(v / c2) + 1e-15), m, v


GRAD_SCALE = 1.0 / 64.0  # the kernel scales the output gradient into FP16 range and undoes it at the end
GRAD_CLAMP = 16384.0     # |dL/dy| per output before the mean's 1 / (3 n)


def grads_fp16(q, target, grid, weights):
    """The gradients of loss_and_grads computed with the training kernel's roundings: FP16
    inputs, weights, hidden activations, output gradient (clamped, scaled by GRAD_SCALE) and
    per-layer deltas; products accumulated in float64 here (FP32 on the tensor cores).
    Returns (summed loss, weight gradients, grid gradients)."""
    r = lambda a: a.astype(np.float16).astype(np.float64)  # noqa: E731
    x = encode(q, grid)
    ws, wo = split(weights.astype(np.float64))
    h = [r(x)]
    for w in ws:
        h.append(r(np.maximum(h[-1] @ r(w).T, 0.0)))
    y = h[-1] @ r(wo).T
    n = len(q)
    d = y - target
    den = y * y + 0.01
    loss = (d * d / den).sum()
    g = r(np.clip(2.0 * d / den, -GRAD_CLAMP, GRAD_CLAMP) * GRAD_SCALE)
    inv = 1.0 / (3.0 * n) / GRAD_SCALE
    g_wo = (g.T @ h[-1]) * inv
    grad = g @ r(wo)
    g_ws = [None] * HIDDEN
    for l in range(HIDDEN - 1, -1, -1):
        delta = r(np.where(h[l + 1] > 0, grad, 0.0))
        g_ws[l] = (delta.T @ h[l]) * inv
        grad = delta @ r(ws[l])
    g_w = np.concatenate([gw.ravel() for gw in g_ws] + [np.vstack([g_wo, np.zeros((OUT_ROWS - 3, WIDTH))]).ravel()])
    g_grid = np.zeros(grid.shape)
    gx = grad[:, :2 * LEVELS] * inv
    for l in range(LEVELS):
        idx, w = corners(q[:, 0:3], l)
        for c in range(8):
            np.add.at(g_grid[l], idx[:, c], w[:, c, None] * gx[:, 2 * l:2 * l + 2])
    return loss, g_w, g_grid
