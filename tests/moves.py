"""Seeded instance motion for the instance-update (refit) tests: each instance is rotated about
its own centre and translated; its inverse and normal transforms follow."""
import numpy as np


def _rotation(rng, angle):
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    k = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(angle) * k + (1 - np.cos(angle)) * (k @ k)


def moved_instances(instances: np.ndarray, rng, max_angle=0.6, max_shift=3.0, scale=0.0) -> np.ndarray:
    """`scale` > 0 also scales each instance about its centre by a factor in [1 - scale, 1 + scale]
    (world-space areas change)."""
    out = instances.copy()
    for i in range(len(out)):
        t = np.asarray(out[i]["transform"], np.float64).reshape(4, 4).T
        m = np.eye(4)
        r = _rotation(rng, rng.uniform(-max_angle, max_angle))
        if scale > 0.0:
            r = r * rng.uniform(1.0 - scale, 1.0 + scale)
        c = t[:3, 3]
        m[:3, :3] = r
        m[:3, 3] = c - r @ c + rng.uniform(-max_shift, max_shift, 3)
        t2 = m @ t
        n = np.asarray(out[i]["normal_transform"], np.float64).reshape(4, 4).T
        n2 = np.eye(4)
        n2[:3, :3] = np.linalg.inv(m[:3, :3]).T @ n[:3, :3]
        out[i]["transform"] = t2.T.ravel().astype(np.float32)
        out[i]["inverse_transform"] = np.linalg.inv(t2).T.ravel().astype(np.float32)
        out[i]["normal_transform"] = n2.T.ravel().astype(np.float32)
    return out
