"""Camera (src/camera.rs) and the glam matrix helpers it uses, restated with numpy.

`Camera.view()` is glam's `Mat4::look_at_rh`; `Camera.proj()` is
`Mat4::perspective_infinite_reverse_rh` with the reference's `z_axis[3] = 1` override
(src/camera.rs:41-45).  Matrices are float32, column-major when flattened (`.T.ravel()`).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

UP = np.array([0.0, 1.0, 0.0])


def look_at_rh(eye: np.ndarray, center: np.ndarray, up: np.ndarray) -> np.ndarray:
    """glam Mat4::look_at_rh (returns a row-major 4x4 float64 matrix M with M @ v)."""
    f = center - eye
    f = f / np.linalg.norm(f)
    s = np.cross(f, up)
    s = s / np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3] = s
    m[1, :3] = u
    m[2, :3] = -f
    m[0, 3] = -np.dot(eye, s)
    m[1, 3] = -np.dot(eye, u)
    m[2, 3] = np.dot(eye, f)
    return m


def perspective_infinite_reverse_rh(fov_y: float, aspect: float, z_near: float) -> np.ndarray:
    f = 1.0 / np.tan(0.5 * fov_y)
    m = np.zeros((4, 4))
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[3, 2] = -1.0
    m[2, 3] = z_near
    return m


def to_col_major(m: np.ndarray) -> np.ndarray:
    """Row-major numpy matrix -> 16 float32 in glam's column-major order."""
    return np.ascontiguousarray(np.asarray(m, np.float64).T.ravel(), dtype=np.float32)


@dataclass
class CameraMove:
    translation: np.ndarray = field(default_factory=lambda: np.zeros(3))
    yaw: float = 0.0
    pitch: float = 0.0


@dataclass
class Camera:
    """src/camera.rs:5-65"""

    position: np.ndarray = field(default_factory=lambda: np.zeros(3))
    yaw: float = 0.0
    pitch: float = 0.0
    z_near: float = 0.1
    z_far: float = 400.0
    fov: float = np.pi / 2.0

    def forward(self) -> np.ndarray:
        v = np.array([np.cos(self.yaw) * np.cos(self.pitch), np.sin(self.pitch), np.sin(self.yaw) * np.cos(self.pitch)])
        return v / np.linalg.norm(v)

    def right(self) -> np.ndarray:
        r = np.cross(self.forward(), UP)
        return -r / np.linalg.norm(r)

    def proj(self, aspect: float) -> np.ndarray:
        p = perspective_infinite_reverse_rh(self.fov, aspect, self.z_near)
        p[3, 2] = 1.0  # proj.z_axis[3] = 1.0
        return p

    def view(self) -> np.ndarray:
        pos = np.asarray(self.position, np.float64)
        return look_at_rh(pos, pos + self.forward(), UP)

    def move_by(self, delta: CameraMove) -> None:
        self.position = np.asarray(self.position, np.float64) + delta.translation
        self.yaw = (self.yaw - delta.yaw) % (2.0 * np.pi)
        self.pitch = float(np.clip(self.pitch - delta.pitch, -1.553, 1.553))

    def different_from(self, other: "Camera") -> bool:
        t = 1e-4
        return (np.max(np.abs(np.asarray(self.position) - np.asarray(other.position))) > t
                or abs(self.yaw - other.yaw) > t or abs(self.pitch - other.pitch) > t or abs(self.fov - other.fov) > t)

    def ray_direction(self, ndc_x: float, ndc_y: float, aspect: float) -> np.ndarray:
        """Direction of integrate.glsl:17-20 for one NDC point (host-side, for placing cameras)."""
        ip = np.linalg.inv(self.proj(aspect))
        iv = np.linalg.inv(self.view())
        v = ip @ np.array([-ndc_x, -ndc_y, 1.0, 1.0])
        d = (iv @ np.array([v[0], v[1], v[2], 0.0]))[:3]
        return d / np.linalg.norm(d)

    @staticmethod
    def looking_at(position, target, fov: float = np.pi / 2.0) -> "Camera":
        """A camera whose rendered image centre looks at `target`.  The reference's ray
        generation (integrate.glsl:17-20 with the z_axis[3] = 1 projection) sends primary
        rays along -forward, so forward is set opposite to the target direction."""
        d = np.asarray(target, np.float64) - np.asarray(position, np.float64)
        d = -d / np.linalg.norm(d)
        pitch = float(np.arcsin(np.clip(d[1], -1.0, 1.0)))
        yaw = float(np.arctan2(d[2], d[0]))
        return Camera(position=np.asarray(position, np.float64), yaw=yaw, pitch=pitch, fov=fov)
