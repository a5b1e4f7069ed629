"""Renderer — the host-side mirror of the reference's public API (src/lib.rs, src/config.rs,
src/scene.rs) over the C ABI of libtinytrace_cuda.so.

Method names, argument meaning and state handling follow `tinytrace::Renderer`:
`set_scene`, `config`/`set_config` (a changed config resets accumulation), `resize`,
`render_to_target` (builds the 368-byte Constants, renders, bumps the accumulated frame
count), `reset_accumulation`, `timings`, `render_to_texture`.  The swapchain path
(`prepare_to_present`/`present`) becomes `tonemap()` into host memory plus `present()`,
which advances the frame index as the reference's present does.
"""
from __future__ import annotations

import ctypes
import enum
from dataclasses import dataclass

import numpy as np

from . import native
from .asset import Scene as AssetScene
from .asset import depth_first_node_tree
from .camera import Camera, to_col_major
from .native import CONSTANTS_DTYPE, EMISSIVE_DTYPE, INSTANCE_DTYPE, SceneDesc, check


class LightSampling(enum.IntEnum):
    """src/config.rs:3-12"""

    ON_HIT = 1
    NEXT_EVENT_ESTIMATION = 2


@dataclass(frozen=True)
class Config:
    """src/config.rs:23-43 (defaults: 4 bounces, 1 sample, tonemap on, NEE)."""

    bounce_count: int = 4
    sample_count: int = 1
    tonemap: bool = True
    light_sampling: LightSampling = LightSampling.NEXT_EVENT_ESTIMATION


@dataclass
class Timings:
    """src/lib.rs:228-232, in seconds of device time."""

    integrate: float
    post_process: float


def _scale_translation(center: np.ndarray, radius: float) -> np.ndarray:
    m = np.eye(4)
    m[:3, :3] *= radius
    m[:3, 3] = center
    return m


def flatten_scene(scene: AssetScene, emissive_fn=None) -> tuple[np.ndarray, np.ndarray]:
    """Scene::new's node-tree walk (src/scene.rs:29-64): one Instance per model with
    position transform = node transform * S(radius) T(centre), inverse, normal transform
    = transform^-T, plus the emissive triangles of emissive models.  `emissive_fn`, when
    given, extracts the triangles of all emissive (mesh index, instance index) models in one
    call (DeviceIngest.emissive_triangles) instead of model by model on the host."""
    instances: list = []
    emissive: list = []
    emissive_models: list = []

    def visit(_index, node, parent):
        transform = parent @ np.asarray(node.transform, np.float64)
        for model in node.models:
            mesh = scene.meshes[model.mesh_index]
            pos_t = transform @ _scale_translation(np.asarray(mesh["center"], np.float64), float(mesh["radius"]))
            inst = np.zeros((), INSTANCE_DTYPE)
            inst["transform"] = to_col_major(pos_t)
            inst["inverse_transform"] = to_col_major(np.linalg.inv(pos_t))
            inst["normal_transform"] = to_col_major(np.linalg.inv(transform).T)
            inst["vertex_offset"] = mesh["vertex_offset"]
            inst["index_offset"] = mesh["index_offset"]
            inst["material_index"] = model.material_index
            inst["mesh_index"] = model.mesh_index
            idx = len(instances)
            instances.append(inst)
            if emissive_fn is not None:
                if model.material_index in scene.emissive_materials:
                    emissive_models.append((model.mesh_index, idx))
                continue
            tris = scene.emissive_triangles_in_model(model, idx)
            if tris is not None:
                emissive.append(tris)
        return transform

    depth_first_node_tree(scene.root, np.eye(4), visit)
    inst_arr = np.array(instances, INSTANCE_DTYPE).reshape(-1) if instances else np.zeros(0, INSTANCE_DTYPE)
    if emissive_fn is not None:
        emissive = [emissive_fn(emissive_models)] if emissive_models else []
    em_arr = np.concatenate(emissive) if emissive else np.zeros(0, EMISSIVE_DTYPE)
    return np.ascontiguousarray(inst_arr), np.ascontiguousarray(em_arr)


class SceneArrays:
    """The byte arrays of one scene exactly as tt_scene_desc borrows them."""

    def __init__(self, scene: AssetScene, emissive_fn=None):
        self.positions = np.ascontiguousarray(scene.positions, np.int16).reshape(-1, 3)
        self.indices = np.ascontiguousarray(scene.indices, np.uint32)
        self.vertices = np.ascontiguousarray(scene.vertices)
        self.materials = np.ascontiguousarray(scene.material_array)
        self.meshes = np.ascontiguousarray(scene.mesh_array)
        self.instances, self.emissive = flatten_scene(scene, emissive_fn)
        # textures: (format, width, height, level count, byte count) rows and all level data
        textures = getattr(scene, "textures", [])
        self.texture_info = np.array([(t.format, t.width, t.height, len(t.levels), len(t.data)) for t in textures],
                                     np.uint64).reshape(-1, 5)
        self.texture_data = np.frombuffer(b"".join(t.data for t in textures), np.uint8).copy()

    FIELDS = ("positions", "indices", "vertices", "materials", "meshes", "instances", "emissive", "texture_info",
              "texture_data")

    def save(self, path, prefix: str = "") -> dict:
        """The arrays as a dict (and, when `path` is given, an .npz file) for reloading with
        `from_arrays` without re-running the scene generator."""
        d = {prefix + k: getattr(self, k) for k in self.FIELDS}
        if path is not None:
            np.savez_compressed(path, **d)
        return d

    @classmethod
    def from_arrays(cls, data, prefix: str = "") -> "SceneArrays":
        self = cls.__new__(cls)
        empty = {"texture_info": np.zeros((0, 5), np.uint64), "texture_data": np.zeros(0, np.uint8)}
        for k in cls.FIELDS:
            v = data[prefix + k] if (prefix + k) in data else empty[k]
            setattr(self, k, np.ascontiguousarray(v))
        return self

    def texture_descs(self):
        """ctypes array of tt_texture pointing into texture_data (kept alive by the caller)."""
        info = np.asarray(self.texture_info, np.uint64).reshape(-1, 5)
        arr = (native.TextureDesc * max(len(info), 1))()
        base = self.texture_data.ctypes.data if self.texture_data.size else None
        at = 0
        for i, (fmt, w, h, levels, nbytes) in enumerate(info.tolist()):
            arr[i].format, arr[i].width, arr[i].height, arr[i].level_count = fmt, w, h, levels
            arr[i].data = (base + at) if base is not None and nbytes else None
            arr[i].bytes = nbytes
            at += nbytes
        return arr

    @property
    def triangle_count(self) -> int:
        return int(sum(int(m["index_count"]) // 3 for m in self.meshes))

    def desc(self) -> SceneDesc:
        d = SceneDesc()
        d.positions = native.ptr(self.positions)
        d.position_count = len(self.positions)
        d.indices = native.ptr(self.indices)
        d.index_count = len(self.indices)
        d.vertices = native.ptr(self.vertices)
        d.vertex_count = len(self.vertices)
        d.materials = native.ptr(self.materials)
        d.material_count = len(self.materials)
        d.mesh_count = len(self.meshes)
        d.meshes = native.ptr(self.meshes)
        d.instances = native.ptr(self.instances)
        d.instance_count = len(self.instances)
        d.emissive_triangle_count = len(self.emissive)
        d.emissive_triangles = native.ptr(self.emissive)
        self._texture_descs = self.texture_descs()
        d.textures = ctypes.addressof(self._texture_descs)
        d.texture_count = len(self.texture_info)
        return d


def make_constants(camera: Camera, extent: tuple[int, int], config: Config, frame_index: int,
                   accumulated_frame_count: int) -> np.ndarray:
    """Constants of Renderer::render_to_target (src/lib.rs:124-142)."""
    w, h = extent
    aspect = float(np.float32(w) / np.float32(h))
    view = camera.view()
    proj = camera.proj(aspect)
    c = np.zeros((), CONSTANTS_DTYPE)
    c["view"] = to_col_major(view)
    c["proj"] = to_col_major(proj)
    c["proj_view"] = to_col_major(proj @ view)
    c["inverse_view"] = to_col_major(np.linalg.inv(view))
    c["inverse_proj"] = to_col_major(np.linalg.inv(proj))
    c["camera_position"] = (*np.asarray(camera.position, np.float32), 0.0)
    c["frame_index"] = frame_index
    c["accumulated_frame_count"] = accumulated_frame_count
    c["sample_count"] = config.sample_count
    c["bounce_count"] = config.bounce_count
    c["screen_size"] = (w, h)
    c["tonemap"] = 1 if config.tonemap else 0
    c["light_sampling"] = int(config.light_sampling)
    return c


class Context:
    """Owner of a tt_context (the backend Context of the reference)."""

    def __init__(self, device: int = 0):
        self.lib = native.load()
        h = ctypes.c_void_p()
        check(self.lib.tt_context_create(device, ctypes.byref(h)))
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self.lib.tt_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def frame_index(self) -> int:
        v = ctypes.c_uint64()
        check(self.lib.tt_frame_index(self.handle, ctypes.byref(v)))
        return v.value

    def create_image(self, lifetime: int, width: int, height: int) -> int:
        h = ctypes.c_uint64()
        check(self.lib.tt_image_create(self.handle, lifetime, width, height, ctypes.byref(h)))
        return h.value

    def create_scene(self, arrays: SceneArrays) -> int:
        d = arrays.desc()
        h = ctypes.c_uint64()
        check(self.lib.tt_scene_create(self.handle, ctypes.byref(d), ctypes.byref(h)))
        return h.value

    def scene_stats(self, scene: int) -> native.SceneStats:
        s = native.SceneStats()
        check(self.lib.tt_scene_stats_get(self.handle, scene, ctypes.byref(s)))
        return s

    def download(self, image: int, width: int, height: int, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((height, width, 4), np.float32)
        check(self.lib.tt_image_download(self.handle, image, native.ptr(out), out.nbytes))
        return out

    def write_image(self, image: int, data: np.ndarray) -> None:
        data = np.ascontiguousarray(data, np.float32)
        check(self.lib.tt_image_write(self.handle, image, native.ptr(data), data.nbytes))

    def clear_lifetime(self, lifetime: int) -> None:
        check(self.lib.tt_clear_lifetime(self.handle, lifetime))


class Renderer:
    """tinytrace::Renderer (src/lib.rs:31-211) without a window."""

    def __init__(self, extent: tuple[int, int], device: int = 0):
        self.context = Context(device)
        self.extent = tuple(extent)
        self.render_target = self.context.create_image(native.TT_LIFETIME_SURFACE, *self.extent)
        self.camera = Camera()
        self._config = Config()
        self.accumulated_frame_count = 0
        self.scene = None
        self.scene_arrays = None
        self.set_scene(AssetScene())

    def set_scene(self, scene: AssetScene) -> None:
        """src/lib.rs:97-102"""
        self.context.clear_lifetime(native.TT_LIFETIME_SCENE)
        arrays = SceneArrays(scene)
        self.scene = self.context.create_scene(arrays)
        self.scene_arrays = arrays

    def config(self) -> Config:
        return self._config

    def set_config(self, config: Config) -> None:
        """src/lib.rs:108-114"""
        if self._config != config:
            self.reset_accumulation()
        self._config = config

    def resize(self, extent: tuple[int, int]) -> None:
        """src/lib.rs:116-122"""
        self.render_target = self.context.create_image(native.TT_LIFETIME_SURFACE, *extent)
        self.extent = tuple(extent)
        self.reset_accumulation()

    def constants(self) -> np.ndarray:
        return make_constants(self.camera, self.extent, self._config, self.context.frame_index(),
                              self.accumulated_frame_count)

    def render_to_target(self) -> None:
        """src/lib.rs:124-161"""
        c = self.constants()
        check(self.context.lib.tt_render(self.context.handle, self.scene, native.ptr(c), self.render_target))
        self.accumulated_frame_count += 1

    def render_restir_to_target(self) -> None:
        """One ReSTIR DI frame (direct light at the primary hit, 1 sample per pixel) into the
        render target, with the same accumulation rule as render_to_target."""
        c = self.constants()
        check(self.context.lib.tt_render_restir(self.context.handle, self.scene, native.ptr(c), self.render_target))
        self.accumulated_frame_count += 1

    def restir_configure(self, candidates: int = 32, temporal_m_cap: float = 20.0, spatial_neighbours: int = 5,
                         spatial_radius: float = 30.0) -> None:
        cfg = native.RestirConfig(candidates, temporal_m_cap, spatial_neighbours, spatial_radius)
        check(self.context.lib.tt_restir_configure(self.context.handle, ctypes.byref(cfg)))

    def restir_reset(self) -> None:
        check(self.context.lib.tt_restir_reset(self.context.handle))

    def restir_reservoirs(self) -> np.ndarray:
        w, h = self.extent
        out = np.zeros((h, w, 8), np.float32)
        check(self.context.lib.tt_restir_download(self.context.handle, native.ptr(out), out.nbytes))
        return out

    def autotune(self, sample_count: int = 8) -> native.TuneResult:
        """Tunes the wavefront integrator's pool size, refill threshold and trace-kernel
        residency for the current scene and camera (tt_autotune) with short renders of
        `sample_count` samples per pixel.  The accumulation restarts afterwards."""
        cfg = Config(bounce_count=self._config.bounce_count, sample_count=sample_count, tonemap=self._config.tonemap,
                     light_sampling=self._config.light_sampling)
        c = make_constants(self.camera, self.extent, cfg, self.context.frame_index(), 0)
        res = native.TuneResult()
        check(self.context.lib.tt_autotune(self.context.handle, self.scene, native.ptr(c), self.render_target,
                                           ctypes.byref(res)))
        self.accumulated_frame_count = 0
        return res

    def reset_accumulation(self) -> None:
        self.accumulated_frame_count = 0

    def timings(self) -> Timings:
        t = native.Timings()
        check(self.context.lib.tt_timings_get(self.context.handle, ctypes.byref(t)))
        return Timings(t.integrate_ns * 1e-9, t.post_process_ns * 1e-9)

    def render_to_texture(self) -> np.ndarray:
        """src/lib.rs:201-210: renders and downloads the RGBA32F target (H x W x 4)."""
        self.render_to_target()
        return self.context.download(self.render_target, *self.extent)

    def tonemap(self, fmt: int = native.TT_FORMAT_RGBA8_UNORM) -> np.ndarray:
        """The display pass (src/post_process/display.glsl) into host memory."""
        c = self.constants()
        w, h = self.extent
        out = np.empty((h, w, 4), np.float32 if fmt == native.TT_FORMAT_RGBA32F else np.uint8)
        check(self.context.lib.tt_tonemap(self.context.handle, self.render_target, native.ptr(c), fmt,
                                          native.ptr(out), out.nbytes))
        return out

    def present(self) -> None:
        """Headless present: advances the frame index like Context::present."""
        check(self.context.lib.tt_advance_frame(self.context.handle))

    def close(self) -> None:
        self.context.close()
