"""tinytrace_gb300 — the tinytrace rendering hot path (path tracer, OpenPBR BSDF, emissive
triangle sampling, neutral tonemap and a GPU LBVH in place of RT-core ray queries) as
hand-written sm_103a CUDA behind a C ABI (include/tinytrace_cuda.h)."""
from .asset import Material, Model, Node, Scene  # noqa: F401
from .camera import Camera, CameraMove  # noqa: F401
from .renderer import Config, LightSampling, Renderer, SceneArrays, Timings  # noqa: F401
