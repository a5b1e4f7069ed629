"""Benchmark: path-traced Msamples/s of the plain path tracer on the 1M-triangle seeded scene
at 1920x1080, 64 samples per pixel, 8 bounces (one step = one Renderer.render_to_target
over the whole image), on N GB300s (one replica per GPU: the path does not shard across
GPUs, every rank renders its own full frame; scaling is weak).

Prints one JSON line (rank 0).  `value` is the device-resident throughput (scene, BVH and
target already in HBM), `e2e` the same metric through Renderer.render_to_texture with the
target downloaded to pinned host memory every step.  `roofline` relates the dominant
kernel's (wf_trace_kernel: extension and shadow rays) algorithmic bytes per launch (BVH
nodes, triangle records, object-ray set-ups, ray state; counted by the instrumented kernels
on the same frame) to its mean CUDA-event launch duration and the measured HBM copy
bandwidth; `traffic` is its DRAM bytes per launch from the committed ncu summary.
`cpu_baseline` times the CPU oracle on a stratified row sample of the same frame, and
`parity` compares those rows with the GPU's frame of the same Constants bit for bit.

--impl reference times the reference path tracer's CPU restatement (the oracle: the
reference itself is Rust + Vulkan/GLSL and cannot run on this machine) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Msamples/s at 1080p, plain path tracer"
UNIT = "Msamples/s"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--spp", type=int, default=64)
    p.add_argument("--depth", type=int, default=8)
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--instances", type=int, default=64)
    p.add_argument("--freq", type=int, default=28)
    p.add_argument("--lights", type=int, default=1000)
    p.add_argument("--cpu-row-stride", type=int, default=ROW_STRIDE,
                   help="the CPU legs render every n-th row of the frame (stratified sample)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--integrator", default="wavefront", choices=["wavefront", "megakernel"])
    p.add_argument("--slots", type=int, default=0, help="wavefront paths in flight (0 = library default)")
    p.add_argument("--host-loop", action="store_true", help="drive the wavefront loop from the host (no CUDA graph)")
    p.add_argument("--no-autotune", action="store_true", help="skip tt_autotune before the warm-up")
    p.add_argument("--no-serve", action="store_true", help="skip the serving sample")
    p.add_argument("--no-restir", action="store_true", help="skip the ReSTIR DI sample")
    p.add_argument("--no-cache", action="store_true", help="skip the radiance-cache sample")
    p.add_argument("--no-textured", action="store_true", help="skip the textured-materials sample")
    p.add_argument("--no-ingest", action="store_true", help="skip the device mesh-ingest sample")
    p.add_argument("--no-light-selection", action="store_true", help="skip the light-selection sample")
    p.add_argument("--no-closed", action="store_true", help="skip the closed-scene (Cornell box) sample")
    p.add_argument("--serve-batch", type=int, default=96, help="requests of the serving sample's capacity run")
    p.add_argument("--serve-inflight", type=int, default=SERVE_INFLIGHT, help="requests the server renders together")
    p.add_argument("--serve-policy", default="smallest_first", choices=["fair", "smallest_first"],
                   help="server scheduling policy (TT_SERVER_POLICY_*)")
    p.add_argument("--serve-requests", type=int, default=512,
                   help="requests at 0.8 x capacity in the serving sample (a quarter as many at 0.5 x and 1.1 x)")
    p.add_argument("--primary", default="raster", choices=["raster", "traverse"],
                   help="camera-ray hits of flat BVH4 scenes: rasterised keys (TT_PRIMARY_RASTER) or traversal")
    p.add_argument("--accel", default="auto", choices=["auto", "flat", "two_level", "wide"],
                   help="acceleration structure (auto = flat up to 2^26 instanced triangles; wide = the flat BVH "
                        "in the compressed 8-wide format)")
    return p.parse_args()


def scan_launches(n: int, per_block: int = 4096) -> int:
    """Kernels of the library's exclusive u32 scan over n values (1024 threads x 4 per block)."""
    blocks = (n + per_block - 1) // per_block
    return 1 if blocks <= 1 else 2 + scan_launches(blocks, per_block)


# ---------------------------------------------------------------- distributed helpers
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def measured_peaks() -> tuple[float, str]:
    path = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(path.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def l2_copy_gbs(device: int) -> dict:
    """Bandwidth of a plain device-to-device copy whose source and destination both stay in
    L2 (copies of 4, 8, 16 and 32 MB; read + write bytes per copy): for each size ~0.3 s of
    back-to-back copies first (clocks up, lines resident), then the best of 3 runs of 400
    copies timed by CUDA events on torch's stream; the best size is kept.  The ceiling for a
    kernel whose bytes L2 serves."""
    import torch

    best, at = 0.0, 0
    with torch.cuda.device(device):
        for mb in (4, 8, 16, 32):
            n = (mb << 20) // 4
            src = torch.ones(n, dtype=torch.float32, device="cuda")
            dst = torch.empty_like(src)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 0.3:
                for _ in range(100):
                    dst.copy_(src)
                torch.cuda.synchronize()
            for _ in range(3):
                e0.record()
                for _ in range(400):
                    dst.copy_(src)
                e1.record()
                torch.cuda.synchronize()
                gbs = 2 * n * 4 * 400 / (e0.elapsed_time(e1) / 1e3) / 1e9
                if gbs > best:
                    best, at = gbs, mb
            del src, dst
        torch.cuda.empty_cache()
    return {"gbs": best, "copy_mb": at, "how": "torch copy_ of an L2-resident buffer (4/8/16/32 MB, best of 3 x 400 "
                                              "copies after 0.3 s of warm-up copies), read + write bytes, CUDA events"}


# Algorithmic bytes per unit of traversal work (wf_trace_kernel): a BVH4 node is one 128-byte
# record (six float4 planes + child references); a triangle test reads one 48-byte record; an
# object-ray set-up reads the instance's three inverse rows and its mesh word (64 bytes); a
# traced ray reads its origin and direction (32 bytes) and writes its result (hit record or
# radiance update, counted as 32 bytes).
NODE_BYTES = 128
WIDE_NODE_BYTES = 80  # compressed 8-wide node (TT_ACCEL_FLAT_WIDE)
TRI_RECORD_BYTES = 48
INSTANCE_RAY_BYTES = 64
RAY_STATE_BYTES = 64
PROFILE = ROOT / "profiles" / "wf_trace_kernel_icosphere_field_1080p.md"


def ncu_traffic_per_launch(rays_per_launch: float) -> float | None:
    """dram__bytes_read.sum + dram__bytes_write.sum per wf_trace_kernel launch of this
    workload: the committed ncu summary's DRAM bytes per traced ray (captured on a small case
    of the same frame: every trace launch of one 1-spp render) times this run's rays per
    launch."""
    if not PROFILE.exists():
        return None
    m = re.search(r"dram_bytes_per_ray:\s*([0-9.eE+]+)", PROFILE.read_text())
    return float(m.group(1)) * rays_per_launch if m else None


def traffic_source() -> str:
    return ("ncu dram__bytes_read.sum + dram__bytes_write.sum per traced ray, every wf_trace_kernel launch of a "
            "1-spp render of the same frame, scaled by this run's rays per launch "
            "(profiles/wf_trace_kernel_icosphere_field_1080p.md)")


def ncu_trace_metrics() -> dict | None:
    """L2 hit rate and warp execution efficiency of the extension-ray trace kernel from the
    committed ncu summary (full capture on a 1-spp case of the same frame)."""
    if not PROFILE.exists():
        return None
    text = PROFILE.read_text()
    l2 = re.search(r"\| L2 hit rate \| ([0-9.]+) %", text)
    tpi = re.search(r"\| threads per instruction \(of 32\) \| ([0-9.]+)", text)
    if not (l2 and tpi):
        return None
    return {"l2_hit_rate": float(l2.group(1)) / 100.0, "warp_execution_efficiency": float(tpi.group(1)) / 32.0,
            "source": "ncu --set full, extension-ray launch, 1 spp (profiles/wf_trace_kernel_icosphere_field_1080p.md)"}


# ---------------------------------------------------------------- workload
def make_workload(a):
    from tinytrace_gb300 import scenes

    return scenes.icosphere_workload(extent=(a.width, a.height), spp=a.spp, depth=a.depth,
                                     instances=a.instances, freq=a.freq, lights=a.lights)


_CPU_SCENES: dict = {}

# The CPU legs render a stratified row sample of the frame: every ROW_STRIDE-th row from
# ROW_STRIDE // 2 on (135 of the 1080 rows at the default stride of 8), the whole width, all
# samples and bounces.  Both legs (cpu_baseline and --impl reference) render the same rows,
# and the GPU's frame of the same Constants is compared with them bit for bit.
ROW_STRIDE = 8


def sample_rows(height: int, stride: int) -> list[int]:
    return list(range(stride // 2, height, stride))


def _oracle_scene(arrays):
    from oracle import oracle

    key = id(arrays)
    t0 = time.perf_counter()
    if key not in _CPU_SCENES:
        _CPU_SCENES[key] = oracle.OracleScene(arrays, flat=True)
    return _CPU_SCENES[key], time.perf_counter() - t0


def render_rows(w, arrays, rows: list[int], target: np.ndarray) -> float:
    """The oracle (a scalar C++ restatement, OpenMP over the pixels of a row on every host
    core, tracing through the flat BVH) renders `rows` of the frame's first render (frame
    index 0, accumulated frame count 0) into `target`; returns the seconds it took."""
    from tinytrace_gb300.renderer import make_constants

    orc, _ = _oracle_scene(arrays)
    c = make_constants(w.camera, w.extent, w.config, 0, 0)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    for y in rows:
        orc.render(c, target, rows=(y, y + 1), threads=threads)
    return time.perf_counter() - t0


def cpu_baseline(w, arrays, stride: int) -> tuple[dict, np.ndarray, list[int]]:
    """Times the oracle on the stratified row sample of the frame; returns the baseline record,
    the CPU image (only the sampled rows written) and the rows."""
    _, build_s = _oracle_scene(arrays)
    W, H = w.extent
    spp = w.config.sample_count
    rows = sample_rows(H, stride)
    target = np.zeros((H, W, 4), np.float32)
    dt = render_rows(w, arrays, rows, target)
    samples = len(rows) * W * spp
    rec = {"value": samples / dt / 1e6, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
           "sample": f"{len(rows)} stratified rows (every {stride}th from row {stride // 2}) x {W} px of the "
                     f"{W}x{H} frame at {spp} spp, depth {w.config.bounce_count} ({samples} samples, {dt:.1f} s; "
                     f"flat BVH build {build_s:.1f} s excluded)"}
    return rec, target, rows


def row_parity(gpu: np.ndarray, cpu: np.ndarray, rows: list[int]) -> dict:
    """Bit-for-bit comparison of the sampled rows (any NaN equals any NaN), plus the largest
    relative difference of the radiance where they differ."""
    g = np.ascontiguousarray(gpu[rows], np.float32)
    c = np.ascontiguousarray(cpu[rows], np.float32)
    same = (g.view(np.uint32) == c.view(np.uint32)) | (np.isnan(g) & np.isnan(c))
    with np.errstate(all="ignore"):
        rel = np.abs(g.astype(np.float64) - c) / np.maximum(np.abs(c.astype(np.float64)), 1e-30)
    rel = np.where(same, 0.0, rel)
    return {"rows": len(rows), "pixels": int(g.shape[0] * g.shape[1]), "values_compared": int(g.size),
            "values_differing": int((~same).sum()), "max_rel_err": float(np.nanmax(rel)) if rel.size else 0.0,
            "bit_exact": bool(same.all()), "frame": "frame index 0, accumulated frame count 0 (no accumulation)",
            "tolerance": "bit for bit (NaN payloads aside); the parity bar is 1e-4 relative per pixel"}


def run_reference(a, dist: Dist):
    """The reference arm: the oracle renders the stratified row sample of the frame once per
    step (W untimed, K timed steps); `ms_per_step` is the measured time of one step and
    `value` the samples of the K steps over their time."""
    if dist.rank != 0:
        return
    from tinytrace_gb300.renderer import SceneArrays

    w = make_workload(a)
    arrays = SceneArrays(w.scene)
    _, build_s = _oracle_scene(arrays)
    W, H = w.extent
    rows = sample_rows(H, a.cpu_row_stride)
    target = np.zeros((H, W, 4), np.float32)
    for _ in range(a.warmup):
        render_rows(w, arrays, rows, target)
    times = [render_rows(w, arrays, rows, target) for _ in range(a.steps)]
    samples = len(rows) * W * w.config.sample_count
    v = samples * a.steps / sum(times) / 1e6
    threads = os.cpu_count() or 1
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": sum(times) / a.steps * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)", "impl": "reference",
           "config": {"workload": w.name, "triangles": arrays.triangle_count, "resolution": [W, H],
                      "spp": w.config.sample_count, "depth": w.config.bounce_count,
                      "step": f"{len(rows)} stratified rows (every {a.cpu_row_stride}th) x {W} px, "
                              f"{samples} samples"},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"{len(rows)} stratified rows (every {a.cpu_row_stride}th from row "
                                      f"{a.cpu_row_stride // 2}) x {W} px of the {W}x{H} frame at "
                                      f"{w.config.sample_count} spp per step ({samples} samples; flat BVH build "
                                      f"{build_s:.1f} s before the first step)"},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "reference arm = the reference path tracer restated on the CPU (oracle/); the reference "
                   "itself (Rust + Vulkan ray queries) cannot run on this machine"}
    print(json.dumps(out))


# ---------------------------------------------------------------- ReSTIR DI sample
# Algorithmic bytes per pixel of the ReSTIR passes (constant materials, uniform candidates),
# for a pixel whose camera ray hits a surface; closest-hit traversal (the G-buffer's camera ray,
# the visibility rays of the initial and shade passes) comes on top.  Records: G-buffer surface
# 64 B, prepared lobes 96 B, reservoir 32 B, material constants 192 B, light record 64 B (the
# four 16-byte rows a light point reads), hit reconstruction 262 B (instance 208, indices 12,
# snorm16 positions 18, vertices 24), target pixel 16 B read + 16 B written.
RESTIR_PASS_BYTES = {
    "restir_gbuffer": 262 + 192 + 64 + 96,
    "restir_initial": 64 + 96 + 192 + 32 * 64 + 32,
    "restir_temporal": 64 + 96 + 192 + 64 + 32 + 32 + 2 * 64 + 32,
    "restir_spatial": 64 + 96 + 192 + 32 + 64 + 5 * (64 + 32 + 64) + 32,
    "restir_shade": 64 + 96 + 192 + 32 + 64 + 32,
}
RESTIR_PROFILE = ROOT / "profiles" / "restir_passes_restir_field_1080p.md"


def restir_initial_flops_per_pixel() -> float | None:
    """FP32 operations per pixel of the initial-candidate pass (FADD + FMUL + 2 x FFMA thread
    instructions per pixel, measured by ncu on a small case of the same scene and camera; the
    committed summary)."""
    if not RESTIR_PROFILE.exists():
        return None
    m = re.search(r"initial_fp32_flops_per_pixel:\s*([0-9.eE+]+)", RESTIR_PROFILE.read_text())
    return float(m.group(1)) if m else None


def run_restir(a, device: int, sm_mhz: float | None) -> dict:
    """ReSTIR DI on the 2.1 M-triangle, 100 k-light scene: 1920x1080, 1 sample per pixel per frame,
    32 candidates, temporal reuse (M cap 20 x), 5 spatial neighbours in 30 px, a 60-frame orbit;
    device time of the 60 frames by CUDA events on the context stream.  Then the same orbit with
    CUDA events around each pass (per-pass time, algorithmic bytes, the initial pass's FP32 rate
    against the FP32 FMA peak at the sampled SM clock), and, at 960x540 over the orbit's first 12
    frames, the oracle's time (cpu_baseline) and its images and reservoirs against the GPU's."""
    import ctypes

    from oracle import oracle
    from tinytrace_gb300 import native, scenes
    from tinytrace_gb300.native import check
    from tinytrace_gb300.renderer import Config, Renderer, make_constants

    W, H, frames = a.width, a.height, 60
    r = Renderer((W, H), device=device)
    scene = scenes.restir_field()
    r.set_scene(scene)
    r.set_config(Config(bounce_count=1, sample_count=1))
    lib, ctx = r.context.lib, r.context.handle

    def orbit(f):
        ang = 2.0 * np.pi * f / frames
        return scenes.Camera.looking_at((95.0 * np.sin(ang), 10.0, 95.0 * np.cos(ang)), (0.0, 0.0, 0.0))

    for f in range(3):
        r.camera = orbit(f)
        r.render_restir_to_target()
        r.present()
    r.restir_reset()
    check(lib.tt_synchronize(ctx))
    check(lib.tt_event_record(ctx, 2))
    for f in range(frames):
        r.camera = orbit(f)
        check(lib.tt_flush_l2(ctx))
        r.render_restir_to_target()
        r.present()
    check(lib.tt_event_record(ctx, 3))
    ms = ctypes.c_float()
    check(lib.tt_event_elapsed_ms(ctx, 2, 3, ctypes.byref(ms)))
    img = r.context.download(r.render_target, W, H)
    stats = r.context.scene_stats(r.scene)

    # the same orbit with CUDA events around every pass
    check(lib.tt_set_option(ctx, native.TT_OPTION_STAGE_TIMING, 1))
    r.restir_reset()
    pass_ns = np.zeros(native.TT_STAGE_COUNT)
    for f in range(frames):
        r.camera = orbit(f)
        check(lib.tt_flush_l2(ctx))
        r.render_restir_to_target()
        r.present()
        stt = native.StageTimings()
        check(lib.tt_stage_timings_get(ctx, ctypes.byref(stt)))
        pass_ns += np.array(stt.ns[:], np.float64)
    check(lib.tt_set_option(ctx, native.TT_OPTION_STAGE_TIMING, 0))
    passes = {}
    for name, stage in (("restir_gbuffer", native.TT_STAGE_RESTIR_GBUFFER),
                        ("restir_initial", native.TT_STAGE_RESTIR_INITIAL),
                        ("restir_temporal", native.TT_STAGE_RESTIR_TEMPORAL),
                        ("restir_spatial", native.TT_STAGE_RESTIR_SPATIAL),
                        ("restir_shade", native.TT_STAGE_RESTIR_SHADE)):
        t = pass_ns[stage] / frames / 1e9
        b = RESTIR_PASS_BYTES[name] * W * H
        passes[name] = {"ms_per_frame": t * 1e3, "algorithmic_bytes_per_frame": b,
                        "algorithmic_gbs": b / t / 1e9 if t > 0 else None}
    r.close()
    peak, _ = measured_peaks()
    t_init = pass_ns[native.TT_STAGE_RESTIR_INITIAL] / frames / 1e9
    flops_px = restir_initial_flops_per_pixel()
    mhz = sm_mhz or 2070.0
    fp32_peak = 152 * 128 * 2 * mhz * 1e6 / 1e12  # TFLOP/s: SMs x FP32 lanes x FMA x clock
    roofline = {"kernel": "restir_initial_kernel", "bound": "alu (FP32 BSDF evaluation of 32 candidates per pixel)",
                "fp32_flops_per_pixel": flops_px,
                "achieved_tflops": flops_px * W * H / t_init / 1e12 if flops_px and t_init > 0 else None,
                "fp32_peak_tflops": fp32_peak,
                "fp32_peak_source": f"nominal: 152 SMs x 128 FP32 lanes x 2 (FMA) x {mhz:.0f} MHz (sampled SM clock)",
                "bytes_per_pixel": RESTIR_PASS_BYTES["restir_initial"],
                "algorithmic_gbs": passes["restir_initial"]["algorithmic_gbs"], "hbm_peak_gbs": peak,
                "flops_source": "ncu FP32 thread-instruction counts on a 480x270 frame of the same orbit "
                                "(profiles/restir_passes_restir_field_1080p.md)"}
    if roofline["achieved_tflops"] is not None:
        roofline["frac"] = roofline["achieved_tflops"] / fp32_peak

    # oracle: CPU time and bit-for-bit parity over the orbit's first frames at a quarter of the pixels
    cw, chh, cframes = W // 2, H // 2, 12
    rs = Renderer((cw, chh), device=device)
    rs.set_scene(scene)
    rs.set_config(Config(bounce_count=1, sample_count=1))
    orc = oracle.OracleScene(rs.scene_arrays, flat=True)
    R = oracle.OracleRestir(orc, cw, chh)
    cpu = np.zeros((chh, cw, 4), np.float32)
    cpu_s, differing, compared = 0.0, 0, 0
    for f in range(cframes):
        rs.camera = orbit(f)
        c = make_constants(rs.camera, (cw, chh), rs.config(), rs.context.frame_index(), rs.accumulated_frame_count)
        rs.render_restir_to_target()
        t0 = time.perf_counter()
        R.frame(c, cpu, threads=os.cpu_count() or 1)
        cpu_s += time.perf_counter() - t0
        for gpu_arr, cpu_arr in ((rs.context.download(rs.render_target, cw, chh), cpu),
                                 (rs.restir_reservoirs(), R.reservoirs())):
            g, k = np.ascontiguousarray(gpu_arr, np.float32), np.ascontiguousarray(cpu_arr, np.float32)
            same = (g.view(np.uint32) == k.view(np.uint32)) | (np.isnan(g) & np.isnan(k))
            differing += int((~same).sum())
            compared += int(same.size)
        rs.present()
    rs.close()
    cpu_rate = cw * chh * cframes / cpu_s / 1e6
    gpu_rate = W * H * frames / (ms.value / 1e3) / 1e6
    return {"workload": f"restir_field_{stats.triangle_count}tri_{int(stats.emissive_count)}lights_{W}x{H}_60frames",
            "ms_per_frame": ms.value / frames, "msamples_per_s": gpu_rate,
            "candidates": 32, "temporal_m_cap": 20, "spatial_neighbours": 5, "spatial_radius_px": 30,
            "l2": "flushed before every frame", "image_mean": float(img[..., :3].mean()),
            "image_finite": bool(np.isfinite(img).all()),
            "passes": passes, "bytes_note": "algorithmic bytes per pixel whose camera ray hits a surface, "
                                             "closest-hit traversal not included (an upper bound for sky pixels)",
            "roofline": roofline,
            "cpu_baseline": {"value": cpu_rate, "unit": "Msamples/s", "cores": os.cpu_count() or 1, "kind": "port",
                             "sample": f"the oracle's ReSTIR frames at {cw}x{chh}, the orbit's first {cframes} "
                                       f"frames, same scene and settings ({cpu_s:.1f} s)"},
            "speedup_vs_cpu": gpu_rate / cpu_rate,
            "parity": {"frames": cframes, "resolution": [cw, chh], "values_compared": compared,
                       "values_differing": differing, "bit_exact": differing == 0,
                       "compared": "images and final reservoirs of every frame"}}


# ---------------------------------------------------------------- radiance-cache sample
CACHE_SPP = (1, 2, 4, 8, 16, 32, 64)


def time_at_error(points: list[dict], target: float) -> tuple[float | None, str]:
    """Time at which an error-vs-time curve (points sorted by time, keys `ms` and `error`) reaches
    `target`, interpolated linearly in log(time) against log(error) between the two points that
    bracket it; (time of the cheapest point, "below") when the cheapest point is already below the
    target, (None, "floor") when no point reaches it."""
    pts = sorted(points, key=lambda p: p["ms"])
    if pts[0]["error"] <= target:
        return pts[0]["ms"], "below"
    for p0, p1 in zip(pts, pts[1:]):
        if p0["error"] >= target >= p1["error"]:
            if p0["error"] == p1["error"]:
                return p1["ms"], "interpolated"
            f = np.log(target / p0["error"]) / np.log(p1["error"] / p0["error"])
            return float(np.exp(np.log(p0["ms"]) + f * (np.log(p1["ms"]) - np.log(p0["ms"])))), "interpolated"
    return None, "floor"


def run_cache(a, device: int) -> dict:
    """Equal-error comparison of the learned radiance cache with the plain path tracer at
    1920x1080, depth 8, on the benchmark field (the 1M-triangle scene of the headline, open: most
    camera paths end in the sky after one bounce) and on the textured Cornell box (closed).
    Reference: the mean of 4 plain renders of 1024 spp.  Both arms render frames of 1, 2, 4, 8,
    16, 32 and 64 spp, 4 frames each with their own seeds (frame index); each frame's device time
    covers the whole render call (for the cache: its queries, the training pairs and the Adam
    steps after the frame).  Error = the mean over pixels and channels of the squared difference
    of tonemapped images, x / (1 + x): bounded per pixel, so that the fireflies of the log-normal
    lights do not decide the comparison (the plain MSE is reported too).  Equal-error speed-up =
    the plain arm's 16-spp time over the time at which the cached arm's error-vs-time curve
    reaches the plain 16-spp error (log-log interpolation between its bracketing points).  The
    cache (C5 configuration: learning rate 1e-2, 65,536 training paths per frame, paths end at the
    first vertex after the primary hit whose path spread exceeds 0.01 of the primary's) trains
    online for 128 frames of 4 spp before its curve is measured."""
    import ctypes

    from tinytrace_gb300 import native, scenes
    from tinytrace_gb300.native import check
    from tinytrace_gb300.renderer import Config, Renderer

    W, H, depth = a.width, a.height, a.depth
    cfg_c5 = (1e-2, 65536, 1, 1, 0.01)
    out = {"reference_spp": 4096, "spp": list(CACHE_SPP), "frames_per_point": 4,
           "error": "tonemapped MSE: mean of (x/(1+x) - ref/(1+ref))^2 over pixels and RGB",
           "config": {"learning_rate": cfg_c5[0], "train_paths_per_frame": cfg_c5[1], "terminate_depth": cfg_c5[2],
                      "spread_threshold": cfg_c5[4]},
           "warmup_frames": 128, "scenes": {}}
    w = make_workload(a)
    cases = [("icosphere_field", w.scene, w.camera),
             ("textured_cornell", scenes.textured_cornell(),
              scenes.Camera.looking_at((0.0, 1.0, 3.4), (0.0, 1.0, 0.0), fov=0.75))]
    for name, scene, camera in cases:
        r = Renderer((W, H), device=device)
        r.set_scene(scene)
        r.camera = camera
        lib, ctx = r.context.lib, r.context.handle

        def frame(spp):
            r.set_config(Config(bounce_count=depth, sample_count=spp))
            r.reset_accumulation()
            check(lib.tt_synchronize(ctx))
            check(lib.tt_event_record(ctx, 4))
            r.render_to_target()
            check(lib.tt_event_record(ctx, 5))
            ms = ctypes.c_float()
            check(lib.tt_event_elapsed_ms(ctx, 4, 5, ctypes.byref(ms)))
            img = r.context.download(r.render_target, W, H)[..., :3].astype(np.float64)
            r.present()
            return img, ms.value

        ref = np.zeros((H, W, 3))
        for _ in range(4):
            ref += frame(1024)[0] / 4.0
        tref = ref / (1.0 + ref)

        def curve():
            pts = []
            for spp in CACHE_SPP:
                ms = err = mse = 0.0
                for _ in range(4):
                    img, t = frame(spp)
                    ms += t / 4.0
                    err += float(np.mean((img / (1.0 + img) - tref) ** 2)) / 4.0
                    mse += float(np.mean((img - ref) ** 2)) / 4.0
                pts.append({"spp": spp, "ms": ms, "error": err, "mse": mse})
            return pts

        plain = curve()
        cfg = native.CacheConfig(*cfg_c5)
        check(lib.tt_cache_configure(ctx, ctypes.byref(cfg)))
        check(lib.tt_set_option(ctx, native.TT_OPTION_RADIANCE_CACHE, 1))
        for _ in range(128):
            frame(4)
        cached = curve()
        # cost breakdown of one cached 16-spp frame (host-driven loop, CUDA events per launch)
        check(lib.tt_set_option(ctx, native.TT_OPTION_STAGE_TIMING, 1))
        frame(16)
        stt = native.StageTimings()
        check(lib.tt_stage_timings_get(ctx, ctypes.byref(stt)))
        check(lib.tt_set_option(ctx, native.TT_OPTION_STAGE_TIMING, 0))
        breakdown = {n: stt.ns[i] / 1e6 for i, n in enumerate(native.STAGE_NAMES) if stt.launches[i]}
        st = native.CacheStatus()
        check(lib.tt_cache_status_get(ctx, ctypes.byref(st)))
        p16 = next(p for p in plain if p["spp"] == 16)
        c16 = next(p for p in cached if p["spp"] == 16)
        t_cached, how = time_at_error(cached, p16["error"])
        t_plain, how_p = time_at_error(plain, c16["error"])
        out["scenes"][name] = {
            "plain": plain, "cached": cached,
            "target_error": p16["error"], "plain_ms_at_target": p16["ms"],
            "cached_ms_at_target": t_cached, "cached_reaches_target": how,
            "equal_rmse_speedup": p16["ms"] / t_cached if t_cached else None,
            "plain_ms_at_cached_16spp_error": t_plain, "plain_reaches_cached_16spp_error": how_p,
            "equal_rmse_speedup_at_cached_16spp": t_plain / c16["ms"] if t_plain else None,
            "cached_16spp_breakdown_ms": breakdown,
            "training": {"steps": int(st.steps), "pairs_last_frame": int(st.pairs), "last_loss": st.last_loss}}
        r.close()
    return out


# ---------------------------------------------------------------- textured-materials sample
def run_textured(a, device: int) -> dict:
    """Texture sampling cost on the benchmark frame: the 1M-triangle field with every sphere
    material textured (BC1 base colour, R8 roughness, BC5 normal maps on half; 168 textures
    with mips) against the same field with constant materials, 1920x1080, 16 spp, depth 8;
    device time by CUDA events around each render (L2 flushed before each), 3 warm-up renders."""
    import ctypes

    from tinytrace_gb300 import native, scenes
    from tinytrace_gb300.native import check
    from tinytrace_gb300.renderer import Config, Renderer

    W, H, spp, frames = a.width, a.height, 16, 3
    out = {}
    for name, textured in (("constant", False), ("textured", True)):
        r = Renderer((W, H), device=device)
        scene = scenes.icosphere_field(instances=a.instances, freq=a.freq, lights=a.lights, textured=textured)
        r.set_scene(scene)
        r.camera = make_workload(a).camera
        r.set_config(Config(bounce_count=a.depth, sample_count=spp))
        lib, ctx = r.context.lib, r.context.handle
        for _ in range(3):
            r.render_to_target()
            r.present()
        total = 0.0
        for _ in range(frames):
            check(lib.tt_flush_l2(ctx))
            check(lib.tt_synchronize(ctx))
            check(lib.tt_event_record(ctx, 6))
            r.render_to_target()
            check(lib.tt_event_record(ctx, 7))
            ms = ctypes.c_float()
            check(lib.tt_event_elapsed_ms(ctx, 6, 7, ctypes.byref(ms)))
            total += ms.value
            r.present()
        img = r.context.download(r.render_target, W, H)
        out[name] = {"ms_per_frame": total / frames, "msamples_per_s": W * H * spp * frames / (total / 1e3) / 1e6,
                     "image_mean": float(img[..., :3].mean()), "image_finite": bool(np.isfinite(img).all())}
        if textured:
            out[name]["textures"] = int(len(r.scene_arrays.texture_info))
            out[name]["texture_bytes"] = int(r.scene_arrays.texture_data.nbytes)
        r.close()
    out["workload"] = f"icosphere_field_{W}x{H}_{spp}spp_d{a.depth}"
    out["textured_over_constant_time"] = out["textured"]["ms_per_frame"] / out["constant"]["ms_per_frame"]
    return out


# ---------------------------------------------------------------- closed-scene sample
def run_closed(a, device: int) -> dict:
    """The per-bounce cost the open benchmark field hides: most of its camera paths leave the
    scene after one bounce (about 1.5 traced rays per sample), while in the closed Cornell box
    of the CPU-runnable configuration every path bounces to full depth.  The box at the
    headline's 1920x1080 and depth 8, 16 spp, autotuned pool: device time (CUDA events, L2
    flushed before each of 3 frames after 3 warm-up frames), Msamples/s, and traced rays per
    sample and per second from an instrumented render of the same frame."""
    import ctypes

    from tinytrace_gb300 import native, scenes
    from tinytrace_gb300.native import check
    from tinytrace_gb300.renderer import Config, Renderer

    W, H, spp, frames = a.width, a.height, 16, 3
    w = scenes.cornell_workload()
    r = Renderer((W, H), device=device)
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(Config(bounce_count=a.depth, sample_count=spp))
    lib, ctx = r.context.lib, r.context.handle
    tune = r.autotune(sample_count=4)
    for _ in range(3):
        r.render_to_target()
        r.present()
    total = 0.0
    for _ in range(frames):
        check(lib.tt_flush_l2(ctx))
        check(lib.tt_synchronize(ctx))
        check(lib.tt_event_record(ctx, 6))
        r.render_to_target()
        check(lib.tt_event_record(ctx, 7))
        ms = ctypes.c_float()
        check(lib.tt_event_elapsed_ms(ctx, 6, 7, ctypes.byref(ms)))
        total += ms.value
        r.present()
    cnt = native.TraversalCounters()
    c = r.constants()
    check(lib.tt_render_counted(ctx, r.scene, native.ptr(c), r.render_target, ctypes.byref(cnt)))
    r.close()
    samples = W * H * spp
    ms = total / frames
    return {"workload": f"cornell_box_{W}x{H}_{spp}spp_d{a.depth}", "ms_per_frame": ms,
            "msamples_per_s": samples / (ms / 1e3) / 1e6, "rays_per_sample": cnt.rays / samples,
            "rays_per_s": cnt.rays / (ms / 1e3), "nodes_per_ray": (cnt.blas_nodes + cnt.tlas_nodes) / max(1, cnt.rays),
            "pool_slots": int(tune.slots), "l2": "flushed before every frame"}


# ---------------------------------------------------------------- light-selection sample
def run_light_selection(a, device: int) -> dict:
    """Power-proportional light selection (TT_LIGHT_SELECTION_POWER, an alias table over the
    1000 log-normal lights) against the reference's uniform pick on the benchmark field at
    960x540, depth 8, 16 spp: device time (CUDA events, 4 frames averaged) and error against a
    16,384-spp uniform reference, by tonemapped MSE and MSE; equal-error speed-up =
    (t_uniform e_uniform) / (t_power e_power).  The two estimators converge to the same image."""
    import ctypes

    from tinytrace_gb300 import native
    from tinytrace_gb300.native import check
    from tinytrace_gb300.renderer import Config, Renderer

    W, H = a.width // 2, a.height // 2
    w = make_workload(a)
    r = Renderer((W, H), device=device)
    r.set_scene(w.scene)
    r.camera = w.camera
    lib, ctx = r.context.lib, r.context.handle

    def frame(spp):
        r.set_config(Config(bounce_count=a.depth, sample_count=spp))
        r.reset_accumulation()
        check(lib.tt_synchronize(ctx))
        check(lib.tt_event_record(ctx, 4))
        r.render_to_target()
        check(lib.tt_event_record(ctx, 5))
        ms = ctypes.c_float()
        check(lib.tt_event_elapsed_ms(ctx, 4, 5, ctypes.byref(ms)))
        img = r.context.download(r.render_target, W, H)[..., :3].astype(np.float64)
        r.present()
        return img, ms.value

    ref = np.zeros((H, W, 3))
    for _ in range(16):
        ref += frame(1024)[0] / 16.0
    tref = ref / (1.0 + ref)
    out = {"workload": f"icosphere_field_{W}x{H}_16spp_d{a.depth}", "reference_spp": 16384, "modes": {}}
    for name, value in (("uniform", native.TT_LIGHT_SELECTION_UNIFORM), ("power", native.TT_LIGHT_SELECTION_POWER)):
        check(lib.tt_set_option(ctx, native.TT_OPTION_LIGHT_SELECTION, value))
        frame(16)
        ms = tm = mse = 0.0
        for _ in range(4):
            img, t = frame(16)
            ms += t / 4.0
            tm += float(np.mean((img / (1.0 + img) - tref) ** 2)) / 4.0
            mse += float(np.mean((img - ref) ** 2)) / 4.0
        out["modes"][name] = {"ms": ms, "tonemapped_mse": tm, "mse": mse, "mean": float(img.mean())}
    u, p = out["modes"]["uniform"], out["modes"]["power"]
    out["equal_error_speedup_tonemapped"] = (u["ms"] * u["tonemapped_mse"]) / (p["ms"] * p["tonemapped_mse"])
    out["equal_error_speedup_mse"] = (u["ms"] * u["mse"]) / (p["ms"] * p["mse"])
    r.close()
    return out


# ---------------------------------------------------------------- device ingest sample
def _grid_mesh(n: int):
    """A height-field grid of n x n vertices, 2 (n - 1)^2 triangles, with texture coordinates."""
    y, x = np.mgrid[0:n, 0:n].astype(np.float32) / np.float32(n - 1)
    z = (0.05 * np.sin(12.0 * x) * np.cos(9.0 * y)).astype(np.float32)
    pos = np.stack([x, z, y], -1).reshape(-1, 3).astype(np.float32)
    uv = np.stack([x, y], -1).reshape(-1, 2).astype(np.float32)
    i = np.arange(n - 1)[:, None] * n + np.arange(n - 1)[None, :]
    quads = np.stack([i, i + n, i + 1, i + 1, i + n, i + n + 1], -1).reshape(-1).astype(np.uint32)
    return pos, uv, quads


def run_ingest(a, device: int) -> dict:
    """Scene::insert_mesh on the device (tt_mesh_ingest: quantisation, generated normals, tangent
    frames, f16 texture coordinates) for a 2.5M-vertex / 5M-triangle mesh, host arrays in and
    out (copies included), against the oracle's sequential CPU restatement and the package's
    numpy host path on the same mesh; then tt_emissive_extract of the mesh as one emissive
    model.  Wall-clock per call after one warm-up call; the GPU output is compared with the
    oracle's bit for bit."""
    from oracle import oracle
    from tinytrace_gb300 import asset
    from tinytrace_gb300.ingest import DeviceIngest
    from tinytrace_gb300.renderer import Context

    pos, uv, idx = _grid_mesh(1582)
    tris = len(idx) // 3
    ctx = Context(device)
    ing = DeviceIngest(ctx)
    ing.process_mesh(pos, uv, idx)
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        q, v, rec = ing.process_mesh(pos, uv, idx)
    gpu_s = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    oq, ov, _ = oracle.mesh_ingest(pos, uv, idx)
    cpu_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    with np.errstate(all="ignore"):
        asset.Scene().insert_mesh(pos, uv, idx)
    host_s = time.perf_counter() - t0
    parity = q.tobytes() == oq.tobytes() and v.tobytes() == ov.tobytes()
    mesh = np.zeros(1, rec.dtype)
    mesh[0] = rec
    ing.emissive_triangles(q, v, idx, mesh, [(0, 0)])
    t0 = time.perf_counter()
    em = ing.emissive_triangles(q, v, idx, mesh, [(0, 0)])
    em_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    oem = oracle.emissive_triangles(q, v, idx, mesh, [(0, 0)])
    em_cpu_s = time.perf_counter() - t0
    ctx.close()
    return {"workload": f"grid_mesh_{len(pos)}v_{tris}tri", "gpu_ms": gpu_s * 1e3,
            "gpu_mtriangles_per_s": tris / gpu_s / 1e6, "oracle_ms": cpu_s * 1e3,
            "oracle_kind": "sequential C restatement, 1 core", "numpy_host_ms": host_s * 1e3,
            "speedup_vs_oracle": cpu_s / gpu_s, "parity_bit_exact": bool(parity),
            "emissive_extract_ms": em_s * 1e3, "emissive_oracle_ms": em_cpu_s * 1e3,
            "emissive_parity": bool(em.tobytes() == oem.tobytes()),
            "timing": "wall clock per call, host arrays in and out (H2D/D2H inside)"}


# ---------------------------------------------------------------- serving sample
SERVE_SCENES = [(1, 7), (4, 11), (16, 18), (64, 28), (128, 44)]  # (instances, frequency): 1e3 .. 5e6 triangles


def serve_requests(rng, pool, logs, n: int, first_frame: int):
    """n requests of the C4 mix: square resolution with side ~U{256..2048} (steps of 16), spp
    ~U{1..256}, depth 8, scene size log-uniform in [1e3, 5e6] triangles (nearest resident scene)."""
    from tinytrace_gb300 import scenes
    from tinytrace_gb300.renderer import Config, make_constants

    cam = scenes.Camera.looking_at((0.0, 10.0, 95.0), (0, 0, 0))
    reqs = []
    for k in range(n):
        side = int(rng.integers(16, 129)) * 16
        spp = int(rng.integers(1, 257))
        scene = pool[int(np.argmin(np.abs(logs - rng.uniform(3.0, np.log10(5e6)))))][1]
        c = make_constants(cam, (side, side), Config(bounce_count=8, sample_count=spp), first_frame + k, 0)
        reqs.append((scene, c, side * side * spp))
    return reqs


SERVE_INFLIGHT = 16  # requests rendered together per round


def serve_run(ctx, reqs, rate: float | None, rng, pool_paths: int, capacity_msamples_s: float | None = None,
              inflight: int = 16, policy: int = 0) -> dict:
    """Submits `reqs` (Poisson arrivals at `rate` per second, or all at once when rate is None),
    waits for all of them and returns latency percentiles and throughput.  Finished requests'
    image buffers are released as the run goes."""
    from tinytrace_gb300.server import RenderServer

    with RenderServer(ctx, hbm_budget_bytes=150 << 30, max_inflight=inflight, pool_paths=pool_paths,
                      policy=policy) as srv:
        t0 = time.perf_counter()
        due = t0
        ids, pending = [], []
        gaps = rng.exponential(1.0 / rate, len(reqs)) if rate else np.zeros(len(reqs))
        for (scene, c, _), gap in zip(reqs, gaps):
            due += gap
            time.sleep(max(0.0, due - time.perf_counter()))
            rid = srv.submit(scene, c)
            ids.append(rid)
            pending.append(rid)
            still = []
            for q in pending:
                if srv.status(q)[0] >= 2:
                    srv.release(q)
                else:
                    still.append(q)
            pending = still
        submit_end = time.perf_counter()
        for q in ids:
            srv.wait(q)
            srv.release(q)
        makespan = time.perf_counter() - t0
        lat = np.array([srv.status(q)[1] for q in ids])
        st = srv.stats()
    samples = sum(n for _, _, n in reqs)
    tenth = max(1, len(lat) // 10)
    # latency against request size: percentiles of the smaller and the larger half (by samples),
    # and of the slowdown, latency over the request's service time at the saturated throughput
    size = np.array([n for _, _, n in reqs], np.float64)
    small = size <= np.median(size)
    by_size = {"smaller_half_p50_ms": float(np.percentile(lat[small], 50)),
               "smaller_half_p99_ms": float(np.percentile(lat[small], 99)),
               "larger_half_p50_ms": float(np.percentile(lat[~small], 50)),
               "larger_half_p99_ms": float(np.percentile(lat[~small], 99))}
    if capacity_msamples_s:
        slow = lat / (size / (capacity_msamples_s * 1e3))
        by_size["slowdown_p50"] = float(np.percentile(slow, 50))
        by_size["slowdown_p99"] = float(np.percentile(slow, 99))
    return {"requests": len(reqs), "arrival_rate_per_s": rate, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()), "max_ms": float(lat.max()),
            "first_tenth_mean_ms": float(lat[:tenth].mean()), "last_tenth_mean_ms": float(lat[-tenth:].mean()),
            "completed_per_s": len(ids) / makespan, "offered_per_s": len(ids) / (submit_end - t0) if rate else None,
            "throughput_msamples_s": samples / makespan / 1e6, "peak_inflight": int(st.peak_inflight),
            "failed": int(st.failed), "makespan_s": makespan,
            "rounds": int(st.rounds), "mean_round_items": st.round_items / max(1, st.rounds),
            "gpu_busy_frac": st.gpu_busy_ns / 1e9 / makespan,
            "msamples_s_while_busy": samples / max(1e-9, st.gpu_busy_ns / 1e9) / 1e6,
            "scheduler_s": {"admit": st.admit_ns / 1e9, "launch": st.launch_ns / 1e9,
                            "copy_out": st.copy_out_ns / 1e9, "wait": st.wait_ns / 1e9},
            "latency_by_size": by_size}


def serve_one_request(ctx, scene, cam, pool_paths: int) -> dict:
    """The cost of the shared-pool kernels: one 1920x1080, 64-spp, depth-8 request on the 1M-
    triangle scene, alone, rendered by tt_render (the single-request kernels; CUDA events) and
    by the server (device time of its rounds from tt_server_stats), same pool size."""
    import ctypes

    from tinytrace_gb300 import native
    from tinytrace_gb300.native import check
    from tinytrace_gb300.renderer import Config, make_constants
    from tinytrace_gb300.server import RenderServer

    lib, h = ctx.lib, ctx.handle
    c = make_constants(cam, (1920, 1080), Config(bounce_count=8, sample_count=64), 7, 0)
    img = ctx.create_image(native.TT_LIFETIME_FRAME, 1920, 1080)
    check(lib.tt_set_option(h, native.TT_OPTION_WAVEFRONT_SLOTS, pool_paths))
    for _ in range(2):
        check(lib.tt_render(h, scene, native.ptr(c), img))
    check(lib.tt_synchronize(h))
    check(lib.tt_event_record(h, 6))
    check(lib.tt_render(h, scene, native.ptr(c), img))
    check(lib.tt_event_record(h, 7))
    ms = ctypes.c_float()
    check(lib.tt_event_elapsed_ms(h, 6, 7, ctypes.byref(ms)))
    with RenderServer(ctx, hbm_budget_bytes=150 << 30, max_inflight=1, pool_paths=pool_paths) as srv:
        srv.wait(srv.submit(scene, c))
        busy0, rounds0 = srv.stats().gpu_busy_ns, srv.stats().rounds
        t0 = time.perf_counter()
        srv.wait(srv.submit(scene, c))
        wall = time.perf_counter() - t0
        st = srv.stats()
    server_ms = (st.gpu_busy_ns - busy0) / 1e6
    return {"request": "1920x1080, 64 spp, depth 8, 1,004,520 triangles", "tt_render_ms": ms.value,
            "server_gpu_ms": server_ms, "server_rounds": int(st.rounds - rounds0), "server_wall_ms": wall * 1e3,
            "server_over_tt_render": server_ms / ms.value}


def run_serving(a, ctx) -> dict:
    """Continuous batching under the C4 request mix on five resident scenes (1e3 .. 5e6
    triangles), HBM budget 150 GB, smallest-first scheduling (a.serve_policy), up to 16 requests
    rendered together per round through one
    shared path pool whose size tt_autotune picks on a render as large as a round (the
    260k-triangle scene at 2048 x 2048, 16 spp, depth 8).  First the server's capacity: a batch of
    a.serve_batch requests submitted at once gives the saturated sample throughput, which over
    the mix's mean request size gives requests per second.  Then
    Poisson arrivals at fractions of that capacity: a.serve_requests requests at 0.8 x capacity and
    a quarter as many at 0.5 x and 1.1 x; a rate is sustained when its completions keep pace with
    its arrivals (completed per second >= 0.95 x offered) and the latency does not grow over the
    run (mean latency of the last tenth of the requests <= 1.5 x that of the first tenth)."""
    import ctypes

    from tinytrace_gb300 import native, scenes
    from tinytrace_gb300.native import check
    from tinytrace_gb300.renderer import Config, SceneArrays, make_constants

    rng = np.random.default_rng(2024)
    pool = []
    for inst, freq in SERVE_SCENES:
        arr = SceneArrays(scenes.icosphere_field(instances=inst, freq=freq, lights=max(4, min(1000, 16 * inst)),
                                                 seed=100 + inst))
        pool.append((arr.triangle_count, ctx.create_scene(arr)))
    logs = np.log10([t for t, _ in pool])
    cam = scenes.Camera.looking_at((0.0, 10.0, 95.0), (0, 0, 0))
    # tuned on a render as large as a round (2048 x 2048 x 16 spp = 2^26 work items), so that the
    # pool sizes a round needs are among the candidates and the ranking is not decided by noise
    img = ctx.create_image(native.TT_LIFETIME_FRAME, 2048, 2048)
    tune = native.TuneResult()
    c = make_constants(cam, (2048, 2048), Config(bounce_count=8, sample_count=16), 0, 0)
    check(ctx.lib.tt_autotune(ctx.handle, pool[2][1], native.ptr(c), img, ctypes.byref(tune)))
    pool_paths = int(tune.slots)
    out = {"scenes_triangles": [int(t) for t, _ in pool], "hbm_budget_gb": 150, "max_inflight": a.serve_inflight,
           "policy": a.serve_policy,
           "pool_paths": pool_paths, "pool_tuning": {"extent": [2048, 2048], "tune_spp": 16,
                                                     "default_ms": tune.default_ms, "tuned_ms": tune.best_ms,
                                                     "renders": int(tune.renders)},
           "round_items": 1 << 26,
           "mix": "side ~U{256..2048} step 16, spp ~U{1..256}, depth 8, scene log-uniform 1e3..5e6 triangles"}
    policy = {"fair": native.TT_SERVER_POLICY_FAIR, "smallest_first": native.TT_SERVER_POLICY_SMALLEST_FIRST}[
        a.serve_policy]
    serve_run(ctx, serve_requests(rng, pool, logs, 8, 0), None, rng, pool_paths, None, a.serve_inflight,
              policy)  # warm-up
    out["one_request"] = serve_one_request(ctx, pool[3][1], cam, pool_paths)
    cap = serve_run(ctx, serve_requests(rng, pool, logs, a.serve_batch, 100), None, rng, pool_paths, None,
                    a.serve_inflight, policy)
    # capacity in requests per second: the sample throughput of the saturated server over the mix's
    # mean request size (E[side^2] E[spp], side = 16 k with k ~ U{16..128}, spp ~ U{1..256}), not
    # the completion rate of one finite batch, whose few large requests decide its makespan
    k = np.arange(16, 129, dtype=np.float64)
    mean_samples = float(np.mean((16.0 * k) ** 2)) * 128.5
    mu = cap["throughput_msamples_s"] * 1e6 / mean_samples
    out["capacity"] = cap
    out["mean_request_msamples"] = mean_samples / 1e6
    out["capacity_per_s"] = mu
    out["rates"] = []
    frame = 10_000
    for frac, n in ((0.5, max(32, a.serve_requests // 4)), (0.8, a.serve_requests), (1.1, max(32, a.serve_requests // 4))):
        res = serve_run(ctx, serve_requests(rng, pool, logs, n, frame), frac * mu, rng, pool_paths,
                        cap["throughput_msamples_s"], a.serve_inflight, policy)
        frame += n
        res["fraction_of_capacity"] = frac
        res["sustained"] = bool(res["completed_per_s"] >= 0.95 * res["offered_per_s"]
                                and res["last_tenth_mean_ms"] <= 1.5 * res["first_tenth_mean_ms"])
        out["rates"].append(res)
    sustained = [r for r in out["rates"] if r["sustained"]]
    best = max(sustained, key=lambda r: r["arrival_rate_per_s"]) if sustained else None
    out["sustainable_rate_per_s"] = best["arrival_rate_per_s"] if best else None
    out["p50_ms_at_sustainable_rate"] = best["p50_ms"] if best else None
    out["p99_ms_at_sustainable_rate"] = best["p99_ms"] if best else None
    out["requests_at_sustainable_rate"] = best["requests"] if best else None
    out["latency_by_size_at_sustainable_rate"] = best["latency_by_size"] if best else None
    return out


def run_ours(a, dist: Dist):
    import ctypes

    from tinytrace_gb300 import native
    from tinytrace_gb300.native import check
    from tinytrace_gb300.renderer import Renderer

    device = dist.local_rank
    w = make_workload(a)
    r = Renderer(w.extent, device=device)
    integ = native.TT_INTEGRATOR_WAVEFRONT if a.integrator == "wavefront" else native.TT_INTEGRATOR_MEGAKERNEL
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_INTEGRATOR, integ))
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_WAVEFRONT_SLOTS, a.slots))
    accel = {"auto": native.TT_ACCEL_AUTO, "flat": native.TT_ACCEL_FLAT, "two_level": native.TT_ACCEL_TWO_LEVEL,
             "wide": native.TT_ACCEL_FLAT_WIDE}
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_ACCEL, accel[a.accel]))
    primary = {"raster": native.TT_PRIMARY_RASTER, "traverse": native.TT_PRIMARY_TRAVERSE}
    check(r.context.lib.tt_set_option(r.context.handle, native.TT_OPTION_PRIMARY_VISIBILITY, primary[a.primary]))
    r.set_scene(w.scene)
    r.camera = w.camera
    r.set_config(w.config)
    lib, ctx = r.context.lib, r.context.handle
    stats = r.context.scene_stats(r.scene)
    W, H = w.extent
    spp = w.config.sample_count
    samples_per_step = W * H * spp

    def step():
        check(lib.tt_flush_l2(ctx))
        r.render_to_target()
        r.present()

    check(lib.tt_set_option(ctx, native.TT_OPTION_GRAPHS, 0 if a.host_loop else 1))
    tuning = None
    if not a.no_autotune and a.integrator == "wavefront" and not a.slots:
        # renders of the same frame at its own sample count (up to 64, one sample chunk), before the
        # warm-up: shorter tuning renders rank pools that the full frame ranks otherwise
        tune_spp = min(spp, 64)
        t = r.autotune(sample_count=tune_spp)
        tuning = {"slots": t.slots, "refill_lanes": t.refill_lanes, "trace_blocks_per_sm": t.trace_blocks_per_sm,
                  "renders": t.renders, "tune_spp": tune_spp, "default_ms": t.default_ms, "tuned_ms": t.best_ms}
    for _ in range(a.warmup):
        step()
    check(lib.tt_synchronize(ctx))
    dist.barrier()
    clocks = ClockSampler(device)
    clocks.start()
    check(lib.tt_synchronize(ctx))
    check(lib.tt_event_record(ctx, 0))
    kernel_ns = []
    for _ in range(a.steps):
        step()
        kernel_ns.append(r.timings().integrate * 1e9)  # synchronises; integrate-kernel events
    check(lib.tt_event_record(ctx, 1))
    ms = ctypes.c_float()
    check(lib.tt_event_elapsed_ms(ctx, 0, 1, ctypes.byref(ms)))
    check(lib.tt_synchronize(ctx))
    clk = clocks.stop()
    dist.barrier()
    total_s = dist.max(ms.value / 1e3)
    value = samples_per_step * a.steps * dist.world / total_s / 1e6

    # per-launch timing: a second loop of the same K steps with CUDA events around every
    # integrator launch on its stream (this drives the loop from the host)
    check(lib.tt_set_option(ctx, native.TT_OPTION_STAGE_TIMING, 1))
    step()
    stage_ns = np.zeros(native.TT_STAGE_COUNT)
    stage_launches = np.zeros(native.TT_STAGE_COUNT, np.int64)
    stage_overflow = False
    timed_ns = []
    for _ in range(a.steps):
        step()
        timed_ns.append(r.timings().integrate * 1e9)
        stt = native.StageTimings()
        check(lib.tt_stage_timings_get(ctx, ctypes.byref(stt)))
        stage_ns += np.array(stt.ns[:], np.float64)
        stage_launches += np.array(stt.launches[:], np.int64)
        stage_overflow |= bool(stt.overflow)
    check(lib.tt_set_option(ctx, native.TT_OPTION_STAGE_TIMING, 0))
    regen_per_step = int(stage_launches[native.TT_STAGE_REGEN]) // a.steps
    reduce_per_step = int(stage_launches[native.TT_STAGE_REDUCE]) // a.steps
    primary_per_step = int(stage_launches[native.TT_STAGE_PRIMARY]) // a.steps
    if a.host_loop or a.integrator != "wavefront":
        launches_per_step = int(stage_launches.sum()) // a.steps
    else:  # graph loop: regen, control, extend, shade and shadow every iteration, then the reduction
        launches_per_step = 5 * regen_per_step + reduce_per_step + primary_per_step
    if primary_per_step:  # the timed set-up counts once: instance, rectangle, two scans, listing and finish kernels
        launches_per_step += 4 + 2 * scan_launches(int(stats.triangle_count) + 1)

    # end to end through the public API: render_to_texture into pinned host memory
    host = ctypes.c_void_p()
    nbytes = W * H * 16
    check(lib.tt_host_alloc(nbytes, ctypes.byref(host)))
    out = np.ctypeslib.as_array((ctypes.c_float * (W * H * 4)).from_address(host.value)).reshape(H, W, 4)
    e2e_steps = max(1, min(a.steps, 3))
    r.render_to_target()
    r.context.download(r.render_target, W, H, out)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        check(lib.tt_flush_l2(ctx))
        r.render_to_target()  # 368-byte Constants host -> device with the launch
        r.context.download(r.render_target, W, H, out)  # W*H*16 bytes device -> host, synchronous
        r.present()
    e2e_s = dist.max(time.perf_counter() - t0)
    check(lib.tt_host_free(host))
    e2e = samples_per_step * e2e_steps * dist.world / e2e_s / 1e6

    # roofline accounting of the dominant kernel (wf_trace_kernel: the extend and shadow
    # stages) from the traversal counters of an instrumented render of the same frame
    cnt = native.TraversalCounters()
    c = r.constants()
    check(lib.tt_render_counted(ctx, r.scene, native.ptr(c), r.render_target, ctypes.byref(cnt)))
    node_size = WIDE_NODE_BYTES if stats.accel == native.TT_ACCEL_FLAT_WIDE else NODE_BYTES
    node_bytes = (cnt.blas_nodes + cnt.tlas_nodes) * node_size
    trace_bytes = (node_bytes + cnt.triangles * TRI_RECORD_BYTES + cnt.instances * INSTANCE_RAY_BYTES
                   + cnt.rays * RAY_STATE_BYTES)
    trace_stages = [native.TT_STAGE_EXTEND, native.TT_STAGE_SHADOW]
    trace_launches = int(stage_launches[trace_stages].sum()) / a.steps  # per frame
    trace_s = float(stage_ns[trace_stages].sum()) / a.steps / 1e9  # per frame
    kernel_s = statistics.mean(kernel_ns) / 1e9
    peak, peak_kind = measured_peaks()
    if trace_launches > 0:
        bytes_per_launch = trace_bytes / trace_launches
        launch_s = trace_s / trace_launches
        achieved = bytes_per_launch / launch_s / 1e9
        node_achieved = node_bytes / trace_s / 1e9
        rays_per_launch = cnt.rays / trace_launches
        default_workload = (W, H, spp, w.config.bounce_count) == (1920, 1080, 64, 8)
        traffic = (ncu_traffic_per_launch(rays_per_launch)
                   if default_workload and stats.accel == native.TT_ACCEL_FLAT else None)
    else:  # the megakernel does everything in one launch
        bytes_per_launch, launch_s = trace_bytes, kernel_s
        achieved = trace_bytes / kernel_s / 1e9
        node_achieved = node_bytes / kernel_s / 1e9
        rays_per_launch, traffic = cnt.rays, None

    l2 = None
    if dist.rank == 0:
        try:
            l2 = l2_copy_gbs(device)
        except Exception:  # torch absent or without CUDA: the L2 reference is left out
            l2 = None
    out_line = None
    if dist.rank == 0:
        cpu, parity = None, None
        if not a.no_cpu_baseline:
            from tinytrace_gb300.renderer import make_constants

            cpu, cpu_img, rows = cpu_baseline(w, r.scene_arrays, a.cpu_row_stride)
            # the GPU's first frame of the same Constants (the image the timed steps render,
            # without their accumulation), compared with the oracle's rows
            c0 = make_constants(w.camera, w.extent, w.config, 0, 0)
            check(lib.tt_render(ctx, r.scene, native.ptr(c0), r.render_target))
            parity = row_parity(r.context.download(r.render_target, W, H), cpu_img, rows)
        stages = {name: {"ms_per_step": stage_ns[i] / a.steps / 1e6,
                         "launches_per_step": int(stage_launches[i]) / a.steps}
                  for i, name in enumerate(native.STAGE_NAMES) if stage_launches[i] > 0}
        out_line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": total_s * 1e3 / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
            "config": {"workload": w.name, "triangles": int(stats.triangle_count),
                       "instances": int(stats.instance_count), "emissive_triangles": int(stats.emissive_count),
                       "resolution": [W, H], "spp": spp, "depth": w.config.bounce_count,
                       "light_sampling": "next_event_estimation",
                       "l2": "flushed before every step (512 MiB memset, inside the timed region)",
                       "parallelism": f"replicas x{dist.world}", "integrator": a.integrator,
                       "accel": {native.TT_ACCEL_FLAT: "flat", native.TT_ACCEL_FLAT_WIDE: "wide"}.get(
                           int(stats.accel), "two_level"),
                       "primary_visibility": a.primary if stats.accel == native.TT_ACCEL_FLAT else "traverse",
                       "autotune": tuning},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 368, "d2h_bytes_per_step": nbytes,
                    "steps": e2e_steps},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                         "traffic": traffic,
                         "kernel": "wf_trace_kernel" if trace_launches > 0 else "integrate_kernel",
                         "launches_per_step": trace_launches, "launch_ms": launch_s * 1e3,
                         "algorithmic_bytes_per_launch": bytes_per_launch, "rays_per_launch": rays_per_launch,
                         "bytes_per_unit": {"node": node_size, "triangle_record": TRI_RECORD_BYTES,
                                            "instance_ray_setup": INSTANCE_RAY_BYTES, "ray_state": RAY_STATE_BYTES},
                         "node_fetch_gbs": node_achieved, "node_fetch_frac": node_achieved / peak,
                         "rays_per_frame": int(cnt.rays), "rays_per_sample": cnt.rays / samples_per_step,
                         "rays_per_s": cnt.rays / (total_s / a.steps),
                         "trace_rays_per_s": cnt.rays / trace_s if trace_launches > 0 else None,
                         "l2_copy": l2, "l2_frac": achieved / l2["gbs"] if l2 else None,
                         "dram_gbs": traffic / launch_s / 1e9 if traffic else None,
                         "dram_frac": traffic / launch_s / 1e9 / peak if traffic else None,
                         "limiter": "latency of dependent L1/L2 node fetches and SIMT efficiency: the algorithmic "
                                    "bytes are served mostly by L1/L2 (see dram_frac and l2_frac), so `frac` "
                                    "measures them against the HBM copy ceiling, not DRAM traffic",
                         "ncu": ncu_trace_metrics(),
                         "traffic_source": traffic_source()},
            "stages": stages,
            "counters": {"rays": cnt.rays, "blas_nodes": cnt.blas_nodes, "tlas_nodes": cnt.tlas_nodes,
                         "triangles": cnt.triangles, "instances": cnt.instances, "hits": cnt.hits,
                         "traversal_step_lane_occupancy": cnt.lane_steps / max(1, 32 * cnt.warp_steps)},
            "scene": {"blas_nodes": int(stats.blas_nodes), "tlas_nodes": int(stats.tlas_nodes),
                      "blas_levels": int(stats.blas_levels), "tlas_levels": int(stats.tlas_levels),
                      "device_bytes": int(stats.device_bytes), "build_ms": None},
            "clocks": clk,
            "gpu_launches": launches_per_step * a.steps,
            "gpu_launches_overflow": stage_overflow,
            "loop": "host-driven" if a.host_loop else "device-side while loop in one CUDA graph per render",
            "cpu_baseline": cpu,
            "parity": parity,
        }
        t = native.Timings()
        check(lib.tt_timings_get(ctx, ctypes.byref(t)))
        out_line["scene"]["build_ms"] = t.scene_build_ns / 1e6
        if not a.no_cache and dist.world == 1:
            try:
                out_line["radiance_cache"] = run_cache(a, device)
            except Exception as e:
                out_line["radiance_cache"] = {"error": f"{type(e).__name__}: {e}"}
        if not a.no_restir and dist.world == 1:
            try:
                out_line["restir"] = run_restir(a, device, clk.get("sm_mhz"))
            except Exception as e:
                out_line["restir"] = {"error": f"{type(e).__name__}: {e}"}
        if not a.no_textured and dist.world == 1:
            try:
                out_line["textured"] = run_textured(a, device)
            except Exception as e:
                out_line["textured"] = {"error": f"{type(e).__name__}: {e}"}
        if not a.no_closed and dist.world == 1:
            try:
                out_line["closed_scene"] = run_closed(a, device)
            except Exception as e:
                out_line["closed_scene"] = {"error": f"{type(e).__name__}: {e}"}
        if not a.no_light_selection and dist.world == 1:
            try:
                out_line["light_selection"] = run_light_selection(a, device)
            except Exception as e:
                out_line["light_selection"] = {"error": f"{type(e).__name__}: {e}"}
        if not a.no_ingest and dist.world == 1:
            try:
                out_line["ingest"] = run_ingest(a, device)
            except Exception as e:
                out_line["ingest"] = {"error": f"{type(e).__name__}: {e}"}
        if not a.no_serve and dist.world == 1:
            try:
                out_line["serving"] = run_serving(a, r.context)
            except Exception as e:  # the serving sample never invalidates the headline line
                out_line["serving"] = {"error": f"{type(e).__name__}: {e}"}
    r.close()
    if out_line is not None:
        print(json.dumps(out_line))


def main():
    a = parse_args()
    dist = Dist()
    try:
        if a.impl == "reference":
            run_reference(a, dist)
        else:
            run_ours(a, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
