"""Writes tests/golden/oracle_golden.npz: inputs and outputs of the CPU oracle on small
seeded cases (elementary functions, BSDF evaluate/sample, closest hits, BVH byte hashes,
two small renders).

The scene arrays are stored too, so that the fixtures do not depend on the scene
generators' floating-point results on another machine.  The reference's own tests hold no
known-answer vectors for this path (its BSDF harness
asserts nothing and its ray queries run on the closed driver BVH), so these fixtures are
the oracle's outputs frozen when they were generated.  They pin the oracle against
regressions and against drift between compilers and CPU architectures (x86-64 here,
aarch64 on the GPU hosts), and the GPU tests compare the CUDA path to them directly.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

OUT = Path(__file__).resolve().parent / "oracle_golden.npz"


def math_inputs() -> dict[int, np.ndarray]:
    rng = np.random.default_rng(1000)
    return {
        0: np.concatenate([rng.uniform(-50, 50, 2044), [0.0, 1e4, -3.0, 7.5]]).astype(np.float32),
        1: np.concatenate([rng.uniform(-50, 50, 2044), [0.0, 1e4, -3.0, 7.5]]).astype(np.float32),
        2: np.concatenate([rng.uniform(-90, 89, 2044), [0.0, -104.0, 88.7, 1.0]]).astype(np.float32),
        3: np.concatenate([np.exp(rng.uniform(-90, 88, 2044)), [1.0, 2.0, 1e-40, 0.5]]).astype(np.float32),
        4: np.concatenate([rng.uniform(-1, 1, 2044), [-1.0, 1.0, 0.0, 0.999]]).astype(np.float32),
    }


def small_field():
    from tinytrace_gb300 import scenes

    return scenes.icosphere_field(instances=6, freq=8, lights=40, seed=11)


def field_rays(arrays, n=4096, seed=1001) -> np.ndarray:
    rng = np.random.default_rng(seed)
    centres = arrays.instances["transform"][:, 12:15].astype(np.float64)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(-40, 40, (n, 3))
    t = centres[rng.integers(0, len(centres), n)] + rng.normal(0, 3.0, (n, 3))
    d = t - rays[:, 0:3]
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 3] = 1e-3
    rays[:, 7] = rng.choice([1000.0, 10000.0, 20.0], n)
    return rays


def render_workloads():
    from tinytrace_gb300 import scenes

    cornell = scenes.cornell_workload(extent=(32, 24), spp=2, depth=4)
    field = scenes.Workload("field_small", small_field(), scenes.Camera.looking_at((0.0, 10.0, 95.0), (0, 0, 0)),
                            (48, 27), scenes.Config(bounce_count=8, sample_count=2))
    return {"cornell": cornell, "field": field}


def bvh_hashes(orc) -> dict[str, str]:
    blas, tris, tlas, bl, tl = orc.bvh()
    nodes, ftris, fl = orc.flat_bvh()
    h = lambda *arrs: hashlib.sha256(b"".join(a.tobytes() for a in arrs)).hexdigest()
    return {"two_level": h(blas, tris, tlas) + f":{bl}:{tl}", "flat": h(nodes, ftris) + f":{fl}"}


def generate() -> dict[str, np.ndarray]:
    from materials import material_suite
    from oracle import oracle
    from tinytrace_gb300 import scenes
    from tinytrace_gb300.renderer import SceneArrays, make_constants

    out: dict[str, np.ndarray] = {}
    for which, x in math_inputs().items():
        out[f"math{which}_x"] = x
        out[f"math{which}_y"] = oracle.math(which, x)
    rng = np.random.default_rng(1002)
    mats = np.stack(material_suite()[:12])
    out["bsdf_materials"] = mats
    ev_in, ev_out, sm_in, sm_out = [], [], [], []
    for m in mats:
        wi = rng.normal(size=(64, 3)).astype(np.float32)
        wi /= np.linalg.norm(wi, axis=1, keepdims=True)
        wi[:48, 2] = np.abs(wi[:48, 2])
        wo = rng.normal(size=(64, 3)).astype(np.float32)
        wo /= np.linalg.norm(wo, axis=1, keepdims=True)
        s = np.zeros((64, 8), np.float32)
        s[:, 0:3], s[:, 4:7] = wi, wo
        s[:, 3] = rng.integers(0, 2**32, 64, dtype=np.uint64).astype(np.uint32).view(np.float32)
        ev_in.append(s)
        ev_out.append(oracle.bsdf_eval(m, s))
        t = np.zeros((64, 4), np.float32)
        t[:, 0:3] = wi
        t[:, 3] = rng.integers(1, 2**32, 64, dtype=np.uint64).astype(np.uint32).view(np.float32)
        sm_in.append(t)
        sm_out.append(oracle.bsdf_sample(m, t))
    out["bsdf_eval_in"], out["bsdf_eval_out"] = np.stack(ev_in), np.stack(ev_out)
    out["bsdf_sample_in"], out["bsdf_sample_out"] = np.stack(sm_in), np.stack(sm_out)
    frozen = {}
    for name, scene in (("cornell", scenes.cornell_box()), ("field", small_field()),
                        ("instanced", scenes.instanced_spheres())):
        frozen[name] = SceneArrays(scene)
        out.update(frozen[name].save(None, prefix=f"scene_{name}_"))
    arrays = frozen["field"]
    orc = oracle.OracleScene(arrays)
    rays = field_rays(arrays)
    out["trace_rays"] = rays
    out["trace_hits"] = orc.trace(rays, cull=False)
    out["trace_hits_cull"] = orc.trace(rays, cull=True)
    for name, arr in frozen.items():
        hs = bvh_hashes(oracle.OracleScene(arr))
        out[f"bvh_{name}_two_level"] = np.array(hs["two_level"])
        out[f"bvh_{name}_flat"] = np.array(hs["flat"])
    for name, w in render_workloads().items():
        c = make_constants(w.camera, w.extent, w.config, 7, 0)
        out[f"render_{name}_constants"] = np.frombuffer(c.tobytes(), np.uint8)
        out[f"render_{name}"] = oracle.OracleScene(frozen[name]).render(c)
    return out


if __name__ == "__main__":
    data = generate()
    np.savez_compressed(OUT, **data)
    print(OUT, OUT.stat().st_size, "bytes,", len(data), "arrays")
