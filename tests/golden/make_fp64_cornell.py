"""Generates tests/golden/cornell_fp64_64x64.npz: the converged float64 render (oracle/fp64_cornell.py)
of the procedural Cornell box at 64x64, depth 4, 4096 samples per pixel, with the constants of
frame 0 (the GPU renders compared with it use the same camera and depth).

Run from the repository root: python tests/golden/make_fp64_cornell.py  (about 10 minutes)."""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import fp64_cornell  # noqa: E402
from tinytrace_gb300 import scenes  # noqa: E402
from tinytrace_gb300.renderer import SceneArrays, make_constants  # noqa: E402

SPP = 4096


def main():
    w = scenes.cornell_workload(extent=(64, 64), spp=SPP, depth=4)
    arrays = SceneArrays(w.scene)
    c = make_constants(w.camera, w.extent, w.config, 0, 0)
    img = fp64_cornell.render(arrays, c, SPP, seed=20261203, batch_pixels=max(1, 65536 // SPP))
    out = Path(__file__).resolve().parent / "cornell_fp64_64x64.npz"
    np.savez_compressed(out, image=img.astype(np.float64), spp=SPP, depth=4, extent=np.array([64, 64]))
    print(out, img.mean(axis=(0, 1)))


if __name__ == "__main__":
    main()
