"""Multi-process host logic of bench.py on CPU (gloo, world size 2).

The path does not shard: N GPUs run N independent replicas and bench.py only needs a
barrier and a max-over-ranks of the timed region.  These tests run that logic as two gloo
ranks on 127.0.0.1, and the reference arm under torchrun, where rank 0 alone works and
prints one JSON line.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str) -> None:
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench

    d = bench.Dist()
    try:
        d.barrier()
        m = d.max(float(rank * 10 + 1))
        d.barrier()
        Path(out_dir, f"rank{rank}.json").write_text(json.dumps({"world": d.world, "max": m}))
    finally:
        d.close()


def test_gloo_max_over_ranks(tmp_path):
    import torch.multiprocessing as mp

    port = free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        res = json.loads((tmp_path / f"rank{r}.json").read_text())
        assert res == {"world": 2, "max": 11.0}


def test_reference_arm_under_torchrun():
    """rank 0 times the CPU path and prints one line; rank 1 exits 0 without work."""
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "1", "--width", "48", "--height", "24", "--spp", "2",
           "--depth", "3", "--instances", "2", "--freq", "4", "--lights", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["higher_is_better"] is True and line["unit"] == "Msamples/s"
    # one step renders the stratified rows; ms_per_step is that measured time, and value is the
    # samples of the timed steps over it
    rows = len(range(4, 24, 8))
    assert "stratified rows" in line["config"]["step"]
    samples = rows * 48 * 2
    assert abs(line["value"] - samples / (line["ms_per_step"] / 1e3) / 1e6) <= 1e-6 * line["value"]


def test_row_sample_and_parity_helpers():
    import numpy as np

    sys.path.insert(0, str(ROOT))
    import bench

    rows = bench.sample_rows(1080, 8)
    assert rows[0] == 4 and rows[-1] == 1076 and len(rows) == 135
    a = np.random.default_rng(0).random((32, 8, 4)).astype(np.float32)
    b = a.copy()
    b[4, 1, 2] = np.nextafter(b[4, 1, 2], np.float32(2))
    b[12, 0, 0] = a[12, 0, 0] = np.nan
    p = bench.row_parity(a, b, [4, 12, 20])
    assert p["values_differing"] == 1 and not p["bit_exact"] and 0 < p["max_rel_err"] < 1e-6
    assert bench.row_parity(a, a, [4, 12, 20])["bit_exact"]


def test_equal_error_interpolation():
    sys.path.insert(0, str(ROOT))
    import bench

    pts = [{"ms": 10.0, "error": 4e-3}, {"ms": 20.0, "error": 2e-3}, {"ms": 40.0, "error": 1e-3}]
    t, how = bench.time_at_error(pts, 2.8284271247461903e-3)  # halfway in log-log between the first two
    assert how == "interpolated" and abs(t - 14.142135623730951) < 1e-9
    assert bench.time_at_error(pts, 5e-3) == (10.0, "below")
    assert bench.time_at_error(pts, 5e-4) == (None, "floor")


@pytest.mark.parametrize("world", [1])
def test_single_process_dist_is_a_no_op(world, monkeypatch):
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    sys.path.insert(0, str(ROOT))
    import bench

    d = bench.Dist()
    assert d.world == world and d.max(3.5) == 3.5
    d.barrier()
    d.close()
