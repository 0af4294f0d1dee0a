"""The benchmark's multi-rank host logic on CPU: two gloo ranks on 127.0.0.1
(the replicas-only layout — every rank renders its own pose batch, no
collective on the data path): barrier, max over ranks of the timed region,
distinct pose batches per rank, and the reference arm's rank 0 alone
reporting."""

import os
import socket
import sys
from pathlib import Path

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    w, r, local = bench.dist_setup()
    assert (w, r) == (world, rank) and dist.get_backend() == "gloo"
    bench.barrier(w)
    t = bench.max_over_ranks(0.5 + rank, w, torch.device("cpu"))
    _, _, _, rt, _ = bench.workload(_Args(), "cpu", seed_offset=rank)
    torch.save({"t": t, "rt": rt}, os.path.join(out_dir, f"rank{rank}.pt"))
    bench.barrier(w)
    dist.destroy_process_group()


class _Args:
    volume = "16x16x16"
    spacing = "1.0,1.0,1.0"
    det = 8
    pixel = 2.0
    batch = 3


def test_two_gloo_ranks_share_the_max_time_and_render_distinct_poses(tmp_path):
    world, port = 2, _free_port()
    mp.spawn(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    r0 = torch.load(tmp_path / "rank0.pt")
    r1 = torch.load(tmp_path / "rank1.pt")
    assert r0["t"] == r1["t"] == pytest.approx(1.5)  # the max over ranks
    assert r0["rt"].shape == r1["rt"].shape == (3, 4, 4)
    assert not torch.equal(r0["rt"], r1["rt"])  # weak scaling: each rank its own pose batch


def _ref_rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench

    w, r, local = bench.dist_setup()
    # ranks other than 0 return at once without work (and without output)
    if r != 0:
        bench.run_reference(None, w, r, local)
        open(os.path.join(out_dir, f"ref{r}.done"), "w").close()
    bench.barrier(w)
    dist.destroy_process_group()


def test_reference_arm_runs_on_rank_zero_only(tmp_path):
    world, port = 2, _free_port()
    mp.spawn(_ref_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    assert (tmp_path / "ref1.done").exists()


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the reference's CPU path restated, on the
    host cores) prints one JSON line with the benchmark's metric, a
    cpu_baseline describing the run and an e2e entry without device copies."""
    import json
    import subprocess

    sys.path.insert(0, str(ROOT))
    import bench

    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "3",
                        "--cpu-rays", "64"], capture_output=True, text=True, timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "frames/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] >= 3
    assert {"value", "unit", "cores", "kind", "sample"} <= set(d["cpu_baseline"])
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert "workload" in d["config"]
