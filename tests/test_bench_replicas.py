"""bench.py's replica path on CPU: `--gpus N` runs N replica processes with a gloo process
group for the barrier and the max-over-ranks timing (one GPU per rank; no collective on the data
path). Here the ranks are CPU processes: the max-over-ranks aggregation of two ranks, and the
reference arm (a CPU-only leg) launched through the replica launcher with world size 2."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_path: str) -> None:
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench

    w, r, local, dist = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(dist)
    # rank r took (r + 1) * 10 ms for 5 steps of 1000 samples
    ms, value = bench.replica_throughput(dist, w, 1000, (r + 1) * 10.0, 5)
    with open(f"{out_path}.{rank}", "w") as f:
        json.dump({"ms": ms, "value": value}, f)
    dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks(tmp_path):
    ctx = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, str(tmp_path / "r"))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(2):
        d = json.loads((tmp_path / f"r.{r}").read_text())
        # the slowest rank's time (20 ms / 5 steps), the samples of both ranks
        assert d["ms"] == pytest.approx(4.0)
        assert d["value"] == pytest.approx(2 * 1000 / 4.0e-3 / 1e6)


def test_reference_arm_through_the_replica_launcher():
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup",
           "0", "--width", "96", "--height", "64"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=str(ROOT))
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout  # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
