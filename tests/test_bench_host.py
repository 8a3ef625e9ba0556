"""bench.py's multi-rank plumbing on CPU: gloo process group, barrier,
max-over-ranks timing, and the reference arm under torchrun with two ranks
(rank 0 prints the one JSON line, rank 1 exits without work)."""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "LOCAL_RANK": str(rank), "WORLD_SIZE": "2"})
    sys.path.insert(0, REPO)
    import bench
    ws, r, local = bench._dist()
    bench._barrier(ws)
    v = bench._max_over_ranks(1.5 + r, ws)
    with open(os.path.join(out, f"rank{r}.json"), "w") as f:
        json.dump({"ws": ws, "rank": r, "max": v}, f)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_gloo_barrier_and_max(tmp_path):
    import torch.multiprocessing as mp
    mp.spawn(_rank_main, args=(_free_port(), str(tmp_path)), nprocs=2, join=True)
    got = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    assert [g["ws"] for g in got] == [2, 2]
    assert [g["max"] for g in got] == [2.5, 2.5]


@pytest.mark.slow
def test_reference_arm_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--particles", "4000", "--steps", "1", "--warmup", "3"]
    p = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "accels/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0


def test_clock_sampler_parsing():
    """Median SM clock, max clock and active throttle reasons from the
    nvidia-smi CSV lines sampled during the timed region."""
    sys.path.insert(0, REPO)
    import bench
    cs = bench.ClockSampler(0)
    cs.proc = type("P", (), {"terminate": lambda self: None, "wait": lambda self, timeout=None: 0})()
    cs.lines = ["0, 2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active",
                "0, 2040, 2070, 1300.0, 0x4, Not Active, Not Active, Not Active, Active",
                "0, 2070, 2070, 1350.0, 0x4, Not Active, Not Active, Not Active, Active",
                "garbage"]
    got = cs.stop()
    assert got["sm_mhz"] == 2070.0 and got["sm_max_mhz"] == 2070.0
    assert got["reasons"] == ["sw_power_cap"] and got["samples"] == 3


def test_workload_description_and_threads():
    sys.path.insert(0, REPO)
    import bench
    d = bench._workload_desc(1_000_000, "fast")
    assert d["workload"].startswith("Plummer sphere N=1,000,000")
    assert d["theta"] == 0.5 and d["softening"] == 0.01 and d["leaf_size"] == 32
    assert "L2 flush" in d["l2"] or "flush" in d["l2"]
    assert bench.host_threads() >= 1
