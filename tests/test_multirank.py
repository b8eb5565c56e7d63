"""The N > 1 path of bench.py on the CPU: two gloo ranks.

Multi-GPU runs are replicas (each rank solves its own copy of the system;
no collective on the data path), so what needs checking is the host logic
around them: the job's time is the slowest rank's, the job's work is the sum
over ranks, only rank 0 reports, and the reference arm's other ranks exit
without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank-dependent local measurements
        t = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
        w = bench.sum_over_ranks(100.0 * (rank + 1), dist, "cpu")
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"max": t, "sum": w}, f)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_reductions_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    got = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for g in got:
        assert g["max"] == 15.0      # the slower rank's time
        assert g["sum"] == 300.0     # both ranks' work


def test_single_process_reductions_are_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.sum_over_ranks(7.0, None, "cpu") == 7.0


def test_reference_arm_other_ranks_exit_without_work():
    # a rank other than 0 of `bench.py --impl reference` prints nothing and
    # exits 0 at once (no GPU, no oracle run)
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "1"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
