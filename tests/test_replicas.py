"""The multi-GPU mode is replicas only: every rank runs the whole workload on
its own GPU, with no data-path collective, and the job's time is the maximum
over the ranks.  These CPU tests cover that host logic with two gloo ranks
(no GPU): the max-over-ranks reduction of bench.py, and the reference arm's
rule that only rank 0 works and prints under torchrun."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out_dir):
    import torch.distributed as tdist
    sys.path.insert(0, ROOT)
    import bench
    tdist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        v = bench.max_over_ranks(1.5 + rank, world, "cpu")
        with open(os.path.join(out_dir, f"r{rank}"), "w") as f:
            f.write(repr(v))
    finally:
        tdist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    got = [float(open(tmp_path / f"r{r}").read()) for r in range(2)]
    assert got == [2.5, 2.5]


def test_max_over_ranks_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, 1, "cpu") == 3.25


def test_reference_arm_nonzero_rank_does_no_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
