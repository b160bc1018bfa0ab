"""The replica path of bench.py on CPU: two gloo ranks (127.0.0.1), each timing its own batch, report
the units of both ranks over the slower rank's time; under torchrun the reference arm runs on rank 0
only and the other ranks exit without output."""
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_path: str) -> None:
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took 10 * (r + 1) ms for its 1000 arena-ticks
        value, ms = bench.replica_rate(1000, 10.0 * (rank + 1), world, "cpu")
        with open(f"{out_path}.{rank}", "w") as f:
            f.write(f"{value} {ms}")
    finally:
        dist.destroy_process_group()


def test_replica_rate_takes_the_slowest_rank(tmp_path):
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    out = str(tmp_path / "rate")
    mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    for r in range(world):
        value, ms = (float(x) for x in open(f"{out}.{r}").read().split())
        assert ms == pytest.approx(20.0)
        assert value == pytest.approx(1000 * world / 0.020)


def test_single_rank_rate_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    value, ms = bench.replica_rate(500, 5.0, 1, "cpu")
    assert (value, ms) == (pytest.approx(100000.0), 5.0)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "3"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
