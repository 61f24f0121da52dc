"""The N > 1 path of bench.py on the CPU: two gloo ranks (replicas) run the bench's own
rank helpers — process-group setup, barrier, max over ranks of the step time and the
whole-job aggregate — with rank-dependent step times.  No GPU."""
import os
import socket
from argparse import Namespace

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, ws: int, port: int, out_dir: str):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    got_ws, got_rank, local = bench.dist_init(Namespace(impl="ours"))
    try:
        bench.barrier(got_ws)
        step = 0.010 * (rank + 1)  # the slower rank decides the job's step time
        job_step = bench.max_over_ranks(got_ws, step)
        tflops = bench.job_tflops(got_ws, 1.0e12, job_step)
        bench.barrier(got_ws)
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
            f.write(f"{got_ws} {got_rank} {local} {dist.get_backend()} {job_step!r} {tflops!r}\n")
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_time_the_job_by_the_slowest_rank(tmp_path):
    ws = 2
    torch.multiprocessing.spawn(_worker, args=(ws, _free_port(), str(tmp_path)), nprocs=ws, join=True)
    rows = [open(tmp_path / f"rank{r}.txt").read().split() for r in range(ws)]
    for r, row in enumerate(rows):
        assert int(row[0]) == ws and int(row[1]) == r and int(row[2]) == r
        assert row[3] == "gloo"
        assert float(row[4]) == pytest.approx(0.020)
        # both ranks' work (2 x 1 TFLOP) over the slowest rank's 20 ms
        assert float(row[5]) == pytest.approx(100.0)
