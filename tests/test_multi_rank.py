"""The N > 1 path of bench.py (one shot replica per rank, no data-path
collective, slowest rank's time) as world-size-2 gloo ranks on CPU: the
max-over-ranks reduction, the whole-job rate, and the reference arm printing
on rank 0 only."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, _ = bench.dist_setup()
        assert (w, r) == (world, rank)
        # rank r took 1 + 1.5 r seconds for its replica
        t = bench.max_over_ranks(1.0 + 1.5 * rank, world, device="cpu")
        rate = bench.whole_job_rate(1000.0, t, world)
        # the reference arm: rank 0 alone samples and prints
        buf = io.StringIO()

        class Args:
            steps, warmup, gpus = 1, 1, world
        if rank != 0:
            with redirect_stdout(buf):
                bench.run_reference(Args())
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
            f.write(f"{t} {rate} {len(buf.getvalue())}\n")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank_and_print_once(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [open(tmp_path / f"rank{r}.txt").read().split() for r in range(world)]
    for t, rate, printed in res:
        assert float(t) == 2.5                       # the slower rank's time on every rank
        assert float(rate) == world * 1000.0 / 2.5   # units of all ranks over that time
    assert int(res[1][2]) == 0                       # rank 1 prints nothing in the reference arm
