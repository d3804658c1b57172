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


def _load_wave():
    sys.path.insert(0, ROOT)
    import __graft_entry__ as g
    return g.load_package()


def test_shot_range_is_the_reference_block_distribution():
    """blockDistribution(numshots, commInterShot) (Simulation.cpp:339-345):
    contiguous blocks of ceil(n / p) shots, every shot in exactly one block."""
    wave = _load_wave()
    for n in (0, 1, 5, 32, 33, 128):
        for p in (1, 2, 3, 4, 8):
            blocks = [wave.shot_range(n, r, p) for r in range(p)]
            covered = [k for lb, ub in blocks for k in range(lb, ub)]
            assert covered == list(range(n)), (n, p, blocks)
            b = (n + p - 1) // p
            assert all(ub - lb <= b for lb, ub in blocks)
    with pytest.raises(wave.WaveError):
        wave.shot_range(4, 2, 2)


def _domains_main(rank, world, port, out_dir, num_shots):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import numpy as np
    import torch.distributed as dist
    wave = _load_wave()
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seen = []

        # per-shot partial results: a "gradient" and a "misfit" that depend on the shot,
        # as the batched adjoint's summed gradient of a block would
        def compute(lb, ub):
            seen.extend(range(lb, ub))
            g = np.zeros(7, np.float64)
            mis = np.zeros(1, np.float64)
            for k in range(lb, ub):
                g += (k + 1) * np.arange(7)
                mis += 0.5 * k * k
            return mis, g

        mis, g = wave.run_shot_domains(num_shots, compute)
        np.save(os.path.join(out_dir, f"dom{rank}.npy"), np.concatenate([mis, g, [len(seen)], seen]))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("num_shots", [5, 1])
def test_two_gloo_ranks_split_the_shots_and_sum_their_results(tmp_path, num_shots):
    """The N > 1 shot-domain path: each rank computes its own block of shots
    (no collective inside), then one sum; with one shot the second rank's
    block is empty and contributes zeros."""
    pytest.importorskip("torch")
    import numpy as np
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_domains_main, args=(world, _free_port(), str(tmp_path), num_shots), nprocs=world, join=True)
    want_g = sum((k + 1) * np.arange(7) for k in range(num_shots))
    want_m = sum(0.5 * k * k for k in range(num_shots))
    blocks = []
    for r in range(world):
        a = np.load(tmp_path / f"dom{r}.npy")
        assert a[0] == want_m and np.array_equal(a[1:8], want_g)      # every rank holds the sums
        n = int(a[8])
        blocks.append([int(v) for v in a[9:9 + n]])
    assert blocks[0] + blocks[1] == list(range(num_shots))            # disjoint, contiguous, complete
    assert len(blocks[0]) == (num_shots + 1) // 2
