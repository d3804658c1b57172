"""Batched multi-shot launches (wave_batch_*): shots with uneven grids stepped
together must give exactly the seismograms of the same shots run one by one
through the single-shot generic kernels, and match the FP64 oracle.

The reference runs shots in separate MPI shot domains (Simulation.cpp:116-121,
339-369); here they share each launch.
"""
import numpy as np
import pytest

from test_gpu_parity import TOL, make_case, rel, to_wave_cfg

pytestmark = pytest.mark.gpu

BATCHES = [
    # (eq, dim, order, fs, boundary, grids)
    ("elastic", 2, 4, 1, 2, [(90, 70, 1), (64, 50, 1), (100, 46, 1)]),
    ("tmem", 2, 6, 0, 2, [(80, 60, 1), (72, 72, 1)]),
    ("acoustic", 3, 4, 0, 1, [(40, 30, 28), (33, 36, 30)]),
    ("viscoelastic", 2, 4, 0, 2, [(70, 50, 1), (60, 64, 1)]),
]


def _eq_name(wave, cfg):
    return [k for k, v in wave.EQUATIONS.items() if v == cfg.equation][0]


@pytest.mark.parametrize("eq,dim,order,fs,boundary,grids", BATCHES)
def test_batch_equals_single_shots_and_oracle(eq, dim, order, fs, boundary, grids, wave, refcpu):
    cases = [make_case(refcpu, eq, dim, order, fs, boundary, dims=g, seed=k) for k, g in enumerate(grids)]
    cfgs = [to_wave_cfg(wave, c[0]) for c in cases]
    singles = []
    for wc, (cfg, model, sidx, stype, sig, ridx, rtype) in zip(cfgs, cases):
        m32 = {k: v.astype(np.float32) for k, v in model.items()}
        singles.append(wave.simulate(wc, m32, sidx, stype, sig.astype(np.float32), ridx, rtype, kernel_path=1))

    b = wave.Batch(cfgs)
    try:
        for shot, (cfg, model, sidx, stype, sig, ridx, rtype) in zip(b.shots, cases):
            shot.prepareForModelling({k: v.astype(np.float32) for k, v in model.items()})
            shot.setSources(sidx, stype, sig.astype(np.float32))
            shot.setReceivers(ridx, rtype)
        b.run(0, b.nt)
        batched = [shot.seismograms() for shot in b.shots]
        per_step = 4 if boundary == 1 else 3
        assert b.launch_count() == per_step * b.nt
    finally:
        b.close()

    for k, (one, many) in enumerate(zip(singles, batched)):
        assert np.abs(one).max() > 0
        assert np.array_equal(one, many), f"shot {k}: batched differs from single-shot run"

    cfg, model, sidx, stype, sig, ridx, rtype = cases[0]
    o = refcpu.Oracle(cfg, model, sidx, stype, sig, ridx, rtype, dtype=np.float64)
    ref = o.run()
    o.close()
    assert rel(batched[0], ref) < TOL


def test_batch_split_time_range_equals_one_call(wave, refcpu):
    cases = [make_case(refcpu, "acoustic", 2, 8, 0, 2, dims=g, seed=k) for k, g in enumerate([(90, 70, 1), (50, 80, 1)])]
    outs = []
    for split in (False, True):
        b = wave.Batch([to_wave_cfg(wave, c[0]) for c in cases])
        try:
            for shot, (cfg, model, sidx, stype, sig, ridx, rtype) in zip(b.shots, cases):
                shot.prepareForModelling({k: v.astype(np.float32) for k, v in model.items()})
                shot.setSources(sidx, stype, sig.astype(np.float32))
                shot.setReceivers(ridx, rtype)
            if split:
                for t0, t1 in ((0, 7), (7, 40), (40, 41), (41, b.nt)):
                    b.run(t0, t1)
            else:
                b.run(0, b.nt)
            outs.append([s.seismograms() for s in b.shots])
        finally:
            b.close()
    for a, c in zip(*outs):
        assert np.array_equal(a, c)


def test_batch_rejects_mixed_equations(wave, refcpu):
    a = make_case(refcpu, "acoustic", 2, 4)[0]
    e = make_case(refcpu, "elastic", 2, 4)[0]
    with pytest.raises(wave.WaveError):
        wave.Batch([to_wave_cfg(wave, a), to_wave_cfg(wave, e)])


def _tm_batch(wave, refcpu, seeds=(0, 1, 2), grids=((80, 60, 1), (72, 72, 1), (100, 40, 1))):
    cases = [make_case(refcpu, "tmem", 2, 4, 0, 2, dims=g, seed=k) for k, g in zip(seeds, grids)]
    return cases, [to_wave_cfg(wave, c[0]) for c in cases]


def _run_batch(wave, cases, cfgs, schedule=None, steps=None):
    b = wave.Batch(cfgs)
    try:
        if schedule is not None:
            b.set_schedule(*schedule)
        for shot, (cfg, model, sidx, stype, sig, ridx, rtype) in zip(b.shots, cases):
            shot.prepareForModelling({k: v.astype(np.float32) for k, v in model.items()})
            shot.setSources(sidx, stype, sig.astype(np.float32))
            shot.setReceivers(ridx, rtype)
        b.run(0, steps or b.nt)
        return [s.seismograms() for s in b.shots], b.schedule()
    finally:
        b.close()


@pytest.mark.parametrize("schedule", [(64, 8, 0), (32, 16, 2), (64, 64, 1), (32, 8, 8), (96, 24, 4)])
def test_every_batch_schedule_gives_the_same_bits(wave, refcpu, schedule):
    """Tile shape and persistent blocks per SM change only which block updates
    a point, not the arithmetic: bit-identical seismograms."""
    cases, cfgs = _tm_batch(wave, refcpu)
    ref, s0 = _run_batch(wave, cases, cfgs, (32, 32, 0))
    got, s1 = _run_batch(wave, cases, cfgs, schedule)
    assert s0["source"] == "set" and (s1["tile_cols"], s1["tile_rows"]) == schedule[:2]
    for a, c in zip(ref, got):
        assert np.abs(a).max() > 0 and np.array_equal(a, c)


def test_autotuner_times_once_then_uses_its_cache(wave, refcpu):
    """The first unstepped batch of a kind is timed over the candidate
    schedules and reset; the result equals a run with the schedule fixed; a
    second batch of the same kind takes the schedule from the cache."""
    cases, cfgs = _tm_batch(wave, refcpu, seeds=(5, 6), grids=((150, 90, 1), (130, 110, 1)))
    tuned, s1 = _run_batch(wave, cases, cfgs)
    assert s1["source"] in ("autotuned", "cache")
    assert s1["tile_cols"] in (32, 64) and s1["tile_rows"] in (8, 16, 32, 64) and s1["blocks_per_sm"] in (0, 1, 2, 4, 8)
    again, s2 = _run_batch(wave, cases, cfgs)
    assert s2["source"] == "cache" and {k: s2[k] for k in ("tile_cols", "tile_rows")} == \
        {k: s1[k] for k in ("tile_cols", "tile_rows")}
    fixed, _ = _run_batch(wave, cases, cfgs, (32, 32, 0))
    for a, b_, c in zip(tuned, again, fixed):
        assert np.array_equal(a, c) and np.array_equal(b_, c)


@pytest.mark.parametrize("schedule", [(32, 8, 0), (64, 16, 0), (64, 32, 2)])
def test_tmz_interior_tiles_equal_single_shots(wave, refcpu, schedule):
    """Lossless TMz: tiles wholly inside a shot's interior (away from the
    operators' edge bands and the CPML slabs) take the batched kernels' lean
    path; the batch still gives the single-shot generic kernels' bits."""
    grids = ((220, 130, 1), (180, 150, 1), (260, 90, 1))
    cases, cfgs = _tm_batch(wave, refcpu, seeds=(7, 8, 9), grids=grids)
    singles = []
    for wc, (cfg, model, sidx, stype, sig, ridx, rtype) in zip(cfgs, cases):
        m32 = {k: v.astype(np.float32) for k, v in model.items()}
        singles.append(wave.simulate(wc, m32, sidx, stype, sig.astype(np.float32), ridx, rtype, kernel_path=1))
    got, s = _run_batch(wave, cases, cfgs, schedule)
    assert (s["tile_cols"], s["tile_rows"]) == schedule[:2]
    for one, many in zip(singles, got):
        assert np.abs(one).max() > 0 and np.array_equal(one, many)
