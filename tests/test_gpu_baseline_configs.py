"""Parity on the benchmarked workloads themselves, through the code paths the
benchmark times: the GPU seismograms (and wavefields) against the FP64 oracle
refcpu<double>, and the oracle's FP32 run refcpu<float> (the reference
formulation in single precision, the stand-in for the reference's own FP32
CPU run) against the same FP64 oracle.

Gate: relative L2 over all traces and samples <= 1e-4 for both
(spec tolerance; Test_CompareSeismogram.cpp:57-88 is the reference's
own seismogram gate style). Each test prints the measured errors, so the
FP32-vs-FP64 drift per workload is in the test log.

* 2-D acoustic 400 x 200, order 4, 20-pt CPML, all NT = 2000 steps, 100
  pressure receivers, sparse and stencil operators.
* 3-D elastic 256^3, order 8, free surface + 20-pt CPML, 6,000 surface traces,
  automatic kernel choice (the two-point streaming kernels on GB300), the
  first 250 steps (the oracle needs ~0.5 s per FP64 step at this size), and
  the nine wavefields after them.
* The same 3-D elastic physics on a 96^3 grid (layers of 12 cells) for all
  NT = 3000 steps: FP32 drift over the full record, with the CPML and the
  free surface reached by the wave. This run uses the zero-padded edge rows
  (edgeOrderReduction = 0): with the current edge-order reduction the
  reference formulation itself grows without bound on this heterogeneous
  model after ~1500 steps, in FP64 as in FP32 (tests/test_oracle_stability.py),
  so no precision comparison is meaningful there.
* 3-D visco-elastic, order 4, L = 2 (Qp 80, Qs 50 by the tau-method), 20-pt
  CPML on a 128 x 64 x 128 sub-grid of the 512 x 256 x 512 workload, 800 steps.
* Batched 2-D TMz: 4 of the 128 shots of the batched workload at full
  NT = 3000, run through the batch API.
"""
import os

import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu
TOL = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def oracle_cfg(refcpu, kw):
    return refcpu.make_config(**kw)


def oracle_run(refcpu, kw, model, acq, steps, dtype, fields=()):
    refcpu.set_threads(os.cpu_count() or 1)
    o = refcpu.Oracle(oracle_cfg(refcpu, kw), {k: np.asarray(v, np.float64) for k, v in model.items()}, acq[0], acq[1],
                      np.asarray(acq[2], np.float64), acq[3], acq[4], dtype=dtype)
    o.step(0, steps)
    seis = o.seismograms()[:, :steps]
    f = {n: o.field(n) for n in fields}
    o.close()
    return seis, f


@pytest.mark.parametrize("stencil", [0, 1])
def test_acoustic_400x200_whole_job(wave, refcpu, stencil):
    kw = dict(bench.AC2_KW, useStencilMatrix=stencil)
    cfg = wave.WaveConfig.make(**kw)
    model = bench.ac2_model()
    s = wave.Factory.Create("2D", "acoustic").initForwardSolver(cfg)
    acq = bench.ac2_acq(s.nt, cfg.DT)
    s.prepareForModelling(model)
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    nt = s.nt
    s.run(0, nt)
    gpu = s.seismograms()
    s.close()
    ref64, _ = oracle_run(refcpu, kw, model, acq, nt, np.float64)
    ref32, _ = oracle_run(refcpu, kw, model, acq, nt, np.float32)
    e_gpu, e32 = rel(gpu, ref64), rel(ref32, ref64)
    print(f"2-D acoustic 400x200 stencil={stencil} NT={nt}: GPU vs FP64 {e_gpu:.3e}, refcpu<float> vs FP64 {e32:.3e}")
    assert nt == 2000 and np.abs(ref64).max() > 0
    assert e_gpu < TOL and e32 < TOL


def test_elastic_256_cube_first_steps_and_wavefields(wave, refcpu):
    steps = 250
    cfg = wave.WaveConfig.make(**bench.CONFIG_KW)
    model = bench.make_model()
    s = wave.Factory.Create("3D", "elastic").initForwardSolver(cfg)
    acq = bench.make_acquisition(s.nt, cfg.DT, wave.wavelet)
    s.prepareForModelling(model)
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    passes = s.streaming_passes()
    s.run(0, steps)
    gpu = s.seismograms()[:, :steps]
    gfields = {f: s.field(f) for f in bench.FIELDS_3D}
    s.close()
    assert gpu.shape[0] == 6000
    ref64, f64 = oracle_run(refcpu, bench.CONFIG_KW, model, acq, steps, np.float64, bench.FIELDS_3D)
    ref32, f32 = oracle_run(refcpu, bench.CONFIG_KW, model, acq, steps, np.float32, bench.FIELDS_3D)
    cat = lambda d: np.concatenate([np.asarray(d[f], np.float64) for f in bench.FIELDS_3D])
    e_gpu, e32 = rel(gpu, ref64), rel(ref32, ref64)
    ef_gpu, ef32 = rel(cat(gfields), cat(f64)), rel(cat(f32), cat(f64))
    print(f"3-D elastic 256^3 o8 FS+CPML, {steps} steps (kernel passes {passes:#x}): seismograms GPU vs FP64 {e_gpu:.3e}, "
          f"refcpu<float> vs FP64 {e32:.3e}; wavefields GPU {ef_gpu:.3e}, refcpu<float> {ef32:.3e}")
    assert np.abs(ref64).max() > 0
    assert e_gpu < TOL and e32 < TOL and ef_gpu < TOL and ef32 < TOL


def _elastic_cube_model(n, seed_layers=2, seed_pert=20260002):
    rng = np.random.default_rng(seed_layers)
    vpk = rng.uniform(1800.0, 4500.0, 8)
    vp = np.repeat(vpk, (n + 7) // 8)[:n, None, None] * np.ones((n, n, n))
    eps = 0.05 * np.clip(np.random.default_rng(seed_pert).standard_normal((n, n, n)), -1, 1)
    vp = (vp * (1 + eps)).astype(np.float32).reshape(-1)
    vs = (vp / 1.73).astype(np.float32)
    rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(np.float32)
    return dict(rho=rho, vp=vp, vs=vs)


def test_elastic_cube_full_record_drift(wave, refcpu):
    """The 256^3 workload's physics (order 8, free surface, 20-pt CPML, DT,
    NT = 3000, Ricker 10 Hz, surface receivers) on a 96^3 grid, every step,
    zero-padded edge rows: the FP32 drift over the whole record with the wave
    through the CPML."""
    n = 96
    kw = dict(bench.CONFIG_KW, NX=n, NY=n, NZ=n, edgeOrderReduction=0)
    cfg = wave.WaveConfig.make(**kw)
    model = _elastic_cube_model(n)
    nt = int(np.float32(np.float32(cfg.T) / np.float32(cfg.DT)) + np.float32(0.5))
    sidx = np.array([n // 2 + n * (n // 2 + n * 20)], np.int64)
    sig = wave.wavelet(1, nt, cfg.DT, 10.0, 1.0, 0.0)[None]
    xs = np.arange(4, n - 4, 6)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    base = (X + n * Z).reshape(-1).astype(np.int64)
    ridx = np.concatenate([base, base, base, base + n * n * 60])
    rtype = np.concatenate([np.full(base.size, t, np.int32) for t in (2, 3, 4, 1)])
    acq = (sidx, np.array([1], np.int32), sig, ridx, rtype)
    gpu = wave.simulate(cfg, model, *acq, kernel_path=3, expect_streaming=True)
    ref64, _ = oracle_run(refcpu, kw, model, acq, nt, np.float64)
    ref32, _ = oracle_run(refcpu, kw, model, acq, nt, np.float32)
    e_gpu, e32 = rel(gpu, ref64), rel(ref32, ref64)
    print(f"3-D elastic 96^3 o8 FS+CPML, all {nt} steps (two-point kernels): GPU vs FP64 {e_gpu:.3e}, "
          f"refcpu<float> vs FP64 {e32:.3e}")
    assert nt == 3000 and np.abs(ref64).max() > 0
    assert e_gpu < TOL and e32 < TOL


def test_viscoelastic_subgrid(wave, refcpu):
    torch = pytest.importorskip("torch")
    NX, NY, NZ, steps = 128, 64, 128, 800
    kw = dict(bench.VI3_KW, NX=NX, NY=NY, NZ=NZ)
    cfg = wave.WaveConfig.make(**kw)
    model = {k: v.cpu().numpy() for k, v in bench.vi3_model(NX, NY, NZ, "cuda").items()}
    s = wave.Factory.Create("3D", "viscoelastic").initForwardSolver(cfg)
    acq = bench.vi3_acq(NX, NY, NZ, s.nt, cfg.DT)
    s.prepareForModelling({k: torch.from_numpy(v).cuda() for k, v in model.items()})
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    s.run(0, steps)
    gpu = s.seismograms()[:, :steps]
    s.close()
    ref64, _ = oracle_run(refcpu, kw, model, acq, steps, np.float64)
    ref32, _ = oracle_run(refcpu, kw, model, acq, steps, np.float32)
    e_gpu, e32 = rel(gpu, ref64), rel(ref32, ref64)
    print(f"3-D visco-elastic 128x64x128 o4 L=2 CPML, {steps} steps: GPU vs FP64 {e_gpu:.3e}, "
          f"refcpu<float> vs FP64 {e32:.3e}")
    assert np.abs(ref64).max() > 0
    assert e_gpu < TOL and e32 < TOL


def test_batched_tmz_four_shots_full_record(wave, refcpu):
    torch = pytest.importorskip("torch")
    shots = bench.tm_shots(128)[:4]
    cfgs = [wave.WaveConfig.make(**bench.tm_cfg_kw(nx, ny)) for nx, ny, _ in shots]
    b = wave.Batch(cfgs)
    acqs = []
    for shot, (nx, ny, m) in zip(b.shots, shots):
        shot.prepareForModelling({k: torch.from_numpy(v).cuda() for k, v in m.items()})
        acq = bench.tm_acq(nx, shot.nt)
        acqs.append(acq)
        shot.setSources(*acq[:3])
        shot.setReceivers(*acq[3:])
    nt = b.shots[0].nt
    b.run(0, nt)
    gpu = [shot.seismograms() for shot in b.shots]
    b.close()
    assert nt == 3000
    for k, ((nx, ny, m), acq) in enumerate(zip(shots, acqs)):
        kw = bench.tm_cfg_kw(nx, ny)
        ref64, _ = oracle_run(refcpu, kw, m, acq, nt, np.float64)
        ref32, _ = oracle_run(refcpu, kw, m, acq, nt, np.float32)
        e_gpu, e32 = rel(gpu[k], ref64), rel(ref32, ref64)
        print(f"batched TMz shot {k} ({nx}x{ny}), all {nt} steps: GPU vs FP64 {e_gpu:.3e}, refcpu<float> vs FP64 {e32:.3e}")
        assert np.abs(ref64).max() > 0
        assert e_gpu < TOL and e32 < TOL
