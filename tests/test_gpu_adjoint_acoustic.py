"""Adjoint gradient of the acoustic misfit in 2-D and 3-D
(wave_adjoint_gradient on an acoustic handle: dJ/dvp, dJ/drho; the vs output
is zero) against the FP64 oracle's own discrete adjoint
(oracle/adjoint_impl.hpp, AcousticAdjoint, pinned to FP64 finite differences
at 1e-6 in tests/test_oracle_adjoint.py), with CPML, ABS, no boundary and the
free surface, sparse and stencil operators, P and VY sources, P / VX / VY
receivers; the checkpoint interval does not change the result and the batched
entry equals the single-shot one bit for bit. The forwards differentiated are
FD2Dacoustic::run (ForwardSolver2Dacoustic.cpp:91-194) and FD3Dacoustic::run
(ForwardSolver3Dacoustic.cpp:91-233); the reference has no adjoint.

Gate: relative L2 <= 1e-4 per parameter (FP32 CUDA adjoint vs FP64)."""
import ctypes

import numpy as np
import pytest

from test_oracle_adjoint import ac_case

pytestmark = pytest.mark.gpu
GRAD_TOL = 1e-4


def _wave_cfg(wave, ocfg):
    c = wave.WaveConfig()
    ctypes.memmove(ctypes.byref(c), ctypes.byref(ocfg), ctypes.sizeof(c))
    return c


def _solver(wave, cfg, model, acq):
    s = wave.Factory.Create("3D" if cfg.dimension == 3 else "2D", "acoustic").initForwardSolver(cfg)
    s.prepareForModelling(model)
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    return s


def _survey(wave, refcpu, dim, fs, boundary, stencil, reduce, order=4):
    size = dict(NX=40, NY=32, NZ=36, nt=260) if dim == 3 else dict(NX=80, NY=64, nt=500)
    ocfg, model, acq = ac_case(refcpu, dim, fs, boundary, stencil, reduce, order=order, **size)
    cfg = _wave_cfg(wave, ocfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    n = m32["vp"].size
    blob = np.exp(-np.linspace(-3, 3, n) ** 2)
    true = dict(m32)
    true["vp"] = (m32["vp"] * (1 + 0.05 * blob)).astype(np.float32)
    true["rho"] = (m32["rho"] * (1 - 0.03 * blob)).astype(np.float32)
    acq32 = (acq[0], acq[1], acq[2].astype(np.float32), acq[3], acq[4])
    s = _solver(wave, cfg, true, acq32)
    s.run(0, s.nt)
    # 0.8 x the true model's data: the residual holds part of the direct wave
    dobs = (0.8 * s.seismograms()).astype(np.float32)
    s.close()
    return ocfg, cfg, m32, acq32, dobs


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("dim,fs,boundary,stencil,reduce,order", [(2, 0, 2, 0, 0, 4), (2, 1, 1, 1, 0, 8), (2, 1, 0, 0, 1, 2),
                                                                  (3, 0, 2, 0, 0, 4), (3, 1, 1, 0, 1, 6), (2, 2, 2, 0, 0, 4),
                                                                  (3, 2, 1, 0, 1, 4)])
def test_acoustic_adjoint_matches_the_fp64_oracle_gradient(wave, refcpu, dim, fs, boundary, stencil, reduce, order):
    ocfg, cfg, m32, acq, dobs = _survey(wave, refcpu, dim, fs, boundary, stencil, reduce, order)
    s = _solver(wave, cfg, m32, acq)
    J, gvp, gvs, grho = s.adjoint_gradient(dobs, checkpoint_every=45)
    s.close()
    o = refcpu.Oracle(ocfg, {k: v.astype(np.float64) for k, v in m32.items()}, acq[0], acq[1], acq[2].astype(np.float64),
                      acq[3], acq[4], dtype=np.float64)
    J64, rvp, _, rrho = o.adjoint_gradient(dobs.astype(np.float64), checkpoint_every=45)
    o.close()
    errs = [_rel(gvp, rvp), _rel(grho, rrho)]
    print(f"acoustic adjoint {dim}-D fs={fs} boundary={boundary} stencil={stencil} reduce={reduce} order={order}: misfit "
          f"{J:.6e} vs FP64 {J64:.6e}; gradient rel L2 vp {errs[0]:.2e} rho {errs[1]:.2e}")
    assert not np.any(gvs)
    assert J > 0 and abs(J - J64) <= 1e-4 * J64
    assert max(errs) <= GRAD_TOL


@pytest.mark.parametrize("dim", [2, 3])
def test_acoustic_checkpoint_interval_and_batch(wave, refcpu, dim):
    ocfg, cfg, m32, acq, dobs = _survey(wave, refcpu, dim, 1, 2, 0, 0)
    nt = dobs.shape[1]
    out = []
    for K in (13, nt + 3):
        s = _solver(wave, cfg, m32, acq)
        out.append(s.adjoint_gradient(dobs, checkpoint_every=K))
        s.close()
    assert abs(out[1][0] - out[0][0]) <= 1e-12 * abs(out[0][0])
    for a, b in zip(out[1][1:], out[0][1:]):
        assert np.array_equal(a, b)
    acqs, obs, single = [], [], []
    for k in range(2):
        a = (acq[0] + 3 * k, acq[1], acq[2], acq[3], acq[4])
        acqs.append(a)
        s = _solver(wave, cfg, m32, a)
        s.run(0, s.nt)
        obs.append((0.8 * s.seismograms()).astype(np.float32))
        s.close()
        s = _solver(wave, cfg, m32, a)
        single.append(s.adjoint_gradient(obs[-1], checkpoint_every=40))
        s.close()
    b = wave.Batch([cfg] * 2)
    try:
        for shot, a in zip(b.shots, acqs):
            shot.prepareForModelling(m32)
            shot.setSources(*a[:3])
            shot.setReceivers(*a[3:])
        mis, gvp, gvs, grho = b.adjoint_gradient(obs, checkpoint_every=40, sum_shots=False)
    finally:
        b.close()
    for k in range(2):
        assert abs(mis[k] - single[k][0]) <= 1e-12 * abs(single[k][0])
        for got, want in zip((gvp[k], grho[k]), (single[k][1], single[k][3])):
            assert np.abs(want).max() > 0 and np.array_equal(got, want)
