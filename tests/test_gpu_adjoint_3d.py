"""Adjoint gradient of the 3-D elastic misfit (wave_adjoint_gradient on a 3-D
elastic handle: dJ/dvp, dJ/dvs, dJ/drho) against the FP64 oracle's own
discrete adjoint (oracle/adjoint_impl.hpp, ElasticAdjoint3D, pinned to FP64
finite differences at 1e-6 in tests/test_oracle_adjoint.py), with CPML, ABS,
no boundary and the free surface, sparse and stencil operators, orders 2-8,
P and VZ sources, P / VX / VY / VZ receivers; the checkpoint interval does not
change the result and the batched entry equals the single-shot one bit for
bit. The forward differentiated is FD3Delastic::run
(ForwardSolver3Delastic.cpp:120-414), run by the library's own forward
kernels (the TMA streaming ones where they apply); the reference has no
adjoint.

Gate: relative L2 <= 1e-4 per parameter (FP32 CUDA adjoint vs FP64)."""
import ctypes

import numpy as np
import pytest

from test_oracle_adjoint import el3_case

pytestmark = pytest.mark.gpu
GRAD_TOL = 1e-4


def _wave_cfg(wave, ocfg):
    c = wave.WaveConfig()
    ctypes.memmove(ctypes.byref(c), ctypes.byref(ocfg), ctypes.sizeof(c))
    return c


def _solver(wave, cfg, model, acq):
    s = wave.Factory.Create("3D", "elastic").initForwardSolver(cfg)
    s.prepareForModelling(model)
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    return s


def _survey(wave, refcpu, fs, boundary, stencil, reduce, order=4):
    ocfg, model, acq = el3_case(refcpu, fs, boundary, stencil, reduce, order=order, NX=40, NY=32, NZ=36, nt=260)
    cfg = _wave_cfg(wave, ocfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    y, z, x = np.mgrid[0:cfg.NY, 0:cfg.NZ, 0:cfg.NX]
    blob = np.exp(-((x - cfg.NX * 0.5) ** 2 + (y - cfg.NY * 0.55) ** 2 + (z - cfg.NZ * 0.5) ** 2) / 40.0).reshape(-1)
    true = dict(m32)
    true["vp"] = (m32["vp"] * (1 + 0.05 * blob)).astype(np.float32)
    true["vs"] = (m32["vs"] * (1 - 0.04 * blob)).astype(np.float32)
    true["rho"] = (m32["rho"] * (1 + 0.03 * blob)).astype(np.float32)
    acq32 = (acq[0], acq[1], acq[2].astype(np.float32), acq[3], acq[4])
    s = _solver(wave, cfg, true, acq32)
    s.run(0, s.nt)
    # 0.8 x the true model's data: the residual holds part of the direct wave
    # (well conditioned in FP32, as in the 2-D surveys)
    dobs = (0.8 * s.seismograms()).astype(np.float32)
    s.close()
    return ocfg, cfg, m32, acq32, dobs


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("fs,boundary,stencil,reduce,order", [(0, 2, 0, 0, 4), (1, 2, 0, 0, 8), (0, 1, 1, 0, 2),
                                                              (1, 0, 0, 1, 6), (1, 1, 0, 0, 4), (2, 2, 0, 0, 4)])
def test_elastic3d_adjoint_matches_the_fp64_oracle_gradient(wave, refcpu, fs, boundary, stencil, reduce, order):
    ocfg, cfg, m32, acq, dobs = _survey(wave, refcpu, fs, boundary, stencil, reduce, order)
    s = _solver(wave, cfg, m32, acq)
    J, gvp, gvs, grho = s.adjoint_gradient(dobs, checkpoint_every=45)
    s.close()
    o = refcpu.Oracle(ocfg, {k: v.astype(np.float64) for k, v in m32.items()}, acq[0], acq[1], acq[2].astype(np.float64),
                      acq[3], acq[4], dtype=np.float64)
    J64, rvp, rvs, rrho = o.adjoint_gradient(dobs.astype(np.float64), checkpoint_every=45)
    o.close()
    errs = [_rel(gvp, rvp), _rel(gvs, rvs), _rel(grho, rrho)]
    print(f"3-D elastic adjoint fs={fs} boundary={boundary} stencil={stencil} reduce={reduce} order={order}: misfit "
          f"{J:.6e} vs FP64 {J64:.6e}; gradient rel L2 vp {errs[0]:.2e} vs {errs[1]:.2e} rho {errs[2]:.2e}")
    assert J > 0 and abs(J - J64) <= 1e-4 * J64
    assert max(errs) <= GRAD_TOL


def test_elastic3d_checkpoint_interval_and_batch(wave, refcpu):
    """K = 9 and NT + 3 give the same gradient bit for bit; two shots in one
    batch equal their single-shot gradients bit for bit."""
    ocfg, cfg, m32, acq, dobs = _survey(wave, refcpu, 1, 2, 0, 0)
    nt = dobs.shape[1]
    out = []
    for K in (9, nt + 3):
        s = _solver(wave, cfg, m32, acq)
        out.append(s.adjoint_gradient(dobs, checkpoint_every=K))
        s.close()
    assert abs(out[1][0] - out[0][0]) <= 1e-12 * abs(out[0][0])
    for a, b in zip(out[1][1:], out[0][1:]):
        assert np.array_equal(a, b)
    acqs, obs, single = [], [], []
    for k in range(2):
        a = (acq[0] + 5 * k, acq[1], acq[2], acq[3], acq[4])
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
        for got, want in zip((gvp[k], gvs[k], grho[k]), single[k][1:]):
            assert np.abs(want).max() > 0 and np.array_equal(got, want)


@pytest.mark.parametrize("L,boundary,stencil,reduce,order,fs", [(1, 2, 0, 0, 4, 0), (2, 1, 0, 1, 6, 0), (2, 0, 1, 0, 2, 0),
                                                                (2, 2, 0, 0, 4, 1), (1, 1, 0, 1, 8, 1), (1, 2, 0, 0, 4, 2)])
def test_visco3d_adjoint_matches_the_fp64_oracle_gradient(wave, refcpu, L, boundary, stencil, reduce, order, fs):
    """3-D visco-elastic (FD3Dviscoelastic::run, ForwardSolver3Dviscoelastic.cpp:132-457): six memory
    variables per mechanism, vp / vs / rho gradients with the relaxation times fixed, against the
    oracle's FP64 adjoint (pinned to FP64 finite differences), with and without the mirror free
    surface (FreeSurface3Dviscoelastic.cpp: sxx, szz and their memory variables exchange with the
    horizontal strain sum and vyy)."""
    ocfg, model, acq = el3_case(refcpu, fs, boundary, stencil, reduce, order=order, NX=40, NY=32, NZ=36, nt=260, L=L)
    cfg = _wave_cfg(wave, ocfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    y, z, x = np.mgrid[0:cfg.NY, 0:cfg.NZ, 0:cfg.NX]
    blob = np.exp(-((x - cfg.NX * 0.5) ** 2 + (y - cfg.NY * 0.55) ** 2 + (z - cfg.NZ * 0.5) ** 2) / 40.0).reshape(-1)
    true = dict(m32)
    true["vp"] = (m32["vp"] * (1 + 0.05 * blob)).astype(np.float32)
    true["vs"] = (m32["vs"] * (1 - 0.04 * blob)).astype(np.float32)
    acq32 = (acq[0], acq[1], acq[2].astype(np.float32), acq[3], acq[4])

    def solver(model_):
        s = wave.Factory.Create("3D", "viscoelastic").initForwardSolver(cfg)
        s.prepareForModelling(model_)
        s.setSources(*acq32[:3])
        s.setReceivers(*acq32[3:])
        return s

    s = solver(true)
    s.run(0, s.nt)
    dobs = (0.8 * s.seismograms()).astype(np.float32)
    s.close()
    s = solver(m32)
    J, gvp, gvs, grho = s.adjoint_gradient(dobs, checkpoint_every=45)
    s.close()
    o = refcpu.Oracle(ocfg, {k: v.astype(np.float64) for k, v in m32.items()}, acq32[0], acq32[1],
                      acq32[2].astype(np.float64), acq32[3], acq32[4], dtype=np.float64)
    J64, rvp, rvs, rrho = o.adjoint_gradient(dobs.astype(np.float64), checkpoint_every=45)
    o.close()
    errs = [_rel(gvp, rvp), _rel(gvs, rvs), _rel(grho, rrho)]
    print(f"3-D visco adjoint L={L} fs={fs} boundary={boundary} stencil={stencil} reduce={reduce} order={order}: misfit {J:.6e} "
          f"vs FP64 {J64:.6e}; gradient rel L2 vp {errs[0]:.2e} vs {errs[1]:.2e} rho {errs[2]:.2e}")
    assert J > 0 and abs(J - J64) <= 1e-4 * J64
    assert max(errs) <= GRAD_TOL
