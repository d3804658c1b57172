"""Adjoint gradients of the lossless 2-D TMz and TEz and 3-D EM misfits
(wave_adjoint_gradient on a TMz / TEz handle: dJ/deps_r, dJ/dsigma, dJ/dmu_r)
against the FP64 oracle's own discrete adjoints (oracle/adjoint_impl.hpp,
TMAdjoint2D / TEAdjoint2D, pinned to FP64 finite differences at 1e-6 in
tests/test_oracle_adjoint.py), with CPML, ABS and no boundary, sparse and
stencil operators; the batched entry equals the single-shot one bit for bit.
The forwards differentiated are FD2Dtmem::run (ForwardSolver2Dtmem.cpp:
108-174) and FD2Demem::run (ForwardSolver2Demem.cpp:112-185); the reference
has no adjoint.

Gate: relative L2 <= 1e-4 per parameter (FP32 CUDA adjoint vs FP64)."""
import ctypes

import numpy as np
import pytest

from test_oracle_adjoint import em3_case, te_case, tm_case

pytestmark = pytest.mark.gpu
GRAD_TOL = 1e-4


def _wave_cfg(wave, ocfg):
    c = wave.WaveConfig()
    ctypes.memmove(ctypes.byref(c), ctypes.byref(ocfg), ctypes.sizeof(c))
    return c


def _survey(wave, refcpu, boundary, stencil, reduce, L=0):
    ocfg, model, acq = tm_case(refcpu, boundary, stencil, reduce, NX=72, NY=60, nt=400, L=L)
    cfg = _wave_cfg(wave, ocfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    yy, xx = np.mgrid[0:cfg.NY, 0:cfg.NX]
    blob = np.exp(-((xx - cfg.NX * 0.5) ** 2 + (yy - cfg.NY * 0.45) ** 2) / 60.0).reshape(-1)
    true = dict(m32)
    true["eps_r"] = (m32["eps_r"] * (1 + 0.1 * blob)).astype(np.float32)
    true["sigma"] = (m32["sigma"] * (1 + 0.5 * blob)).astype(np.float32)
    acq32 = (acq[0], acq[1], acq[2].astype(np.float32), acq[3], acq[4])
    s = wave.Factory.Create("2D", _tm_key(cfg)).initForwardSolver(cfg)
    s.prepareForModelling(true)
    s.setSources(*acq32[:3])
    s.setReceivers(*acq32[3:])
    s.run(0, s.nt)
    # observed data scaled so that the residual is a large part of the signal:
    # the TMz forward's FP32 rounding (this survey runs at a small Courant
    # number) then stays far below the residual the adjoint propagates
    dobs = (0.6 * s.seismograms()).astype(np.float32)
    s.close()
    return ocfg, cfg, m32, acq32, dobs


def _te_key(cfg):
    return "viscoemem" if cfg.numRelaxationMechanisms > 0 else "emem"


def _tm_key(cfg):
    return "viscotmem" if cfg.numRelaxationMechanisms > 0 else "tmem"


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("boundary,stencil,reduce,L", [(2, 0, 0, 0), (0, 1, 0, 0), (1, 0, 0, 0), (2, 0, 1, 0), (2, 0, 0, 1),
                                                      (1, 1, 0, 2)])
def test_tmz_adjoint_matches_the_fp64_oracle_gradient(wave, refcpu, boundary, stencil, reduce, L):
    """L > 0: visco-TMz (FD2Dviscotmem::run, ForwardSolver2Dviscotmem.cpp:130-205), tau_eps and
    tau_sigma fixed."""
    ocfg, cfg, m32, acq, dobs = _survey(wave, refcpu, boundary, stencil, reduce, L)
    s = wave.Factory.Create("2D", _tm_key(cfg)).initForwardSolver(cfg)
    s.prepareForModelling(m32)
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    J, ge, gs, gm = s.adjoint_gradient(dobs, checkpoint_every=45)
    s.close()
    o = refcpu.Oracle(ocfg, {k: v.astype(np.float64) for k, v in m32.items()}, acq[0], acq[1], acq[2].astype(np.float64),
                      acq[3], acq[4], dtype=np.float64)
    J64, re, rs, rm = o.adjoint_gradient(dobs.astype(np.float64), checkpoint_every=45)
    o.close()
    errs = [_rel(a, b) for a, b in ((ge, re), (gs, rs), (gm, rm))]
    print(f"TMz adjoint L={L} boundary={boundary} stencil={stencil} reduce={reduce}: misfit {J:.6e} vs FP64 {J64:.6e}; "
          f"gradient rel L2 eps_r {errs[0]:.2e} sigma {errs[1]:.2e} mu_r {errs[2]:.2e}")
    assert J > 0 and abs(J - J64) <= 1e-4 * J64
    assert max(errs) <= GRAD_TOL


def test_tmz_batched_adjoint_equals_single_shots(wave, refcpu):
    ocfg, cfg, m32, acq, dobs0 = _survey(wave, refcpu, 2, 0, 0)
    acqs, dobs, single = [], [], []
    for k in range(2):
        sidx = np.array([acq[0][0] + 9 * k], np.int64)
        a = (sidx, acq[1], acq[2], acq[3], acq[4])
        acqs.append(a)
        s = wave.Factory.Create("2D", _tm_key(cfg)).initForwardSolver(cfg)
        s.prepareForModelling(m32)
        s.setSources(*a[:3])
        s.setReceivers(*a[3:])
        s.run(0, s.nt)
        dobs.append(0.8 * s.seismograms())
        single.append(s.adjoint_gradient(dobs[-1], checkpoint_every=30))
        s.close()
    b = wave.Batch([cfg] * 2)
    try:
        for shot, a in zip(b.shots, acqs):
            shot.prepareForModelling(m32)
            shot.setSources(*a[:3])
            shot.setReceivers(*a[3:])
        mis, g1, g2, g3 = b.adjoint_gradient(dobs, checkpoint_every=30, sum_shots=False)
    finally:
        b.close()
    for k in range(2):
        assert abs(mis[k] - single[k][0]) <= 1e-12 * abs(single[k][0])
        for got, want in zip((g1[k], g2[k], g3[k]), single[k][1:]):
            assert np.abs(want).max() > 0 and np.array_equal(got, want)


def test_tmz_adjoint_rejects_other_receiver_components(wave, refcpu):
    ocfg, cfg, m32, acq, dobs = _survey(wave, refcpu, 0, 0, 0)
    s = wave.Factory.Create("2D", _tm_key(cfg)).initForwardSolver(cfg)
    s.prepareForModelling(m32)
    s.setSources(*acq[:3])
    with pytest.raises(wave.WaveError) as e:
        # an Ex receiver on a TMz grid: refused when set, or by the adjoint
        s.setReceivers(acq[3][:2], np.array([1, 2], np.int32))
        s.adjoint_gradient(np.zeros((2, s.nt), np.float32))
    assert e.value.code in (wave.WAVE_ERR_UNSUPPORTED, wave.WAVE_ERR_ARG)
    s.close()


def _te_survey(wave, refcpu, boundary, stencil, reduce, order=4, L=0):
    ocfg, model, acq = te_case(refcpu, boundary, stencil, reduce, order=order, NX=72, NY=60, nt=400, L=L)
    cfg = _wave_cfg(wave, ocfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    yy, xx = np.mgrid[0:cfg.NY, 0:cfg.NX]
    blob = np.exp(-((xx - cfg.NX * 0.5) ** 2 + (yy - cfg.NY * 0.45) ** 2) / 60.0).reshape(-1)
    true = dict(m32)
    true["eps_r"] = (m32["eps_r"] * (1 + 0.1 * blob)).astype(np.float32)
    true["sigma"] = (m32["sigma"] * (1 + 0.5 * blob)).astype(np.float32)
    true["mu_r"] = (m32["mu_r"] * (1 + 0.05 * blob)).astype(np.float32)
    acq32 = (acq[0], acq[1], acq[2].astype(np.float32), acq[3], acq[4])
    s = wave.Factory.Create("2D", _te_key(cfg)).initForwardSolver(cfg)
    s.prepareForModelling(true)
    s.setSources(*acq32[:3])
    s.setReceivers(*acq32[3:])
    s.run(0, s.nt)
    # scaled as in the TMz survey: the residual holds part of the direct wave
    dobs = (0.6 * s.seismograms()).astype(np.float32)
    s.close()
    return ocfg, cfg, m32, acq32, dobs


@pytest.mark.parametrize("boundary,stencil,reduce,order,L", [(2, 0, 0, 4, 0), (0, 1, 0, 2, 0), (1, 0, 0, 6, 0), (2, 0, 1, 8, 0),
                                                             (2, 0, 0, 4, 1), (1, 1, 0, 6, 2)])
def test_tez_adjoint_matches_the_fp64_oracle_gradient(wave, refcpu, boundary, stencil, reduce, order, L):
    """Ey and Hz sources (the Hz source exercises the re-formed pre-taper hz),
    Ex, Ey and Hz receivers; L > 0: visco-TEz (FD2Dviscoemem::run,
    ForwardSolver2Dviscoemem.cpp:142-228), tau_eps and tau_sigma fixed."""
    ocfg, cfg, m32, acq, dobs = _te_survey(wave, refcpu, boundary, stencil, reduce, order, L)
    s = wave.Factory.Create("2D", _te_key(cfg)).initForwardSolver(cfg)
    s.prepareForModelling(m32)
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    J, ge, gs, gm = s.adjoint_gradient(dobs, checkpoint_every=45)
    s.close()
    o = refcpu.Oracle(ocfg, {k: v.astype(np.float64) for k, v in m32.items()}, acq[0], acq[1], acq[2].astype(np.float64),
                      acq[3], acq[4], dtype=np.float64)
    J64, re, rs, rm = o.adjoint_gradient(dobs.astype(np.float64), checkpoint_every=45)
    o.close()
    errs = [_rel(a, b) for a, b in ((ge, re), (gs, rs), (gm, rm))]
    print(f"TEz adjoint L={L} boundary={boundary} stencil={stencil} reduce={reduce} order={order}: misfit {J:.6e} vs FP64 "
          f"{J64:.6e}; gradient rel L2 eps_r {errs[0]:.2e} sigma {errs[1]:.2e} mu_r {errs[2]:.2e}")
    assert J > 0 and abs(J - J64) <= 1e-4 * J64
    assert max(errs) <= GRAD_TOL


def test_tez_batched_adjoint_equals_single_shots(wave, refcpu):
    ocfg, cfg, m32, acq, dobs0 = _te_survey(wave, refcpu, 1, 0, 0)
    acqs, dobs, single = [], [], []
    for k in range(2):
        a = (acq[0] + 7 * k, acq[1], acq[2], acq[3], acq[4])
        acqs.append(a)
        s = wave.Factory.Create("2D", _te_key(cfg)).initForwardSolver(cfg)
        s.prepareForModelling(m32)
        s.setSources(*a[:3])
        s.setReceivers(*a[3:])
        s.run(0, s.nt)
        dobs.append(0.8 * s.seismograms())
        single.append(s.adjoint_gradient(dobs[-1], checkpoint_every=30))
        s.close()
    b = wave.Batch([cfg] * 2)
    try:
        for shot, a in zip(b.shots, acqs):
            shot.prepareForModelling(m32)
            shot.setSources(*a[:3])
            shot.setReceivers(*a[3:])
        mis, g1, g2, g3 = b.adjoint_gradient(dobs, checkpoint_every=30, sum_shots=False)
    finally:
        b.close()
    for k in range(2):
        assert abs(mis[k] - single[k][0]) <= 1e-12 * abs(single[k][0])
        for got, want in zip((g1[k], g2[k], g3[k]), single[k][1:]):
            assert np.abs(want).max() > 0 and np.array_equal(got, want)


@pytest.mark.parametrize("boundary,stencil,reduce,order,L", [(2, 0, 0, 4, 0), (1, 1, 0, 2, 0), (0, 0, 1, 6, 0), (2, 0, 0, 4, 1),
                                                             (1, 0, 1, 2, 2)])
def test_em3d_adjoint_matches_the_fp64_oracle_gradient(wave, refcpu, boundary, stencil, reduce, order, L):
    """3-D EM (FD3Demem::run, ForwardSolver3Demem.cpp:119-237; L > 0: FD3Dviscoemem::run,
    ForwardSolver3Dviscoemem.cpp:161-309 with the taus fixed; Ez and Hz sources, Ez / Ex / Ey / Hz
    receivers) against the oracle's FP64 3-D EM adjoint (EM3Adjoint, pinned to FP64 finite
    differences at 1e-6)."""
    ocfg, model, acq = em3_case(refcpu, boundary, stencil, reduce, order=order, NX=40, NY=32, NZ=36, nt=260, L=L)
    cfg = _wave_cfg(wave, ocfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    y, z, x = np.mgrid[0:cfg.NY, 0:cfg.NZ, 0:cfg.NX]
    blob = np.exp(-((x - cfg.NX * 0.5) ** 2 + (y - cfg.NY * 0.5) ** 2 + (z - cfg.NZ * 0.5) ** 2) / 40.0).reshape(-1)
    true = dict(m32)
    true["eps_r"] = (m32["eps_r"] * (1 + 0.1 * blob)).astype(np.float32)
    true["sigma"] = (m32["sigma"] * (1 + 0.5 * blob)).astype(np.float32)
    acq32 = (acq[0], acq[1], acq[2].astype(np.float32), acq[3], acq[4])

    def solver(model_):
        s = wave.Factory.Create("3D", "viscoemem" if L else "emem").initForwardSolver(cfg)
        s.prepareForModelling(model_)
        s.setSources(*acq32[:3])
        s.setReceivers(*acq32[3:])
        return s

    s = solver(true)
    s.run(0, s.nt)
    dobs = (0.6 * s.seismograms()).astype(np.float32)
    s.close()
    s = solver(m32)
    J, ge, gs, gm = s.adjoint_gradient(dobs, checkpoint_every=45)
    s.close()
    o = refcpu.Oracle(ocfg, {k: v.astype(np.float64) for k, v in m32.items()}, acq32[0], acq32[1],
                      acq32[2].astype(np.float64), acq32[3], acq32[4], dtype=np.float64)
    J64, re, rs, rm = o.adjoint_gradient(dobs.astype(np.float64), checkpoint_every=45)
    o.close()
    errs = [_rel(a, b) for a, b in ((ge, re), (gs, rs), (gm, rm))]
    print(f"3-D EM adjoint L={L} boundary={boundary} stencil={stencil} reduce={reduce} order={order}: misfit {J:.6e} vs FP64 "
          f"{J64:.6e}; gradient rel L2 eps_r {errs[0]:.2e} sigma {errs[1]:.2e} mu_r {errs[2]:.2e}")
    assert J > 0 and abs(J - J64) <= 1e-4 * J64
    assert max(errs) <= GRAD_TOL
