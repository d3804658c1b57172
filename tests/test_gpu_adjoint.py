"""Adjoint gradient of the 2-D elastic seismogram misfit (wave_adjoint_gradient)
against central finite differences of the misfit computed with the forward
solver itself, for vp, vs and rho along smooth perturbation directions; the
checkpoint interval must not change the result; unsupported set-ups are
rejected. The reference has no adjoint; the forward it differentiates is
FD2Delastic::run (ForwardSolver2Delastic.cpp:117-297).

Tolerance: |<g, dm> - (J(m + h dm) - J(m - h dm)) / 2h| <= 2e-2 |FD| (FP32
forward and adjoint, relative step 1e-3 of the parameter: the FP32 forward's
rounding bounds this check). The tight checks are against the FP64 oracle
gradient (oracle/adjoint_impl.hpp, itself pinned to FP64 finite differences
at 1e-6): relative L2 <= 1e-4 per parameter, with the free surface and ABS,
through a test-only torch.autograd.Function, and on a sub-grid of the
32-shot FWI workload.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
NX, NY, DH = 72, 60, 5.0
FD_TOL = 2e-2


def _blob(cx, cy, s):
    y, x = np.mgrid[0:NY, 0:NX]
    return np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2.0 * s * s)).reshape(-1)


def _models():
    y = np.arange(NY)[:, None] * np.ones((1, NX))
    vp = np.where(y < 25, 2200.0, 2900.0) + 150.0 * (y / NY)
    vs = vp / 1.75
    rho = 310.0 * vp ** 0.25
    true = dict(vp=vp.reshape(-1) * (1 + 0.06 * _blob(36, 32, 5)), vs=vs.reshape(-1) * (1 - 0.05 * _blob(30, 36, 5)),
                rho=rho.reshape(-1))
    start = dict(vp=vp.reshape(-1), vs=vs.reshape(-1), rho=rho.reshape(-1))
    return ({k: v.astype(np.float32) for k, v in true.items()}, {k: v.astype(np.float32) for k, v in start.items()})


def _config(wave, order=4, boundary=2, fs=0, stencil=0, dim=2, reduce=1):
    vmax = 3300.0
    DT = 0.3 * DH / (vmax * np.sqrt(2) * 1.3)
    return wave.WaveConfig.make(dimension=dim, equation="elastic", NX=NX, NY=NY, NZ=1 if dim == 2 else 20, DH=DH, DT=DT,
                                T=420 * DT, spatialFDorder=order, FreeSurface=fs, DampingBoundary=boundary,
                                BoundaryWidth=10, DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=15.0,
                                VMaxCPML=vmax, useStencilMatrix=stencil, edgeOrderReduction=reduce)


def _acq(wave, cfg, nt):
    sig = wave.wavelet(1, nt, cfg.DT, 3300.0 / (10 * DH), 1.0, 0.0)
    sidx = np.array([NX // 2 + NX * 8, 14 + NX * 10], np.int64)
    stype = np.array([1, 3], np.int32)
    xs = np.arange(6, NX - 6, 4)
    ridx = np.concatenate([xs + NX * 6, xs + NX * 6, xs[::3] + NX * 50]).astype(np.int64)
    rtype = np.concatenate([np.full(xs.size, 2), np.full(xs.size, 3), np.full(xs[::3].size, 1)]).astype(np.int32)
    return sidx, stype, np.stack([sig, 0.5 * sig]), ridx, rtype


def _solver(wave, cfg, model, acq):
    s = wave.Factory.Create("2D", "elastic").initForwardSolver(cfg)
    s.prepareForModelling(model)
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    return s


def _misfit(wave, cfg, model, acq, dobs):
    s = _solver(wave, cfg, model, acq)
    s.run(0, s.nt)
    r = s.seismograms().astype(np.float64) - dobs
    s.close()
    return 0.5 * float(np.sum(r * r))


@pytest.mark.parametrize("order,boundary,stencil", [(4, 2, 0), (8, 2, 0), (2, 0, 1), (6, 2, 1)])
def test_adjoint_gradient_matches_finite_differences(wave, order, boundary, stencil):
    cfg = _config(wave, order=order, boundary=boundary, stencil=stencil)
    true, start = _models()
    s = wave.Factory.Create("2D", "elastic").initForwardSolver(cfg)
    nt = s.nt
    s.close()
    acq = _acq(wave, cfg, nt)
    st = _solver(wave, cfg, true, acq)
    st.run(0, nt)
    dobs = st.seismograms().astype(np.float64)
    st.close()
    sa = _solver(wave, cfg, start, acq)
    J, gvp, gvs, grho = sa.adjoint_gradient(dobs.astype(np.float32), checkpoint_every=50)
    sa.close()
    J0 = _misfit(wave, cfg, start, acq, dobs)
    assert J > 0 and abs(J - J0) <= 1e-5 * J0
    dirs = {"vp": _blob(40, 28, 6), "vs": _blob(28, 34, 6), "rho": _blob(34, 40, 6)}
    grads = {"vp": gvp, "vs": gvs, "rho": grho}
    for name, d in dirs.items():
        h = 1e-3 * float(np.mean(start[name]))
        mp = dict(start); mp[name] = (start[name] + h * d).astype(np.float32)
        mm = dict(start); mm[name] = (start[name] - h * d).astype(np.float32)
        # the step actually applied after rounding to FP32
        dp = (mp[name].astype(np.float64) - mm[name].astype(np.float64)) / 2.0
        fd = (_misfit(wave, cfg, mp, acq, dobs) - _misfit(wave, cfg, mm, acq, dobs)) / 2.0
        ad = float(np.dot(grads[name].astype(np.float64), dp))
        assert abs(fd) > 0
        assert abs(ad - fd) <= FD_TOL * abs(fd), f"{name}: adjoint {ad:.6e} vs finite difference {fd:.6e}"


def test_checkpoint_interval_does_not_change_the_gradient(wave):
    cfg = _config(wave)
    true, start = _models()
    s = wave.Factory.Create("2D", "elastic").initForwardSolver(cfg)
    nt = s.nt
    s.close()
    acq = _acq(wave, cfg, nt)
    st = _solver(wave, cfg, true, acq)
    st.run(0, nt)
    dobs = st.seismograms()
    st.close()
    out = []
    for K in (7, 50, nt + 3):
        sa = _solver(wave, cfg, start, acq)
        out.append(sa.adjoint_gradient(dobs, checkpoint_every=K))
        sa.close()
    for o in out[1:]:
        assert abs(o[0] - out[0][0]) <= 1e-12 * abs(out[0][0])
        for a, b in zip(o[1:], out[0][1:]):
            assert np.array_equal(a, b)


def test_batched_adjoint_equals_single_shot_adjoints(wave):
    cfg = _config(wave)
    true, start = _models()
    s = wave.Factory.Create("2D", "elastic").initForwardSolver(cfg)
    nt = s.nt
    s.close()
    base = _acq(wave, cfg, nt)
    acqs = []
    for k in range(3):
        sidx = np.array([12 + 20 * k + NX * 8], np.int64)
        acqs.append((sidx, base[1][:1], base[2][:1], base[3], base[4]))
    dobs, single = [], []
    for acq in acqs:
        st = _solver(wave, cfg, true, acq)
        st.run(0, nt)
        dobs.append(st.seismograms())
        st.close()
        sa = _solver(wave, cfg, start, acq)
        single.append(sa.adjoint_gradient(dobs[-1], checkpoint_every=40))
        sa.close()
    b = wave.Batch([cfg] * 3)
    try:
        for shot, acq in zip(b.shots, acqs):
            shot.prepareForModelling(start)
            shot.setSources(*acq[:3])
            shot.setReceivers(*acq[3:])
        mis, gvp, gvs, grho = b.adjoint_gradient(dobs, checkpoint_every=40, sum_shots=False)
        mis_sum, svp, svs, srho = b.adjoint_gradient(dobs, checkpoint_every=40, sum_shots=True)
    finally:
        b.close()
    for k in range(3):
        # the misfit is a double-precision atomic sum: equal up to summation order
        assert abs(mis[k] - single[k][0]) <= 1e-12 * abs(single[k][0])
        assert np.array_equal(gvp[k], single[k][1])
        assert np.array_equal(gvs[k], single[k][2])
        assert np.array_equal(grho[k], single[k][3])
    assert np.allclose(mis_sum, mis, rtol=1e-12, atol=0)
    for summed, parts in ((svp, gvp), (svs, gvs), (srho, grho)):
        ref = np.sum([p.astype(np.float64) for p in parts], axis=0)
        assert np.linalg.norm(summed - ref) <= 1e-6 * np.linalg.norm(ref)


# ----------------------------------------------------------------------------
# against the FP64 oracle gradient
# ----------------------------------------------------------------------------
# Gate: 1e-4 relative L2 per parameter. The observed data of the two-layer
# survey below are 0.8 x the true model's seismograms, so that the residual
# holds part of the direct wave: with the unscaled data the residual at the
# receivers next to the sources is a small difference of large direct
# arrivals, and FP32 rounding alone moves the gradient by 2e-4 .. 6e-4 (the
# oracle's own FP32 adjoint shows the same); scaled, the oracle's FP32 and
# FP64 gradients agree to ~2e-5.
GRAD_TOL = 1e-4


def _oracle_gradient(refcpu, cfg, model, acq, dobs, K=50):
    ocfg = refcpu.WaveConfig()
    import ctypes
    ctypes.memmove(ctypes.byref(ocfg), ctypes.byref(cfg), ctypes.sizeof(ocfg))
    o = refcpu.Oracle(ocfg, {k: np.asarray(v, np.float64) for k, v in model.items()}, acq[0], acq[1],
                      np.asarray(acq[2], np.float64), acq[3], acq[4], dtype=np.float64)
    out = o.adjoint_gradient(np.asarray(dobs, np.float64), checkpoint_every=K)
    o.close()
    return out


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def _survey(wave, **kw):
    cfg = _config(wave, **kw)
    true, start = _models()
    s = wave.Factory.Create("2D", "elastic").initForwardSolver(cfg)
    nt = s.nt
    s.close()
    acq = _acq(wave, cfg, nt)
    if kw.get("fs"):
        # sources below the surface row, receivers on it
        acq = (acq[0] + NX * 2, acq[1], acq[2], np.where(acq[3] < NX * 10, acq[3] % NX, acq[3]), acq[4])
    st = _solver(wave, cfg, true, acq)
    st.run(0, nt)
    dobs = (0.8 * st.seismograms()).astype(np.float32)
    st.close()
    return cfg, start, acq, dobs


@pytest.mark.parametrize("kw", [dict(order=4, boundary=2), dict(order=2, boundary=0, stencil=1),
                                dict(order=4, boundary=2, fs=1), dict(order=4, boundary=1),
                                dict(order=6, boundary=1, fs=1), dict(order=8, boundary=2, fs=1, stencil=1),
                                dict(order=4, boundary=2, fs=1, reduce=0), dict(order=4, boundary=1, reduce=0),
                                dict(order=4, boundary=2, fs=2)])
def test_adjoint_gradient_matches_the_fp64_oracle_gradient(wave, refcpu, kw):
    """P and VY sources (the VY source exercises the re-formed pre-taper
    velocities), P / VX / VY receivers; every free-surface / ABS / CPML
    combination the adjoint supports."""
    cfg, start, acq, dobs = _survey(wave, **kw)
    sa = _solver(wave, cfg, start, acq)
    J, gvp, gvs, grho = sa.adjoint_gradient(dobs, checkpoint_every=50)
    sa.close()
    J64, g64vp, g64vs, g64rho = _oracle_gradient(refcpu, cfg, start, acq, dobs)
    errs = [_rel(g, r) for g, r in ((gvp, g64vp), (gvs, g64vs), (grho, g64rho))]
    print(f"adjoint {kw}: misfit {J:.6e} vs FP64 {J64:.6e}; gradient rel L2 vp {errs[0]:.2e} vs {errs[1]:.2e} "
          f"rho {errs[2]:.2e}")
    assert abs(J - J64) <= 1e-4 * J64
    assert max(errs) <= GRAD_TOL


def _smooth(rng, ny=NY, nx=NX):
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(rng.standard_normal((ny, nx)), 4.0, mode="nearest").reshape(-1)


def _fwi_survey(wave, NXs, NYs, nt, shots=3, fs=0):
    """The FWI workload's physics (order 4, DH 5 m, DT 5e-4, 20-pt CPML,
    layered model with two +-10 % anomalies, smoothed start model, Ricker
    10 Hz P sources at depth 10, two-component receivers) on a small grid:
    [(cfg, start, acq, dobs)] per shot, dobs from the FP32 forward on the
    true model."""
    import bench
    kw = dict(bench.FWI_KW, NX=NXs, NY=NYs, T=(nt - 0.4) * bench.FWI_KW["DT"], VMaxCPML=4400.0, FreeSurface=fs)
    cfg = wave.WaveConfig.make(**kw)
    true, start = bench.fwi_models(NXs, NYs)
    out = []
    for k in range(shots):
        sidx = np.array([30 + (NXs - 60) * k // max(1, shots - 1) + NXs * (2 if fs else 10)], np.int64)
        sig = wave.wavelet(1, nt, cfg.DT, 10.0, 1.0, 0.0)[None]
        xs = 10 + 4 * np.arange((NXs - 20) // 4)
        ry = 0 if fs else 10
        ridx = np.concatenate([xs + NXs * ry, xs + NXs * ry]).astype(np.int64)
        rtype = np.concatenate([np.full(xs.size, 2), np.full(xs.size, 3)]).astype(np.int32)
        acq = (sidx, np.array([1], np.int32), sig, ridx, rtype)
        st = _solver(wave, cfg, true, acq)
        st.run(0, nt)
        dobs = st.seismograms()
        st.close()
        out.append((cfg, start, acq, dobs))
    return out


def _oracle_misfit(refcpu, cfg, model, acq, dobs):
    import ctypes
    ocfg = refcpu.WaveConfig()
    ctypes.memmove(ctypes.byref(ocfg), ctypes.byref(cfg), ctypes.sizeof(ocfg))
    o = refcpu.Oracle(ocfg, model, acq[0], acq[1], np.asarray(acq[2], np.float64), acq[3], acq[4], dtype=np.float64)
    d = o.run()
    o.close()
    return 0.5 * float(np.sum((d - np.asarray(dobs, np.float64)) ** 2))


def test_autograd_gradient_against_fp64_finite_differences(wave, refcpu):
    """Through the test-only torch.autograd.Function: the gradients equal the
    C ABI's, and their projections on 8 seeded smooth directions (per
    parameter) and 16 single points (the largest gradient entries) match
    central finite differences of the FP64 oracle's misfit (relative step
    1e-4) within 1e-4 (directions) / 1e-3 of the largest entry (points)."""
    torch = pytest.importorskip("torch")
    import adjoint_autograd
    cfg, start, acq, dobs = _fwi_survey(wave, 100, 60, 600, shots=1, fs=1)[0]
    t = {k: torch.tensor(v, dtype=torch.float32, requires_grad=True) for k, v in start.items()}
    sa = _solver(wave, cfg, start, acq)
    J = adjoint_autograd.misfit(t["vp"], t["vs"], t["rho"], sa, dobs, 50)
    J.backward()
    _, gvp, gvs, grho = sa.adjoint_gradient(dobs, checkpoint_every=50)
    sa.close()
    grads = {"vp": t["vp"].grad.numpy(), "vs": t["vs"].grad.numpy(), "rho": t["rho"].grad.numpy()}
    for k, g in (("vp", gvp), ("vs", gvs), ("rho", grho)):
        assert np.array_equal(grads[k], g)
    m64 = {k: v.astype(np.float64) for k, v in start.items()}
    rng = np.random.default_rng(20260005)
    worst = 0.0
    ny, nx = cfg.NY, cfg.NX
    for name in ("vp", "vs", "rho"):
        for _ in range(8):
            d = _smooth(rng, ny, nx) * m64[name]
            h = 1e-4
            mp, mm = dict(m64), dict(m64)
            mp[name] = m64[name] + h * d
            mm[name] = m64[name] - h * d
            fd = (_oracle_misfit(refcpu, cfg, mp, acq, dobs) - _oracle_misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)
            ad = float(np.dot(grads[name].astype(np.float64), d))
            worst = max(worst, abs(ad - fd) / abs(fd))
            assert abs(ad - fd) <= 1e-4 * abs(fd), (name, ad, fd)
    g_all = np.concatenate([grads["vp"], grads["vs"], grads["rho"]]).astype(np.float64)
    top = np.argsort(-np.abs(g_all))[:16]
    for k in top:
        name, i = ("vp", "vs", "rho")[k // cfg.N], int(k % cfg.N)
        h = 1e-4 * m64[name][i]
        mp, mm = dict(m64), dict(m64)
        mp[name] = m64[name].copy()
        mm[name] = m64[name].copy()
        mp[name][i] += h
        mm[name][i] -= h
        fd = (_oracle_misfit(refcpu, cfg, mp, acq, dobs) - _oracle_misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)
        assert abs(grads[name][i] - fd) <= 1e-3 * abs(fd), (name, i, grads[name][i], fd)
    print(f"autograd directional derivatives: worst relative error {worst:.2e}")


def test_fwi_workload_subgrid_batched_against_fp64(wave, refcpu):
    """The 32-shot FWI-gradient workload's physics (order 4, DH 5 m, DT 5e-4,
    20-pt CPML, layered model with two +-10 % anomalies, smoothed start
    model, P sources at depth 10, 136 two-component receivers rows) on a
    200 x 100 sub-grid, 1000 steps, 3 shots in one batch with the gradients
    summed, checkpoints every 50 steps: against the sum of the FP64 oracle's
    per-shot gradients."""
    NXs, NYs, nt = 200, 100, 1000
    shots = _fwi_survey(wave, NXs, NYs, nt, shots=3)
    cfg, start = shots[0][0], shots[0][1]
    acqs = [x[2] for x in shots]
    dobs = [x[3] for x in shots]
    b = wave.Batch([cfg] * 3)
    try:
        for shot, acq in zip(b.shots, acqs):
            shot.prepareForModelling(start)
            shot.setSources(*acq[:3])
            shot.setReceivers(*acq[3:])
        mis, gvp, gvs, grho = b.adjoint_gradient(dobs, checkpoint_every=50, sum_shots=True)
    finally:
        b.close()
    ref = [np.zeros(cfg.N) for _ in range(3)]
    J64 = 0.0
    for acq, d in zip(acqs, dobs):
        J, a, bb, c = _oracle_gradient(refcpu, cfg, start, acq, d)
        J64 += J
        for r, g in zip(ref, (a, bb, c)):
            r += g
    errs = [_rel(g, r) for g, r in zip((gvp, gvs, grho), ref)]
    print(f"FWI sub-grid 200x100, 3 shots, NT={nt}: misfit {sum(mis):.6e} vs FP64 {J64:.6e}; "
          f"gradient rel L2 vp {errs[0]:.2e} vs {errs[1]:.2e} rho {errs[2]:.2e}")
    assert abs(sum(mis) - J64) <= 1e-4 * J64
    assert max(errs) <= GRAD_TOL
