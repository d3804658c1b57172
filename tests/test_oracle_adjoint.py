"""The oracle's FP64 discrete adjoint of the 2-D elastic step
(oracle/adjoint_impl.hpp), checked without a GPU against central finite
differences of the FP64 oracle's own misfit: along seeded smooth directions
and at single grid points, for vp, vs and rho, with CPML, no boundary, ABS and
the free surface, both edge rules and stencil operators. This pins the FP64
gradient the CUDA adjoint is compared with (tests/test_gpu_adjoint.py).

Gate: relative error of the directional derivative <= 1e-6 (FP64 forward
with a relative step of 1e-4: truncation ~1e-8, rounding ~1e-11)."""
import numpy as np
import pytest


def case(refcpu, fs=0, boundary=2, stencil=0, reduce=1, order=4, seed=3, NX=44, NY=36, nt=160, L=0):
    """2-D elastic survey; L > 0: visco-elastic with L relaxation mechanisms."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:NY, 0:NX]
    vp = 2000.0 + 600.0 * (y / NY) + 80.0 * np.sin(x / 5.0) + 30 * rng.standard_normal((NY, NX))
    vs = vp / 1.75
    rho = 310.0 * vp ** 0.25
    fields = dict(vp=vp, vs=vs, rho=rho)
    if L:
        fields["taup"] = 0.04 + 0.01 * np.sin(x / 6.0) + 0.005 * (y / NY)
        fields["taus"] = 0.05 + 0.01 * np.cos(y / 5.0)
    model = {k: v.reshape(-1).astype(np.float64) for k, v in fields.items()}
    DH, DT = 5.0, 4e-4
    cfg = refcpu.make_config(dimension=2, equation="viscoelastic" if L else "elastic", NX=NX, NY=NY, NZ=1, DH=DH, DT=DT,
                             T=(nt - 0.4) * DT, spatialFDorder=order, FreeSurface=fs, DampingBoundary=boundary,
                             BoundaryWidth=8, DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=20.0, VMaxCPML=2700.0,
                             useStencilMatrix=stencil, edgeOrderReduction=reduce, numRelaxationMechanisms=L,
                             relaxationFrequency=[15.0, 40.0][:L])
    sidx = np.array([refcpu.grid_index(cfg, NX // 2, 2 if fs else 6, 0)], np.int64)
    sig = refcpu.ricker(nt, DT, 25.0, 1.0, -0.02, np.float64)[None]
    rx = np.arange(4, NX - 4, 3)
    ry = 0 if fs else 5
    ridx = np.concatenate([rx + NX * ry, rx + NX * ry, rx + NX * (NY - 6)]).astype(np.int64)
    rtype = np.concatenate([np.full(rx.size, 2), np.full(rx.size, 3), np.full(rx.size, 1)]).astype(np.int32)
    return cfg, model, (sidx, np.array([1], np.int32), sig, ridx, rtype)


def misfit(refcpu, cfg, model, acq, dobs):
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    d = o.run()
    o.close()
    return 0.5 * float(np.sum((d - dobs) ** 2))


def smooth_direction(rng, NY, NX):
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(rng.standard_normal((NY, NX)), 3.0, mode="nearest").reshape(-1)


@pytest.mark.parametrize("fs,boundary,stencil,reduce", [(0, 2, 0, 1), (0, 0, 0, 0), (1, 2, 0, 1), (0, 1, 0, 1),
                                                        (1, 1, 1, 0), (2, 2, 0, 1)])
def test_oracle_adjoint_matches_fp64_finite_differences(refcpu, fs, boundary, stencil, reduce):
    cfg, model, acq = case(refcpu, fs, boundary, stencil, reduce)
    # observed data: the same survey on a perturbed model
    true = dict(model)
    yy, xx = np.mgrid[0:cfg.NY, 0:cfg.NX]
    blob = np.exp(-((xx - cfg.NX * 0.4) ** 2 + (yy - cfg.NY * 0.6) ** 2) / 40.0).reshape(-1)
    true["vp"] = model["vp"] * (1 + 0.05 * blob)
    true["vs"] = model["vs"] * (1 - 0.04 * blob)
    o = refcpu.Oracle(cfg, true, *acq, dtype=np.float64)
    dobs = o.run()
    o.close()
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    J, gvp, gvs, grho = o.adjoint_gradient(dobs, checkpoint_every=37)
    o.close()
    assert J == pytest.approx(misfit(refcpu, cfg, model, acq, dobs), rel=1e-12)
    rng = np.random.default_rng(11)
    grads = dict(vp=gvp, vs=gvs, rho=grho)
    for name in ("vp", "vs", "rho"):
        d = smooth_direction(rng, cfg.NY, cfg.NX) * model[name]
        h = 1e-4
        mp, mm = dict(model), dict(model)
        mp[name] = model[name] + h * d
        mm[name] = model[name] - h * d
        fd = (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)
        ad = float(np.dot(grads[name], d))
        assert abs(ad - fd) <= 1e-6 * abs(fd), (name, ad, fd)
    # one single-point probe per parameter, at the point of the largest gradient
    for name in ("vp", "vs", "rho"):
        k = int(np.argmax(np.abs(grads[name])))
        h = 1e-4 * model[name][k]
        mp, mm = dict(model), dict(model)
        mp[name] = model[name].copy()
        mm[name] = model[name].copy()
        mp[name][k] += h
        mm[name][k] -= h
        fd = (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)
        assert abs(grads[name][k] - fd) <= 1e-6 * abs(fd), (name, k, grads[name][k], fd)


def test_oracle_adjoint_is_independent_of_the_checkpoint_interval(refcpu):
    cfg, model, acq = case(refcpu, fs=1, boundary=2)
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    d = o.run()
    dobs = 0.9 * d
    g1 = o.adjoint_gradient(dobs, checkpoint_every=1)
    g2 = o.adjoint_gradient(dobs, checkpoint_every=1000)
    o.close()
    assert g1[0] == g2[0]
    for a, b in zip(g1[1:], g2[1:]):
        assert np.array_equal(a, b)


def tm_case(refcpu, boundary=2, stencil=0, reduce=1, order=4, NX=48, NY=40, nt=220, L=0):
    """2-D TMz survey; L > 0: visco-TMz with L relaxation mechanisms."""
    rng = np.random.default_rng(5)
    y, x = np.mgrid[0:NY, 0:NX]
    eps = 6.0 + 8.0 * (y > NY // 2) + 0.5 * np.sin(x / 4.0) + 0.2 * rng.standard_normal((NY, NX))
    sig = 10 ** (-3.0 + 0.5 * np.cos(y / 6.0))
    mur = 1.0 + 0.05 * (x > NX // 2)
    fields = dict(eps_r=eps, sigma=sig, mu_r=mur)
    if L:
        fields["tau_eps"] = 0.15 + 0.05 * np.sin(x / 5.0)
        fields["tau_sigma"] = 0.1 + 0.05 * np.cos(y / 4.0)
    model = {k: v.reshape(-1).astype(np.float64) for k, v in fields.items()}
    DH = 0.02
    DT = 0.3 * DH / (3e8 * np.sqrt(2) * 1.3)
    cfg = refcpu.make_config(dimension=2, equation="viscotmem" if L else "tmem", NX=NX, NY=NY, NZ=1, DH=DH, DT=DT,
                             T=(nt - 0.4) * DT, spatialFDorder=order, DampingBoundary=boundary, BoundaryWidth=8,
                             DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=4e8, VMaxCPML=1.5e8,
                             useStencilMatrix=stencil, edgeOrderReduction=reduce, numRelaxationMechanisms=L,
                             relaxationFrequency=[3e8, 9e8][:L])
    sidx = np.array([refcpu.grid_index(cfg, NX // 2, 6, 0)], np.int64)
    sig_t = refcpu.ricker(nt, DT, 6e8, 1.0, 0.0, np.float64)[None]
    rx = np.arange(4, NX - 4, 3)
    ridx = np.concatenate([rx + NX * 5, rx + NX * (NY - 6)]).astype(np.int64)
    return cfg, model, (sidx, np.array([1], np.int32), sig_t, ridx, np.ones(ridx.size, np.int32))


@pytest.mark.parametrize("boundary,stencil,reduce,L", [(2, 0, 1, 0), (0, 1, 0, 0), (1, 0, 1, 0), (2, 0, 1, 1), (1, 1, 0, 2)])
def test_oracle_tmz_adjoint_matches_fp64_finite_differences(refcpu, boundary, stencil, reduce, L):
    """The oracle's FP64 adjoint of the lossless TMz step and of the visco-TMz
    step (L mechanisms, tau_eps and tau_sigma fixed; gradients with respect to
    eps_r, sigma, mu_r) against central finite differences of its own misfit,
    with CPML, no boundary and ABS."""
    cfg, model, acq = tm_case(refcpu, boundary, stencil, reduce, L=L)
    true = dict(model)
    yy, xx = np.mgrid[0:cfg.NY, 0:cfg.NX]
    blob = np.exp(-((xx - cfg.NX * 0.5) ** 2 + (yy - cfg.NY * 0.4) ** 2) / 30.0).reshape(-1)
    true["eps_r"] = model["eps_r"] * (1 + 0.1 * blob)
    true["sigma"] = model["sigma"] * (1 + 0.5 * blob)
    o = refcpu.Oracle(cfg, true, *acq, dtype=np.float64)
    dobs = o.run()
    o.close()
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    J, ge, gs, gm = o.adjoint_gradient(dobs, checkpoint_every=41)
    o.close()
    assert J > 0 and J == pytest.approx(misfit(refcpu, cfg, model, acq, dobs), rel=1e-12)
    rng = np.random.default_rng(12)
    grads = dict(eps_r=ge, sigma=gs, mu_r=gm)
    for name in ("eps_r", "sigma", "mu_r"):
        d = smooth_direction(rng, cfg.NY, cfg.NX) * model[name]
        h = 1e-4
        mp, mm = dict(model), dict(model)
        mp[name] = model[name] + h * d
        mm[name] = model[name] - h * d
        fd = (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)
        ad = float(np.dot(grads[name], d))
        assert abs(fd) > 0
        assert abs(ad - fd) <= 1e-6 * abs(fd), (name, ad, fd)


def sh_case(refcpu, fs=0, boundary=2, stencil=0, reduce=1, order=4, NX=44, NY=36, nt=180, L=0):
    """2-D SH survey; L > 0: visco-SH with L relaxation mechanisms."""
    rng = np.random.default_rng(7)
    y, x = np.mgrid[0:NY, 0:NX]
    vs = 1200.0 + 500.0 * (y / NY) + 60.0 * np.sin(x / 5.0) + 20 * rng.standard_normal((NY, NX))
    rho = 1800.0 + 300.0 * (y > NY // 2) + 40.0 * np.cos(x / 7.0)
    fields = dict(vs=vs, rho=rho)
    if L:
        fields["taus"] = 0.05 + 0.01 * np.cos(y / 5.0) + 0.005 * np.sin(x / 4.0)
    model = {k: v.reshape(-1).astype(np.float64) for k, v in fields.items()}
    DH, DT = 5.0, 6e-4
    cfg = refcpu.make_config(dimension=2, equation="viscosh" if L else "sh", NX=NX, NY=NY, NZ=1, DH=DH, DT=DT,
                             T=(nt - 0.4) * DT, spatialFDorder=order, FreeSurface=fs, DampingBoundary=boundary,
                             BoundaryWidth=8, DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=20.0, VMaxCPML=1800.0,
                             useStencilMatrix=stencil, edgeOrderReduction=reduce, numRelaxationMechanisms=L,
                             relaxationFrequency=[15.0, 40.0][:L])
    sidx = np.array([refcpu.grid_index(cfg, NX // 2, 2 if fs else 6, 0)], np.int64)
    sig = refcpu.ricker(nt, DT, 20.0, 1.0, -0.02, np.float64)[None]
    rx = np.arange(4, NX - 4, 3)
    ridx = np.concatenate([rx + NX * (0 if fs else 5), rx + NX * (NY - 6)]).astype(np.int64)
    return cfg, model, (sidx, np.array([4], np.int32), sig, ridx, np.full(ridx.size, 4, np.int32))


@pytest.mark.parametrize("fs,boundary,stencil,reduce,L", [(0, 2, 0, 1, 0), (0, 0, 1, 0, 0), (1, 2, 0, 1, 0), (0, 1, 0, 1, 0),
                                                          (1, 1, 1, 0, 0), (0, 2, 0, 1, 1), (1, 1, 0, 0, 2)])
def test_oracle_sh_adjoint_matches_fp64_finite_differences(refcpu, fs, boundary, stencil, reduce, L):
    """The oracle's FP64 adjoint of the 2-D SH step (gradients with respect
    to vs and rho; the vp gradient is zero) against central finite
    differences of its own misfit (relative step 1e-5) along smooth
    directions and at the point of the largest gradient, with CPML, no
    boundary, ABS and the free surface, and for visco-SH with one and two
    relaxation mechanisms (the relaxation times fixed)."""
    cfg, model, acq = sh_case(refcpu, fs, boundary, stencil, reduce, L=L)
    true = dict(model)
    yy, xx = np.mgrid[0:cfg.NY, 0:cfg.NX]
    blob = np.exp(-((xx - cfg.NX * 0.45) ** 2 + (yy - cfg.NY * 0.55) ** 2) / 40.0).reshape(-1)
    true["vs"] = model["vs"] * (1 + 0.06 * blob)
    true["rho"] = model["rho"] * (1 - 0.04 * blob)
    o = refcpu.Oracle(cfg, true, *acq, dtype=np.float64)
    dobs = o.run()
    o.close()
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    J, gvp, gvs, grho = o.adjoint_gradient(dobs, checkpoint_every=43)
    o.close()
    assert J > 0 and J == pytest.approx(misfit(refcpu, cfg, model, acq, dobs), rel=1e-12)
    assert not np.any(gvp)
    rng = np.random.default_rng(13)
    grads = dict(vs=gvs, rho=grho)
    for name in ("vs", "rho"):
        d = smooth_direction(rng, cfg.NY, cfg.NX) * model[name]
        h = 1e-5   # the SH misfit's curvature puts the truncation at ~1e-6 for 1e-4
        mp, mm = dict(model), dict(model)
        mp[name] = model[name] + h * d
        mm[name] = model[name] - h * d
        fd = (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)
        ad = float(np.dot(grads[name], d))
        assert abs(fd) > 0
        assert abs(ad - fd) <= 1e-6 * abs(fd), (name, ad, fd)
        k = int(np.argmax(np.abs(grads[name])))
        hk = 1e-5 * model[name][k]
        mp, mm = dict(model), dict(model)
        mp[name] = model[name].copy()
        mm[name] = model[name].copy()
        mp[name][k] += hk
        mm[name][k] -= hk
        fd = (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * hk)
        assert abs(grads[name][k] - fd) <= 1e-6 * abs(fd), (name, k, grads[name][k], fd)


def te_case(refcpu, boundary=2, stencil=0, reduce=1, order=4, NX=48, NY=40, nt=220, L=0):
    """2-D TEz survey; L > 0: visco-TEz with L relaxation mechanisms."""
    rng = np.random.default_rng(9)
    y, x = np.mgrid[0:NY, 0:NX]
    eps = 5.0 + 7.0 * (y > NY // 2) + 0.5 * np.cos(x / 4.0) + 0.2 * rng.standard_normal((NY, NX))
    sig = 10 ** (-3.0 + 0.5 * np.sin(y / 5.0))
    mur = 1.0 + 0.05 * (x > NX // 3)
    fields = dict(eps_r=eps, sigma=sig, mu_r=mur)
    if L:
        fields["tau_eps"] = 0.15 + 0.05 * np.cos(x / 5.0)
        fields["tau_sigma"] = 0.1 + 0.05 * np.sin(y / 4.0)
    model = {k: v.reshape(-1).astype(np.float64) for k, v in fields.items()}
    DH = 0.02
    DT = 0.3 * DH / (3e8 * np.sqrt(2) * 1.3)
    cfg = refcpu.make_config(dimension=2, equation="viscoemem" if L else "emem", NX=NX, NY=NY, NZ=1, DH=DH, DT=DT,
                             T=(nt - 0.4) * DT, spatialFDorder=order, DampingBoundary=boundary, BoundaryWidth=8,
                             DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=4e8, VMaxCPML=1.5e8,
                             useStencilMatrix=stencil, edgeOrderReduction=reduce, numRelaxationMechanisms=L,
                             relaxationFrequency=[3e8, 9e8][:L])
    sidx = np.array([refcpu.grid_index(cfg, NX // 2, 6, 0), refcpu.grid_index(cfg, NX // 3, 9, 0)], np.int64)
    sig_t = refcpu.ricker(nt, DT, 6e8, 1.0, 0.0, np.float64)
    rx = np.arange(4, NX - 4, 3)
    ridx = np.concatenate([rx + NX * 5, rx + NX * 5, rx + NX * (NY - 6)]).astype(np.int64)
    rtype = np.concatenate([np.full(rx.size, 2), np.full(rx.size, 3), np.full(rx.size, 4)]).astype(np.int32)
    return cfg, model, (sidx, np.array([3, 4], np.int32), np.stack([sig_t, 300.0 * sig_t]), ridx, rtype)


@pytest.mark.parametrize("boundary,stencil,reduce,L", [(2, 0, 1, 0), (0, 1, 0, 0), (1, 0, 1, 0), (2, 0, 1, 1), (1, 1, 0, 2)])
def test_oracle_tez_adjoint_matches_fp64_finite_differences(refcpu, boundary, stencil, reduce, L):
    """The oracle's FP64 adjoint of the lossless TEz step (gradients with
    respect to eps_r, sigma, mu_r; Ey and Hz sources, Ex, Ey and Hz
    receivers; L > 0: visco-TEz with tau_eps and tau_sigma fixed) against
    Richardson-extrapolated central finite differences of its own misfit,
    with CPML, no boundary and ABS."""
    cfg, model, acq = te_case(refcpu, boundary, stencil, reduce, L=L)
    true = dict(model)
    yy, xx = np.mgrid[0:cfg.NY, 0:cfg.NX]
    blob = np.exp(-((xx - cfg.NX * 0.5) ** 2 + (yy - cfg.NY * 0.4) ** 2) / 30.0).reshape(-1)
    true["eps_r"] = model["eps_r"] * (1 + 0.1 * blob)
    true["sigma"] = model["sigma"] * (1 + 0.5 * blob)
    true["mu_r"] = model["mu_r"] * (1 + 0.05 * blob)
    o = refcpu.Oracle(cfg, true, *acq, dtype=np.float64)
    dobs = o.run()
    o.close()
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    J, ge, gs, gm = o.adjoint_gradient(dobs, checkpoint_every=41)
    o.close()
    assert J > 0 and J == pytest.approx(misfit(refcpu, cfg, model, acq, dobs), rel=1e-12)
    rng = np.random.default_rng(17)
    grads = dict(eps_r=ge, sigma=gs, mu_r=gm)
    for name in ("eps_r", "sigma", "mu_r"):
        d = smooth_direction(rng, cfg.NY, cfg.NX) * model[name]

        def central(h):
            mp, mm = dict(model), dict(model)
            mp[name] = model[name] + h * d
            mm[name] = model[name] - h * d
            return (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)

        # Richardson-extrapolated central difference (steps 2e-4, 4e-4): the visco surveys' eps_r
        # derivative is small against the misfit, so a single step's truncation or rounding shows
        h = 2e-4
        d1 = central(h)
        fd = d1 - (central(2 * h) - d1) / 3
        ad = float(np.dot(grads[name], d))
        assert abs(fd) > 0
        assert abs(ad - fd) <= 1e-6 * abs(fd), (name, ad, fd)


def el3_case(refcpu, fs=0, boundary=2, stencil=0, reduce=1, order=4, NX=24, NY=20, NZ=18, nt=110, L=0):
    """3-D elastic survey; L > 0: visco-elastic with L relaxation mechanisms."""
    rng = np.random.default_rng(21)
    y, z, x = np.mgrid[0:NY, 0:NZ, 0:NX]   # index x + NX (z + NZ y)
    vp = 2000.0 + 500.0 * (y / NY) + 60.0 * np.sin(x / 4.0) + 40.0 * np.cos(z / 3.0) + 20 * rng.standard_normal((NY, NZ, NX))
    vs = vp / 1.8
    rho = 300.0 * vp ** 0.25
    fields = dict(vp=vp, vs=vs, rho=rho)
    if L:
        fields["taup"] = 0.04 + 0.01 * np.sin(x / 5.0) + 0.005 * np.cos(z / 4.0)
        fields["taus"] = 0.05 + 0.01 * np.cos(y / 4.0)
    model = {k: v.reshape(-1).astype(np.float64) for k, v in fields.items()}
    DH, DT = 5.0, 4e-4
    cfg = refcpu.make_config(dimension=3, equation="viscoelastic" if L else "elastic", NX=NX, NY=NY, NZ=NZ, DH=DH, DT=DT,
                             T=(nt - 0.4) * DT, spatialFDorder=order, FreeSurface=fs, DampingBoundary=boundary,
                             BoundaryWidth=5, DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=25.0, VMaxCPML=2600.0,
                             useStencilMatrix=stencil, edgeOrderReduction=reduce, numRelaxationMechanisms=L,
                             relaxationFrequency=[20.0, 50.0][:L])
    sidx = np.array([refcpu.grid_index(cfg, NX // 2, 2 if fs else 5, NZ // 2),
                     refcpu.grid_index(cfg, NX // 3, 7, NZ // 3)], np.int64)
    sig = refcpu.ricker(nt, DT, 30.0, 1.0, -0.015, np.float64)
    rx = np.arange(3, NX - 3, 3)
    ry = 0 if fs else 4
    ridx = np.concatenate([rx + NX * (NZ // 2 + NZ * ry), rx + NX * (NZ // 3 + NZ * ry), rx + NX * (5 + NZ * (NY - 5)),
                           rx + NX * (12 + NZ * (NY - 5))]).astype(np.int64)
    rtype = np.concatenate([np.full(rx.size, 2), np.full(rx.size, 3), np.full(rx.size, 4), np.full(rx.size, 1)]).astype(np.int32)
    return cfg, model, (sidx, np.array([1, 4], np.int32), np.stack([sig, 3e-4 * sig]), ridx, rtype)


def smooth3(rng, cfg):
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(rng.standard_normal((cfg.NY, cfg.NZ, cfg.NX)), 2.5, mode="nearest").reshape(-1)


@pytest.mark.parametrize("fs,boundary,stencil,reduce", [(0, 2, 0, 1), (1, 2, 0, 1), (0, 1, 1, 0), (1, 0, 0, 0),
                                                        (2, 2, 0, 1)])
def test_oracle_elastic3d_adjoint_matches_fp64_finite_differences(refcpu, fs, boundary, stencil, reduce):
    """The oracle's FP64 adjoint of the 3-D elastic step (gradients with
    respect to vp, vs, rho; P and VZ sources, P / VX / VY / VZ receivers)
    against central finite differences of its own misfit along smooth
    directions, with CPML, ABS, no boundary and the free surface."""
    cfg, model, acq = el3_case(refcpu, fs, boundary, stencil, reduce)
    true = dict(model)
    y, z, x = np.mgrid[0:cfg.NY, 0:cfg.NZ, 0:cfg.NX]
    blob = np.exp(-((x - cfg.NX * 0.5) ** 2 + (y - cfg.NY * 0.55) ** 2 + (z - cfg.NZ * 0.5) ** 2) / 18.0).reshape(-1)
    true["vp"] = model["vp"] * (1 + 0.05 * blob)
    true["vs"] = model["vs"] * (1 - 0.04 * blob)
    true["rho"] = model["rho"] * (1 + 0.03 * blob)
    o = refcpu.Oracle(cfg, true, *acq, dtype=np.float64)
    dobs = 0.9 * o.run()
    o.close()
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    J, gvp, gvs, grho = o.adjoint_gradient(dobs, checkpoint_every=37)
    o.close()
    assert J > 0 and J == pytest.approx(misfit(refcpu, cfg, model, acq, dobs), rel=1e-12)
    rng = np.random.default_rng(23)
    grads = dict(vp=gvp, vs=gvs, rho=grho)
    for name in ("vp", "vs", "rho"):
        d = smooth3(rng, cfg) * model[name]
        h = 1e-5
        mp, mm = dict(model), dict(model)
        mp[name] = model[name] + h * d
        mm[name] = model[name] - h * d
        fd = (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)
        ad = float(np.dot(grads[name], d))
        assert abs(fd) > 0
        assert abs(ad - fd) <= 1e-6 * abs(fd), (name, ad, fd)


@pytest.mark.parametrize("L,boundary,stencil,reduce,fs", [(1, 2, 0, 1, 0), (2, 0, 1, 0, 0), (2, 1, 0, 1, 0), (1, 2, 0, 1, 1),
                                                           (2, 1, 1, 0, 1), (1, 2, 0, 1, 2)])
def test_oracle_visco_adjoint_matches_fp64_finite_differences(refcpu, L, boundary, stencil, reduce, fs):
    """The oracle's FP64 adjoint of the 2-D visco-elastic step (memory
    variables of one or two relaxation mechanisms; gradients with respect to
    vp, vs, rho with the relaxation times held fixed) against central finite
    differences of its own misfit, with CPML, no boundary, ABS and the free
    surface (its visco exchange, FreeSurface2Dviscoelastic.cpp)."""
    cfg, model, acq = case(refcpu, fs, boundary, stencil, reduce, L=L)
    true = dict(model)
    yy, xx = np.mgrid[0:cfg.NY, 0:cfg.NX]
    blob = np.exp(-((xx - cfg.NX * 0.4) ** 2 + (yy - cfg.NY * 0.6) ** 2) / 40.0).reshape(-1)
    true["vp"] = model["vp"] * (1 + 0.05 * blob)
    true["vs"] = model["vs"] * (1 - 0.04 * blob)
    o = refcpu.Oracle(cfg, true, *acq, dtype=np.float64)
    dobs = 0.9 * o.run()
    o.close()
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    J, gvp, gvs, grho = o.adjoint_gradient(dobs, checkpoint_every=37)
    o.close()
    assert J > 0 and J == pytest.approx(misfit(refcpu, cfg, model, acq, dobs), rel=1e-12)
    rng = np.random.default_rng(29)
    grads = dict(vp=gvp, vs=gvs, rho=grho)
    for name in ("vp", "vs", "rho"):
        d = smooth_direction(rng, cfg.NY, cfg.NX) * model[name]
        h = 1e-5
        mp, mm = dict(model), dict(model)
        mp[name] = model[name] + h * d
        mm[name] = model[name] - h * d
        fd = (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)
        ad = float(np.dot(grads[name], d))
        assert abs(fd) > 0
        assert abs(ad - fd) <= 1e-6 * abs(fd), (name, ad, fd)


def ac_case(refcpu, dim=2, fs=0, boundary=2, stencil=0, reduce=1, order=4, NX=44, NY=36, NZ=20, nt=180):
    rng = np.random.default_rng(31)
    NZ = NZ if dim == 3 else 1
    y, z, x = np.mgrid[0:NY, 0:NZ, 0:NX]
    vp = 1800.0 + 600.0 * (y / NY) + 70.0 * np.sin(x / 5.0) + 30.0 * np.cos(z / 4.0) + 25 * rng.standard_normal((NY, NZ, NX))
    rho = 1700.0 + 300.0 * (y > NY // 2) + 40.0 * np.cos(x / 6.0)
    model = {k: v.reshape(-1).astype(np.float64) for k, v in dict(vp=vp, rho=rho).items()}
    DH, DT = 5.0, 4e-4
    cfg = refcpu.make_config(dimension=dim, equation="acoustic", NX=NX, NY=NY, NZ=NZ, DH=DH, DT=DT, T=(nt - 0.4) * DT,
                             spatialFDorder=order, FreeSurface=fs, DampingBoundary=boundary, BoundaryWidth=6,
                             DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=25.0, VMaxCPML=2500.0,
                             useStencilMatrix=stencil, edgeOrderReduction=reduce)
    zc = NZ // 2
    sidx = np.array([refcpu.grid_index(cfg, NX // 2, 2 if fs else 6, zc), refcpu.grid_index(cfg, NX // 3, 9, zc)], np.int64)
    sig = refcpu.ricker(nt, DT, 25.0, 1.0, -0.02, np.float64)
    rx = np.arange(4, NX - 4, 3)
    ry = 1 if fs else 5
    ridx = np.concatenate([rx + NX * (zc + NZ * ry), rx + NX * (zc + NZ * ry), rx + NX * (zc + NZ * (NY - 6))]).astype(np.int64)
    rtype = np.concatenate([np.full(rx.size, 1), np.full(rx.size, 3), np.full(rx.size, 2)]).astype(np.int32)
    return cfg, model, (sidx, np.array([1, 3], np.int32), np.stack([sig, 2e-3 * sig]), ridx, rtype)


@pytest.mark.parametrize("dim,fs,boundary,stencil,reduce", [(2, 0, 2, 0, 1), (2, 1, 1, 1, 0), (2, 1, 0, 0, 1),
                                                            (3, 0, 2, 0, 1), (3, 1, 1, 0, 0), (2, 2, 2, 0, 1),
                                                            (3, 2, 1, 0, 1)])
def test_oracle_acoustic_adjoint_matches_fp64_finite_differences(refcpu, dim, fs, boundary, stencil, reduce):
    """The oracle's FP64 adjoint of the 2-D and 3-D acoustic steps (gradients
    with respect to vp and rho; P and VY sources, P / VX / VY receivers)
    against central finite differences of its own misfit, with CPML, ABS, no
    boundary and the free surface."""
    cfg, model, acq = ac_case(refcpu, dim, fs, boundary, stencil, reduce)
    true = dict(model)
    n = model["vp"].size
    blob = np.exp(-np.linspace(-3, 3, n) ** 2)
    true["vp"] = model["vp"] * (1 + 0.05 * blob)
    true["rho"] = model["rho"] * (1 - 0.03 * blob)
    o = refcpu.Oracle(cfg, true, *acq, dtype=np.float64)
    dobs = 0.9 * o.run()
    o.close()
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    J, gvp, gvs, grho = o.adjoint_gradient(dobs, checkpoint_every=37)
    o.close()
    assert J > 0 and J == pytest.approx(misfit(refcpu, cfg, model, acq, dobs), rel=1e-12)
    assert not np.any(gvs)
    rng = np.random.default_rng(37)
    grads = dict(vp=gvp, rho=grho)
    for name in ("vp", "rho"):
        d = (smooth3(rng, cfg) if dim == 3 else smooth_direction(rng, cfg.NY, cfg.NX)) * model[name]
        h = 1e-5
        mp, mm = dict(model), dict(model)
        mp[name] = model[name] + h * d
        mm[name] = model[name] - h * d
        fd = (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)
        ad = float(np.dot(grads[name], d))
        assert abs(fd) > 0
        assert abs(ad - fd) <= 1e-6 * abs(fd), (name, ad, fd)


@pytest.mark.parametrize("L,boundary,stencil,reduce,fs", [(1, 2, 0, 1, 0), (2, 1, 1, 0, 0), (2, 0, 0, 1, 0), (1, 2, 0, 1, 1),
                                                           (2, 0, 1, 0, 1), (1, 2, 0, 1, 2)])
def test_oracle_visco3d_adjoint_matches_fp64_finite_differences(refcpu, L, boundary, stencil, reduce, fs):
    """The oracle's FP64 adjoint of the 3-D visco-elastic step (six memory
    variables per mechanism; vp, vs, rho with the relaxation times fixed)
    against central finite differences of its own misfit, with and without
    the free surface (its visco exchange, FreeSurface3Dviscoelastic.cpp)."""
    cfg, model, acq = el3_case(refcpu, fs, boundary, stencil, reduce, L=L)
    true = dict(model)
    y, z, x = np.mgrid[0:cfg.NY, 0:cfg.NZ, 0:cfg.NX]
    blob = np.exp(-((x - cfg.NX * 0.5) ** 2 + (y - cfg.NY * 0.55) ** 2 + (z - cfg.NZ * 0.5) ** 2) / 18.0).reshape(-1)
    true["vp"] = model["vp"] * (1 + 0.05 * blob)
    true["vs"] = model["vs"] * (1 - 0.04 * blob)
    o = refcpu.Oracle(cfg, true, *acq, dtype=np.float64)
    dobs = 0.9 * o.run()
    o.close()
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    J, gvp, gvs, grho = o.adjoint_gradient(dobs, checkpoint_every=37)
    o.close()
    assert J > 0 and J == pytest.approx(misfit(refcpu, cfg, model, acq, dobs), rel=1e-12)
    rng = np.random.default_rng(41)
    grads = dict(vp=gvp, vs=gvs, rho=grho)
    for name in ("vp", "vs", "rho"):
        d = smooth3(rng, cfg) * model[name]
        h = 1e-5
        mp, mm = dict(model), dict(model)
        mp[name] = model[name] + h * d
        mm[name] = model[name] - h * d
        fd = (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)
        ad = float(np.dot(grads[name], d))
        assert abs(fd) > 0
        assert abs(ad - fd) <= 1e-6 * abs(fd), (name, ad, fd)


def em3_case(refcpu, boundary=2, stencil=0, reduce=1, order=4, NX=24, NY=20, NZ=18, nt=120, L=0):
    """3-D EM survey; L > 0: 3-D visco-EM with L relaxation mechanisms."""
    rng = np.random.default_rng(43)
    y, z, x = np.mgrid[0:NY, 0:NZ, 0:NX]
    eps = 5.0 + 6.0 * (y > NY // 2) + 0.4 * np.cos(x / 4.0) + 0.3 * np.sin(z / 3.0) + 0.1 * rng.standard_normal((NY, NZ, NX))
    sig = 10 ** (-3.0 + 0.4 * np.sin(y / 5.0))
    mur = 1.0 + 0.05 * (x > NX // 3)
    fields = dict(eps_r=eps, sigma=sig, mu_r=mur)
    if L:
        fields["tau_eps"] = 0.15 + 0.05 * np.cos(x / 5.0) + 0.02 * np.sin(z / 4.0)
        fields["tau_sigma"] = 0.1 + 0.05 * np.sin(y / 4.0)
    model = {k: v.reshape(-1).astype(np.float64) for k, v in fields.items()}
    DH = 0.02
    DT = 0.3 * DH / (3e8 * np.sqrt(3) * 1.3)
    cfg = refcpu.make_config(dimension=3, equation="viscoemem" if L else "emem", NX=NX, NY=NY, NZ=NZ, DH=DH, DT=DT,
                             T=(nt - 0.4) * DT, spatialFDorder=order, DampingBoundary=boundary, BoundaryWidth=5,
                             DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=5e8, VMaxCPML=1.5e8,
                             useStencilMatrix=stencil, edgeOrderReduction=reduce, numRelaxationMechanisms=L,
                             relaxationFrequency=[3e8, 9e8][:L])
    sidx = np.array([refcpu.grid_index(cfg, NX // 2, 5, NZ // 2), refcpu.grid_index(cfg, NX // 3, 8, NZ // 3)], np.int64)
    sig_t = refcpu.ricker(nt, DT, 7e8, 1.0, 0.0, np.float64)
    rx = np.arange(3, NX - 3, 3)
    ridx = np.concatenate([rx + NX * (NZ // 2 + NZ * 4), rx + NX * (NZ // 2 + NZ * 4), rx + NX * (5 + NZ * (NY - 5)),
                           rx + NX * (12 + NZ * (NY - 5))]).astype(np.int64)
    rtype = np.concatenate([np.full(rx.size, 1), np.full(rx.size, 2), np.full(rx.size, 3), np.full(rx.size, 4)]).astype(np.int32)
    return cfg, model, (sidx, np.array([1, 4], np.int32), np.stack([sig_t, 300.0 * sig_t]), ridx, rtype)


@pytest.mark.parametrize("boundary,stencil,reduce,L", [(2, 0, 1, 0), (1, 1, 0, 0), (0, 0, 1, 0), (2, 0, 1, 1), (1, 0, 0, 2)])
def test_oracle_em3d_adjoint_matches_fp64_finite_differences(refcpu, boundary, stencil, reduce, L):
    """The oracle's FP64 adjoint of the lossless 3-D EM step (gradients with
    respect to eps_r, sigma, mu_r; Ez and Hz sources, Ez / Ex / Ey / Hz
    receivers; L > 0: 3-D visco-EM with the taus fixed) against
    Richardson-extrapolated central finite differences of its own misfit,
    with CPML, ABS and no boundary."""
    cfg, model, acq = em3_case(refcpu, boundary, stencil, reduce, L=L)
    true = dict(model)
    y, z, x = np.mgrid[0:cfg.NY, 0:cfg.NZ, 0:cfg.NX]
    blob = np.exp(-((x - cfg.NX * 0.5) ** 2 + (y - cfg.NY * 0.5) ** 2 + (z - cfg.NZ * 0.5) ** 2) / 18.0).reshape(-1)
    true["eps_r"] = model["eps_r"] * (1 + 0.1 * blob)
    true["sigma"] = model["sigma"] * (1 + 0.5 * blob)
    true["mu_r"] = model["mu_r"] * (1 + 0.05 * blob)
    o = refcpu.Oracle(cfg, true, *acq, dtype=np.float64)
    dobs = 0.9 * o.run()
    o.close()
    o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
    J, ge, gs, gm = o.adjoint_gradient(dobs, checkpoint_every=41)
    o.close()
    assert J > 0 and J == pytest.approx(misfit(refcpu, cfg, model, acq, dobs), rel=1e-12)
    rng = np.random.default_rng(47)
    grads = dict(eps_r=ge, sigma=gs, mu_r=gm)
    for name in ("eps_r", "sigma", "mu_r"):
        d = smooth3(rng, cfg) * model[name]

        def central(h):
            mp, mm = dict(model), dict(model)
            mp[name] = model[name] + h * d
            mm[name] = model[name] - h * d
            return (misfit(refcpu, cfg, mp, acq, dobs) - misfit(refcpu, cfg, mm, acq, dobs)) / (2 * h)

        d1 = central(2e-4)
        fd = d1 - (central(4e-4) - d1) / 3
        ad = float(np.dot(grads[name], d))
        assert abs(fd) > 0
        assert abs(ad - fd) <= 1e-6 * abs(fd), (name, ad, fd)
