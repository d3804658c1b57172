"""Oracle checks for the EM solvers that have no reference golden: visco-TM,
visco-TE, 3-D EM and 3-D visco-EM (ForwardSolverEM/*.cpp). With all relaxation
parameters zero the visco-EM step reduces algebraically to the elastic-free EM
step (effective optical permittivity = static permittivity, C_d = 0), so the
two must agree bit for bit; with relaxation the fields must stay finite and
change. CPU only."""
import numpy as np
import pytest

from oracle import refcpu


def _run(eq, dim, dims, tau=(0.0, 0.0), boundary=2, order=4, nt=160):
    NX, NY, NZ = dims
    n = NX * NY * NZ
    rng = np.random.default_rng(3)
    DH = 0.02
    model = dict(eps_r=rng.uniform(4, 9, n), sigma=10 ** rng.uniform(-4, -2, n), mu_r=np.ones(n),
                 tau_eps=np.full(n, tau[0]), tau_sigma=np.full(n, tau[1]))
    vmax = 3e8 / 2
    DT = 0.35 * DH / (vmax * np.sqrt(dim) * 1.3)
    cfg = refcpu.make_config(dimension=dim, equation=eq, NX=NX, NY=NY, NZ=NZ, DH=DH, DT=DT, T=nt * DT,
                             spatialFDorder=order, FreeSurface=0, DampingBoundary=boundary, BoundaryWidth=6,
                             DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=2e8, VMaxCPML=vmax,
                             numRelaxationMechanisms=2 if eq.startswith("visco") else 0,
                             relaxationFrequency=[1e8, 6e8, 0, 0])
    nt = refcpu.nt_of(cfg)
    sig = refcpu.ricker(nt, DT, vmax / (10 * DH), 1.0, 0.0, np.float64)[None]
    tm = eq.endswith("tmem")
    st = 1 if (tm or dim == 3) else 4
    rtypes = [1] if tm else ([1, 2, 3, 4] if dim == 3 else [2, 3, 4])
    sidx = [refcpu.grid_index(cfg, NX // 2, NY // 2, NZ // 2)]
    ridx = [refcpu.grid_index(cfg, 3 + 5 * k, NY // 3, NZ // 3) for k in range(len(rtypes))]
    o = refcpu.Oracle(cfg, model, np.array(sidx), np.array([st]), sig, np.array(ridx), np.array(rtypes), dtype=np.float64)
    s = o.run()
    o.close()
    return s


@pytest.mark.parametrize("plain,visco,dim,dims,boundary", [
    ("tmem", "viscotmem", 2, (40, 34, 1), 2),
    ("emem", "viscoemem", 2, (40, 34, 1), 1),
    ("emem", "viscoemem", 3, (22, 18, 20), 2),
])
def test_visco_em_without_relaxation_equals_plain_em(plain, visco, dim, dims, boundary):
    a = _run(plain, dim, dims, boundary=boundary)
    b = _run(visco, dim, dims, boundary=boundary)
    assert np.abs(a).max() > 0
    assert np.array_equal(a, b)


@pytest.mark.parametrize("eq,dim,dims", [("viscotmem", 2, (40, 34, 1)), ("viscoemem", 2, (40, 34, 1)),
                                         ("viscoemem", 3, (22, 18, 20))])
def test_visco_em_relaxation_changes_the_response(eq, dim, dims):
    a = _run(eq, dim, dims)
    b = _run(eq, dim, dims, tau=(0.3, 0.5))
    assert np.isfinite(b).all()
    assert np.linalg.norm(a - b) > 1e-3 * np.linalg.norm(a)


def test_3d_em_is_finite_and_absorbed():
    s = _run("emem", 3, (22, 18, 20), boundary=2, nt=400)
    assert np.isfinite(s).all()
    # the CPML absorbs: the late part of the traces is much weaker than the peak
    assert np.abs(s[:, -40:]).max() < 0.2 * np.abs(s).max()


@pytest.mark.parametrize("boundary", [0, 2])
def test_lossless_tmz_oracle_equals_the_pinned_acoustic_oracle(boundary, refcpu):
    """The reference has no EM golden. Lossless 2-D TMz is the 2-D acoustic
    system under Ez <-> p, Hy <-> vx, -Hx <-> vy, 1/eps <-> M, mu <-> rho
    (ForwardSolver2Dtmem.cpp:108-174 against ForwardSolver2Dacoustic.cpp:
    91-190), and the CPML profiles are the same functions of VMaxCPML, DH and
    DT; so on a homogeneous model the EM oracle must reproduce the acoustic
    oracle, which the reference's goldens pin. FP64, CPML or no boundary."""
    eps0, mu0 = 8.854187817e-12, 4e-7 * np.pi
    NX, NY, DH, eps_r, mu_r = 120, 100, 0.02, 4.0, 1.0
    c = 1.0 / np.sqrt(eps_r * eps0 * mu_r * mu0)
    DT = 0.3 * DH / (c * np.sqrt(2.0))
    kw = dict(dimension=2, NX=NX, NY=NY, DH=DH, DT=DT, T=400 * DT, spatialFDorder=4, DampingBoundary=boundary,
              BoundaryWidth=10, NPower=4.0, CenterFrequencyCPML=2e8, VMaxCPML=float(c))
    cfg_a = refcpu.make_config(equation="acoustic", **kw)
    cfg_e = refcpu.make_config(equation="tmem", **kw)
    nt, n = refcpu.nt_of(cfg_a), NX * NY
    sidx = np.array([NX // 2 + NX * (NY // 2)])
    sig = refcpu.ricker(nt, DT, 6e8, 1.0, 0.0, np.float64)[None]
    ridx = np.array([10 + NX * 10, NX - 20 + NX * 30, 40 + NX * (NY - 15), NX // 2 + NX * 3])
    o = refcpu.Oracle(cfg_a, dict(rho=np.full(n, mu_r * mu0), vp=np.full(n, c)), sidx, np.array([1]), sig, ridx,
                      np.ones(4, int), dtype=np.float64)
    p = o.run()
    o.close()
    o = refcpu.Oracle(cfg_e, dict(eps_r=np.full(n, eps_r), sigma=np.zeros(n), mu_r=np.full(n, mu_r)), sidx,
                      np.array([1]), sig, ridx, np.ones(4, int), dtype=np.float64)
    ez = o.run()
    o.close()
    assert np.abs(p).max() > 0
    assert np.linalg.norm(ez - p) / np.linalg.norm(p) < 1e-8


def te_sh_pair(refcpu, order, NX=120, NY=100, nt=150, eps_r=6.0, mu_r=1.2):
    """A lossless TEz survey and the 2-D SH survey it maps onto: rho = mu_r mu0,
    shear modulus 1 / (eps_r eps0) (so vs is the EM wave speed), and every SH
    point one cell up in x and y from its TEz point:
        vz[x, y] = hz[x-1, y-1],  sxz[x, y] = -ey[x, y-1],  syz[x, y] = ex[x-1, y].
    Interior rows satisfy Dxb f[x] = Dxf f[x-1], so the SH update of vz from
    Dxb sxz + Dyb syz is the TEz update of hz from -(Dxf ey - Dyf ex), and the
    SH stress updates from Dxf vz, Dyf vz are the TEz updates of ey, ex from
    Dxb hz, Dyb hz (Ca = 1, Cb = 1 / eps on a homogeneous lossless grid); the
    edge rows differ, so the wavefield must not reach them (no damping
    boundary, a short run). FD2Demem::run (ForwardSolver2Demem.cpp:112-185),
    FD2Dsh::run (ForwardSolver2Dsh.cpp:108-196)."""
    eps0, mu0 = 8.8541878176e-12, 1.2566370614e-6
    DH = 0.02
    c = 3e8 / np.sqrt(eps_r * mu_r)
    DT = 0.3 * DH / (c * np.sqrt(2))
    n = NX * NY
    kw = dict(dimension=2, NX=NX, NY=NY, NZ=1, DH=DH, DT=DT, T=(nt - 0.4) * DT, spatialFDorder=order, DampingBoundary=0,
              FreeSurface=0, edgeOrderReduction=0)
    te = refcpu.make_config(equation="emem", **kw)
    sh = refcpu.make_config(equation="sh", **kw)
    x0, y0 = NX // 2, NY // 2
    sig = refcpu.ricker(nt, DT, c / (12 * DH), 1.0, 0.0, np.float64)[None]
    rx = np.arange(30, 90, 7)
    ry = np.full(rx.size, 35)
    te_model = dict(eps_r=np.full(n, eps_r), sigma=np.zeros(n), mu_r=np.full(n, mu_r))
    sh_model = dict(rho=np.full(n, mu_r * mu0), vs=np.full(n, np.sqrt(1.0 / (eps_r * eps0) / (mu_r * mu0))))
    te_acq = (np.array([x0 + NX * y0], np.int64), np.array([4], np.int32), sig, (rx + NX * ry).astype(np.int64),
              np.full(rx.size, 4, np.int32))
    sh_acq = (np.array([(x0 + 1) + NX * (y0 + 1)], np.int64), np.array([4], np.int32), sig,
              ((rx + 1) + NX * (ry + 1)).astype(np.int64), np.full(rx.size, 4, np.int32))
    return (te, te_model, te_acq), (sh, sh_model, sh_acq)


@pytest.mark.parametrize("order", [2, 4, 8])
def test_lossless_tez_oracle_equals_the_pinned_sh_oracle(order, refcpu):
    """The TEz restatement equals the SH restatement (pinned to the reference's
    2-D SH golden) under the TE/SH analogy: Hz traces equal the mapped vz
    traces bit for bit and the mapped fields agree to rounding."""
    (te, tm, ta), (sh, sm, sa) = te_sh_pair(refcpu, order)
    o = refcpu.Oracle(te, tm, *ta, dtype=np.float64)
    d_te = o.run()
    hz, ex, ey = (o.field(k).reshape(te.NY, te.NX) for k in ("hz", "ex", "ey"))
    o.close()
    o = refcpu.Oracle(sh, sm, *sa, dtype=np.float64)
    d_sh = o.run()
    vz, sxz, syz = (o.field(k).reshape(sh.NY, sh.NX) for k in ("vz", "sxz", "syz"))
    o.close()
    assert np.abs(d_sh).max() > 0
    assert np.array_equal(d_te, d_sh)
    assert np.abs(vz[1:, 1:] - hz[:-1, :-1]).max() <= 1e-12 * np.abs(vz).max()
    assert np.abs(sxz[1:, :] + ey[:-1, :]).max() <= 1e-12 * np.abs(sxz).max()
    assert np.abs(syz[:, 1:] - ex[:, :-1]).max() <= 1e-12 * np.abs(syz).max()


def em3_split_case(refcpu, order, NX=64, NY=56, NZ=48, nt=90, eps_r=5.0, mu_r=1.1):
    """A lossless 3-D EM survey with z-invariant line sources (Ez along z, and a
    Hz line a few cells away) and receivers on the middle z slice, and the
    lossless TMz and TEz surveys its middle slice splits into: with the
    fields constant along z the interior z-derivatives vanish, and the 3-D
    update (ForwardSolver3Demem.cpp:140-237) separates into the TMz step
    (hx, hy, ez; ForwardSolver2Dtmem.cpp:108-174) and the TEz step (hz, ex,
    ey; ForwardSolver2Demem.cpp:112-185). The z edges break the invariance;
    the middle slice stays clear of them for the run's length (no damping
    boundary). Returns (3-D case, TMz case, TEz case), each (cfg, model, acq)."""
    DH = 0.02
    c = 3e8 / np.sqrt(eps_r * mu_r)
    DT = 0.3 * DH / (c * np.sqrt(3))
    base = dict(DH=DH, DT=DT, T=(nt - 0.4) * DT, spatialFDorder=order, DampingBoundary=0, FreeSurface=0,
                edgeOrderReduction=0, NX=NX, NY=NY)
    c3 = refcpu.make_config(dimension=3, equation="emem", NZ=NZ, **base)
    ctm = refcpu.make_config(dimension=2, equation="tmem", NZ=1, **base)
    cte = refcpu.make_config(dimension=2, equation="emem", NZ=1, **base)
    sig = refcpu.ricker(nt, DT, c / (12 * DH), 1.0, 0.0, np.float64)
    x0, y0, zc = NX // 2, NY // 2, NZ // 2
    rx = np.arange(16, 48, 5)
    ry = np.full(rx.size, 18)
    n3, n2 = NX * NY * NZ, NX * NY
    m3 = dict(eps_r=np.full(n3, eps_r), sigma=np.zeros(n3), mu_r=np.full(n3, mu_r))
    m2 = dict(eps_r=np.full(n2, eps_r), sigma=np.zeros(n2), mu_r=np.full(n2, mu_r))
    zs = np.arange(NZ)
    acq3 = (np.concatenate([x0 + NX * (zs + NZ * y0), (x0 - 5) + NX * (zs + NZ * (y0 + 3))]).astype(np.int64),
            np.concatenate([np.full(NZ, 1), np.full(NZ, 4)]).astype(np.int32),
            np.concatenate([np.tile(sig, (NZ, 1)), np.tile(300.0 * sig, (NZ, 1))]),
            np.concatenate([rx + NX * (zc + NZ * ry), rx + NX * (zc + NZ * ry)]).astype(np.int64),
            np.concatenate([np.full(rx.size, 1), np.full(rx.size, 4)]).astype(np.int32))
    acqtm = (np.array([x0 + NX * y0], np.int64), np.array([1], np.int32), sig[None], (rx + NX * ry).astype(np.int64),
             np.full(rx.size, 1, np.int32))
    acqte = (np.array([(x0 - 5) + NX * (y0 + 3)], np.int64), np.array([4], np.int32), 300.0 * sig[None],
             (rx + NX * ry).astype(np.int64), np.full(rx.size, 4, np.int32))
    return (c3, m3, acq3), (ctm, m2, acqtm), (cte, m2, acqte)


@pytest.mark.parametrize("order", [2, 4, 8])
def test_lossless_3d_em_oracle_splits_into_the_pinned_tmz_and_tez(order, refcpu):
    """The 3-D EM restatement on z-invariant sources equals, on its middle
    slice, the TMz and TEz restatements (pinned to the acoustic and SH goldens
    by the maps above): Ez and Hz traces to 1e-11 relative (the residual is
    the z edges' reach through the stencils)."""
    out = []
    for cfg, model, acq in em3_split_case(refcpu, order):
        o = refcpu.Oracle(cfg, model, *acq, dtype=np.float64)
        out.append(o.run())
        o.close()
    d3, dtm, dte = out
    k = dtm.shape[0]
    assert np.abs(dtm).max() > 0 and np.abs(dte).max() > 0
    assert np.linalg.norm(d3[:k] - dtm) <= 1e-11 * np.linalg.norm(dtm)
    assert np.linalg.norm(d3[k:] - dte) <= 1e-11 * np.linalg.norm(dte)
