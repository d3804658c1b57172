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
