"""The FP64 adjoint of the acoustic variable-grid step (oracle/vargrid_adjoint.py)
against FP64 central finite differences of its own forward (oracle/vargrid.py
AcousticVarGrid, pinned to the reference's variable-grid goldens): CPML, ABS
or no damping boundary, with and without the mirror free surface, 2-D and
3-D, 1:3 and 1:3:1 grids."""
import numpy as np
import pytest

FD_TOL = 1e-6


def vg_case(refcpu, dim=2, fs=1, boundary=2, edge=1, nt=150, seed=3, equation="acoustic"):
    """A small acoustic variable-grid survey: the oracle's grid, model and
    acquisition, and the config the library takes for the same run."""
    from oracle import vargrid
    if dim == 2:
        NX, NY, NZ, grid = 31, 39, 1, [(0, 1, 4), (12, 3, 4), (27, 1, 4)]
    else:
        NX, NY, NZ, grid = 19, 27, 19, [(0, 1, 4), (12, 3, 2)]
    DH, vmax = 5.0, 3200.0
    DT = 0.3 * DH / (vmax * np.sqrt(dim) * 1.3)
    cfg = refcpu.make_config(dimension=dim, equation=equation, NX=NX, NY=NY, NZ=NZ, DH=DH, DT=DT, T=(nt - 0.5) * DT,
                             spatialFDorder=grid[0][2], FreeSurface=fs, DampingBoundary=boundary,
                             BoundaryWidth=6 if boundary else 0, DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=12.0,
                             VMaxCPML=vmax, edgeOrderReduction=edge, useVariableGrid=1, useVariableFDoperators=1,
                             grid=grid)
    nt = refcpu.nt_of(cfg)
    g = vargrid.VarGrid(NX, NY, NZ, DH, [r[0] for r in grid], [r[1] for r in grid])
    NX, NY, NZ = g.NX, g.NY, g.NZ   # the extents the layering reduces the grid to
    rng = np.random.default_rng(seed)
    vp = 2500.0 + 500.0 * g.y / NY + 60.0 * np.sin(g.x / 4.0) + 20.0 * rng.standard_normal(g.N)
    rho = 1900.0 + 200.0 * (g.y > NY // 2) + 30.0 * np.cos(g.x / 5.0)
    vs = vp / 1.8 + 15.0 * np.cos(g.y / 3.0)
    fc = 4.5 / (nt * DT)
    src = np.asarray(g.coordinate2index([NX // 2], [2 if fs else 5], [NZ // 2]), np.int64)
    sig = refcpu.ricker(nt, DT, fc, 1.0, 0.0, np.float64)[None]
    ys = [1 if fs else 3, grid[1][0] - 1, grid[1][0] + 3, NY - 4, NY // 2]
    types = [1, 2, 3, 1, 4 if dim == 3 else 2]
    rx = [(7 * i + 5) % NX for i in range(len(ys))]
    rz = [(5 * i + 3) % NZ for i in range(len(ys))]
    # receivers on points of the grid (coarse layers hold every third x, y, z)
    y0, y1 = grid[1][0], grid[2][0] if len(grid) > 2 else NY
    f = [3 if y0 <= y < y1 else 1 for y in ys]
    ys = [y - (y - y0) % 3 if y0 <= y < y1 else y for y in ys]
    rx = [x - x % k for x, k in zip(rx, f)]
    rz = [0 if dim == 2 else z - z % k for z, k in zip(rz, f)]
    ridx = np.array([int(g.coordinate2index(x, y, z)) for x, y, z in zip(rx, ys, rz)], np.int64)
    cp = damp = None
    if boundary == 2:
        cp = vargrid.cpml_coefficients(g, 6, 4.0, 12.0, vmax, DT, fs != 0, np.float64)
    elif boundary == 1:
        damp = vargrid.abs_damping(g, 6, 8.0, fs != 0, np.float64)
    return dict(cfg=cfg, g=g, orders=[r[2] for r in grid], nt=nt, DT=DT, fs=fs, cpml=cp, damping=damp, vp=vp, vs=vs, rho=rho,
                src_idx=src, src_type=np.array([1], np.int32), signals=sig, rec_idx=ridx,
                rec_type=np.array(types, np.int32), edge=bool(edge))


def vg_seismograms(c, vp, rho):
    from oracle import vargrid
    sim = vargrid.AcousticVarGrid(c["g"], c["orders"], c["DT"], rho, vp, c["fs"], c["cpml"], c["src_idx"], c["src_type"],
                                  c["signals"], c["rec_idx"], c["rec_type"], dtype=np.float64, edge=c["edge"],
                                  damping=c["damping"])
    return sim.run(c["nt"])


def vg_observed(c):
    """0.8 x the data of a model with a smooth velocity anomaly."""
    g = c["g"]
    blob = np.exp(-((g.x - g.NX * 0.5) ** 2 + (g.y - g.NY * 0.6) ** 2 + (g.z - g.NZ * 0.5) ** 2) / 40.0)
    return 0.8 * vg_seismograms(c, c["vp"] * (1 + 0.05 * blob), c["rho"])


def _misfit(c, vp, rho, dobs):
    r = vg_seismograms(c, vp, rho) - dobs
    return 0.5 * float(np.sum(r * r))


def _gradient(c, dobs):
    from oracle.vargrid_adjoint import adjoint_gradient
    return adjoint_gradient(c["g"], c["orders"], c["DT"], c["rho"], c["vp"], c["fs"], c["cpml"], c["src_idx"],
                            c["src_type"], c["signals"], c["rec_idx"], c["rec_type"], dobs, damping=c["damping"],
                            edge=c["edge"])


@pytest.mark.parametrize("dim,fs,boundary,edge", [(2, 1, 2, 1), (2, 0, 1, 0), (2, 1, 0, 1), (3, 1, 2, 1), (3, 0, 1, 1),
                                                 (2, 2, 2, 1)])
def test_oracle_vargrid_adjoint_matches_fp64_finite_differences(refcpu, dim, fs, boundary, edge):
    c = vg_case(refcpu, dim, fs, boundary, edge, nt=120 if dim == 3 else 150)
    dobs = vg_observed(c)
    J, gvp, grho = _gradient(c, dobs)
    assert abs(J - _misfit(c, c["vp"], c["rho"], dobs)) <= 1e-12 * J
    g = c["g"]
    rng = np.random.default_rng(11)
    for name, grad in (("vp", gvp), ("rho", grho)):
        base = c[name]
        smooth = np.sin(g.x / 3.0 + rng.uniform(0, 6)) * np.cos(g.y / 4.0 + rng.uniform(0, 6)) + 0.3 * np.sin(g.z / 2.5)
        dm = smooth * base
        h = 1e-5
        args = {k: c[k] for k in ("vp", "rho")}
        plus = dict(args, **{name: base + h * dm})
        minus = dict(args, **{name: base - h * dm})
        fd = (_misfit(c, plus["vp"], plus["rho"], dobs) - _misfit(c, minus["vp"], minus["rho"], dobs)) / (2 * h)
        ad = float(np.dot(grad, dm))
        assert abs(fd) > 0
        assert abs(ad - fd) <= FD_TOL * abs(fd), f"{name}: adjoint {ad:.9e} vs finite difference {fd:.9e}"


def vge_seismograms(c, vp, vs, rho):
    from oracle.vargrid_elastic import ElasticVarGrid2D, ElasticVarGrid3D
    sim = (ElasticVarGrid3D if c["g"].NZ > 1 else ElasticVarGrid2D)(c["g"], c["orders"], c["DT"], rho, vp, vs, c["cpml"], c["src_idx"], c["src_type"], c["signals"],
                           c["rec_idx"], c["rec_type"], dtype=np.float64, edge=c["edge"], free_surface=c["fs"] == 1,
                           damping=c["damping"])
    return sim.run(c["nt"])


def vge_observed(c):
    """0.8 x the data of a model with smooth vp and vs anomalies."""
    g = c["g"]
    blob = np.exp(-((g.x - g.NX * 0.5) ** 2 + (g.y - g.NY * 0.6) ** 2 + (g.z - g.NZ * 0.5) ** 2) / 40.0)
    return 0.8 * vge_seismograms(c, c["vp"] * (1 + 0.05 * blob), c["vs"] * (1 - 0.04 * blob), c["rho"])


def vge_gradient(c, dobs):
    from oracle.vargrid_adjoint import elastic_adjoint_gradient_2d, elastic_adjoint_gradient_3d
    fn = elastic_adjoint_gradient_3d if c["g"].NZ > 1 else elastic_adjoint_gradient_2d
    return fn(c["g"], c["orders"], c["DT"], c["rho"], c["vp"], c["vs"], c["cpml"], c["src_idx"],
                                       c["src_type"], c["signals"], c["rec_idx"], c["rec_type"], dobs,
                                       damping=c["damping"], free_surface=c["fs"] == 1, edge=c["edge"])


@pytest.mark.parametrize("dim,fs,boundary,edge", [(2, 1, 2, 1), (2, 0, 1, 0), (2, 1, 0, 1), (2, 0, 2, 1), (3, 1, 2, 1),
                                                 (3, 0, 1, 1)])
def test_oracle_elastic_vargrid_adjoint_matches_fp64_finite_differences(refcpu, dim, fs, boundary, edge):
    c = vg_case(refcpu, dim, fs, boundary, edge, nt=160 if dim == 2 else 110, equation="elastic")
    dobs = vge_observed(c)
    J, gvp, gvs, grho = vge_gradient(c, dobs)
    r = vge_seismograms(c, c["vp"], c["vs"], c["rho"]) - dobs
    assert abs(J - 0.5 * float(np.sum(r * r))) <= 1e-12 * J
    g = c["g"]
    rng = np.random.default_rng(13)
    for name, grad in (("vp", gvp), ("vs", gvs), ("rho", grho)):
        base = c[name]
        dm = (np.sin(g.x / 3.0 + rng.uniform(0, 6)) * np.cos(g.y / 4.0 + rng.uniform(0, 6))) * base
        h = 1e-5
        fd = []
        for sgn in (1.0, -1.0):
            m = {k: c[k] for k in ("vp", "vs", "rho")}
            m[name] = base + sgn * h * dm
            rr = vge_seismograms(c, m["vp"], m["vs"], m["rho"]) - dobs
            fd.append(0.5 * float(np.sum(rr * rr)))
        fd = (fd[0] - fd[1]) / (2 * h)
        ad = float(np.dot(grad, dm))
        assert abs(fd) > 0
        assert abs(ad - fd) <= FD_TOL * abs(fd), f"{name}: adjoint {ad:.9e} vs finite difference {fd:.9e}"
