"""GPU parity of the 2-D elastic step on the variable grid (vargrid.cu:
vge_vel / vge_str with the interface interpolations, through the C ABI)
against the FP64 variable-grid elastic oracle (oracle/vargrid_elastic.py,
itself tied to the pinned regular-grid oracle in
tests/test_oracle_vargrid_elastic.py).

The step is FD2Delastic::run (ForwardSolver2Delastic.cpp:117-297) and
FD3Delastic::run (ForwardSolver3Delastic.cpp:120-414) on the layered grid of
Coordinates (Coordinates.cpp:119-245), with DyfStaggeredX / DybStaggeredX
(Derivatives.cpp:852-1011), DyfStaggeredZ / DybStaggeredZ (:1012-1168) and
the StaggeredXZ interpolation (:1568-1661), CPML, ABS or no damping
boundary, with or without the mirror free surface (DybStaggeredX / ZFreeSurface,
DyfFreeSurface and the surface exchange).

Tolerance: relative L2 over all traces and samples <= 1e-4 against FP64."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-4

# (NX, NY, grid rows (first y, dhFactor, order), variable grid, damping boundary, edge reduction, free surface)
CASES = [
    (122, 100, [(0, 1, 4), (31, 3, 4), (70, 1, 4)], 1, 2, 0, 0),
    (122, 100, [(0, 1, 4), (31, 3, 6), (70, 1, 4)], 1, 2, 1, 0),
    (113, 96, [(0, 1, 2), (30, 3, 2), (57, 9, 2)], 1, 0, 0, 0),
    (90, 80, [(0, 1, 2), (40, 1, 8)], 0, 2, 1, 0),
    (122, 100, [(0, 1, 4), (31, 3, 6), (70, 1, 4)], 1, 2, 1, 1),
    (113, 96, [(0, 1, 6), (30, 3, 2), (57, 9, 2)], 1, 0, 0, 1),
    (122, 100, [(0, 1, 4), (31, 3, 4), (70, 1, 4)], 1, 1, 0, 0),
    (113, 96, [(0, 1, 4), (30, 3, 2), (57, 9, 2)], 1, 1, 1, 1),
]


def _case(refcpu, k):
    from oracle import vargrid
    NX, NY, grid, vgrid, boundary, edge, fs = CASES[k]
    DH, vmax = 5.0, 3200.0
    DT = 0.3 * DH / (vmax * np.sqrt(2.0) * 1.3)
    nt = 500
    cfg = refcpu.make_config(dimension=2, equation="elastic", NX=NX, NY=NY, NZ=1, DH=DH, DT=DT, T=nt * DT,
                             spatialFDorder=grid[0][2], FreeSurface=fs, DampingBoundary=boundary,
                             BoundaryWidth=12 if boundary else 0, DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=12.0,
                             VMaxCPML=vmax, edgeOrderReduction=edge, useVariableGrid=vgrid,
                             useVariableFDoperators=1, grid=grid)
    g = vargrid.VarGrid(NX, NY, 1, DH, [r[0] for r in grid], [r[1] for r in grid] if vgrid else [1] * len(grid))
    nt = refcpu.nt_of(cfg)
    rng = np.random.default_rng(40 + k)
    vp = rng.uniform(2600.0, vmax, g.N).astype(np.float32)
    vs = (vp / rng.uniform(1.7, 1.9, g.N)).astype(np.float32)
    rho = (310.0 * vp.astype(np.float64) ** 0.25 * rng.uniform(0.9, 1.1, g.N)).astype(np.float32)
    fc = 4.5 / (nt * DT)
    src = g.coordinate2index([g.NX // 2], [4 if fs else g.NY // 5], [0])
    sig = refcpu.ricker(nt, DT, fc, 1.0, 0.0, np.float64)[None]
    ys = [0 if fs else 3, grid[1][0] - 1, grid[1][0] + 4, g.NY - 3, g.NY // 2, grid[1][0], 0, 1]
    types = [1, 2, 3, 1, 2, 3, 2, 3]
    rx = [(7 * i + 5) % g.NX for i in range(len(ys))]
    ridx = np.array([int(g.coordinate2index(x, y, 0)) for x, y in zip(rx, ys)], np.int64)
    return dict(cfg=cfg, g=g, orders=[r[2] for r in grid], nt=nt, model=dict(rho=rho, vp=vp, vs=vs),
                src=np.asarray(src, np.int64), stype=np.array([1], np.int32), sig=sig, ridx=ridx,
                rtype=np.array(types, np.int32))


def _oracle(case, dtype=np.float64):
    from oracle import vargrid, vargrid_elastic
    cfg, g = case["cfg"], case["g"]
    cp = None
    if cfg.DampingBoundary == 2:
        cp = vargrid.cpml_coefficients(g, cfg.BoundaryWidth, cfg.NPower, cfg.CenterFrequencyCPML, cfg.VMaxCPML, cfg.DT,
                                       cfg.FreeSurface != 0, dtype)
    damp = vargrid.abs_damping(g, cfg.BoundaryWidth, cfg.DampingCoeff, cfg.FreeSurface != 0, dtype) \
        if cfg.DampingBoundary == 1 else None
    m = {k: v.astype(dtype) for k, v in case["model"].items()}
    sim = vargrid_elastic.ElasticVarGrid2D(g, case["orders"], cfg.DT, m["rho"], m["vp"], m["vs"], cp, case["src"],
                                           case["stype"], case["sig"].astype(dtype), case["ridx"], case["rtype"],
                                           dtype=dtype, var_order=bool(cfg.useVariableFDoperators),
                                           edge=bool(cfg.edgeOrderReduction), var_grid=bool(cfg.useVariableGrid),
                                           free_surface=cfg.FreeSurface != 0, damping=damp)
    return sim.run(case["nt"])


def _gpu(wave, case, kernel_path=0):
    c = wave.WaveConfig()
    ctypes.memmove(ctypes.byref(c), ctypes.byref(case["cfg"]), ctypes.sizeof(c))
    return wave.simulate(c, case["model"], case["src"], case["stype"], case["sig"].astype(np.float32), case["ridx"],
                         case["rtype"], kernel_path=kernel_path)


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def _rel_groups(a, b, rtype):
    """Relative L2 of the pressure traces and of the velocity traces, each
    over its own group (velocities are some 1e-7 of the stresses in SI
    units, so a pooled figure would not see them): the larger of the two."""
    p = rtype == 1
    return max(_rel(a[g], b[g]) for g in (p, ~p) if g.any())


@pytest.mark.parametrize("k", range(len(CASES)))
def test_elastic_vargrid_matches_fp64_oracle(k, wave, refcpu):
    case = _case(refcpu, k)
    gpu = _gpu(wave, case)
    ref = _oracle(case)
    assert np.abs(ref).max() > 0 and np.isfinite(gpu).all()
    err = _rel_groups(gpu, ref, case["rtype"])
    print(f"elastic variable grid case {k}: rel L2 vs FP64 oracle {err:.2e}")
    assert err < TOL, err


def test_elastic_vargrid_fused_and_separate_source_launch_agree(wave, refcpu):
    """Sources and receivers ride in the stress interpolation launch unless
    kernel path 1 asks for the separate launch: the same bits."""
    case = _case(refcpu, 0)
    np.testing.assert_array_equal(_gpu(wave, case, 0), _gpu(wave, case, 1))


# (NX, NY, NZ, grid rows, variable grid, damping boundary, edge reduction, free surface)
CASES_3D = [
    (49, 60, 49, [(0, 1, 4), (21, 3, 4), (42, 1, 4)], 1, 2, 0, 0),
    (55, 48, 37, [(0, 1, 2), (12, 3, 6), (30, 9, 2)], 1, 0, 1, 0),
    (40, 38, 36, [(0, 1, 4), (20, 1, 6)], 0, 2, 1, 0),
    (49, 60, 49, [(0, 1, 4), (21, 3, 4), (42, 1, 4)], 1, 2, 0, 1),
    (49, 60, 49, [(0, 1, 4), (21, 3, 4), (42, 1, 4)], 1, 1, 0, 1),
]


def _case3d(refcpu, k):
    from oracle import vargrid
    NX, NY, NZ, grid, vgrid, boundary, edge, fs = CASES_3D[k]
    DH, vmax = 5.0, 3200.0
    DT = 0.3 * DH / (vmax * np.sqrt(3.0) * 1.3)
    nt = 300
    cfg = refcpu.make_config(dimension=3, equation="elastic", NX=NX, NY=NY, NZ=NZ, DH=DH, DT=DT, T=nt * DT,
                             spatialFDorder=grid[0][2], FreeSurface=fs, DampingBoundary=boundary,
                             BoundaryWidth=8 if boundary else 0, DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=15.0,
                             VMaxCPML=vmax, edgeOrderReduction=edge, useVariableGrid=vgrid,
                             useVariableFDoperators=1, grid=grid)
    g = vargrid.VarGrid(NX, NY, NZ, DH, [r[0] for r in grid], [r[1] for r in grid] if vgrid else [1] * len(grid))
    nt = refcpu.nt_of(cfg)
    rng = np.random.default_rng(70 + k)
    vp = rng.uniform(2600.0, vmax, g.N).astype(np.float32)
    vs = (vp / rng.uniform(1.7, 1.9, g.N)).astype(np.float32)
    rho = (310.0 * vp.astype(np.float64) ** 0.25 * rng.uniform(0.9, 1.1, g.N)).astype(np.float32)
    fc = 4.5 / (nt * DT)
    src = g.coordinate2index([g.NX // 2], [4 if fs else g.NY // 5], [g.NZ // 2])
    sig = refcpu.ricker(nt, DT, fc, 1.0, 0.0, np.float64)[None]
    # stored points away from the side frames, spread over the index space
    # (every layer, interface rows included)
    inner = np.nonzero((g.x >= 5) & (g.x < g.NX - 5) & (g.z >= 5) & (g.z < g.NZ - 5))[0]
    ridx = inner[np.linspace(0, len(inner) - 1, 9).astype(np.int64)].astype(np.int64)
    types = [1, 2, 3, 4, 1, 4, 3, 2, 1]
    if fs:   # surface receivers as well
        top = g.coordinate2index([g.NX // 3, g.NX // 2 + 4, g.NX // 4], [0, 0, 1], [g.NZ // 2, g.NZ // 3, g.NZ // 2 + 3])
        ridx = np.concatenate([ridx, np.asarray(top, np.int64)])
        types = types + [2, 3, 4]
    return dict(cfg=cfg, g=g, orders=[r[2] for r in grid], nt=nt, model=dict(rho=rho, vp=vp, vs=vs),
                src=np.asarray(src, np.int64), stype=np.array([1], np.int32), sig=sig, ridx=ridx,
                rtype=np.array(types, np.int32))


def _oracle3d(case, dtype=np.float64):
    from oracle import vargrid, vargrid_elastic
    cfg, g = case["cfg"], case["g"]
    cp = None
    if cfg.DampingBoundary == 2:
        cp = vargrid.cpml_coefficients(g, cfg.BoundaryWidth, cfg.NPower, cfg.CenterFrequencyCPML, cfg.VMaxCPML, cfg.DT,
                                       cfg.FreeSurface != 0, dtype)
    damp = vargrid.abs_damping(g, cfg.BoundaryWidth, cfg.DampingCoeff, cfg.FreeSurface != 0, dtype) \
        if cfg.DampingBoundary == 1 else None
    m = {k: v.astype(dtype) for k, v in case["model"].items()}
    sim = vargrid_elastic.ElasticVarGrid3D(g, case["orders"], cfg.DT, m["rho"], m["vp"], m["vs"], cp, case["src"],
                                           case["stype"], case["sig"].astype(dtype), case["ridx"], case["rtype"],
                                           dtype=dtype, var_order=bool(cfg.useVariableFDoperators),
                                           edge=bool(cfg.edgeOrderReduction), var_grid=bool(cfg.useVariableGrid),
                                           free_surface=cfg.FreeSurface != 0, damping=damp)
    return sim.run(case["nt"])


@pytest.mark.parametrize("k", range(len(CASES_3D)))
def test_3d_elastic_vargrid_matches_fp64_oracle(k, wave, refcpu):
    case = _case3d(refcpu, k)
    gpu = _gpu(wave, case)
    ref = _oracle3d(case)
    assert np.abs(ref).max() > 0 and np.isfinite(gpu).all()
    err = _rel_groups(gpu, ref, case["rtype"])
    print(f"3-D elastic variable grid case {k}: rel L2 vs FP64 oracle {err:.2e}")
    assert err < TOL, err
