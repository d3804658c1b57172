"""The variable-grid oracle against the reference's variable-grid goldens
(par/ci/seismogram.{2D,3D}.acoustic.varGrid.ref.p.mtx, gate of
Test_CompareSeismogram.cpp:57-88), and the library's grid index space
(wave_grid_*, no GPU needed) against the oracle's restatement of
Acquisition/Coordinates.cpp."""
import numpy as np
import pytest

import ci_cases

GATE = 5e-7


def test_vargrid_oracle_matches_2d_golden(refcpu):
    case = ci_cases.load_vargrid_case("2D.acoustic.varGrid")
    seis = ci_cases.run_vargrid_oracle(case, np.float32)
    g = case["golden"]
    assert seis.shape == g.shape
    assert refcpu.reference_misfit(seis, g) < GATE


def test_vargrid_oracle_matches_3d_golden(refcpu):
    case = ci_cases.load_vargrid_case("3D.acoustic.varGrid")
    seis = ci_cases.run_vargrid_oracle(case, np.float32)
    g = case["golden"]
    assert seis.shape == g.shape
    assert refcpu.reference_misfit(seis, g) < GATE


def test_vargrid_goldens_predate_edge_order_reduction(refcpu):
    """As for the regular-grid goldens: with the current edge rule
    (Derivatives.cpp:166-179) the 2-D variable-grid golden fails the gate."""
    case = ci_cases.load_vargrid_case("2D.acoustic.varGrid", edge_order_reduction=1)
    case["cfg"].edgeOrderReduction = 1
    seis = ci_cases.run_vargrid_oracle(case, np.float32)
    assert refcpu.reference_misfit(seis, case["golden"]) > 10 * GATE


GRIDS = [
    # (dimension, NX, NY, NZ, [(interface, dhFactor, order), ...])
    (2, 305, 303, 1, [(0, 1, 2), (30, 3, 6), (150, 1, 2), (200, 3, 6)]),     # the CI grid
    (3, 104, 303, 104, [(0, 1, 2), (30, 3, 6), (150, 1, 2), (200, 3, 6)]),
    (2, 120, 100, 1, [(0, 1, 4), (31, 3, 4), (70, 9, 2)]),                    # interfaces moved to whole cells
    (3, 40, 61, 47, [(0, 1, 4), (20, 3, 6)]),
    (2, 50, 60, 1, [(0, 1, 2), (25, 1, 8)]),                                  # variable FD orders only
]


def _cfg(wave, refcpu, dim, NX, NY, NZ, grid, var_grid=True):
    kw = dict(dimension=dim, equation="acoustic", NX=NX, NY=NY, NZ=NZ, DH=10.0, DT=1e-3, T=0.1,
              spatialFDorder=2, useVariableGrid=int(var_grid), useVariableFDoperators=1, grid=grid)
    return wave.WaveConfig.make(**kw), refcpu.make_config(**kw)


@pytest.mark.parametrize("k", range(len(GRIDS)))
def test_library_grid_index_space_matches_oracle(k, wave, refcpu):
    from oracle import vargrid
    dim, NX, NY, NZ, grid = GRIDS[k]
    var_grid = any(r[1] != 1 for r in grid)
    c, _ = _cfg(wave, refcpu, dim, NX, NY, NZ, grid, var_grid)
    g = vargrid.VarGrid(NX, NY, NZ, 10.0, [r[0] for r in grid], [r[1] for r in grid] if var_grid else [1] * len(grid))
    assert wave.grid_num_points(c) == g.N
    x, y, z, ext = wave.grid_coordinates(c)
    assert ext == (g.NX, g.NY, g.NZ)
    np.testing.assert_array_equal(x, g.x)
    np.testing.assert_array_equal(y, g.y)
    np.testing.assert_array_equal(z, g.z)
    rng = np.random.default_rng(k)
    for _ in range(200):
        X, Y, Z = rng.integers(0, g.NX), rng.integers(0, g.NY), rng.integers(0, g.NZ)
        try:
            want = int(g.coordinate2index(X, Y, Z))
        except IndexError:
            with pytest.raises(wave.WaveError):
                wave.grid_index(c, X, Y, Z)
            continue
        assert wave.grid_index(c, X, Y, Z) == want
    # index -> coordinate -> index is the identity
    sel = rng.integers(0, g.N, 500)
    np.testing.assert_array_equal(g.coordinate2index(g.x[sel], g.y[sel], g.z[sel]), sel)


def test_regular_grid_index_space(wave):
    c = wave.WaveConfig.make(dimension=3, NX=7, NY=5, NZ=3, DH=1.0, DT=1e-3, T=0.01)
    assert wave.grid_num_points(c) == 105
    assert wave.grid_index(c, 2, 3, 1) == 2 + 1 * 7 + 3 * 21
    x, y, z, ext = wave.grid_coordinates(c)
    assert ext == (7, 5, 3)
    assert (x[2 + 7 + 63], y[2 + 7 + 63], z[2 + 7 + 63]) == (2, 3, 1)


@pytest.mark.parametrize("name", sorted(ci_cases.VARGRID_CASES))
def test_parameter_reader_reads_the_grid_configuration(name, wave, refcpu):
    import ctypes
    import os
    path = os.path.join(ci_cases.CI, ci_cases.VARGRID_CASES[name][0])
    mine = wave.WaveConfig.from_file(path)
    ref = refcpu.config_from_parameters(refcpu.read_parameter_file(path), base_dir=ci_cases.CI)
    for f, _ in wave.WaveConfig._fields_:
        a, b = getattr(mine, f), getattr(ref, f)
        assert (list(a) == list(b)) if isinstance(a, ctypes.Array) else (a == b), f
    assert mine.useVariableGrid == 1 and mine.gridLayers == 4
    assert list(mine.gridDHFactor)[:4] == [1, 3, 1, 3] and list(mine.gridFDOrder)[:4] == [2, 6, 2, 6]


def test_invalid_grid_configurations_are_rejected(wave, refcpu):
    bad = [
        [(1, 1, 2), (30, 3, 2)],          # first interface not at y = 0
        [(0, 1, 2), (30, 2, 2)],          # factor 2
        [(0, 1, 2), (30, 9, 2)],          # jump 1 -> 9
        [(0, 1, 2), (30, 3, 5)],          # odd order
    ]
    for grid in bad:
        c, _ = _cfg(wave, refcpu, 2, 100, 100, 1, grid)
        with pytest.raises(wave.WaveError):
            wave.grid_num_points(c)


OPERATOR_CASES = [
    # (configuration, edge rule, free surface); the CI grids and a 3-D 1:3:1 grid
    ("2D.acoustic.varGrid", 0, None),
    ("2D.acoustic.varGrid", 1, 0),
    ("3D.acoustic.varGrid", 0, None),
]


def _ell_to_csr(cols, vals, n):
    import scipy.sparse as sp
    w = cols.shape[0]
    rows = np.tile(np.arange(n), w)
    m = sp.csr_matrix((vals.ravel().astype(np.float64), (rows, cols.ravel())), shape=(n, n))
    m.eliminate_zeros()
    return m


@pytest.mark.parametrize("name,edge,fs", OPERATOR_CASES)
def test_library_operators_equal_the_oracle_entry_for_entry(name, edge, fs, wave, refcpu):
    """The library's host-assembled variable-grid operators (wave_grid_operator)
    against the oracle's row-by-row restatement of Derivatives.cpp: every
    column and every FP32 weight equal, for the six derivative operators and
    the three interface interpolations."""
    import ctypes
    from oracle import vargrid
    case = ci_cases.load_vargrid_case(name, edge_order_reduction=edge)
    cfg = case["cfg"]
    if fs is not None:
        cfg.FreeSurface = fs
    c = wave.WaveConfig()
    ctypes.memmove(ctypes.byref(c), ctypes.byref(cfg), ctypes.sizeof(c))
    g = case["grid"]
    op = vargrid.Operators(g, case["orders"], cfg.DT, cfg.FreeSurface == 1, np.float32, True, bool(edge), True)
    mats = [op.Dxf, op.Dyf, getattr(op, "Dzf", None), op.Dxb, op.Dyb, getattr(op, "Dzb", None),
            op.IFull, op.IStagX, getattr(op, "IStagZ", None)]
    for k, want in enumerate(mats):
        if want is None:
            continue
        cols, vals = wave.grid_operator(c, k)
        got = _ell_to_csr(cols, vals, g.N)
        want = want.astype(np.float64).tocsr()
        want.eliminate_zeros()
        diff = abs(got - want)
        assert diff.nnz == 0 or diff.max() == 0, (k, diff.max())


@pytest.mark.parametrize("dim,edge,fs,boundary", [(2, 1, 1, 2), (2, 0, 0, 2), (3, 1, 0, 2), (2, 1, 1, 1), (2, 0, 0, 1),
                                                   (3, 1, 1, 1)])
def test_single_layer_vargrid_oracle_equals_the_regular_grid_oracle(dim, edge, fs, boundary, refcpu):
    """With one layer the variable-grid restatement must reduce to the regular
    grid: the two oracles (scipy CSR and the C++ refcpu) agree in FP64, with
    CPML or ABS."""
    from oracle import vargrid
    NX, NY, NZ = (60, 50, 1) if dim == 2 else (24, 22, 20)
    DH, order = 5.0, 4
    DT = 0.3 * DH / (3000.0 * np.sqrt(dim))
    nt = 150
    cfg = refcpu.make_config(dimension=dim, equation="acoustic", NX=NX, NY=NY, NZ=NZ, DH=DH, DT=DT, T=nt * DT,
                             spatialFDorder=order, FreeSurface=fs, DampingBoundary=boundary, BoundaryWidth=8, NPower=4.0,
                             CenterFrequencyCPML=20.0, VMaxCPML=3000.0, edgeOrderReduction=edge, DampingCoeff=8.0)
    nt = refcpu.nt_of(cfg)
    rng = np.random.default_rng(dim)
    n = NX * NY * NZ
    vp = rng.uniform(2400.0, 3000.0, n)
    rho = 310.0 * vp ** 0.25
    sidx = np.array([NX // 2 + NX * NZ * (3 if fs else NY // 3) + NX * (NZ // 2)])
    sig = refcpu.ricker(nt, DT, 30.0, 1.0, 0.0, np.float64)[None]
    ridx = np.array([5 + NX * NZ * 10, NX - 6 + NX * NZ * (NY - 4), 7 + NX * NZ * 20])
    rtype = np.array([1, 2, 3])
    o = refcpu.Oracle(cfg, dict(rho=rho, vp=vp), sidx, np.array([1]), sig, ridx, rtype, dtype=np.float64)
    ref = o.run()
    o.close()
    g = vargrid.VarGrid(NX, NY, NZ, DH, [0], [1])
    cp = vargrid.cpml_coefficients(g, 8, 4.0, 20.0, 3000.0, DT, fs != 0, np.float64) if boundary == 2 else None
    damp = vargrid.abs_damping(g, 8, 8.0, fs != 0, np.float64) if boundary == 1 else None
    sim = vargrid.AcousticVarGrid(g, [order], DT, rho, vp, fs, cp, sidx, [1], sig, ridx, rtype, dtype=np.float64,
                                  var_order=False, edge=bool(edge), var_grid=False, damping=damp)
    got = sim.run(nt)
    assert np.abs(ref).max() > 0
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-9
