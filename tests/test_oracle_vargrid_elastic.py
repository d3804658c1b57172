"""The 2-D elastic variable-grid oracle (oracle/vargrid_elastic.py), checker
of the variable-grid elastic GPU path (tests/test_gpu_vargrid_elastic.py). The reference has no elastic
variable-grid golden, so it is tied to the pinned regular-grid oracle: with
one layer the two must agree to rounding, and on a 1:3:1 grid the receivers
in the fine layers must track an all-fine regular run."""
import numpy as np
import pytest


def _model(n, rng):
    vp = rng.uniform(2400.0, 3000.0, n)
    return 310.0 * vp ** 0.25, vp, vp / 1.8


@pytest.mark.parametrize("boundary,fs", [(2, 0), (0, 0), (2, 1), (0, 1), (1, 0), (1, 1)])
def test_single_layer_elastic_vargrid_equals_regular_oracle(boundary, fs, refcpu):
    from oracle import vargrid as vg, vargrid_elastic as ve
    NX, NY, DH, order, vmax = 70, 60, 5.0, 4, 3000.0
    DT = 0.3 * DH / (vmax * np.sqrt(2.0))
    cfg = refcpu.make_config(dimension=2, equation="elastic", NX=NX, NY=NY, DH=DH, DT=DT, T=300 * DT,
                             spatialFDorder=order, DampingBoundary=boundary, BoundaryWidth=8, NPower=4.0,
                             CenterFrequencyCPML=20.0, VMaxCPML=vmax, edgeOrderReduction=0, FreeSurface=fs,
                             DampingCoeff=8.0)
    nt = refcpu.nt_of(cfg)
    rho, vp, vs = _model(NX * NY, np.random.default_rng(1))
    sidx = np.array([NX // 2 + NX * (NY // 3)])
    sig = refcpu.ricker(nt, DT, 30.0, 1.0, 0.0, np.float64)[None]
    ridx = np.array([5 + NX * 10, NX - 6 + NX * (NY - 4), 7 + NX * 20])
    rtype = np.array([1, 2, 3])
    o = refcpu.Oracle(cfg, dict(rho=rho, vp=vp, vs=vs), sidx, np.array([1]), sig, ridx, rtype, dtype=np.float64)
    ref = o.run()
    o.close()
    g = vg.VarGrid(NX, NY, 1, DH, [0], [1])
    cp = vg.cpml_coefficients(g, 8, 4.0, 20.0, vmax, DT, fs != 0, np.float64) if boundary == 2 else None
    damp = vg.abs_damping(g, 8, 8.0, fs != 0, np.float64) if boundary == 1 else None
    sim = ve.ElasticVarGrid2D(g, [order], DT, rho, vp, vs, cp, sidx, [1], sig, ridx, rtype, dtype=np.float64,
                              var_order=False, edge=False, var_grid=False, free_surface=fs != 0, damping=damp)
    got = sim.run(nt)
    assert np.abs(ref).max() > 0
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12


def test_elastic_vargrid_tracks_the_all_fine_grid(refcpu):
    from oracle import vargrid as vg, vargrid_elastic as ve
    NX, NY, DH = 122, 100, 5.0
    vp0, vs0, rho0, fc = 3000.0, 1700.0, 2200.0, 8.0
    DT = 0.3 * DH / (vp0 * np.sqrt(2.0) * 1.2)
    nt = 1400
    grid = [(0, 1, 4), (40, 3, 4), (70, 1, 4)]
    g = vg.VarGrid(NX, NY, 1, DH, [r[0] for r in grid], [r[1] for r in grid])
    sig = refcpu.ricker(nt, DT, fc, 1.0, 0.0, np.float64)[None]
    sx, sy = 60, 20
    recs = [(30, 10), (90, 25), (60, 85)]          # fine layers above and below the coarse one
    cp = vg.cpml_coefficients(g, 12, 4.0, fc, vp0, DT, False, np.float64)
    sidx = g.coordinate2index([sx], [sy], [0])
    ridx = g.coordinate2index([r[0] for r in recs], [r[1] for r in recs], [0] * len(recs))
    sim = ve.ElasticVarGrid2D(g, [r[2] for r in grid], DT, np.full(g.N, rho0), np.full(g.N, vp0), np.full(g.N, vs0),
                              cp, sidx, [1], sig, ridx, [1] * len(recs), dtype=np.float64, edge=False)
    a = sim.run(nt)
    cfg = refcpu.make_config(dimension=2, equation="elastic", NX=g.NX, NY=g.NY, DH=DH, DT=DT, T=nt * DT,
                             spatialFDorder=4, DampingBoundary=2, BoundaryWidth=12, NPower=4.0,
                             CenterFrequencyCPML=fc, VMaxCPML=vp0, edgeOrderReduction=0)
    n = g.NX * g.NY
    o = refcpu.Oracle(cfg, dict(rho=np.full(n, rho0), vp=np.full(n, vp0), vs=np.full(n, vs0)),
                      np.array([sx + g.NX * sy]), np.array([1]), sig[:, :refcpu.nt_of(cfg)],
                      np.array([r[0] + g.NX * r[1] for r in recs]), np.ones(len(recs), int), dtype=np.float64)
    b = o.run()
    o.close()
    m = min(a.shape[1], b.shape[1])
    assert np.isfinite(a).all()
    for k in range(len(recs)):
        assert np.linalg.norm(a[k, :m] - b[k, :m]) / np.linalg.norm(b[k, :m]) < 0.02


@pytest.mark.parametrize("grid,NX,NY", [
    ([(0, 1, 2), (30, 3, 6), (150, 1, 2), (200, 3, 6)], 305, 303),    # the CI grid
    ([(0, 1, 4), (31, 3, 6), (70, 1, 4)], 122, 100),
    ([(0, 1, 2), (30, 3, 2), (57, 9, 2)], 113, 96),
])
def test_library_staggered_operators_equal_the_oracle(grid, NX, NY, wave, refcpu):
    """DyfStaggeredX / DybStaggeredX as the library assembles them on the host
    (wave_grid_operator 9, 10) against the oracle, entry for entry."""
    import scipy.sparse as sp
    from oracle import vargrid as vg, vargrid_elastic as ve
    DT = 4e-4
    kw = dict(dimension=2, equation="elastic", NX=NX, NY=NY, NZ=1, DH=10.0, DT=DT, T=0.01, spatialFDorder=grid[0][2],
              useVariableGrid=1, useVariableFDoperators=1, grid=grid)
    c = wave.WaveConfig.make(**kw)
    g = vg.VarGrid(NX, NY, 1, 10.0, [r[0] for r in grid], [r[1] for r in grid])
    op = vg.Operators(g, [r[2] for r in grid], DT, False, np.float32, True, True, True)
    for k, fwd in ((9, True), (10, False)):
        cols, vals = wave.grid_operator(c, k)
        w = cols.shape[0]
        got = sp.csr_matrix((vals.ravel().astype(np.float64), (np.tile(np.arange(g.N), w), cols.ravel())), shape=(g.N, g.N))
        got.eliminate_zeros()
        want = ve.staggered_x_operator(op, [r[2] for r in grid], True, fwd).astype(np.float64).tocsr()
        want.eliminate_zeros()
        diff = abs(got - want)
        assert diff.nnz == 0 or diff.max() == 0, (k, diff.max())


@pytest.mark.parametrize("boundary,fs", [(2, 0), (0, 0), (2, 1), (1, 0), (1, 1)])
def test_single_layer_3d_elastic_vargrid_equals_regular_oracle(boundary, fs, refcpu):
    """The 3-D elastic variable-grid oracle (staggered-Z operators, the XZ /
    YZ shear averages, the 3-D interpolation set) on one layer against the
    pinned regular 3-D elastic oracle, FP64."""
    from oracle import vargrid as vg, vargrid_elastic as ve
    NX, NY, NZ, DH, order, vmax = 30, 28, 26, 5.0, 4, 3000.0
    DT = 0.3 * DH / (vmax * np.sqrt(3.0))
    cfg = refcpu.make_config(dimension=3, equation="elastic", NX=NX, NY=NY, NZ=NZ, DH=DH, DT=DT, T=160 * DT,
                             spatialFDorder=order, DampingBoundary=boundary, BoundaryWidth=6, NPower=4.0,
                             CenterFrequencyCPML=20.0, VMaxCPML=vmax, edgeOrderReduction=0, FreeSurface=fs,
                             DampingCoeff=8.0)
    nt = refcpu.nt_of(cfg)
    rho, vp, vs = _model(NX * NY * NZ, np.random.default_rng(2))
    g = vg.VarGrid(NX, NY, NZ, DH, [0], [1])
    sidx = g.coordinate2index([NX // 2], [NY // 3], [NZ // 2])
    sig = refcpu.ricker(nt, DT, 40.0, 1.0, 0.0, np.float64)[None]
    ridx = g.coordinate2index([5, NX - 6, 7, 12], [10, NY - 4, 20, 5], [4, 9, NZ - 5, 13])
    rtype = np.array([1, 2, 3, 4])
    o = refcpu.Oracle(cfg, dict(rho=rho, vp=vp, vs=vs), sidx, np.array([1]), sig, ridx, rtype, dtype=np.float64)
    ref = o.run()
    o.close()
    cp = vg.cpml_coefficients(g, 6, 4.0, 20.0, vmax, DT, fs != 0, np.float64) if boundary == 2 else None
    damp = vg.abs_damping(g, 6, 8.0, fs != 0, np.float64) if boundary == 1 else None
    sim = ve.ElasticVarGrid3D(g, [order], DT, rho, vp, vs, cp, sidx, [1], sig, ridx, rtype, dtype=np.float64,
                              var_order=False, edge=False, var_grid=False, free_surface=fs != 0, damping=damp)
    got = sim.run(nt)
    assert np.abs(ref).max() > 0
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12


def test_3d_elastic_vargrid_tracks_the_all_fine_grid(refcpu):
    """A 1:3:1 3-D grid (every staggered-X / Z operator shift and the
    StaggeredX / Z / XZ and Full interpolations in play): receivers in the fine
    layers stay within 2 % of an all-fine regular run (the misfit is the
    coarse layer's dispersion: 4 % at a 10 Hz peak, 0.6 % at 6 Hz), and two
    receivers that mirror each other under x <-> z record the same trace (the
    x- and z-staggered operators and interpolations agree)."""
    from oracle import vargrid as vg, vargrid_elastic as ve
    NX, NY, NZ, DH = 49, 60, 49, 5.0
    vp0, vs0, rho0, fc = 3000.0, 1700.0, 2200.0, 6.0
    DT = 0.3 * DH / (vp0 * np.sqrt(3.0) * 1.2)
    nt = 700
    grid = [(0, 1, 4), (21, 3, 4), (42, 1, 4)]
    g = vg.VarGrid(NX, NY, NZ, DH, [r[0] for r in grid], [r[1] for r in grid])
    sig = refcpu.ricker(nt, DT, fc, 1.0, 0.0, np.float64)[None]
    src = (g.NX // 2, 12, g.NZ // 2)
    recs = [(12, 8, 20), (36, 15, 30), (24, 50, 24), (24, 50, 10), (10, 50, 24)]
    cp = vg.cpml_coefficients(g, 9, 4.0, fc, vp0, DT, False, np.float64)
    sidx = g.coordinate2index([src[0]], [src[1]], [src[2]])
    ridx = g.coordinate2index([r[0] for r in recs], [r[1] for r in recs], [r[2] for r in recs])
    sim = ve.ElasticVarGrid3D(g, [r[2] for r in grid], DT, np.full(g.N, rho0), np.full(g.N, vp0), np.full(g.N, vs0),
                              cp, sidx, [1], sig, ridx, [1] * len(recs), dtype=np.float64, edge=False)
    a = sim.run(nt)
    cfg = refcpu.make_config(dimension=3, equation="elastic", NX=g.NX, NY=g.NY, NZ=g.NZ, DH=DH, DT=DT, T=nt * DT,
                             spatialFDorder=4, DampingBoundary=2, BoundaryWidth=9, NPower=4.0,
                             CenterFrequencyCPML=fc, VMaxCPML=vp0, edgeOrderReduction=0)
    n = g.NX * g.NY * g.NZ
    o = refcpu.Oracle(cfg, dict(rho=np.full(n, rho0), vp=np.full(n, vp0), vs=np.full(n, vs0)),
                      np.array([src[0] + g.NX * (src[2] + g.NZ * src[1])]), np.array([1]), sig[:, :refcpu.nt_of(cfg)],
                      np.array([r[0] + g.NX * (r[2] + g.NZ * r[1]) for r in recs]), np.ones(len(recs), int),
                      dtype=np.float64)
    b = o.run()
    o.close()
    m = min(a.shape[1], b.shape[1])
    assert np.isfinite(a).all()
    for k in range(len(recs)):
        assert np.linalg.norm(a[k, :m] - b[k, :m]) / np.linalg.norm(b[k, :m]) < 0.02, k
    assert np.linalg.norm(a[3] - a[4]) <= 1e-10 * np.linalg.norm(a[3])


@pytest.mark.parametrize("grid,dims,fs", [
    ([(0, 1, 4), (21, 3, 4), (42, 1, 4)], (49, 60, 49), 0),
    ([(0, 1, 2), (12, 3, 6), (30, 9, 2)], (55, 48, 37), 0),
    ([(0, 1, 6), (12, 3, 6), (30, 9, 2)], (55, 48, 37), 1),
    ([(0, 3, 4), (12, 1, 4)], (49, 40, 49), 1),
])
def test_library_3d_staggered_operators_equal_the_oracle(grid, dims, fs, wave, refcpu):
    """DyfStaggeredX / DybStaggeredX / DyfStaggeredZ / DybStaggeredZ (with
    FreeSurface=1 the backward ones are their image variants) and the
    StaggeredXZ interpolation as the library assembles them on the host
    (wave_grid_operator 9-13) against the oracle, entry for entry, on 3-D
    variable grids."""
    import scipy.sparse as sp
    from oracle import vargrid as vg, vargrid_elastic as ve
    NX, NY, NZ = dims
    DT = 4e-4
    kw = dict(dimension=3, equation="elastic", NX=NX, NY=NY, NZ=NZ, DH=10.0, DT=DT, T=0.01, spatialFDorder=grid[0][2],
              useVariableGrid=1, useVariableFDoperators=1, grid=grid, FreeSurface=fs)
    c = wave.WaveConfig.make(**kw)
    g = vg.VarGrid(NX, NY, NZ, 10.0, [r[0] for r in grid], [r[1] for r in grid])
    orders = [r[2] for r in grid]
    op = vg.Operators(g, orders, DT, fs != 0, np.float32, True, True, True)
    want = {9: ve.staggered_operator(op, orders, True, True, "x"),
            10: ve.staggered_operator(op, orders, True, False, "x", fs != 0),
            11: ve.staggered_operator(op, orders, True, True, "z"),
            12: ve.staggered_operator(op, orders, True, False, "z", fs != 0), 13: op.IStagXZ}
    for k, w_ in want.items():
        cols, vals = wave.grid_operator(c, k)
        w = cols.shape[0]
        got = sp.csr_matrix((vals.ravel().astype(np.float64), (np.tile(np.arange(g.N), w), cols.ravel())), shape=(g.N, g.N))
        got.eliminate_zeros()
        ref = w_.astype(np.float64).tocsr()
        ref.eliminate_zeros()
        diff = abs(got - ref)
        assert diff.nnz == 0 or diff.max() == 0, (k, diff.max())
