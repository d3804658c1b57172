"""GPU parity of the variable-grid acoustic path (vargrid.cu, through the C ABI)
against the reference's variable-grid goldens (gate of
Test_CompareSeismogram.cpp:57-88) and against the FP64 variable-grid oracle
(oracle/vargrid.py).

Tolerance: relative L2 over all traces and samples <= 1e-4 against the FP64
oracle; the reference's gate (average misfit per sample <= 5e-7) against the
goldens."""
import ctypes

import numpy as np
import pytest

import ci_cases

pytestmark = pytest.mark.gpu
TOL = 1e-4
GATE = 5e-7


def to_wave_cfg(wave, cfg):
    c = wave.WaveConfig()
    ctypes.memmove(ctypes.byref(c), ctypes.byref(cfg), ctypes.sizeof(c))
    return c


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run_gpu(wave, case):
    cfg = to_wave_cfg(wave, case["cfg"])
    m = {k: v.astype(np.float32) for k, v in case["model"].items()}
    return wave.simulate(cfg, m, case["src_idx"], case["src_type"], case["signals"].astype(np.float32),
                         case["rec_idx"], case["rec_type"])


def test_gpu_matches_2d_vargrid_golden(wave, refcpu):
    case = ci_cases.load_vargrid_case("2D.acoustic.varGrid")
    seis = run_gpu(wave, case)
    assert refcpu.reference_misfit(seis.astype(np.float64), case["golden"]) < GATE
    c64 = ci_cases.load_vargrid_case("2D.acoustic.varGrid", np.float64)
    ref = ci_cases.run_vargrid_oracle(c64, np.float64)
    assert rel(seis, ref) < TOL


def test_gpu_matches_3d_vargrid_golden(wave, refcpu):
    case = ci_cases.load_vargrid_case("3D.acoustic.varGrid")
    seis = run_gpu(wave, case)
    g = case["golden"]
    assert refcpu.reference_misfit(seis.astype(np.float64), g) < GATE
    assert rel(seis, g) < 1e-3


# (dimension, NX, NY, NZ, grid rows, variable grid, free surface, damping boundary, edge reduction)
SYNTH = [
    (2, 122, 100, 1, [(0, 1, 4), (31, 3, 6), (70, 1, 4)], 1, 1, 2, 1),
    (2, 113, 96, 1, [(0, 1, 2), (30, 3, 2), (57, 9, 2)], 1, 1, 0, 0),
    (2, 90, 80, 1, [(0, 1, 2), (40, 1, 8)], 0, 0, 2, 1),
    (3, 41, 60, 41, [(0, 1, 4), (20, 3, 4)], 1, 0, 2, 0),
    (3, 44, 54, 38, [(0, 1, 6), (18, 3, 2), (36, 1, 4)], 1, 1, 2, 1),
    (2, 122, 100, 1, [(0, 1, 4), (31, 3, 6), (70, 1, 4)], 1, 1, 1, 1),
    (3, 41, 60, 41, [(0, 1, 4), (20, 3, 4)], 1, 0, 1, 0),
]


def synth_case(refcpu, k):
    from oracle import vargrid
    dim, NX, NY, NZ, grid, vgrid, fs, boundary, edge = SYNTH[k]
    DH = 5.0
    vmax = 3200.0
    DT = 0.3 * DH / (vmax * np.sqrt(dim) * 1.3)
    nt = 500
    cfg = refcpu.make_config(dimension=dim, equation="acoustic", NX=NX, NY=NY, NZ=NZ, DH=DH, DT=DT, T=nt * DT,
                             spatialFDorder=grid[0][2], FreeSurface=fs, DampingBoundary=boundary,
                             BoundaryWidth=12 if boundary else 0, DampingCoeff=8.0, NPower=4.0, CenterFrequencyCPML=12.0,
                             VMaxCPML=vmax, edgeOrderReduction=edge, useVariableGrid=vgrid,
                             useVariableFDoperators=1, grid=grid)
    g = vargrid.VarGrid(NX, NY, NZ, DH, [r[0] for r in grid], [r[1] for r in grid] if vgrid else [1] * len(grid))
    nt = refcpu.nt_of(cfg)
    rng = np.random.default_rng(k)
    vp = rng.uniform(2500.0, vmax, g.N).astype(np.float32)
    rho = (310.0 * vp.astype(np.float64) ** 0.25 * rng.uniform(0.9, 1.1, g.N)).astype(np.float32)
    fc = 4.5 / (nt * DT)   # the Ricker peak (1.5/fc) at a third of the record
    sx, sy, sz = g.NX // 2, 3 if fs else g.NY // 5, g.NZ // 2
    src = g.coordinate2index([sx], [sy], [sz])
    sig = refcpu.ricker(nt, DT, fc, 1.0, 0.0, np.float64)[None]
    ys = [0 if fs else 2, grid[1][0] - 1, grid[1][0] + 4, g.NY - 3, g.NY // 2]
    types = [1, 2, 3, 1, 4 if dim == 3 else 2]
    rx = [(7 * i + 5) % g.NX for i in range(len(ys))]
    rz = [(5 * i + 3) % g.NZ for i in range(len(ys))]
    ridx = [int(g.coordinate2index(x, y, z)) for x, y, z in zip(rx, ys, rz)]
    return dict(cfg=cfg, grid=g, orders=[r[2] for r in grid], nt=nt, model=dict(rho=rho, vp=vp),
                src_idx=np.asarray(src, np.int64), src_type=np.array([1], np.int32), signals=sig,
                rec_idx=np.array(ridx, np.int64), rec_type=np.array(types, np.int32))


@pytest.mark.parametrize("k", range(len(SYNTH)))
def test_gpu_vargrid_heterogeneous_model_matches_fp64_oracle(k, wave, refcpu):
    case = synth_case(refcpu, k)
    gpu = run_gpu(wave, case)
    c64 = dict(case)
    c64["model"] = {kk: v.astype(np.float64) for kk, v in case["model"].items()}
    ref = ci_cases.run_vargrid_oracle(c64, np.float64)
    assert np.abs(ref).max() > 0
    assert rel(gpu, ref) < TOL, rel(gpu, ref)


def test_gpu_vargrid_chunked_stepping_is_bit_identical(wave, refcpu):
    case = synth_case(refcpu, 0)
    cfg = to_wave_cfg(wave, case["cfg"])
    m = {k: v.astype(np.float32) for k, v in case["model"].items()}
    whole = wave.simulate(cfg, m, case["src_idx"], case["src_type"], case["signals"].astype(np.float32),
                          case["rec_idx"], case["rec_type"])
    s = wave.Factory.Create("2d", "acoustic").initForwardSolver(cfg)
    try:
        s.prepareForModelling(m)
        s.setSources(case["src_idx"], case["src_type"], case["signals"].astype(np.float32))
        s.setReceivers(case["rec_idx"], case["rec_type"])
        t = 0
        for chunk in (1, 7, 1, 64, 200):
            s.run(t, min(t + chunk, s.nt))
            t = min(t + chunk, s.nt)
        s.run(t, s.nt)
        parts = s.seismograms()
    finally:
        s.close()
    np.testing.assert_array_equal(parts, whole)


def test_gpu_vargrid_rejects_what_it_does_not_build(wave, refcpu):
    base = dict(dimension=2, NX=122, NY=100, NZ=1, DH=5.0, DT=5e-4, T=0.01, spatialFDorder=4,
                useVariableGrid=1, useVariableFDoperators=1, grid=[(0, 1, 4), (31, 3, 4)])
    for eq, extra in (("sh", {}), ("elastic", dict(FreeSurface=2)),
                      ("viscoelastic", dict(numRelaxationMechanisms=1, relaxationFrequency=[5.0, 0, 0, 0])),
                      ("tmem", {})):
        cfg = wave.WaveConfig.make(equation=eq, **dict(base, **extra))
        with pytest.raises(wave.WaveError):
            wave.Factory.Create("3d" if extra.get("dimension") == 3 else "2d", eq).initForwardSolver(cfg)


@pytest.mark.parametrize("k", [0, 1, 4])
def test_gpu_vargrid_stencil_classes_equal_the_ell_operators(k, wave, refcpu):
    """The default kernels read each row's entries from its stencil class;
    kernel path 1 streams the ELL blocks. Same entries in the same order:
    bit-identical seismograms."""
    case = synth_case(refcpu, k)
    cfg = to_wave_cfg(wave, case["cfg"])
    m = {kk: v.astype(np.float32) for kk, v in case["model"].items()}
    args = (case["src_idx"], case["src_type"], case["signals"].astype(np.float32), case["rec_idx"], case["rec_type"])
    a = wave.simulate(cfg, m, *args, kernel_path=0)
    b = wave.simulate(cfg, m, *args, kernel_path=1)
    np.testing.assert_array_equal(a, b)
