"""Wavefield decomposition (decomposeWavefieldType 1 and 2, 2-D acoustic) on
the GPU against the CPU restatement (oracle/decompose.py) of
Wavefields2Dacoustic.cpp:119-300, applied to the GPU's own wavefields before
and after the step."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_wave_cfg(wave, cfg):
    c = wave.WaveConfig()
    ctypes.memmove(ctypes.byref(c), ctypes.byref(cfg), ctypes.sizeof(c))
    return c


@pytest.mark.parametrize("kind,reduce", [(1, 1), (2, 0)])
def test_gpu_decomposition_matches_restatement(kind, reduce, wave, refcpu):
    from oracle import decompose, vargrid
    NX, NY, DH, order = 120, 90, 5.0, 4
    DT = 0.3 * DH / (3000.0 * np.sqrt(2))
    kw = dict(dimension=2, equation="acoustic", NX=NX, NY=NY, NZ=1, DH=DH, DT=DT, T=400 * DT,
              spatialFDorder=order, FreeSurface=0, DampingBoundary=2, BoundaryWidth=10, NPower=4.0,
              CenterFrequencyCPML=10.0, VMaxCPML=3000.0, edgeOrderReduction=reduce)
    cfg = refcpu.make_config(**kw)
    rng = np.random.default_rng(kind)
    vp = rng.uniform(2200.0, 3000.0, NX * NY).astype(np.float32)
    rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(np.float32)
    nt = refcpu.nt_of(cfg)
    sig = refcpu.ricker(nt, DT, 25.0, 1.0, 0.0, np.float32)[None]
    s = wave.Factory.Create("2d", "acoustic").initForwardSolver(to_wave_cfg(wave, cfg))
    try:
        s.prepareForModelling(dict(rho=rho, vp=vp))
        s.setSources(np.array([NX // 2 + NX * (NY // 3)]), np.array([1]), sig)
        s.setReceivers(np.array([5 + NX * 5]), np.array([1]))
        s.set_decomposition(kind)
        t = 150
        s.run(0, t)
        old = [s.field(n) for n in ("P", "VX", "VY")]
        s.run(t, t + 1)
        cur = [s.field(n) for n in ("P", "VX", "VY")]
        names = ["up", "down"] if kind == 1 else ["left", "right"]
        got = [s.field(f"{f}.{n}") for f in ("P", "VX", "VY") for n in names]
    finally:
        s.close()
    g = vargrid.VarGrid(NX, NY, 1, DH, [0], [1])
    op = vargrid.Operators(g, [order], DT, False, np.float32, var_order=False, edge=bool(reduce), var_grid=False)
    want = decompose.decompose_2d_acoustic(kind, cur, old, op.Dyf if kind == 1 else op.Dxf, DT)
    for k, (a, b) in enumerate(zip(got, want)):
        F = cur[k // 2]
        assert np.abs(F).max() > 0
        # the split may differ only where the Poynting estimate is at rounding level
        differ = a != b
        assert differ.mean() < 2e-3, (k, differ.mean())
        np.testing.assert_array_equal(a[~differ], b[~differ])
        # each part is the field or zero, and the two parts cover the field
        assert np.all((a == F) | (a == 0))
    for q in range(3):
        up, down = got[2 * q], got[2 * q + 1]
        F = cur[q]
        assert np.all((up == F) | (down == F))


@pytest.mark.parametrize("kind", [1, 2])
def test_gpu_tmz_decomposition_matches_restatement(kind, wave, refcpu):
    from oracle import decompose, vargrid
    NX, NY, DH = 110, 90, 0.02
    DT = 0.3 * DH / (1.5e8 * np.sqrt(2))
    kw = dict(dimension=2, equation="tmem", NX=NX, NY=NY, NZ=1, DH=DH, DT=DT, T=300 * DT, spatialFDorder=4,
              DampingBoundary=2, BoundaryWidth=10, NPower=4.0, CenterFrequencyCPML=2e8, VMaxCPML=1.5e8)
    cfg = refcpu.make_config(**kw)
    rng = np.random.default_rng(kind)
    n = NX * NY
    model = dict(eps_r=rng.uniform(4.0, 9.0, n).astype(np.float32), sigma=np.full(n, 1e-3, np.float32),
                 mu_r=np.ones(n, np.float32))
    nt = refcpu.nt_of(cfg)
    sig = refcpu.ricker(nt, DT, 6e8, 1.0, 0.0, np.float32)[None]
    s = wave.Factory.Create("2d", "tmem").initForwardSolver(to_wave_cfg(wave, cfg))
    try:
        s.prepareForModelling(model)
        s.setSources(np.array([NX // 2 + NX * (NY // 2)]), np.array([1]), sig)
        s.setReceivers(np.array([5 + NX * 5]), np.array([1]))
        s.set_decomposition(kind)
        t = 120
        s.run(0, t)
        old = s.field("EZ")
        s.run(t, t + 1)
        cur = [s.field(n_) for n_ in ("EZ", "HX", "HY")]
        names = ["up", "down"] if kind == 1 else ["left", "right"]
        got = [s.field(f"EZ.{n_}") for n_ in names]
    finally:
        s.close()
    g = vargrid.VarGrid(NX, NY, 1, DH, [0], [1])
    op = vargrid.Operators(g, [4], DT, False, np.float32, var_order=False, edge=True, var_grid=False)
    want = decompose.decompose_2d_tmem(kind, cur, old, op.Dyf if kind == 1 else op.Dxf, DT)
    F = cur[0]
    assert np.abs(F).max() > 0
    for a, b in zip(got, want):
        differ = a != b
        assert differ.mean() < 2e-3, differ.mean()
        np.testing.assert_array_equal(a[~differ], b[~differ])
        assert np.all((a == F) | (a == 0))
    assert np.all((got[0] == F) | (got[1] == F))


def test_decomposition_is_2d_acoustic_and_tmz_only(wave, refcpu):
    kw = dict(dimension=2, equation="elastic", NX=40, NY=40, NZ=1, DH=5.0, DT=5e-4, T=0.01, spatialFDorder=4)
    s = wave.Factory.Create("2d", "elastic").initForwardSolver(to_wave_cfg(wave, refcpu.make_config(**kw)))
    try:
        with pytest.raises(wave.WaveError):
            s.set_decomposition(1)
    finally:
        s.close()
