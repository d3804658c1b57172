"""Seismogram output path on the GPU against numpy restatements of the
reference: resampling to seismoDT (Common::calcResampleMat, Common.hpp:202-230,
applied in Seismogram::write, Seismogram.cpp:109) and per-trace normalisation
(Seismogram::normalizeTrace, Seismogram.cpp:215-240)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def resample_reference(d, dt, sdt):
    coeff = np.float32(sdt) / np.float32(dt)
    nt = d.shape[1]
    n_new = int(np.floor(np.float32(nt - 1) / coeff)) + 1
    out = np.zeros((d.shape[0], n_new), np.float32)
    for k in range(n_new):
        rel = np.float32(k) * coeff
        c0 = int(np.floor(rel))
        w1 = np.fmod(rel, np.float32(1.0))
        w0 = np.float32(1.0) - w1
        s = np.zeros(d.shape[0], np.float32)
        if c0 < nt:
            s = s + w0 * d[:, c0]
        if c0 + 1 < nt:
            s = s + w1 * d[:, c0 + 1]
        out[:, k] = s
    return out


@pytest.mark.parametrize("nt,dt,sdt", [(1000, 2e-4, 2e-4), (1000, 2e-4, 1e-3), (777, 1.5e-4, 4e-4), (64, 1e-3, 3.3e-3),
                                       (500, 5e-4, 3e-4)])
def test_resample_matches_reference_formula(wave, nt, dt, sdt):
    d = np.random.default_rng(nt).standard_normal((9, nt)).astype(np.float32)
    got = wave.resample_traces(d, dt, sdt)
    ref = resample_reference(d, dt, sdt)
    assert got.shape == ref.shape
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6)
    if sdt == dt:
        assert np.array_equal(got, d)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_normalize_matches_reference(wave, mode):
    d = np.random.default_rng(mode).standard_normal((11, 300)).astype(np.float32) * 1e-3
    d[4] = 0.0                                   # a zero trace is divided by 1
    got = wave.normalize_traces(d, mode)
    if mode == 0:
        ref = d
    else:
        n = np.abs(d).max(axis=1) if mode == 1 else np.sqrt((d.astype(np.float64) ** 2).sum(axis=1))
        n = np.where(n == 0, 1, n).astype(np.float32)
        ref = d / n[:, None]
    np.testing.assert_allclose(got, ref, rtol=2e-6, atol=0)
    assert np.array_equal(got[4], d[4])
