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


def _next_pow2(n):
    t = np.float32(np.log(np.float32(n)))
    t = np.float32(t / np.log(2.0))
    return int(np.float32(2.0) ** np.ceil(t))


def hilbert_reference(d):
    """HilbertFFT (HilbertFFT.cpp): zero padding to the next power of two of
    nt-1, weights 1 / 2 / 0 over the spectrum, 1/N, inverse FFT, imaginary part."""
    nt = d.shape[1]
    N = max(_next_pow2(nt - 1), nt)
    f = np.fft.fft(d.astype(np.float64), n=N, axis=1)
    w = np.zeros(N)
    if N % 2 == 0:
        w[0] = w[N // 2] = 1.0
        w[1:N // 2] = 2.0
    else:
        w[0] = 1.0
        w[1:(N + 1) // 2] = 2.0
    return np.fft.ifft(f * w, axis=1).imag[:, :nt]


@pytest.mark.parametrize("nt", [1000, 513, 64, 37])
def test_envelope_matches_fft_hilbert(wave, nt):
    rng = np.random.default_rng(nt)
    t = np.arange(nt)
    d = (np.sin(0.07 * t)[None, :] * rng.uniform(0.5, 2, (5, 1)) + 0.1 * rng.standard_normal((5, nt))).astype(np.float32)
    got = wave.envelope(d)
    ref = np.sqrt(d.astype(np.float64) ** 2 + hilbert_reference(d) ** 2)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5


@pytest.mark.parametrize("ptype", [1, 2, 3])
def test_instantaneous_phase_as_reference(wave, ptype):
    d = np.random.default_rng(ptype).standard_normal((4, 200)).astype(np.float32)
    got = wave.instantaneous_phase(d, ptype)
    imag = -d.astype(np.float64)              # Common.hpp:301-302: the imaginary part is -data there
    if ptype == 1:
        ref = np.arctan(imag / d)
    else:
        ref = np.arctan2(imag, d)
        if ptype == 3:
            ref = np.unwrap(ref, axis=1)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-5)


def test_normalize_mode4_envelope(wave):
    d = np.random.default_rng(9).standard_normal((6, 300)).astype(np.float32)
    got = wave.normalize_traces(d, 4)
    l2 = d / np.sqrt((d.astype(np.float64) ** 2).sum(axis=1, keepdims=True))
    env = np.sqrt(l2 ** 2 + hilbert_reference(l2) ** 2)
    ref = l2 / (env + 1e-3 * env.max(axis=1, keepdims=True))
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-5
