"""Seismogram output path on the GPU against numpy restatements of the
reference: resampling to seismoDT (Common::calcResampleMat, Common.hpp:202-230,
applied in Seismogram::write, Seismogram.cpp:109), per-trace normalisation
(Seismogram::normalizeTrace, Seismogram.cpp:215-240) and AGC normalisation
(Seismogram::calcInverseAGC, Seismogram.cpp:323-387)."""
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


def agc_reference(d, dt, f):
    """normalizeTraces 3 restated in FP32 (Seismogram::calcInverseAGC,
    Seismogram.cpp:323-387, then normalizeTrace(3), :235-237): l2-normalised
    traces, inverse AGC from a backward running window sum of squares, product."""
    d = np.asarray(d, np.float32)
    ntr, nt = d.shape
    norm = np.sqrt((d.astype(np.float64) ** 2).sum(axis=1)).astype(np.float32)
    norm = np.where(norm == 0, np.float32(1), norm)
    nd = (d / norm[:, None]).astype(np.float32)
    x = 1.0 / float(np.float32(f) * np.float32(dt))
    nagc = min(int(np.floor(x + 0.5)), nt // 2)
    total = np.float32(np.sqrt((nd.astype(np.float64) ** 2).sum()))
    wl0 = np.float32(1e-3 * float(total) / nt / ntr)
    inv = np.zeros_like(nd)
    f32 = np.float32
    for tr in range(ntr):
        row = nd[tr]
        ss = f32(0)
        for t in range(nt):
            ss = f32(ss + f32(row[t] * row[t]))
        l2 = f32(np.sqrt(ss))
        wl = f32(f32(l2 * l2) / f32(nt))
        wl = f32(float(wl) * 1e-3) if wl != 0 else wl0
        acc, win = f32(0), f32(nagc)
        for t in range(nt - nagc, nt):
            acc = f32(acc + f32(row[t] * row[t]))
            acc = f32(acc + wl)
        for t in range(nt - 1, -1, -1):
            if t >= nt - nagc:
                v = row[t - nagc]
                acc = f32(f32(acc + f32(v * v)) + wl)
                win = f32(win + f32(1))
            elif t >= nagc:
                a, b = row[t - nagc], row[t + nagc]
                acc = f32(f32(acc + f32(a * a)) - f32(b * b))
            else:
                b = row[t + nagc]
                acc = f32(f32(acc - f32(b * b)) - wl)
                win = f32(win - f32(1))
            with np.errstate(divide="ignore", invalid="ignore"):
                r = f32(acc / win)
            inv[tr, t] = f32(f32(1) / f32(np.sqrt(r))) if r > 0 else f32(0)
    return (nd * inv).astype(np.float32), inv


@pytest.mark.parametrize("ntr,nt,dt,f", [(7, 400, 1e-3, 15.0), (5, 301, 2e-3, 1.0), (4, 256, 5e-4, 500.0)])
def test_agc_normalisation_matches_reference_formula(wave, ntr, nt, dt, f):
    rng = np.random.default_rng(nt)
    d = (rng.standard_normal((ntr, nt)) * np.exp(-np.linspace(0, 4, nt))[None, :]).astype(np.float32)
    d[1] = 0.0                                   # a zero trace takes the global water level
    got, inv = wave.agc_normalize_traces(d, dt, f)
    ref, ref_inv = agc_reference(d, dt, f)
    np.testing.assert_allclose(inv, ref_inv, rtol=1e-5, atol=0)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-12)
    assert np.all(np.isfinite(got))


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
