"""Receiver-side encoding of seismograms (Receivers::encode / decode,
Receivers.cpp:354-573): properties of the restatement in
oracle/encode_traces.py on the CPU, and the CUDA wave_encode_traces against
it (GPU tests, relative L2 <= 1e-5: FP32 traces, FP64 projections)."""
import numpy as np
import pytest

from oracle import encode_traces as et


def _survey(seed=1, nshots=4, nrec=13, nt=300, overlap=True):
    rng = np.random.default_rng(seed)
    mark = np.zeros((nshots, nrec), np.int32)
    for s in range(nshots):
        lo = s * (nrec // nshots)
        hi = min(nrec - 1, lo + (nrec // nshots) + (2 if overlap else 0))
        mark[s, lo:hi] = 1
    super_mark = (mark.sum(0) > 0).astype(np.int32)
    super_mark[-1] = 1   # a super-shot receiver no shot records
    amp = np.where(rng.random(nshots) < 0.5, -1.0, 1.0).astype(np.float32) * rng.uniform(0.5, 2.0, nshots).astype(np.float32)
    shots = [rng.standard_normal((int(mark[s].sum()), nt)).astype(np.float32) for s in range(nshots)]
    fc = rng.uniform(5.0, 40.0, nshots).astype(np.float32)
    return mark, super_mark, amp, shots, fc


def test_restatement_encode_places_signed_traces():
    mark, sm, amp, shots, _ = _survey(overlap=False)
    sup = et.encode(shots, mark, sm, amp)
    rows = np.flatnonzero(sm)
    for s in range(len(amp)):
        rs = np.flatnonzero(mark[s])
        for j, r in enumerate(rs):
            k = int(np.flatnonzero(rows == r)[0])
            assert np.array_equal(sup[k], shots[s][j].astype(np.float64) * np.sign(amp[s]))
    assert not np.any(sup[-1])
    back = et.decode(sup, mark, sm, amp)
    for s in range(len(amp)):
        assert np.allclose(back[s], shots[s], rtol=0, atol=1e-6)


def test_restatement_single_frequency_filter():
    """The projection keeps one frequency: a trace that is a sinusoid at that
    frequency keeps its shape (up to the block's max normalisation), and a
    filtered trace is a sinusoid of that frequency."""
    nt, DT = 512, 1e-3
    nfft = 512   # next power of two of nt - 1
    df = 1.0 / (nfft * DT)
    w = 2 * np.pi * 20 * df
    t = np.arange(nt) * DT
    tr = np.cos(w * t)[None]
    out = et.single_frequency(tr, 20 * df, DT, matrix=True)
    assert np.allclose(out, tr / np.abs(tr).max(), atol=1e-9)
    rng = np.random.default_rng(0)
    f = et.single_frequency(rng.standard_normal(nt), 20 * df, DT, matrix=False)[0]
    # f = a cos(w t) + b sin(w t): fit and check the residual
    A = np.stack([np.cos(w * t), np.sin(w * t)], 1)
    coef, *_ = np.linalg.lstsq(A, f, rcond=None)
    assert np.linalg.norm(A @ coef - f) <= 1e-9 * np.linalg.norm(f)


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("filtered", [False, True])
@pytest.mark.parametrize("overlap", [False, True])
def test_gpu_multi_offset_encode_decode_match_restatement(wave, filtered, overlap):
    mark, sm, amp, shots, fc = _survey(overlap=overlap)
    DT = 2e-3
    f = fc if filtered else None
    sup = wave.encode_traces(False, mark, sm, amp, f, DT, shot_data=shots)
    want = et.encode(shots, mark, sm, amp, f, DT)
    assert _rel(sup, want) <= 1e-5
    back = wave.encode_traces(True, mark, sm, amp, f, DT, super_data=want.astype(np.float32))
    want_back = et.decode(want, mark, sm, amp, f, DT)
    for g, w in zip(back, want_back):
        assert g.shape == w.shape and _rel(g, w) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("filtered", [False, True])
def test_gpu_common_offset_encode_decode_match_restatement(wave, filtered):
    rng = np.random.default_rng(5)
    n, nt, DT = 8, 400, 1e-3
    mark = np.eye(n, dtype=np.int32)
    mark[3, 3] = 0   # a shot whose own receiver is not recorded
    sm = np.ones(n, np.int32)
    sm[6] = 0        # a shot outside the super-shot
    amp = rng.choice([-1.0, 1.0], n).astype(np.float32)
    shots = [rng.standard_normal((1, nt)).astype(np.float32) for _ in range(n)]
    f = rng.uniform(5, 60, n).astype(np.float32) if filtered else None
    sup = wave.encode_traces(False, mark, sm, amp, f, DT, common_offset=True, shot_data=shots)
    want = et.encode(shots, mark, sm, amp, f, DT, common_offset=True)
    assert sup.shape == want.shape and _rel(sup, want) <= 1e-5
    back = wave.encode_traces(True, mark, sm, amp, f, DT, common_offset=True, super_data=want.astype(np.float32))
    want_back = et.decode(want, mark, sm, amp, f, DT, common_offset=True)
    for g, w in zip(back, want_back):
        assert g.shape == w.shape
        assert _rel(g, w) <= 1e-5 if np.any(w) else not np.any(g)
