"""TEST INFRASTRUCTURE ONLY — restatement of the reference's source encoding,
Sources::calcSourceSettingsEncode (src/Acquisition/Sources.cpp:569-660) for
time-domain and frequency-domain (gradientDomain != 0) modelling, the checker
of wave_encode_sources, wave_encode_frequencies and
wave_encode_sources_frequency. The random numbers
come from the C library's srand/rand through ctypes, the generator the
reference calls (std::srand/std::rand)."""
from __future__ import annotations

import ctypes
import ctypes.util
import math

import numpy as np

_libc = ctypes.CDLL(ctypes.util.find_library("c"))
_libc.srand.argtypes = [ctypes.c_uint]
_libc.rand.restype = ctypes.c_int


def encode(mode: int, num_domains: int, seed: int, amp):
    """(super-shot numbers, signed amplitudes) of n shots, one source row each."""
    n = len(amp)
    per_super = math.ceil(np.float32(n) / np.float32(num_domains))
    base = num_domains * 1e4 + 1
    out_no = [0] * n
    out_amp = [np.float32(a) for a in amp]
    _libc.srand(seed & 0xFFFFFFFF)
    history = [0] * num_domains
    if mode == 1:
        for i in range(n):
            if i < num_domains:
                k = i
            else:
                k = _libc.rand() % num_domains
                while history[k] >= per_super:
                    k = _libc.rand() % num_domains
            history[k] += 1
            out_no[i] = int(base + k)
        for i in range(n):
            s = _libc.rand() % 2
            out_amp[i] = np.float32(out_amp[i] * (1.0 if s > 0 else -1.0))
    elif mode == 2:
        out_no = [int(base + i % num_domains) for i in range(n)]
    else:
        out_no = [int(base + i // per_super) for i in range(n)]
    return np.array(out_no, np.int32), np.array(out_amp, np.float32)


def frequencies(encoded: bool, fc1: float, fc2: float, T: float, DT: float, cpml_fc: float) -> np.ndarray:
    """The frequency list (Sources.cpp:587-611) in the reference's float
    arithmetic: NT = (T / DT) + 0.5, nFFT = Common::calcNextPowTwo(NT - 1),
    df = 1 / (nFFT DT), band indices ceil(fc / df); a list of n values
    start + k step (lama::linearDenseVector)."""
    f32 = np.float32
    T, DT, fc1, fc2 = f32(T), f32(DT), f32(fc1), f32(fc2)
    if fc2 == 0:
        fc2 = f32(f32(cpml_fc) * f32(2))
    NT = int(float(T / DT) + 0.5)
    e = f32(np.log(f32(NT - 1)))
    e = f32(float(e) / math.log(2.0))
    e = f32(np.ceil(e))
    nfft = int(np.power(f32(2.0), e))
    df = f32(f32(1.0) / (f32(nfft) * DT))
    i1, i2 = int(np.ceil(f32(fc1 / df))), int(np.ceil(f32(fc2 / df)))
    if not encoded:
        i1 = int(np.ceil(f32(f32(i1) / f32(2))))
        i2 *= 2
        if i1 == 0:
            i1 = 1
        n = int(np.ceil(f32(i2 - i1 + 1)))
        step = df
    else:
        if i1 == 0:
            i1 = 2
        if i1 % 2 == 1:
            i1 += 1
        n = int(np.ceil(f32(f32(i2 - i1 + 1) / f32(2))))
        step = f32(f32(2) * df)
    start = f32(f32(i1) * df)
    return np.array([f32(start + f32(k) * step) for k in range(max(n, 0))], np.float32)


def encode_frequency(mode: int, num_domains: int, seed: int, amp, fc1, fc2, T, DT, cpml_fc):
    """Frequency-domain encoding: the time-domain assignment, then for each
    super-shot in order of first appearance each of its shots a distinct
    random frequency of the encoded list (Sources.cpp:641-660), the same
    rand() stream continuing."""
    n = len(amp)
    f = frequencies(True, fc1, fc2, T, DT, cpml_fc)
    per_super = math.ceil(np.float32(n) / np.float32(num_domains))
    if len(f) < per_super:
        raise ValueError("fewer frequencies than shots per super-shot")
    no, a = encode(mode, num_domains, seed, amp)   # seeds and draws the same stream
    # continue the stream after encode(): replay its draws to reach the same state
    _libc.srand(seed & 0xFFFFFFFF)
    _replay_draws(mode, num_domains, n)
    order = []
    for s in no:
        if s not in order:
            order.append(int(s))
    fc = np.zeros(n, np.float32)
    for k in range(min(num_domains, len(order))):
        used = [0] * len(f)
        for i in range(n):
            if no[i] != order[k]:
                continue
            j = _libc.rand() % len(f)
            while used[j] > 0:
                j = _libc.rand() % len(f)
            used[j] += 1
            fc[i] = f[j]
    return no, a, fc


def _replay_draws(mode: int, num_domains: int, n: int):
    """The rand() draws encode() makes for mode (mode 1 only draws)."""
    if mode != 1:
        return
    per_super = math.ceil(np.float32(n) / np.float32(num_domains))
    history = [0] * num_domains
    for i in range(n):
        if i < num_domains:
            k = i
        else:
            k = _libc.rand() % num_domains
            while history[k] >= per_super:
                k = _libc.rand() % num_domains
        history[k] += 1
    for _ in range(n):
        _libc.rand()
