"""TEST INFRASTRUCTURE ONLY — restatement of the reference's source encoding,
Sources::calcSourceSettingsEncode (src/Acquisition/Sources.cpp:569-660) for
time-domain modelling, the checker of wave_encode_sources. The random numbers
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
