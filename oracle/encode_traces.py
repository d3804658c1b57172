"""TEST INFRASTRUCTURE ONLY — restatement of the reference's receiver-side
encoding of seismograms, Receivers::encode / Receivers::decode
(src/Acquisition/Receivers.cpp:354-573), and of the single-frequency "ideal"
band-pass it applies for frequency-domain modelling (Filter::init,
calcIdealBp with order 1 and apply, src/Filter/Filter.cpp:8-18, 239-342); the
checker of wave_encode_traces. FP64.

Multi-offset data: each shot s of a super-shot owns the rows of its marked
receivers (mark[s, r] != 0) among the super-shot's receivers
(super_mark[r] != 0), in receiver order. Encoding sums, over the shots in
order, sign_s x filter_s(shot data) into the super-shot rows; decoding copies
the super-shot rows back out, then applies the sign and the filter. The
matrix filter projects each row on exp(j w t), w = 2 pi ceil(fc / df) df,
df = 1 / (nFFT DT) (nFFT the next power of two of NT - 1), scales by 2 / nFFT
and then divides the whole block by its largest magnitude.

Common-offset data (as many shots as receivers, one trace per shot): super-shot
row k belongs to the k-th shot whose receiver is in the super-shot; a shot
adds (or receives) its trace only if its own receiver is marked for it, and
the vector filter scales by 1 / NT without the maximum normalisation."""
from __future__ import annotations

import math

import numpy as np


def _next_pow2(n: int) -> int:
    e = np.float32(np.log(np.float32(n)))
    e = np.float32(float(e) / math.log(2.0))
    return int(np.power(np.float32(2.0), np.float32(np.ceil(e))))


def single_frequency(d: np.ndarray, fc: float, DT: float, matrix: bool) -> np.ndarray:
    """Filter::apply of calcIdealBp(order 1) on a block of traces (rows)."""
    d = np.atleast_2d(np.asarray(d, np.float64))
    nt = d.shape[1]
    nfft = _next_pow2(nt - 1)
    df = 1.0 / (nfft * DT)
    w = 2.0 * math.pi * float(np.ceil(np.float32(fc) / np.float32(df))) * df   # the index in the reference's float
    t = np.arange(nt) * DT
    X = d @ np.exp(-1j * w * t)
    out = np.real(np.outer(X, np.exp(1j * w * t)))
    if matrix:
        out *= 2.0 / nfft
        m = np.abs(out).max()
        if m > 0:
            out /= m
    else:
        out /= nt
    return out


def encode(shot_data, mark, super_mark, amp, fc=None, DT=None, common_offset=False):
    """Receivers::encode: the super-shot block from the shots' blocks."""
    mark = np.asarray(mark)
    sup = np.flatnonzero(super_mark)
    nt = np.asarray(shot_data[0]).shape[-1]
    if common_offset:
        shots = [s for s in range(len(amp)) if super_mark[s]]
        out = np.zeros((len(shots), nt))
        for k, s in enumerate(shots):
            if not mark[s, s]:
                continue
            row = np.asarray(shot_data[s], np.float64).reshape(-1)[:nt] * (-1.0 if amp[s] < 0 else 1.0)
            if fc is not None:
                row = single_frequency(row, fc[s], DT, matrix=False)[0]
            out[k] += row
        return out
    out = np.zeros((sup.size, nt))
    row_of = {r: k for k, r in enumerate(sup)}
    for s in range(len(amp)):
        rs = [r for r in sup if mark[s, r]]
        D = np.asarray(shot_data[s], np.float64).reshape(len(rs), nt) * (-1.0 if amp[s] < 0 else 1.0)
        if fc is not None and len(rs):
            D = single_frequency(D, fc[s], DT, matrix=True)
        for j, r in enumerate(rs):
            out[row_of[r]] += D[j]
    return out


def decode(super_data, mark, super_mark, amp, fc=None, DT=None, common_offset=False):
    """Receivers::decode: the shots' blocks from the super-shot block."""
    mark = np.asarray(mark)
    sup = np.flatnonzero(super_mark)
    super_data = np.asarray(super_data, np.float64)
    nt = super_data.shape[-1]
    outs = []
    if common_offset:
        k = 0
        for s in range(len(amp)):
            row = np.zeros(nt)
            if super_mark[s]:
                if mark[s, s]:
                    row = super_data[k] * (-1.0 if amp[s] < 0 else 1.0)
                    if fc is not None:
                        row = single_frequency(row, fc[s], DT, matrix=False)[0]
                k += 1
            outs.append(row[None])
        return outs
    row_of = {r: k for k, r in enumerate(sup)}
    for s in range(len(amp)):
        rs = [r for r in sup if mark[s, r]]
        D = np.array([super_data[row_of[r]] for r in rs]).reshape(len(rs), nt) * (-1.0 if amp[s] < 0 else 1.0)
        if fc is not None and len(rs):
            D = single_frequency(D, fc[s], DT, matrix=True)
        outs.append(D)
    return outs
