"""TEST INFRASTRUCTURE ONLY — CPU restatement of the reference's wavefield
decomposition of the 2-D acoustic and 2-D TMz wavefields, the checker of the
GPU decomposition kernels (FD2Dtmem::decompose: src/WavefieldsEM/
Wavefields2Dtmem.cpp:109-160, EZ only, S1 = EZ*HX or -(EZ*HY)).

Simulation.cpp:450-461 forms the time derivative of one step as
(old - new) * (-1/DT); FD2Dacoustic::decompose (src/Wavefields/
Wavefields2Dacoustic.cpp:119-300) then splits P, VX and VY by the sign of a
Poynting-vector estimate: type 1 up/down with Dyf and S1 = -P*VY, type 2
left/right with Dxf and S1 = -P*VX. Each vector operation is one rounded step
in the value type, as in the reference. sign(NaN) is taken as 0.
"""
from __future__ import annotations

import numpy as np


def _split(F, Fo, s1, D, DT, dtype):
    """The up/left and down/right parts of one field."""
    d = np.dtype(dtype).type
    neg_dtinv = d(-(d(1) / d(DT)))
    dfdt = ((np.asarray(Fo, dtype=dtype) - F).astype(dtype) * neg_dtinv).astype(dtype)
    s2 = -((D @ F).astype(dtype) * dfdt).astype(dtype)
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = d(d(np.abs(s1).max()) / d(np.abs(s2).max()))
        q = ((s2 * ratio).astype(dtype) + s1).astype(dtype)
    sg = np.sign(np.nan_to_num(q, nan=0.0))
    up = (np.abs(sg - 1) > 0).astype(dtype) * F         # sign(|sign(Q) - 1|) * F
    down = ((sg + 1) > 0).astype(dtype) * F             # sign(sign(Q) + 1) * F
    return up.astype(dtype), down.astype(dtype)


def decompose_2d_tmem(kind: int, cur, old_ez, D, DT: float, dtype=np.float32):
    """cur: (EZ, HX, HY) after the step; old_ez before it. Returns
    (EZ.up/left, EZ.down/right)."""
    EZ, HX, HY = (np.asarray(a, dtype=dtype) for a in cur)
    s1 = (EZ * HX).astype(dtype) if kind == 1 else -(EZ * HY).astype(dtype)
    return list(_split(EZ, old_ez, s1, D, DT, dtype))


def decompose_2d_acoustic(kind: int, cur, old, D, DT: float, dtype=np.float32):
    """cur, old: (P, VX, VY) after and before the step; D: the DT-scaled Dyf
    (kind 1) or Dxf (kind 2) as a sparse matrix. Returns the six parts in the
    order F.up/left, F.down/right for F = P, VX, VY."""
    d = np.dtype(dtype).type
    P, VX, VY = (np.asarray(a, dtype=dtype) for a in cur)
    s1 = ((-P) * (VY if kind == 1 else VX)).astype(dtype)
    neg_dtinv = d(-(d(1) / d(DT)))
    out = []
    for F, Fo in zip((P, VX, VY), old):
        dfdt = ((np.asarray(Fo, dtype=dtype) - F).astype(dtype) * neg_dtinv).astype(dtype)
        s2 = -((D @ F).astype(dtype) * dfdt).astype(dtype)
        with np.errstate(divide="ignore", invalid="ignore"):
            ratio = d(d(np.abs(s1).max()) / d(np.abs(s2).max()))
            q = ((s2 * ratio).astype(dtype) + s1).astype(dtype)
        sg = np.sign(np.nan_to_num(q, nan=0.0))
        up = (np.abs(sg - 1) > 0).astype(dtype) * F         # sign(|sign(Q) - 1|) * F
        down = ((sg + 1) > 0).astype(dtype) * F             # sign(sign(Q) + 1) * F
        out += [up.astype(dtype), down.astype(dtype)]
    return out
