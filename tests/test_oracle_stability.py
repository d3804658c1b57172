"""Finding kept under test: the current sparse-operator edge rule of the
reference (the FD order is lowered near the grid edges until the stencil fits,
Derivatives.cpp:166-179 and 743-756) makes the elastic time step unstable on a
heterogeneous model, whatever the time step: on a 64 x 64 grid, order 8, a
+-5 % point-wise random velocity model and no damping boundary, the FP64 oracle
grows without bound after a few hundred steps, while the zero-padded edge rows
(edgeOrderReduction = 0, the rule the reference's CI golden seismograms were
made with) stay bounded. The CUDA path reproduces the growth (it follows the
oracle step for step), so long records on heterogeneous models use
edgeOrderReduction = 0 or enough damping."""
import os

import numpy as np
import pytest


def _max_vx_history(refcpu, reduce, steps=1500, chunk=500, n=64, dt=2e-4):
    refcpu.set_threads(os.cpu_count() or 1)
    rng = np.random.default_rng(1)
    vp = 3000.0 * (1 + 0.05 * np.clip(rng.standard_normal(n * n), -1, 1))
    model = dict(vp=vp, vs=vp / 1.73, rho=310.0 * vp ** 0.25)
    cfg = refcpu.make_config(dimension=2, equation="elastic", NX=n, NY=n, NZ=1, DH=2.0, DT=dt, T=steps * dt,
                             spatialFDorder=8, DampingBoundary=0, edgeOrderReduction=reduce)
    sig = refcpu.ricker(refcpu.nt_of(cfg), dt, 10.0, 1.0, 0.0, np.float64)[None]
    o = refcpu.Oracle(cfg, model, np.array([n // 2 + n * (n // 2)]), np.array([1]), sig, np.array([5 + n * 5]),
                      np.array([2]), dtype=np.float64)
    out = []
    for k in range(0, steps, chunk):
        o.step(k, k + chunk)
        out.append(float(np.abs(o.field("vx")).max()))
    o.close()
    return out


@pytest.mark.parametrize("dt", [2e-4, 1e-4])
def test_edge_order_reduction_grows_on_a_heterogeneous_model(refcpu, dt):
    grown = _max_vx_history(refcpu, 1, dt=dt, steps=1500 if dt == 2e-4 else 3000, chunk=500 if dt == 2e-4 else 1000)
    padded = _max_vx_history(refcpu, 0, dt=dt, steps=1500 if dt == 2e-4 else 3000, chunk=500 if dt == 2e-4 else 1000)
    assert grown[-1] > 1e4 * grown[0]          # exponential growth (half the CFL step too)
    assert padded[-1] < 10 * padded[0]         # bounded with zero-padded edge rows
