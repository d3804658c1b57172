"""The adjoint gradient on the acoustic variable grid (vargrid.cu
vargrid_adjoint, through wave_adjoint_gradient) against the FP64 oracle
adjoint (oracle/vargrid_adjoint.py, pinned to FP64 finite differences at 1e-6
in tests/test_oracle_vargrid_adjoint.py): acoustic and elastic, 2-D and 3-D, CPML, ABS or no damping boundary, with and without the mirror free
surface, 1:3 and 1:3:1 grids. Gate: 1e-4 relative L2 on each gradient, 1e-4
on the misfit."""
import ctypes

import numpy as np
import pytest

from test_oracle_vargrid_adjoint import _gradient, vg_case, vg_observed, vge_gradient, vge_observed

pytestmark = pytest.mark.gpu
GRAD_TOL = 1e-4


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("dim,fs,boundary,edge", [(2, 1, 2, 1), (2, 0, 1, 0), (2, 1, 0, 1), (3, 1, 2, 1), (3, 0, 1, 1)])
def test_vargrid_adjoint_matches_the_fp64_oracle_gradient(wave, refcpu, dim, fs, boundary, edge):
    c = vg_case(refcpu, dim, fs, boundary, edge, nt=300 if dim == 2 else 200)
    dobs = vg_observed(c).astype(np.float32)
    cfg = wave.WaveConfig()
    ctypes.memmove(ctypes.byref(cfg), ctypes.byref(c["cfg"]), ctypes.sizeof(cfg))
    s = wave.Factory.Create("3D" if dim == 3 else "2D", "acoustic").initForwardSolver(cfg)
    try:
        assert s.nt == c["nt"]
        s.prepareForModelling(dict(vp=c["vp"].astype(np.float32), rho=c["rho"].astype(np.float32)))
        s.setSources(c["src_idx"], c["src_type"], c["signals"].astype(np.float32))
        s.setReceivers(c["rec_idx"], c["rec_type"])
        J, gvp, gvs, grho = s.adjoint_gradient(dobs, checkpoint_every=37)
    finally:
        s.close()
    J64, rvp, rrho = _gradient(c, dobs.astype(np.float64))
    errs = [_rel(gvp, rvp), _rel(grho, rrho)]
    print(f"variable-grid adjoint {dim}-D fs={fs} boundary={boundary} edge={edge}: misfit {J:.6e} vs FP64 {J64:.6e}; "
          f"gradient rel L2 vp {errs[0]:.2e} rho {errs[1]:.2e}")
    assert not np.any(gvs)
    assert J > 0 and abs(J - J64) <= 1e-4 * J64
    assert max(errs) <= GRAD_TOL


def _solver(wave, c, dim, equation, model):
    cfg = wave.WaveConfig()
    ctypes.memmove(ctypes.byref(cfg), ctypes.byref(c["cfg"]), ctypes.sizeof(cfg))
    s = wave.Factory.Create("3D" if dim == 3 else "2D", equation).initForwardSolver(cfg)
    s.prepareForModelling({k: v.astype(np.float32) for k, v in model.items()})
    s.setSources(c["src_idx"], c["src_type"], c["signals"].astype(np.float32))
    s.setReceivers(c["rec_idx"], c["rec_type"])
    return s


@pytest.mark.parametrize("dim,fs,boundary,edge", [(2, 1, 2, 1), (2, 0, 1, 0), (2, 1, 0, 1), (2, 0, 2, 1), (3, 1, 2, 1),
                                                 (3, 0, 1, 1), (3, 1, 0, 1)])
def test_elastic_vargrid_adjoint_matches_the_fp64_oracle_gradient(wave, refcpu, dim, fs, boundary, edge):
    """Elastic on the variable grid (vge_vel / vge_str with the staggered operators, the shear
    averages and the surface exchange), 2-D and 3-D, against the oracle's FP64 adjoint."""
    c = vg_case(refcpu, dim, fs, boundary, edge, nt=300 if dim == 2 else 200, equation="elastic")
    dobs = vge_observed(c).astype(np.float32)
    s = _solver(wave, c, dim, "elastic", dict(vp=c["vp"], vs=c["vs"], rho=c["rho"]))
    try:
        assert s.nt == c["nt"]
        J, gvp, gvs, grho = s.adjoint_gradient(dobs, checkpoint_every=41)
    finally:
        s.close()
    J64, rvp, rvs, rrho = vge_gradient(c, dobs.astype(np.float64))
    errs = [_rel(gvp, rvp), _rel(gvs, rvs), _rel(grho, rrho)]
    print(f"variable-grid elastic adjoint {dim}-D fs={fs} boundary={boundary} edge={edge}: misfit {J:.6e} vs FP64 {J64:.6e}; "
          f"gradient rel L2 vp {errs[0]:.2e} vs {errs[1]:.2e} rho {errs[2]:.2e}")
    assert J > 0 and abs(J - J64) <= 1e-4 * J64
    assert max(errs) <= GRAD_TOL
