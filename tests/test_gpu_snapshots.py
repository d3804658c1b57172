"""Snapshots around the time loop against the FP64 oracle: wavefields
(wave_get_field, the data of Wavefields*::write snapType 1/2) and the snapType 3
curl and divergence energies (Wavefields2Delastic.cpp:218-250,
Wavefields3Delastic.cpp:197-240), after a number of steps."""
import numpy as np
import pytest

from test_gpu_parity import make_case, rel, to_wave_cfg

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.mark.parametrize("eq,dim,order,fs,boundary", [("elastic", 2, 4, 1, 2), ("elastic", 3, 8, 0, 2),
                                                      ("viscoelastic", 2, 6, 0, 1), ("elastic", 3, 4, 1, 1)])
def test_fields_and_energies_match_oracle(wave, refcpu, eq, dim, order, fs, boundary):
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, eq, dim, order, fs, boundary)
    steps = 180
    o = refcpu.Oracle(cfg, model, sidx, stype, sig, ridx, rtype, dtype=np.float64)
    o.step(0, steps)
    wc = to_wave_cfg(wave, cfg)
    s = wave.Factory.Create("3D" if dim == 3 else "2D", eq).initForwardSolver(wc)
    s.prepareForModelling({k: v.astype(np.float32) for k, v in model.items()})
    s.set_kernel_path(1)
    s.setSources(sidx, stype, sig.astype(np.float32))
    s.setReceivers(ridx, rtype)
    s.run(0, steps)
    names = ["vx", "vy", "sxx", "syy", "sxy"] + (["vz", "szz", "sxz", "syz"] if dim == 3 else [])
    for n in names:
        ref = o.field(n)
        assert rel(s.field(n.upper() if n.startswith("v") else "S" + n[1:]), ref) < TOL, n
    curl, div = s.curl_div()
    rc, rd = o.curl_div()
    assert np.abs(rc).max() > 0 and np.abs(rd).max() > 0
    assert rel(curl, rc) < TOL
    assert rel(div, rd) < TOL
    with pytest.raises(wave.WaveError):
        s.field("EZ")
    s.close()
    o.close()
