"""The NVTX ranges around the library's phases (csrc/trace.h, the counterpart
of the reference's SCAI_REGION markers) are host-side only: a run with the
ranges switched off (WAVE_TRACE=0) gives bit-identical seismograms and
gradients to a run with them on, and the same misfit to its atomic sum's
rounding."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import __graft_entry__ as g
wave = g.load_package()
cfg = wave.WaveConfig.make(dimension=2, equation="elastic", NX=60, NY=50, DH=5.0, DT=4e-4, T=0.08,
                           spatialFDorder=4, DampingBoundary=2, BoundaryWidth=10, NPower=4.0,
                           CenterFrequencyCPML=15.0, VMaxCPML=3000.0, FreeSurface=1)
n = cfg.N
rng = np.random.default_rng(5)
m = dict(vp=rng.uniform(2500, 3000, n).astype(np.float32), vs=rng.uniform(1400, 1700, n).astype(np.float32),
         rho=rng.uniform(1800, 2200, n).astype(np.float32))
s = wave.Factory.Create("2D", "elastic").initForwardSolver(cfg)
s.prepareForModelling(m)
sig = wave.wavelet(1, s.nt, cfg.DT, 15.0, 1.0, 0.0)[None]
s.setSources(np.array([30 + 60 * 10], np.int64), np.array([1], np.int32), sig)
s.setReceivers(np.array([10 + 60 * 5, 45 + 60 * 30], np.int64), np.array([2, 1], np.int32))
s.run(0, s.nt)
seis = s.seismograms()
J, gvp, gvs, grho = s.adjoint_gradient((0.8 * seis).astype(np.float32), checkpoint_every=40)
s.close()
print(json.dumps(dict(seis=seis.tobytes().hex(), J=J, g=np.concatenate([gvp, gvs, grho]).tobytes().hex())))
"""


def _run(trace):
    env = dict(os.environ, WAVE_TRACE=trace)
    out = subprocess.run([sys.executable, "-c", CHILD, ROOT], env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return json.loads(out.stdout.strip().splitlines()[-1])


def test_trace_switch_does_not_change_results():
    on, off = _run("1"), _run("0")
    seis = np.frombuffer(bytes.fromhex(on["seis"]), np.float32)
    assert np.abs(seis).max() > 0
    assert on["seis"] == off["seis"]
    # the misfit is a double-precision atomic sum over the residual samples, its
    # last bits follow the order the additions land in (as between any two runs)
    assert on["J"] > 0 and abs(on["J"] - off["J"]) <= 1e-12 * on["J"]
    assert on["g"] == off["g"]
