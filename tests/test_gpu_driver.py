"""The C++ driver (wave_simulation, the Simulation.cpp-style loop over shots)
end to end on the reference's 2-D acoustic CI case: parameter file, source and
receiver files, the time loop on the GPU, and the seismogram output path
(SeismogramFormat 4 = SU as the CI file asks, and MatrixMarket with trace
normalisation and resampling), compared with the reference's golden seismogram
(par/ci/seismogram.2D.acoustic.ref.p.mtx) under the reference's gate."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import refcpu
from test_gpu_seismo import resample_reference

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ci")
GATE = 5e-7


def _setup(tmp_path, edits):
    ci = tmp_path / "ci"
    ci.mkdir()
    for f in ("sources_ci.2D.txt", "receiver_ci.2D.txt"):
        shutil.copy(os.path.join(GOLDEN, f), ci / f)
    text = open(os.path.join(GOLDEN, "configuration_ci.2D.acoustic.txt")).read().splitlines()
    out, seen = [], set()
    for line in text:
        key = line.split("=")[0].strip() if "=" in line else None
        if key in edits:
            seen.add(key)
        out.append(f"{key}={edits[key]}" if key in edits else line)
    out += [f"{k}={v}" for k, v in edits.items() if k not in seen]
    cfg = ci / "configuration.txt"
    cfg.write_text("\n".join(out) + "\n")
    return cfg, ci


def _run(wave, cfg):
    exe = os.path.join(os.path.dirname(wave.LIB_PATH), "wave_simulation")
    r = subprocess.run([exe, str(cfg)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr


def test_driver_su_output_matches_reference_golden(wave, tmp_path):
    cfg, ci = _setup(tmp_path, {})
    _run(wave, cfg)
    raw = open(ci / "seismogram.2D.acoustic.ci.shot_1.p.su", "rb").read()
    ns = int(np.frombuffer(raw, dtype="<u2", count=1, offset=114)[0])
    trace = np.frombuffer(raw, dtype="<f4", count=ns, offset=240)[None, :].astype(np.float64)
    golden = refcpu.read_mtx_array(os.path.join(GOLDEN, "seismogram.2D.acoustic.ref.p.mtx"))
    assert trace.shape == golden.shape
    assert refcpu.reference_misfit(trace, golden) < GATE
    assert np.linalg.norm(trace - golden) / np.linalg.norm(golden) < 1e-4


def test_driver_mtx_output_with_normalisation_and_resampling(wave, tmp_path):
    cfg, ci = _setup(tmp_path, {"SeismogramFormat": "1", "normalizeTraces": "1", "seismoDT": "6.0e-03"})
    _run(wave, cfg)
    got = refcpu.read_mtx_array(str(ci / "seismogram.2D.acoustic.ci.shot_1.p.mtx"))
    golden = refcpu.read_mtx_array(os.path.join(GOLDEN, "seismogram.2D.acoustic.ref.p.mtx")).astype(np.float32)
    ref = resample_reference(golden / np.abs(golden).max(axis=1, keepdims=True), 2e-3, 6e-3)
    assert got.shape == ref.shape
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-4


def test_driver_agc_normalisation_writes_the_inverse_agc(wave, tmp_path):
    """normalizeTraces=3 (Simulation.cpp:521-525): the inverse AGC is written as
    <seismogram>.shot_1.p.inverseAGC.mtx and the seismogram is the l2-normalised
    trace times it; the AGC window comes from CenterFrequencyCPML."""
    from test_gpu_seismo import agc_reference
    cfg, ci = _setup(tmp_path, {"SeismogramFormat": "1", "normalizeTraces": "3", "CenterFrequencyCPML": "5.0"})
    _run(wave, cfg)
    got = refcpu.read_mtx_array(str(ci / "seismogram.2D.acoustic.ci.shot_1.p.mtx"))
    inv = refcpu.read_mtx_array(str(ci / "seismogram.2D.acoustic.ci.shot_1.p.inverseAGC.mtx"))
    keys = dict(line.split("#")[0].split("=", 1) for line in open(cfg).read().splitlines() if "=" in line.split("#")[0])
    keys = {k.strip(): v.strip() for k, v in keys.items()}
    dt, fc = float(keys["DT"]), float(keys.get("CenterFrequencyCPML", "5"))
    golden = refcpu.read_mtx_array(os.path.join(GOLDEN, "seismogram.2D.acoustic.ref.p.mtx")).astype(np.float32)
    ref, ref_inv = agc_reference(golden, dt, fc)
    assert got.shape == ref.shape and inv.shape == ref_inv.shape
    # the GPU seismogram differs from the reference golden at the 1e-5 level; the AGC output follows
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-3
    assert np.linalg.norm(inv - ref_inv) / np.linalg.norm(ref_inv) < 1e-3


def test_driver_snapshots_equal_the_solver_fields(wave, tmp_path):
    cfg, ci = _setup(tmp_path, {"snapType": "1", "tFirstSnapshot": "0.2", "tlastSnapshot": "0.6", "tincSnapshot": "0.2",
                                "WavefieldFileName": "ci/wavefield"})
    _run(wave, cfg)
    wc = wave.WaveConfig.from_file(str(cfg))
    s = wave.Factory.Create("2D", "acoustic").initForwardSolver(wc)
    s.prepareForModelling(dict(rho=np.full(wc.N, 2000.0, np.float32), vp=np.full(wc.N, 3500.0, np.float32)))
    src = [l.split() for l in open(ci / "sources_ci.2D.txt") if l.strip() and not l.startswith("#")][0]
    x, y, z, typ, shape, fc, amp, ts = (int(src[1]), int(src[2]), int(src[3]), int(src[4]), int(src[6]), float(src[7]),
                                        float(src[8]), float(src[9]))
    s.setSources(np.array([x + wc.NX * y], np.int64), np.array([typ], np.int32),
                 wave.wavelet(shape, s.nt, wc.DT, fc, amp, ts)[None])
    rec = [l.split() for l in open(ci / "receiver_ci.2D.txt") if l.strip() and not l.startswith("#")]
    s.setReceivers(np.array([int(r[0]) + wc.NX * int(r[1]) for r in rec], np.int64), np.array([int(r[3]) for r in rec], np.int32))
    t = 0
    for step in (100, 200, 300):
        s.run(t, step + 1)
        t = step + 1
        for name in ("VX", "VY"):
            snap = refcpu.read_mtx_array(str(ci / f"wavefield.shot_1.{name}.{step}.mtx"))[:, 0]
            assert np.array_equal(snap.astype(np.float32), s.field(name)), (name, step)
    s.close()


def test_driver_runs_the_variable_grid_ci_case(wave, tmp_path):
    """The 2-D variable-grid CI case through the driver: gridConfigurationFilename
    read relative to the parameter file, sources and receivers mapped with
    Coordinates::coordinate2index, the seismogram under the reference's gate."""
    ci = tmp_path / "ci"
    ci.mkdir()
    for f in ("sources_ci.2D.varGrid.txt", "receiver_ci.2D.varGrid.txt", "gridConfig.txt"):
        shutil.copy(os.path.join(GOLDEN, f), ci / f)
    text = open(os.path.join(GOLDEN, "configuration_ci.2D.acoustic.varGrid.txt")).read()
    cfg = ci / "configuration.txt"
    cfg.write_text(text + "\nedgeOrderReduction=0\n")
    _run(wave, cfg)
    got = refcpu.read_mtx_array(str(ci / "seismogram.2D.acoustic.varGrid.ci.shot_0.p.mtx"))
    golden = refcpu.read_mtx_array(os.path.join(GOLDEN, "seismogram.2D.acoustic.varGrid.ref.p.mtx"))
    assert got.shape == golden.shape
    assert refcpu.reference_misfit(got, golden) < GATE


def test_driver_writes_the_decomposition_snapshots(wave, tmp_path):
    """decomposeWavefieldType=1 with snapType=4: the driver writes P, VX, VY
    and their up/down parts (Wavefields2Dacoustic.cpp:86-95); each part is the
    field or zero and the two parts cover the field."""
    cfg, ci = _setup(tmp_path, {"snapType": "4", "decomposeWavefieldType": "1", "tFirstSnapshot": "0.3",
                                "tlastSnapshot": "0.3", "tincSnapshot": "0.1", "WavefieldFileName": "ci/wavefield"})
    _run(wave, cfg)
    step = 150
    for f in ("P", "VX", "VY"):
        F = refcpu.read_mtx_array(str(ci / f"wavefield.shot_1.{f}.{step}.mtx"))[:, 0]
        up = refcpu.read_mtx_array(str(ci / f"wavefield.shot_1.{f}.up.{step}.mtx"))[:, 0]
        down = refcpu.read_mtx_array(str(ci / f"wavefield.shot_1.{f}.down.{step}.mtx"))[:, 0]
        assert np.abs(F).max() > 0
        assert np.all((up == F) | (up == 0)) and np.all((down == F) | (down == 0))
        assert np.all((up == F) | (down == F))
        assert np.any(up != F) and np.any(down != F)


def test_driver_runs_a_visco_tm_parameter_file(wave, tmp_path):
    """equationType=viscotmem through the C++ plugin mirror and the driver:
    the relaxation times come from the tauEpsilon / tauSigmar keys
    (ViscoTMEM.cpp:206), are passed by prepareForModelling, and the
    seismogram equals the same run through the Python binding and the FP64
    oracle within 1e-4."""
    DT, nt = 4.0e-11, 500
    edits = {"equationType": "viscotmem", "DH": "0.02", "DT": f"{DT:.3e}", "T": f"{(nt - 0.4) * DT:.6e}",
             "spatialFDorder": "4", "DampingBoundary": "2", "BoundaryWidth": "10", "centerfrequencycpml": "1.0e8",
             "vmaxcpml": "1.0e8", "numRelaxationMechanisms": "1", "relaxationFrequency": "1.0e8", "epsilonr": "9.0",
             "sigma": "0.005", "mur": "1.0", "tauEpsilon": "0.1", "tauSigmar": "0.1", "SeismogramFormat": "1",
             "seismoDT": f"{DT:.3e}",
             "useStencilMatrix": "0", "SourceFilename": "ci/sources_em", "ReceiverFilename": "ci/receiver_em",
             "SeismogramFilename": "ci/seismogram.em"}
    cfg, ci = _setup(tmp_path, edits)
    (ci / "sources_em.txt").write_text("1 49 49 0 1 1 1 4.0e8 1.0 0.0\n")
    (ci / "receiver_em.txt").write_text("69 69 0 1\n30 40 0 1\n")
    _run(wave, cfg)
    got = refcpu.read_mtx_array(str(ci / "seismogram.em.shot_1.ez.mtx"))
    wc = wave.WaveConfig.from_file(str(cfg))
    assert wc.equation == wave.EQUATIONS["viscotmem"] and wc.numRelaxationMechanisms == 1
    n = wc.N
    model = dict(eps_r=np.full(n, 9.0), sigma=np.full(n, 0.005), mu_r=np.ones(n), tau_eps=np.full(n, 0.1),
                 tau_sigma=np.full(n, 0.1))
    nt = refcpu.nt_of(wc)
    sidx = np.array([49 + 100 * 49], np.int64)
    sig = wave.wavelet(1, nt, wc.DT, 4.0e8, 1.0, 0.0)[None].astype(np.float64)
    ridx = np.array([69 + 100 * 69, 30 + 100 * 40], np.int64)
    stype, rtype = np.array([1], np.int32), np.array([1, 1], np.int32)
    py = wave.simulate(wc, {k: v.astype(np.float32) for k, v in model.items()}, sidx, stype, sig.astype(np.float32),
                       ridx, rtype)
    ocfg = refcpu.WaveConfig()
    wave.WaveConfig.copy_from(ocfg, wc)
    o = refcpu.Oracle(ocfg, model, sidx, stype, sig, ridx, rtype, dtype=np.float64)
    ref = o.run()
    o.close()
    assert got.shape == ref.shape
    assert np.abs(ref).max() > 0
    assert np.linalg.norm(got - py) / np.linalg.norm(py) < 1e-6
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-4
