"""Host-side checks of the C ABI that need no GPU: the library loads and exports
every entry point include/wave.h declares, the parameter-file reader follows
the reference's rules, the wavelets match, and argument errors come back as
status codes before any CUDA call."""
import ctypes
import os
import re

import numpy as np
import pytest

import ci_cases

ROOT = ci_cases.ROOT


def header_symbols():
    text = open(os.path.join(ROOT, "include", "wave.h")).read()
    return set(re.findall(r"\b(wave_[a-z_]+)\s*\(", text))


def test_library_exports_every_declared_symbol(wave):
    L = wave.lib()
    declared = header_symbols()
    assert declared == set(wave.ABI_SYMBOLS)
    for name in declared:
        assert hasattr(L, name), name


@pytest.mark.parametrize("name", sorted(n for n in ci_cases.CASES if not n.endswith("visco")))
def test_parameter_file_reader_matches_reference_rules(name, wave, refcpu):
    path = os.path.join(ci_cases.CI, ci_cases.CASES[name][0])
    mine = wave.WaveConfig.from_file(path)
    ref = refcpu.config_from_parameters(refcpu.read_parameter_file(path))
    for f, _ in wave.WaveConfig._fields_:
        a, b = getattr(mine, f), getattr(ref, f)
        if isinstance(a, ctypes.Array):
            assert list(a) == list(b), f
        else:
            assert a == b, f


def test_legacy_visco_key_is_rejected_like_the_current_factory(wave):
    """The visco CI files say equationType=visco, which the current factory
    rejects (ForwardSolverFactory.cpp:13); the key is "viscoelastic" now."""
    with pytest.raises(wave.WaveError) as e:
        wave.WaveConfig.from_file(os.path.join(ci_cases.CI, "configuration_ci.2D.visco.txt"))
    assert e.value.code == wave.WAVE_ERR_ARG


def test_parameter_file_missing_key_is_an_error(wave, tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("dimension=2D\nequationType=acoustic\nNX=10\n")
    with pytest.raises(wave.WaveError) as e:
        wave.WaveConfig.from_file(str(p))
    assert e.value.code == wave.WAVE_ERR_ARG
    with pytest.raises(wave.WaveError) as e:
        wave.WaveConfig.from_file(str(tmp_path / "missing.txt"))
    assert e.value.code == wave.WAVE_ERR_IO


def test_ricker_matches_reference_formula(wave, refcpu):
    for fc, amp, ts in ((5.0, 5.0, 0.0), (15.0, 1.0, 0.01), (200e6, 1.0, 0.0)):
        dt = 2e-3 if fc < 100 else 7e-11
        a = wave.wavelet(1, 1000, dt, fc, amp, ts)
        b = refcpu.ricker(1000, dt, fc, amp, ts, np.float32)
        assert np.allclose(a, b, rtol=1e-5, atol=1e-6 * amp)


@pytest.mark.parametrize("shape", range(1, 10))
def test_every_wavelet_shape_is_finite(wave, shape):
    s = wave.wavelet(shape, 500, 1e-3, 10.0, 2.0, 0.05)
    assert np.all(np.isfinite(s)) and np.abs(s).max() > 0


def test_wavelet_rejects_bad_shape(wave):
    with pytest.raises(wave.WaveError):
        wave.wavelet(42, 10, 1e-3, 10.0, 1.0, 0.0)


@pytest.mark.parametrize("kw,code", [
    (dict(spatialFDorder=5), 1),                       # unsupported FD order
    (dict(dimension=3, equation="sh", NZ=8), 5),       # no 3-D SH solver in the factory
    (dict(DampingBoundary=2, BoundaryWidth=0), 1),     # CPML without a width
    (dict(equation="viscoelastic", numRelaxationMechanisms=0), 1),
    (dict(DT=-1.0), 1),
])
def test_create_rejects_bad_configs_without_touching_the_gpu(wave, kw, code):
    base = dict(dimension=2, equation="acoustic", NX=16, NY=16, DH=1.0, DT=1e-4, T=0.01, spatialFDorder=4)
    base.update(kw)
    cfg = wave.WaveConfig.make(**base)
    h = ctypes.c_void_p()
    rc = wave.lib().wave_solver_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc == code
    assert wave.lib().wave_last_error(None)


def test_nt_rule(wave, refcpu):
    for T, DT in ((2.0, 2e-3), (0.45, 1.5e-4), (0.4, 2e-4), (2.0, 5e-4)):
        cfg = wave.WaveConfig.make(NX=4, NY=4, DH=1.0, DT=DT, T=T)
        nt = ctypes.c_int()
        assert wave.lib().wave_config_nt(ctypes.byref(cfg), ctypes.byref(nt)) == 0
        assert nt.value == refcpu.nt_of(cfg)


def test_null_handle_errors(wave):
    L = wave.lib()
    assert L.wave_solver_step(None, 0, 1) == wave.WAVE_ERR_ARG
    assert L.wave_solver_destroy(None) == wave.WAVE_ERR_ARG
    assert L.wave_check_finite(None) == wave.WAVE_ERR_ARG


def test_noalloc_wrapper_rejects_host_tensors_without_touching_the_gpu(wave):
    torch = pytest.importorskip("torch")
    t = torch.ones(64)
    with pytest.raises(wave.WaveError) as e:
        wave.average_shear_modulus_noalloc(t, t, (4, 4, 4), 0)
    assert "CUDA tensor" in str(e.value)
