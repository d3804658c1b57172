"""Python host binding of the GB300 forward solver (libwavegpu.so, include/wave.h).

It mirrors the reference's plugin interface for the time-stepping hot path so
that tests read like the reference's own:

* ``Factory.Create(dimension, equationType)`` ~ ForwardSolver::Factory<float>::Create
  (src/ForwardSolver/ForwardSolverFactory.cpp:4-67), case-insensitive keys;
* ``ForwardSolver.initForwardSolver(config)`` / ``prepareForModelling(model)`` /
  ``run(t)`` / ``resetCPML()`` ~ the virtual methods of ForwardSolver
  (src/ForwardSolver/ForwardSolver.hpp:25-70);
* errors raise ``WaveError`` with the library's message (the reference throws
  COMMON_THROWEXCEPTION / SCAI_ASSERT_ERROR).

There is no CPU fallback: every call goes through the CUDA library, and loading
fails loudly when it is missing.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libwavegpu.so")

WAVE_OK, WAVE_ERR_ARG, WAVE_ERR_CUDA, WAVE_ERR_NONFINITE, WAVE_ERR_TIMEOUT, WAVE_ERR_UNSUPPORTED, WAVE_ERR_STATE, WAVE_ERR_IO = range(8)
MEM_HOST, MEM_DEVICE = 0, 1
EQUATIONS = {"acoustic": 0, "elastic": 1, "viscoelastic": 2, "sh": 3, "viscosh": 4,
             "tmem": 5, "emem": 6, "viscotmem": 7, "viscoemem": 8}

# every entry point declared in include/wave.h
ABI_SYMBOLS = (
    "wave_config_nt", "wave_config_from_file", "wave_solver_create", "wave_solver_destroy",
    "wave_set_model", "wave_set_model_em", "wave_set_sources", "wave_set_receivers",
    "wave_solver_step", "wave_solver_reset", "wave_get_seismograms", "wave_check_finite",
    "wave_get_state_size", "wave_get_state", "wave_set_state", "wave_get_nt",
    "wave_get_num_receivers", "wave_device_bytes", "wave_get_stream", "wave_get_launch_count", "wave_set_timing",
    "wave_get_kernel_times", "wave_last_error", "wave_wavelet", "wave_set_kernel_path",
    "wave_get_kernel_path", "wave_average_shear_modulus", "wave_batch_create", "wave_batch_destroy",
    "wave_batch_shot", "wave_batch_step", "wave_batch_get_stream", "wave_batch_get_launch_count",
    "wave_batch_last_error", "wave_batch_set_schedule", "wave_batch_get_schedule", "wave_average_shear_modulus_noalloc", "wave_adjoint_gradient",
    "wave_batch_adjoint_gradient", "wave_resample_traces", "wave_normalize_traces", "wave_read_mtx",
    "wave_write_mtx", "wave_write_su", "wave_get_field", "wave_get_curl_div", "wave_envelope",
    "wave_instantaneous_phase", "wave_selftest_bounded_wait", "wave_set_dependent_launch",
    "wave_agc_normalize_traces", "wave_grid_num_points", "wave_grid_index", "wave_grid_coordinates",
    "wave_set_decomposition", "wave_grid_operator", "wave_encode_sources", "wave_encode_frequencies",
    "wave_encode_sources_frequency", "wave_encode_traces",
)


class WaveError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[wave error {code}] {msg}")
        self.code = code


class WaveConfig(ctypes.Structure):
    """ctypes mirror of ``wave_config`` (include/wave.h)."""
    _fields_ = [
        ("dimension", ctypes.c_int),
        ("equation", ctypes.c_int),
        ("NX", ctypes.c_int64), ("NY", ctypes.c_int64), ("NZ", ctypes.c_int64),
        ("DH", ctypes.c_double), ("DT", ctypes.c_double), ("T", ctypes.c_double),
        ("spatialFDorder", ctypes.c_int),
        ("FreeSurface", ctypes.c_int),
        ("DampingBoundary", ctypes.c_int),
        ("BoundaryWidth", ctypes.c_int),
        ("DampingCoeff", ctypes.c_double),
        ("NPower", ctypes.c_double),
        ("CenterFrequencyCPML", ctypes.c_double),
        ("VMaxCPML", ctypes.c_double),
        ("numRelaxationMechanisms", ctypes.c_int),
        ("relaxationFrequency", ctypes.c_double * 4),
        ("useStencilMatrix", ctypes.c_int),
        ("edgeOrderReduction", ctypes.c_int),
        ("useVariableGrid", ctypes.c_int),
        ("useVariableFDoperators", ctypes.c_int),
        ("gridLayers", ctypes.c_int),
        ("gridInterface", ctypes.c_int * 16),
        ("gridDHFactor", ctypes.c_int * 16),
        ("gridFDOrder", ctypes.c_int * 16),
    ]

    @classmethod
    def from_file(cls, path: str) -> "WaveConfig":
        c = cls()
        _check(None, lib().wave_config_from_file(path.encode(), ctypes.byref(c)))
        return c

    @classmethod
    def make(cls, **kw) -> "WaveConfig":
        c = cls()
        c.dimension = kw.get("dimension", 2)
        eq = kw.get("equation", "acoustic")
        c.equation = EQUATIONS[eq.lower()] if isinstance(eq, str) else int(eq)
        c.NX, c.NY, c.NZ = kw["NX"], kw["NY"], kw.get("NZ", 1)
        c.DH, c.DT, c.T = kw["DH"], kw["DT"], kw["T"]
        c.spatialFDorder = kw.get("spatialFDorder", 2)
        c.FreeSurface = kw.get("FreeSurface", 0)
        c.DampingBoundary = kw.get("DampingBoundary", 0)
        c.BoundaryWidth = kw.get("BoundaryWidth", 0)
        c.DampingCoeff = kw.get("DampingCoeff", 8.0)
        c.NPower = kw.get("NPower", 4.0)
        c.CenterFrequencyCPML = kw.get("CenterFrequencyCPML", 5.0)
        c.VMaxCPML = kw.get("VMaxCPML", 3500.0)
        c.numRelaxationMechanisms = kw.get("numRelaxationMechanisms", 0)
        rf = list(kw.get("relaxationFrequency", [])) + [0.0] * 4
        for i in range(4):
            c.relaxationFrequency[i] = rf[i]
        c.useStencilMatrix = kw.get("useStencilMatrix", 0)
        c.edgeOrderReduction = kw.get("edgeOrderReduction", 1)
        # variable grid: grid = [(first depth index, dhFactor, FD order), ...]
        # (the rows of the reference's gridConfigurationFilename)
        c.useVariableGrid = kw.get("useVariableGrid", 0)
        c.useVariableFDoperators = kw.get("useVariableFDoperators", 0)
        grid = kw.get("grid", [])
        if len(grid) > 16:
            raise ValueError("at most 16 grid layers")
        c.gridLayers = len(grid)
        for i, row in enumerate(grid):
            c.gridInterface[i], c.gridDHFactor[i] = int(row[0]), int(row[1])
            c.gridFDOrder[i] = int(row[2]) if len(row) > 2 else c.spatialFDorder
        return c

    def copy_from(self, other) -> "WaveConfig":
        """Copies the fields of another ctypes config with the same layout."""
        ctypes.memmove(ctypes.byref(self), ctypes.byref(other), ctypes.sizeof(WaveConfig))
        return self

    @property
    def N(self) -> int:
        """Number of grid points (the variable grid's layered points, or NX*NY*NZ)."""
        return grid_num_points(self)


_lib = None


def build(verbose: bool = False) -> str:
    """Compiles libwavegpu.so for sm_103a with nvcc (Makefile next to this file)."""
    jobs = str(min(8, os.cpu_count() or 1))
    out = None if verbose else subprocess.DEVNULL
    subprocess.run(["make", "-s", "-j", jobs, "-C", HERE], check=True, stdout=out)
    return LIB_PATH


def lib():
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it first (__graft_entry__.build())")
    L = ctypes.CDLL(LIB_PATH)
    P, I, CP = ctypes.c_void_p, ctypes.c_int, ctypes.POINTER
    L.wave_last_error.restype = ctypes.c_char_p
    L.wave_last_error.argtypes = [P]
    L.wave_config_from_file.argtypes = [ctypes.c_char_p, CP(WaveConfig)]
    L.wave_config_nt.argtypes = [CP(WaveConfig), CP(I)]
    L.wave_solver_create.argtypes = [CP(WaveConfig), CP(P)]
    L.wave_solver_destroy.argtypes = [P]
    L.wave_set_model.argtypes = [P, P, P, P, P, P, ctypes.c_size_t, I]
    L.wave_set_model_em.argtypes = [P, P, P, P, P, P, ctypes.c_size_t, I]
    L.wave_set_sources.argtypes = [P, I, P, P, P, I]
    L.wave_set_receivers.argtypes = [P, I, P, P]
    L.wave_solver_step.argtypes = [P, I, I]
    L.wave_solver_reset.argtypes = [P]
    L.wave_get_seismograms.argtypes = [P, P, ctypes.c_size_t, I]
    L.wave_check_finite.argtypes = [P]
    L.wave_get_state_size.argtypes = [P, CP(ctypes.c_size_t)]
    L.wave_get_state.argtypes = [P, P, ctypes.c_size_t, I]
    L.wave_set_state.argtypes = [P, P, ctypes.c_size_t, I]
    L.wave_get_nt.argtypes = [P, CP(I)]
    L.wave_get_num_receivers.argtypes = [P, CP(I)]
    L.wave_device_bytes.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    L.wave_get_stream.argtypes = [P, CP(P)]
    L.wave_get_launch_count.argtypes = [P, CP(ctypes.c_longlong)]
    L.wave_set_timing.argtypes = [P, I]
    L.wave_get_kernel_times.argtypes = [P, CP(ctypes.c_double), CP(ctypes.c_double), CP(ctypes.c_longlong)]
    L.wave_wavelet.argtypes = [I, I, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, P]
    L.wave_set_kernel_path.argtypes = [P, I]
    L.wave_set_dependent_launch.argtypes = [P, I]
    L.wave_set_decomposition.argtypes = [P, I]
    L.wave_get_kernel_path.argtypes = [P, CP(I)]
    L.wave_average_shear_modulus.argtypes = [P, P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, I, I]
    L.wave_average_shear_modulus_noalloc.argtypes = [P, P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, I, P]
    L.wave_adjoint_gradient.argtypes = [P, P, I, I, ctypes.POINTER(ctypes.c_double), P, P, P, I]
    i64 = ctypes.c_int64
    L.wave_resample_traces.argtypes = [P, i64, i64, ctypes.c_double, ctypes.c_double, P, ctypes.POINTER(i64), I]
    L.wave_normalize_traces.argtypes = [P, i64, i64, I, I]
    L.wave_agc_normalize_traces.argtypes = [P, i64, i64, ctypes.c_double, ctypes.c_double, P, I]
    L.wave_read_mtx.argtypes = [ctypes.c_char_p, P, i64, ctypes.POINTER(i64), ctypes.POINTER(i64)]
    L.wave_write_mtx.argtypes = [ctypes.c_char_p, P, i64, i64]
    L.wave_write_su.argtypes = [ctypes.c_char_p, P, i64, i64, ctypes.c_double, P, i64, i64, i64, i64, ctypes.c_double]
    L.wave_selftest_bounded_wait.argtypes = [ctypes.POINTER(ctypes.c_int)]
    L.wave_get_field.argtypes = [P, ctypes.c_char_p, P, I]
    L.wave_get_curl_div.argtypes = [P, P, P, I]
    L.wave_envelope.argtypes = [P, i64, i64, I]
    L.wave_instantaneous_phase.argtypes = [P, i64, i64, I, I]
    L.wave_batch_adjoint_gradient.argtypes = [P, P, I, I, ctypes.POINTER(ctypes.c_double), P, P, P, I, I]
    L.wave_batch_create.argtypes = [P, I, CP(P)]
    L.wave_batch_destroy.argtypes = [P]
    L.wave_batch_shot.argtypes = [P, I, CP(P)]
    L.wave_batch_step.argtypes = [P, I, I]
    L.wave_batch_get_stream.argtypes = [P, CP(P)]
    L.wave_batch_get_launch_count.argtypes = [P, CP(ctypes.c_longlong)]
    L.wave_batch_set_schedule.argtypes = [P, I, I, I]
    L.wave_batch_get_schedule.argtypes = [P, CP(I), CP(I), CP(I), CP(I)]
    L.wave_grid_num_points.argtypes = [CP(WaveConfig), ctypes.POINTER(i64)]
    L.wave_grid_index.argtypes = [CP(WaveConfig), i64, i64, i64, ctypes.POINTER(i64)]
    L.wave_grid_coordinates.argtypes = [CP(WaveConfig), P, P, P, i64, P]
    L.wave_grid_operator.argtypes = [CP(WaveConfig), I, CP(I), P, P, i64]
    L.wave_encode_sources.argtypes = [I, I, ctypes.c_uint, I, P, P, P, P]
    D = ctypes.c_double
    L.wave_encode_frequencies.argtypes = [I, D, D, D, D, D, P, I, CP(I)]
    L.wave_encode_sources_frequency.argtypes = [I, I, ctypes.c_uint, I, P, D, D, D, D, D, P, P, P]
    L.wave_encode_traces.argtypes = [I, I, I, ctypes.c_int64, P, P, P, P, D, I, P, P, I]
    L.wave_batch_last_error.restype = ctypes.c_char_p
    L.wave_batch_last_error.argtypes = [P]
    _lib = L
    return L


def _check(h, rc: int):
    if rc != WAVE_OK:
        raise WaveError(rc, lib().wave_last_error(h).decode())


def _ptr(a):
    """Pointer of a numpy array (host) or a torch tensor (host or device)."""
    if a is None:
        return None, MEM_HOST
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr()), (MEM_DEVICE if a.is_cuda else MEM_HOST)
    return a.ctypes.data_as(ctypes.c_void_p), MEM_HOST


def _f32(a):
    if a is None or hasattr(a, "data_ptr"):
        return a
    return np.ascontiguousarray(a, dtype=np.float32)


def grid_num_points(cfg: WaveConfig) -> int:
    """Points of the configuration's grid: NX*NY*NZ, or the variable grid's
    layered points (Coordinates::getNGridpoints)."""
    n = ctypes.c_int64()
    _check(None, lib().wave_grid_num_points(ctypes.byref(cfg), ctypes.byref(n)))
    return int(n.value)


def grid_index(cfg: WaveConfig, x: int, y: int, z: int) -> int:
    """Coordinates::coordinate2index of a fine-grid coordinate (x, y = depth, z)."""
    i = ctypes.c_int64()
    _check(None, lib().wave_grid_index(ctypes.byref(cfg), int(x), int(y), int(z), ctypes.byref(i)))
    return int(i.value)


def grid_coordinates(cfg: WaveConfig):
    """Coordinates::index2coordinate of every index: (x, y, z) int64 arrays and
    the (NX, NY, NZ) the variable grid reduced the extents to."""
    n = grid_num_points(cfg)
    xyz = [np.zeros(n, dtype=np.int64) for _ in range(3)]
    ext = np.zeros(3, dtype=np.int64)
    _check(None, lib().wave_grid_coordinates(ctypes.byref(cfg), *(a.ctypes.data_as(ctypes.c_void_p) for a in xyz), n,
                                             ext.ctypes.data_as(ctypes.c_void_p)))
    return xyz[0], xyz[1], xyz[2], tuple(int(v) for v in ext)


def grid_operator(cfg: WaveConfig, op: int):
    """The host-assembled operator `op` of a variable-grid configuration
    (wave_grid_operator: 0 Dxf, 1 Dyf, 2 Dzf, 3 Dxb, 4 Dyb, 5 Dzb, 6-8 the
    interface interpolations) as (cols, vals), each W x N."""
    n = grid_num_points(cfg)
    w = ctypes.c_int()
    _check(None, lib().wave_grid_operator(ctypes.byref(cfg), int(op), ctypes.byref(w), None, None, 0))
    cols = np.zeros((w.value, n), dtype=np.int32)
    vals = np.zeros((w.value, n), dtype=np.float32)
    _check(None, lib().wave_grid_operator(ctypes.byref(cfg), int(op), ctypes.byref(w), cols.ctypes.data_as(ctypes.c_void_p),
                                          vals.ctypes.data_as(ctypes.c_void_p), cols.size))
    return cols, vals


def encode_sources(mode: int, num_domains: int, seed: int, shot_no, amp):
    """Source encoding (wave_encode_sources): (super-shot numbers, signed
    amplitudes) for one source row per shot."""
    no = np.ascontiguousarray(shot_no, dtype=np.int32)
    a = np.ascontiguousarray(amp, dtype=np.float32)
    no_out = np.zeros_like(no)
    a_out = np.zeros_like(a)
    _check(None, lib().wave_encode_sources(int(mode), int(num_domains), int(seed) & 0xFFFFFFFF, len(no),
                                           no.ctypes.data_as(ctypes.c_void_p), a.ctypes.data_as(ctypes.c_void_p),
                                           no_out.ctypes.data_as(ctypes.c_void_p), a_out.ctypes.data_as(ctypes.c_void_p)))
    return no_out, a_out


def encode_frequencies(encoded: bool, fc1: float, fc2: float, T: float, DT: float, cpml_fc: float) -> np.ndarray:
    """The frequency list of frequency-domain modelling (wave_encode_frequencies)."""
    n = ctypes.c_int(0)
    _check(None, lib().wave_encode_frequencies(int(encoded), fc1, fc2, T, DT, cpml_fc, None, 0, ctypes.byref(n)))
    out = np.zeros(max(n.value, 1), np.float32)
    _check(None, lib().wave_encode_frequencies(int(encoded), fc1, fc2, T, DT, cpml_fc, out.ctypes.data_as(ctypes.c_void_p),
                                               out.size, ctypes.byref(n)))
    return out[:n.value]


def encode_sources_frequency(mode: int, num_domains: int, seed: int, amp, fc1: float, fc2: float, T: float, DT: float,
                             cpml_fc: float):
    """Frequency-domain source encoding (wave_encode_sources_frequency):
    (super-shot numbers, signed amplitudes, per-shot frequencies)."""
    a = np.ascontiguousarray(amp, np.float32)
    no = np.zeros(a.size, np.int32)
    ao = np.zeros(a.size, np.float32)
    fo = np.zeros(a.size, np.float32)
    _check(None, lib().wave_encode_sources_frequency(int(mode), int(num_domains), int(seed) & 0xFFFFFFFF, a.size,
                                                     a.ctypes.data_as(ctypes.c_void_p), fc1, fc2, T, DT, cpml_fc,
                                                     no.ctypes.data_as(ctypes.c_void_p), ao.ctypes.data_as(ctypes.c_void_p),
                                                     fo.ctypes.data_as(ctypes.c_void_p)))
    return no, ao, fo


def encode_traces(decode: bool, mark, super_mark, amp, fc=None, DT: float = 0.0, common_offset: bool = False,
                  shot_data=None, super_data=None, nt: int = 0):
    """Receiver-side encoding (wave_encode_traces) on host arrays: decode=False
    returns the super-shot block from the list of per-shot blocks, decode=True
    the list of per-shot blocks from the super-shot block."""
    mark = np.ascontiguousarray(mark, np.int32)
    sm = np.ascontiguousarray(super_mark, np.int32)
    a = np.ascontiguousarray(amp, np.float32)
    ns, nr = mark.shape
    f = None if fc is None else np.ascontiguousarray(fc, np.float32)
    if common_offset:
        rows = [1] * ns
        nsup = int(np.count_nonzero(sm))
    else:
        rows = [int(np.count_nonzero((mark[s] != 0) & (sm != 0))) for s in range(ns)]
        nsup = int(np.count_nonzero(sm))
    if decode:
        sup = np.ascontiguousarray(super_data, np.float32)
        nt = sup.shape[-1]
        shots = [np.zeros((r, nt), np.float32) for r in rows]
    else:
        shots = [np.ascontiguousarray(d, np.float32).reshape(r, -1) for d, r in zip(shot_data, rows)]
        nt = shots[0].shape[-1]
        sup = np.zeros((nsup, nt), np.float32)
    ptrs = (ctypes.c_void_p * ns)(*[d.ctypes.data_as(ctypes.c_void_p).value for d in shots])
    _check(None, lib().wave_encode_traces(int(decode), ns, nr, nt, mark.ctypes.data_as(ctypes.c_void_p),
                                          sm.ctypes.data_as(ctypes.c_void_p), a.ctypes.data_as(ctypes.c_void_p),
                                          None if f is None else f.ctypes.data_as(ctypes.c_void_p), float(DT), int(common_offset),
                                          ptrs, sup.ctypes.data_as(ctypes.c_void_p), MEM_HOST))
    return shots if decode else sup


def wavelet(shape: int, nt: int, dt: float, fc: float, amp: float, tshift: float) -> np.ndarray:
    """Source time function (Sources.cpp:157-215 shapes 1..9)."""
    out = np.zeros(nt, dtype=np.float32)
    _check(None, lib().wave_wavelet(shape, nt, dt, fc, amp, tshift, out.ctypes.data_as(ctypes.c_void_p)))
    return out


def average_shear_modulus(mu, dims, mode: int, out=None):
    """Harmonic S-modulus average with the reference's vacuum rules
    (ModelparameterSeismic.cpp:421-432); dims = (NX, NY, NZ); mode 0..2 = XY/XZ/YZ
    4-point, 3/4 = 2-point along x/y. numpy (host) or torch cuda arrays."""
    mu = _f32(mu)
    if out is None:
        out = np.zeros(int(np.prod(dims)), dtype=np.float32) if not hasattr(mu, "data_ptr") else mu.new_zeros(mu.shape)
    (pm, mem), (po, _) = _ptr(mu), _ptr(out)
    _check(None, lib().wave_average_shear_modulus(pm, po, dims[0], dims[1], dims[2], mode, mem))
    return out


def resample_traces(data, dt: float, seismo_dt: float):
    """Seismogram resampling to seismo_dt (wave_resample_traces); data: ntr x nt."""
    d = np.ascontiguousarray(data, dtype=np.float32)
    ntr, nt = d.shape
    nout = ctypes.c_int64()
    _check(None, lib().wave_resample_traces(None, ntr, nt, dt, seismo_dt, None, ctypes.byref(nout), MEM_HOST))
    out = np.zeros((ntr, nout.value), dtype=np.float32)
    _check(None, lib().wave_resample_traces(d.ctypes.data_as(ctypes.c_void_p), ntr, nt, dt, seismo_dt,
                                            out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nout), MEM_HOST))
    return out


def agc_normalize_traces(data, dt: float, f_agc: float):
    """normalizeTraces 3 (wave_agc_normalize_traces): returns (AGC-normalised
    traces, inverse AGC), both new arrays."""
    d = np.ascontiguousarray(np.array(data, dtype=np.float32, copy=True))
    inv = np.zeros_like(d)
    _check(None, lib().wave_agc_normalize_traces(d.ctypes.data_as(ctypes.c_void_p), d.shape[0], d.shape[1], dt, f_agc,
                                                 inv.ctypes.data_as(ctypes.c_void_p), MEM_HOST))
    return d, inv


def normalize_traces(data, mode: int):
    """Seismogram::normalizeTrace modes 0, 1, 2, 4 (wave_normalize_traces); returns a new array."""
    d = np.array(data, dtype=np.float32, order="C", copy=True)
    _check(None, lib().wave_normalize_traces(d.ctypes.data_as(ctypes.c_void_p), d.shape[0], d.shape[1], mode, MEM_HOST))
    return d


def envelope(data):
    """Trace envelopes (wave_envelope); data: ntr x nt."""
    d = np.array(data, dtype=np.float32, order="C", copy=True)
    _check(None, lib().wave_envelope(d.ctypes.data_as(ctypes.c_void_p), d.shape[0], d.shape[1], MEM_HOST))
    return d


def instantaneous_phase(data, phase_type: int):
    d = np.array(data, dtype=np.float32, order="C", copy=True)
    _check(None, lib().wave_instantaneous_phase(d.ctypes.data_as(ctypes.c_void_p), d.shape[0], d.shape[1], phase_type, MEM_HOST))
    return d


def read_mtx(path: str) -> np.ndarray:
    """A MatrixMarket file as a rows x cols float32 array (wave_read_mtx)."""
    r, c = ctypes.c_int64(), ctypes.c_int64()
    _check(None, lib().wave_read_mtx(path.encode(), None, 0, ctypes.byref(r), ctypes.byref(c)))
    out = np.zeros((r.value, c.value), dtype=np.float32)
    _check(None, lib().wave_read_mtx(path.encode(), out.ctypes.data_as(ctypes.c_void_p), out.size, ctypes.byref(r), ctypes.byref(c)))
    return out


def write_mtx(path: str, data) -> None:
    d = np.ascontiguousarray(data, dtype=np.float32)
    if d.ndim == 1:
        d = d[:, None]
    _check(None, lib().wave_write_mtx(path.encode(), d.ctypes.data_as(ctypes.c_void_p), d.shape[0], d.shape[1]))


def write_su(path: str, data, dt: float, rec_idx, src_idx: int, dims, DH: float) -> None:
    d = np.ascontiguousarray(data, dtype=np.float32)
    r = np.ascontiguousarray(rec_idx, dtype=np.int64)
    _check(None, lib().wave_write_su(path.encode(), d.ctypes.data_as(ctypes.c_void_p), d.shape[0], d.shape[1], dt,
                                     r.ctypes.data_as(ctypes.c_void_p), int(src_idx), dims[0], dims[1], dims[2], DH))


def average_shear_modulus_noalloc(mu, out, dims, mode: int, stream: int = 0):
    """wave_average_shear_modulus_noalloc: the same average with no device
    allocation (fixed 2^22-point scratch). mu and out are torch cuda float32
    tensors; the work is queued on `stream` (a raw cudaStream_t, 0 = default)."""
    n = int(dims[0]) * int(dims[1]) * int(dims[2])
    for name, t in (("mu", mu), ("out", out)):
        # the C ABI cannot see a tensor's length: a short one would be read or written past its end
        if not (hasattr(t, "data_ptr") and getattr(t, "is_cuda", False)):
            raise WaveError(WAVE_ERR_ARG, f"{name} must be a CUDA tensor")
        if str(t.dtype) != "torch.float32" or not t.is_contiguous():
            raise WaveError(WAVE_ERR_ARG, f"{name} must be a contiguous float32 tensor")
        if t.numel() < n:
            raise WaveError(WAVE_ERR_ARG, f"{name} holds {t.numel()} values, fewer than NX*NY*NZ = {n}")
    _check(None, lib().wave_average_shear_modulus_noalloc(ctypes.c_void_p(mu.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                                          dims[0], dims[1], dims[2], mode, ctypes.c_void_p(stream or None)))
    return out


class ForwardSolver:
    """One solver handle (ForwardSolver<float> + its boundary objects, on the GPU)."""

    def __init__(self, dimension: str, equation_type: str):
        self.dimension = dimension
        self.equation_type = equation_type
        self.h = None
        self.cfg = None

    # ForwardSolver::initForwardSolver (ForwardSolver.hpp:52)
    def initForwardSolver(self, config: WaveConfig):
        cfg = WaveConfig().copy_from(config)
        d = 3 if self.dimension.lower() == "3d" else 2
        if cfg.dimension != d or cfg.equation != EQUATIONS[self.equation_type.lower()]:
            raise WaveError(WAVE_ERR_ARG, "configuration does not match the factory keys")
        h = ctypes.c_void_p()
        _check(None, lib().wave_solver_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h, self.cfg = h, cfg
        nt = ctypes.c_int()
        _check(self.h, lib().wave_get_nt(self.h, ctypes.byref(nt)))
        self.nt = nt.value
        return self

    # Modelparameter::prepareForModelling + ForwardSolver::prepareForModelling (ForwardSolver.hpp:42)
    def prepareForModelling(self, model: dict):
        n = self.cfg.N
        if self.cfg.equation >= EQUATIONS["tmem"]:
            arrs = [_f32(model.get(k)) for k in ("eps_r", "sigma", "mu_r", "tau_eps", "tau_sigma")]
            fn = lib().wave_set_model_em
        else:
            arrs = [_f32(model.get(k)) for k in ("rho", "vp", "vs", "taup", "taus")]
            fn = lib().wave_set_model
        ptrs = [_ptr(a) for a in arrs]
        mems = {m for (p, m) in ptrs if p is not None}
        if len(mems) > 1:
            raise WaveError(WAVE_ERR_ARG, "model arrays must all be host or all be device")
        self._model_keep = arrs
        _check(self.h, fn(self.h, *[p for (p, _) in ptrs], n, mems.pop() if mems else MEM_HOST))

    def setSources(self, idx, types, signals):
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        types = np.ascontiguousarray(types, dtype=np.int32)
        sig = _f32(signals)
        p, mem = _ptr(sig)
        _check(self.h, lib().wave_set_sources(self.h, len(idx), idx.ctypes.data_as(ctypes.c_void_p),
                                              types.ctypes.data_as(ctypes.c_void_p), p, mem))

    def setReceivers(self, idx, types):
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        types = np.ascontiguousarray(types, dtype=np.int32)
        self.nrec = len(idx)
        _check(self.h, lib().wave_set_receivers(self.h, len(idx), idx.ctypes.data_as(ctypes.c_void_p),
                                                types.ctypes.data_as(ctypes.c_void_p)))

    # ForwardSolver::run(..., t) for one or many steps (ForwardSolver.hpp:38)
    def run(self, t_begin: int, t_end: int | None = None):
        _check(self.h, lib().wave_solver_step(self.h, t_begin, t_begin + 1 if t_end is None else t_end))

    # Wavefields::resetWavefields + ForwardSolver::resetCPML (ForwardSolver.hpp:40)
    def resetCPML(self):
        _check(self.h, lib().wave_solver_reset(self.h))

    def seismograms(self, out=None):
        if out is None:
            out = np.zeros((self.nrec, self.nt), dtype=np.float32)
        p, mem = _ptr(out)
        _check(self.h, lib().wave_get_seismograms(self.h, p, self.nrec * self.nt, mem))
        return out

    def check_finite(self) -> bool:
        rc = lib().wave_check_finite(self.h)
        if rc == WAVE_ERR_NONFINITE:
            return False
        _check(self.h, rc)
        return True

    def state(self) -> np.ndarray:
        n = ctypes.c_size_t()
        _check(self.h, lib().wave_get_state_size(self.h, ctypes.byref(n)))
        buf = np.zeros(n.value, dtype=np.uint8)
        _check(self.h, lib().wave_get_state(self.h, buf.ctypes.data_as(ctypes.c_void_p), n.value, MEM_HOST))
        return buf

    def set_state(self, buf: np.ndarray):
        _check(self.h, lib().wave_set_state(self.h, buf.ctypes.data_as(ctypes.c_void_p), buf.nbytes, MEM_HOST))

    def stream(self) -> int:
        s = ctypes.c_void_p()
        _check(self.h, lib().wave_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def launch_count(self) -> int:
        c = ctypes.c_longlong()
        _check(self.h, lib().wave_get_launch_count(self.h, ctypes.byref(c)))
        return c.value

    # ForwardSolver::estimateMemory (ForwardSolver.hpp:46), measured: the handle's device bytes
    def estimateMemory(self) -> int:
        b = ctypes.c_int64()
        _check(self.h, lib().wave_device_bytes(self.h, ctypes.byref(b)))
        return int(b.value)

    def set_kernel_path(self, path: int):
        """0 = automatic (fastest kernel per pass, timed when the model is set),
        1 = generic kernels (and the separate source/receiver kernel), 2 =
        one-point streaming TMA kernels, 3 = two-point streaming TMA kernels
        (2 and 3 wherever they apply)."""
        _check(self.h, lib().wave_set_kernel_path(self.h, path))

    def set_dependent_launch(self, on: bool):
        """Programmatic dependent launch of the per-point kernels (default on);
        the results do not depend on it."""
        _check(self.h, lib().wave_set_dependent_launch(self.h, 1 if on else 0))

    def set_decomposition(self, kind: int):
        """decomposeWavefieldType: 1 up/down, 2 left/right parts of P, VX, VY
        after every step (2-D acoustic); read them with field("P.up") etc."""
        _check(self.h, lib().wave_set_decomposition(self.h, int(kind)))

    def adjoint_gradient(self, dobs, checkpoint_every: int = 50):
        """Misfit J = 1/2 ||d - d_obs||^2 and its gradient by the discrete
        adjoint: w.r.t. (vp, vs, rho) for 2-D and 3-D elastic and visco-elastic
        (relaxation times held fixed; elastic also on a variable grid),
        2-D and 3-D acoustic, also on a variable grid (where the vs gradient is
        zero) and 2-D SH and visco-SH (where the vp
        gradient is zero), (eps_r, sigma, mu_r) for 2-D TMz and TEz and 3-D EM and their visco
        variants. d_obs: n_receivers x NT (numpy or torch cuda).
        Returns (J, g1, g2, g3) as float64 / numpy arrays."""
        d = _f32(dobs)
        pd, mem = _ptr(d)
        n = self.cfg.N
        g = [np.zeros(n, dtype=np.float32) for _ in range(3)]
        J = ctypes.c_double(0.0)
        _check(self.h, lib().wave_adjoint_gradient(self.h, pd, mem, int(checkpoint_every), ctypes.byref(J),
                                                    g[0].ctypes.data_as(ctypes.c_void_p), g[1].ctypes.data_as(ctypes.c_void_p),
                                                    g[2].ctypes.data_as(ctypes.c_void_p), MEM_HOST))
        return J.value, g[0], g[1], g[2]

    def field(self, name: str) -> np.ndarray:
        """One wavefield (wave_get_field), e.g. "VX", "Sxx", "EZ"."""
        out = np.zeros(self.cfg.N, dtype=np.float32)
        _check(self.h, lib().wave_get_field(self.h, name.encode(), out.ctypes.data_as(ctypes.c_void_p), MEM_HOST))
        return out

    def curl_div(self):
        """snapType 3 energies (wave_get_curl_div): (curl, div)."""
        c = np.zeros(self.cfg.N, dtype=np.float32)
        d = np.zeros(self.cfg.N, dtype=np.float32)
        _check(self.h, lib().wave_get_curl_div(self.h, c.ctypes.data_as(ctypes.c_void_p), d.ctypes.data_as(ctypes.c_void_p), MEM_HOST))
        return c, d

    def streaming_passes(self) -> int:
        """Bit 0: the velocity pass runs a streaming kernel; bit 1: the stress pass;
        bits 2 / 3: that kernel is the two-points-per-thread one."""
        v = ctypes.c_int()
        _check(self.h, lib().wave_get_kernel_path(self.h, ctypes.byref(v)))
        return v.value

    def streaming_active(self) -> bool:
        return self.streaming_passes() != 0

    def set_timing(self, on: bool):
        _check(self.h, lib().wave_set_timing(self.h, int(on)))

    def kernel_times(self):
        a, b, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_longlong()
        _check(self.h, lib().wave_get_kernel_times(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(n)))
        return a.value, b.value, n.value

    def close(self):
        if self.h:
            lib().wave_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _ShotView(ForwardSolver):
    """A shot of a batch: the per-shot handle, owned by the batch."""

    def __init__(self, h, cfg):
        super().__init__("3d" if cfg.dimension == 3 else "2d", [k for k, v in EQUATIONS.items() if v == cfg.equation][0])
        self.h, self.cfg = h, cfg
        nt = ctypes.c_int()
        _check(self.h, lib().wave_get_nt(self.h, ctypes.byref(nt)))
        self.nt = nt.value

    def run(self, *a):
        raise WaveError(WAVE_ERR_STATE, "step the batch, not a single shot")

    def close(self):
        self.h = None   # owned by the batch


class Batch:
    """Many shots with uneven grids stepped together (wave_batch_*)."""

    def __init__(self, configs):
        arr = (WaveConfig * len(configs))()
        for i, c in enumerate(configs):
            arr[i].copy_from(c)
        self._cfgs = arr
        b = ctypes.c_void_p()
        rc = lib().wave_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(configs), ctypes.byref(b))
        if rc != WAVE_OK:
            raise WaveError(rc, lib().wave_batch_last_error(None).decode())
        self.b = b
        self.shots = []
        for i in range(len(configs)):
            h = ctypes.c_void_p()
            self._check(lib().wave_batch_shot(self.b, i, ctypes.byref(h)))
            self.shots.append(_ShotView(h, arr[i]))
        self.nt = self.shots[0].nt

    def _check(self, rc):
        if rc != WAVE_OK:
            raise WaveError(rc, lib().wave_batch_last_error(self.b).decode())

    def run(self, t0: int, t1: int):
        self._check(lib().wave_batch_step(self.b, t0, t1))

    def adjoint_gradient(self, dobs, checkpoint_every: int = 50, sum_shots: bool = True):
        """Misfits and (vp, vs, rho) gradients of every shot (wave_batch_adjoint_gradient).
        dobs: one n_receivers x NT array per shot. With sum_shots the shots' gradients
        are summed (shots on one grid). Returns (misfits, g_vp, g_vs, g_rho); the
        gradients are arrays (summed) or lists of arrays (per shot)."""
        ns = len(self.shots)
        d = [np.ascontiguousarray(x, dtype=np.float32) for x in dobs]
        dptr = (ctypes.c_void_p * ns)(*[x.ctypes.data for x in d])
        nout = 1 if sum_shots else ns
        sizes = [self.shots[k].cfg.N for k in range(nout)]
        g = [[np.zeros(n, dtype=np.float32) for n in sizes] for _ in range(3)]
        ptrs = [(ctypes.c_void_p * nout)(*[a.ctypes.data for a in gk]) for gk in g]
        mis = (ctypes.c_double * ns)()
        self._check(lib().wave_batch_adjoint_gradient(self.b, ctypes.cast(dptr, ctypes.c_void_p), MEM_HOST, int(checkpoint_every),
                                                      mis, ctypes.cast(ptrs[0], ctypes.c_void_p), ctypes.cast(ptrs[1], ctypes.c_void_p),
                                                      ctypes.cast(ptrs[2], ctypes.c_void_p), MEM_HOST, int(sum_shots)))
        if sum_shots:
            return list(mis), g[0][0], g[1][0], g[2][0]
        return list(mis), g[0], g[1], g[2]

    def set_schedule(self, tile_cols: int, tile_rows: int, blocks_per_sm: int):
        """Fixes the batched launches' schedule (wave_batch_set_schedule); (0, 0, 0) returns to the autotuner."""
        self._check(lib().wave_batch_set_schedule(self.b, int(tile_cols), int(tile_rows), int(blocks_per_sm)))

    def schedule(self) -> dict:
        """The schedule in use and its source (wave_batch_get_schedule)."""
        c, r, p, src = (ctypes.c_int() for _ in range(4))
        self._check(lib().wave_batch_get_schedule(self.b, ctypes.byref(c), ctypes.byref(r), ctypes.byref(p), ctypes.byref(src)))
        return {"tile_cols": c.value, "tile_rows": r.value, "blocks_per_sm": p.value,
                "source": ("default", "autotuned", "cache", "set")[src.value]}

    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._check(lib().wave_batch_get_stream(self.b, ctypes.byref(s)))
        return s.value or 0

    def launch_count(self) -> int:
        c = ctypes.c_longlong()
        self._check(lib().wave_batch_get_launch_count(self.b, ctypes.byref(c)))
        return c.value

    def close(self):
        if getattr(self, "b", None):
            for s in self.shots:
                s.h = None
            lib().wave_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Factory:
    """ForwardSolver::Factory<float>::Create (ForwardSolverFactory.cpp:4-67)."""

    @staticmethod
    def Create(dimension: str, equation_type: str) -> ForwardSolver:
        d, t = dimension.lower(), equation_type.lower()
        if d not in ("2d", "3d"):
            raise WaveError(WAVE_ERR_ARG, "Unkown dimension")
        if t not in EQUATIONS:
            raise WaveError(WAVE_ERR_ARG, "Unkown type")
        return ForwardSolver(d, t)


def simulate(config: WaveConfig, model: dict, src_idx, src_type, signals, rec_idx, rec_type,
             kernel_path: int = 0, expect_streaming: bool | None = None) -> np.ndarray:
    """Runs one shot through the whole time loop (Simulation.cpp:432-533) and
    returns the seismograms (n_receivers x NT)."""
    dim = "3d" if config.dimension == 3 else "2d"
    eq = [k for k, v in EQUATIONS.items() if v == config.equation][0]
    s = Factory.Create(dim, eq).initForwardSolver(config)
    try:
        s.prepareForModelling(model)
        s.set_kernel_path(kernel_path)
        if expect_streaming is not None and s.streaming_active() != expect_streaming:
            raise WaveError(WAVE_ERR_STATE, f"streaming kernels active={s.streaming_active()}, expected {expect_streaming}")
        s.setSources(src_idx, src_type, signals)
        s.setReceivers(rec_idx, rec_type)
        s.run(0, s.nt)
        out = s.seismograms()
        if not s.check_finite():
            raise WaveError(WAVE_ERR_NONFINITE, "Infinite or NaN value in seismogram or/and velocity wavefield!")
        return out
    finally:
        s.close()


# ---------------------------------------------------------------------------
# Shot domains across processes (one process per GPU)
# ---------------------------------------------------------------------------
def shot_range(num_shots: int, domain: int, num_domains: int) -> tuple:
    """Shots [lb, ub) of shot domain `domain` out of `num_domains`: contiguous
    blocks of ceil(num_shots / num_domains) shots, the block distribution
    the reference builds over its inter-shot communicator
    (Simulation.cpp:339-345, blockDistribution(numshots, commInterShot)); the
    last domains may get fewer shots or none."""
    if num_shots < 0 or num_domains < 1 or not 0 <= domain < num_domains:
        raise WaveError(WAVE_ERR_ARG, "shot_range: invalid shot or domain count")
    block = (num_shots + num_domains - 1) // num_domains
    lb = min(domain * block, num_shots)
    return lb, min(lb + block, num_shots)


def sum_over_shot_domains(local, group=None):
    """Sum of a per-process partial result (seismograms, gradients, misfits)
    over all processes of the torch.distributed group, as the reference sums
    its seismograms over the inter-shot communicator (SeismogramHandler.cpp:
    479). `local` is a numpy array (reduced through a CPU tensor: gloo) or a
    torch tensor (reduced in place on its device: NCCL for CUDA tensors).
    Without an initialised process group the input comes back unchanged."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size(group) == 1:
        return local
    if isinstance(local, torch.Tensor):
        dist.all_reduce(local, op=dist.ReduceOp.SUM, group=group)
        return local
    t = torch.from_numpy(np.ascontiguousarray(local)).clone()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy()


def run_shot_domains(num_shots: int, compute, group=None):
    """Runs this process's block of shots and sums the result over all
    processes: compute(lb, ub) returns the partial result of shots [lb, ub)
    (a numpy array or a tuple of them, zeros for an empty block), and every
    process receives the sums. One process per GPU; no collective runs inside
    `compute`, only the final sum."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        rank, world = dist.get_rank(group), dist.get_world_size(group)
    else:
        rank, world = 0, 1
    lb, ub = shot_range(num_shots, rank, world)
    part = compute(lb, ub)
    if isinstance(part, tuple):
        return tuple(sum_over_shot_domains(p, group) for p in part)
    return sum_over_shot_domains(part, group)


def fwi_gradient_shot_domains(config: WaveConfig, model: dict, acquisitions, dobs, checkpoint_every: int = 50,
                              group=None):
    """Summed misfit and vp / vs / rho gradients over all shots, the shots
    split into contiguous blocks over the processes of the torch.distributed
    group: each process runs its block as one batch on its own GPU
    (wave_batch_adjoint_gradient, gradients summed on the device), then one
    sum over the processes. acquisitions[k] = (src_idx, src_type, signals,
    rec_idx, rec_type) and dobs[k] are shot k's."""
    n = config.N

    def compute(lb, ub):
        if ub <= lb:
            z = np.zeros(n, np.float64)
            return np.zeros(1, np.float64), z, z.copy(), z.copy()
        b = Batch([config] * (ub - lb))
        try:
            for shot, k in zip(b.shots, range(lb, ub)):
                shot.prepareForModelling(model)
                shot.setSources(*acquisitions[k][:3])
                shot.setReceivers(*acquisitions[k][3:])
            mis, gvp, gvs, grho = b.adjoint_gradient(list(dobs[lb:ub]), checkpoint_every=checkpoint_every, sum_shots=True)
        finally:
            b.close()
        f = lambda a: np.asarray(a, np.float64)
        return np.array([float(np.sum(mis))]), f(gvp), f(gvs), f(grho)

    mis, gvp, gvs, grho = run_shot_domains(len(acquisitions), compute, group)
    return float(mis[0]), gvp, gvs, grho
