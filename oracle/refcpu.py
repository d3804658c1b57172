"""TEST INFRASTRUCTURE ONLY — ctypes front end of the oracle (refcpu).

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module, as the checker / the timed CPU baseline. It also holds the small
host-side restatements the tests need to reproduce the reference's CI cases:

* a parameter-file reader with the reference's KEY=VALUE rules
  (src/Configuration/Configuration.cpp:45-100, Configuration.hpp:95-143);
* source / receiver acquisition-file readers (src/Acquisition/AcquisitionSettings.hpp:55-109;
  receivers: ``x y z type`` rows);
* the Ricker wavelet (src/Acquisition/SourceSignal/Ricker.cpp:29-53) in the value type;
* the TwoLayer model of the CI (src/Tools/CreateModel/TwoLayer.cpp:25-62);
* a MatrixMarket ``array real general`` reader (format of par/ci/*.ref.*.mtx).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle_refcpu.so")

EQ = {"acoustic": 0, "elastic": 1, "viscoelastic": 2, "sh": 3, "viscosh": 4,
      "tmem": 5, "emem": 6, "viscotmem": 7, "viscoemem": 8}


class WaveConfig(ctypes.Structure):
    """Mirror of ``wave_config`` in include/wave.h."""
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


def make_config(**kw) -> WaveConfig:
    c = WaveConfig()
    c.dimension = kw.get("dimension", 2)
    eq = kw.get("equation", 0)
    c.equation = EQ[eq] if isinstance(eq, str) else int(eq)
    c.NX, c.NY = kw["NX"], kw["NY"]
    c.NZ = kw.get("NZ", 1)
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
    rf = list(kw.get("relaxationFrequency", [0.0, 0.0, 0.0, 0.0])) + [0.0] * 4
    for i in range(4):
        c.relaxationFrequency[i] = rf[i]
    c.useStencilMatrix = kw.get("useStencilMatrix", 0)
    c.edgeOrderReduction = kw.get("edgeOrderReduction", 1)
    c.useVariableGrid = kw.get("useVariableGrid", 0)
    c.useVariableFDoperators = kw.get("useVariableFDoperators", 0)
    grid = kw.get("grid", [])
    c.gridLayers = len(grid)
    for i, row in enumerate(grid):
        c.gridInterface[i], c.gridDHFactor[i] = int(row[0]), int(row[1])
        c.gridFDOrder[i] = int(row[2]) if len(row) > 2 else c.spatialFDorder
    return c


def nt_of(cfg: WaveConfig) -> int:
    """NT = int(T/DT + 0.5) in single precision (Common.hpp:240-243)."""
    return int(np.float32(np.float32(cfg.T) / np.float32(cfg.DT)) + np.float32(0.5))


# --------------------------------------------------------------------------
# reference parameter files
# --------------------------------------------------------------------------
def read_parameter_file(path: str) -> dict:
    """KEY=VALUE reader with the reference's rules: keys lower-cased, whole-line
    '#' comments skipped, trailing '# comment' cut (Configuration.cpp:45-100)."""
    out = {}
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            end = len(line)
            p = line.find("#")
            if p != -1:
                if p == 0:
                    continue
                end = p
            e = line.find("=")
            if e == -1:
                continue
            out[line[:e].lower()] = line[e + 1:end]
    return out


def _tok(v: str) -> str:
    s = v.split()
    return s[0] if s else ""


def _num(v: str, cast):
    """istringstream >> T semantics: leading numeric prefix of the first token."""
    t = _tok(v)
    for k in range(len(t), 0, -1):
        try:
            return cast(t[:k])
        except ValueError:
            continue
    raise ValueError(v)


def config_from_parameters(p: dict, base_dir: str | None = None) -> WaveConfig:
    """base_dir: folder against which gridConfigurationFilename is resolved
    (tried as given, then base_dir/name, then base_dir/../name)."""
    g = lambda k, cast=float, default=None: (_num(p[k.lower()], cast) if k.lower() in p else default)
    dim = 3 if _tok(p["dimension"]).lower() == "3d" else 2
    kw = dict(
        dimension=dim, equation=_tok(p["equationtype"]).lower(),
        NX=g("NX", int), NY=g("NY", int), NZ=g("NZ", int, 1),
        DH=g("DH"), DT=g("DT"), T=g("T"),
        spatialFDorder=g("spatialFDorder", int),
        FreeSurface=g("FreeSurface", int, 0),
        DampingBoundary=g("DampingBoundary", int, 0),
        BoundaryWidth=g("BoundaryWidth", int, 0),
        DampingCoeff=g("DampingCoeff", float, 8.0),
        NPower=g("NPower", float, 4.0),
        CenterFrequencyCPML=g("CenterFrequencyCPML", float, 5.0),
        VMaxCPML=g("VMaxCPML", float, 3500.0),
        numRelaxationMechanisms=max(0, g("numRelaxationMechanisms", int, 0)),
        relaxationFrequency=[g("relaxationFrequency", float, 0.0), g("relaxationFrequency2", float, 0.0),
                             g("relaxationFrequency3", float, 0.0), g("relaxationFrequency4", float, 0.0)],
        useStencilMatrix=g("useStencilMatrix", int, 0),
        edgeOrderReduction=g("edgeOrderReduction", int, 1),
        useVariableGrid=g("useVariableGrid", int, 0),
        useVariableFDoperators=g("useVariableFDoperators", int, 0),
    )
    if kw["equation"] == "visco":
        kw["equation"] = "viscoelastic"
    if kw["useVariableGrid"] or kw["useVariableFDoperators"]:
        from oracle import vargrid
        name = _tok(p["gridconfigurationfilename"])
        tries = [name] + ([os.path.join(base_dir, name), os.path.join(base_dir, "..", name)] if base_dir else [])
        path = next(t for t in tries if os.path.exists(t))
        iface, dhf, order = vargrid.read_grid_config(path)
        kw["grid"] = [(a, b, c if order else kw["spatialFDorder"]) for a, b, c in
                      zip(iface, dhf, order or [0] * len(iface))]
    return make_config(**kw)


def read_sources(path: str) -> list:
    """10-column source rows (AcquisitionSettings.hpp:55-109)."""
    rows = []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s or s.startswith("#"):
                continue
            v = s.split()
            if len(v) != 10:
                raise ValueError("Wrong number of parameters in line of source acquisition file")
            rows.append(dict(no=int(v[0]), x=int(v[1]), y=int(v[2]), z=int(v[3]), type=int(v[4]),
                             wtype=int(v[5]), shape=int(v[6]), fc=float(v[7]), amp=float(v[8]),
                             tshift=float(v[9])))
    return rows


def read_receivers(path: str) -> list:
    rows = []
    with open(path) as f:
        for line in f:
            s = line.strip()
            if not s or s.startswith("#"):
                continue
            v = s.split()
            rows.append(dict(x=int(v[0]), y=int(v[1]), z=int(v[2]), type=int(v[3])))
    return rows


def grid_index(cfg: WaveConfig, x, y, z):
    nz = 1 if cfg.dimension == 2 else cfg.NZ
    return np.int64(x) + np.int64(z) * cfg.NX + np.int64(y) * cfg.NX * nz


def ricker(nt: int, dt: float, fc: float, amp: float, tshift: float, dtype=np.float32) -> np.ndarray:
    """Ricker::calc (Ricker.cpp:29-53) evaluated in the value type."""
    d = np.dtype(dtype).type
    t = d(0) + np.arange(nt).astype(dtype) * d(dt)
    help_ = d(d(1.5) / d(fc) + d(tshift))
    tau = (t - help_).astype(dtype)
    tau = (tau * d(np.pi * d(fc))).astype(dtype)
    h = (tau * tau).astype(dtype)
    e = np.exp((d(-1.0) * h).astype(dtype)).astype(dtype)
    h2 = (d(1.0) - d(2.0) * h).astype(dtype)
    return (d(amp) * h2 * e).astype(dtype)


def two_layer(cfg: WaveConfig, dtype=np.float32) -> dict:
    """TwoLayer model (TwoLayer.cpp:25-62): layer 2 from depth index y >= 40."""
    nz = 1 if cfg.dimension == 2 else cfg.NZ
    shape = (cfg.NY, nz, cfg.NX)
    out = {}
    for name, a, b in (("vp", 3500, 4550), ("vs", 2000, 2600), ("rho", 2000, 2600),
                       ("taup", 0.1, 0.1), ("taus", 0.1, 0.1)):
        arr = np.full(shape, a, dtype=dtype)
        arr[40:] = b
        out[name] = arr.reshape(-1)
    return out


def read_mtx_array(path: str) -> np.ndarray:
    """MatrixMarket 'array real general' -> (rows, cols), column-major values."""
    with open(path) as f:
        lines = [l for l in f.read().splitlines() if l and not l.startswith("%")]
    r, c = (int(v) for v in lines[0].split()[:2])
    vals = np.array([float(v) for v in lines[1:1 + r * c]], dtype=np.float64)
    return vals.reshape(c, r).T


def reference_misfit(test: np.ndarray, ref: np.ndarray) -> float:
    """Test_CompareSeismogram.cpp:57-88: sum of per-component L2 norms of the
    difference / (max amplitude * samples * traces)."""
    mx = max(np.abs(ref).max(), np.abs(test).max())
    return float(np.linalg.norm(test - ref) / (mx * ref.shape[0] * ref.shape[1]))


# --------------------------------------------------------------------------
# the oracle library
# --------------------------------------------------------------------------
_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.refcpu_create_f32.restype = P
        L.refcpu_create_f64.restype = P
        for fn in (L.refcpu_create_f32, L.refcpu_create_f64):
            fn.argtypes = [ctypes.POINTER(WaveConfig), P, ctypes.c_int, P, P, P, ctypes.c_int, P, P]
        L.refcpu_step.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.refcpu_seismograms.argtypes = [P, P]
        L.refcpu_field.argtypes = [P, ctypes.c_char_p, P]
        L.refcpu_curl_div.argtypes = [P, P, P]
        L.refcpu_nt.argtypes = [P]
        L.refcpu_destroy.argtypes = [P]
        L.refcpu_last_error.restype = ctypes.c_char_p
        L.refcpu_set_threads.argtypes = [ctypes.c_int]
        L.refcpu_adjoint_elastic2d.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.POINTER(ctypes.c_double), P, P, P]
        L.refcpu_adjoint_tmz.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.POINTER(ctypes.c_double), P, P, P]
        L.refcpu_adjoint_sh.argtypes = [P, P, P, P, ctypes.c_int, ctypes.POINTER(ctypes.c_double), P, P]
        L.refcpu_adjoint_acoustic.argtypes = [P, P, P, P, ctypes.c_int, ctypes.POINTER(ctypes.c_double), P, P]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


MODEL_KEYS = ("rho", "vp", "vs", "taup", "taus", "eps_r", "sigma", "mu_r", "tau_eps", "tau_sigma")


@dataclass
class Oracle:
    """One refcpu simulation (float32 or float64)."""
    cfg: WaveConfig
    model: dict
    src_idx: np.ndarray
    src_type: np.ndarray
    signals: np.ndarray
    rec_idx: np.ndarray
    rec_type: np.ndarray
    dtype: type = np.float64
    _keep: list = field(default_factory=list)

    def __post_init__(self):
        L = lib()
        d = np.dtype(self.dtype)
        arrs = []
        for k in MODEL_KEYS:
            v = self.model.get(k)
            arrs.append(None if v is None else np.ascontiguousarray(v, dtype=d))
        self._keep = arrs
        ptrs = (ctypes.c_void_p * len(arrs))(*[(_ptr(a) if a is not None else None) for a in arrs])
        self._sidx = np.ascontiguousarray(self.src_idx, dtype=np.int64)
        self._stype = np.ascontiguousarray(self.src_type, dtype=np.int32)
        self._sig = np.ascontiguousarray(self.signals, dtype=d)
        self._ridx = np.ascontiguousarray(self.rec_idx, dtype=np.int64)
        self._rtype = np.ascontiguousarray(self.rec_type, dtype=np.int32)
        create = L.refcpu_create_f64 if d == np.float64 else L.refcpu_create_f32
        self.h = create(ctypes.byref(self.cfg), ctypes.cast(ptrs, ctypes.c_void_p), len(self._sidx),
                        _ptr(self._sidx), _ptr(self._stype), _ptr(self._sig), len(self._ridx),
                        _ptr(self._ridx), _ptr(self._rtype))
        if not self.h:
            raise RuntimeError(L.refcpu_last_error().decode())
        self.nt = L.refcpu_nt(self.h)

    def step(self, t0: int, t1: int, copy_state: bool = False) -> float:
        sec = ctypes.c_double(0)
        if lib().refcpu_step(self.h, t0, t1, int(copy_state), ctypes.byref(sec)) != 0:
            raise RuntimeError(lib().refcpu_last_error().decode())
        return sec.value

    def run(self) -> np.ndarray:
        self.step(0, self.nt)
        return self.seismograms()

    def seismograms(self) -> np.ndarray:
        out = np.zeros((len(self._ridx), self.nt), dtype=np.float64)
        lib().refcpu_seismograms(self.h, _ptr(out))
        return out

    def field(self, name: str) -> np.ndarray:
        n = self.cfg.NX * self.cfg.NY * (1 if self.cfg.dimension == 2 else self.cfg.NZ)
        out = np.zeros(n, dtype=np.float64)
        if lib().refcpu_field(self.h, name.encode(), _ptr(out)) != 0:
            raise KeyError(name)
        return out

    def curl_div(self):
        """snapType 3 energies (curl, div) of the current wavefields."""
        n = self.cfg.NX * self.cfg.NY * (1 if self.cfg.dimension == 2 else self.cfg.NZ)
        c = np.zeros(n, dtype=np.float64)
        d = np.zeros(n, dtype=np.float64)
        if lib().refcpu_curl_div(self.h, _ptr(c), _ptr(d)) != 0:
            raise RuntimeError(lib().refcpu_last_error().decode())
        return c, d

    def adjoint_gradient(self, dobs: np.ndarray, checkpoint_every: int = 50):
        """Misfit 1/2 sum (d - dobs)^2 and its gradients with respect to vp, vs
        and rho (2-D and 3-D elastic, 2-D visco-elastic with the relaxation
        times held fixed; 2-D SH: the vp gradient is zero; 2-D and 3-D
        acoustic: the vs gradient is zero) or eps_r, sigma
        and mu_r (lossless 2-D TMz and TEz), by the oracle's own discrete adjoint
        (adjoint_impl.hpp) in this oracle's value type."""
        n = self.cfg.NX * self.cfg.NY * (self.cfg.NZ if self.cfg.dimension == 3 else 1)
        em = self.cfg.equation >= 5
        if self.cfg.equation == EQ["acoustic"]:
            m = [np.ascontiguousarray(self.model[k], dtype=np.float64) for k in ("vp", "rho")]
            d = np.ascontiguousarray(dobs, dtype=np.float64)
            if d.size != len(self._ridx) * self.nt:
                raise ValueError("dobs must hold n_receivers x NT samples")
            g = [np.zeros(n, dtype=np.float64) for _ in range(2)]
            J = ctypes.c_double(0)
            if lib().refcpu_adjoint_acoustic(self.h, _ptr(m[0]), _ptr(m[1]), _ptr(d), int(checkpoint_every),
                                             ctypes.byref(J), _ptr(g[0]), _ptr(g[1])) != 0:
                raise RuntimeError(lib().refcpu_last_error().decode())
            return J.value, g[0], np.zeros(n, dtype=np.float64), g[1]
        if self.cfg.equation in (EQ["sh"], EQ["viscosh"]):
            m = [np.ascontiguousarray(self.model[k], dtype=np.float64) for k in ("vs", "rho")]
            d = np.ascontiguousarray(dobs, dtype=np.float64)
            if d.size != len(self._ridx) * self.nt:
                raise ValueError("dobs must hold n_receivers x NT samples")
            g = [np.zeros(n, dtype=np.float64) for _ in range(2)]
            J = ctypes.c_double(0)
            if lib().refcpu_adjoint_sh(self.h, _ptr(m[0]), _ptr(m[1]), _ptr(d), int(checkpoint_every), ctypes.byref(J),
                                       _ptr(g[0]), _ptr(g[1])) != 0:
                raise RuntimeError(lib().refcpu_last_error().decode())
            return J.value, np.zeros(n, dtype=np.float64), g[0], g[1]
        keys = ("eps_r", "sigma", "mu_r") if em else ("vp", "vs", "rho")
        m = [np.ascontiguousarray(self.model[k], dtype=np.float64) for k in keys]
        d = np.ascontiguousarray(dobs, dtype=np.float64)
        if d.size != len(self._ridx) * self.nt:
            raise ValueError("dobs must hold n_receivers x NT samples")
        g = [np.zeros(n, dtype=np.float64) for _ in range(3)]
        J = ctypes.c_double(0)
        fn = lib().refcpu_adjoint_tmz if em else lib().refcpu_adjoint_elastic2d
        if fn(self.h, *(_ptr(a) for a in m), _ptr(d), int(checkpoint_every), ctypes.byref(J), *(_ptr(a) for a in g)) != 0:
            raise RuntimeError(lib().refcpu_last_error().decode())
        return J.value, g[0], g[1], g[2]

    def close(self):
        if getattr(self, "h", None):
            lib().refcpu_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def set_threads(n: int) -> int:
    return lib().refcpu_set_threads(n)
