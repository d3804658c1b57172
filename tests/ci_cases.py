"""The reference's CI integration cases (par/ci), rebuilt from the committed
fixtures in tests/golden/ci/: parameter file, acquisition files, TwoLayer model
(for ModelRead=1) and the golden seismogram of the first shot.

Mirrors par/start_tests.sh:24-98 + src/Tests/IntegrationTest/Test_CompareSeismogram.cpp.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
from oracle import refcpu  # noqa: E402

CI = os.path.join(ROOT, "tests", "golden", "ci")

# name -> (config file, golden file). The variable-grid cases are in
# VARGRID_CASES below.
CASES = {
    "2D.acoustic": ("configuration_ci.2D.acoustic.txt", "seismogram.2D.acoustic.ref.p.mtx"),
    "2D.sh": ("configuration_ci.2D.sh.txt", "seismogram.2D.sh.ref.vz.mtx"),
    "2D.elastic": ("configuration_ci.2D.elastic.txt", "seismogram.2D.elastic.ref.vy.mtx"),
    "3D.acoustic": ("configuration_ci.3D.acoustic.txt", "seismogram.3D.acoustic.ref.p.mtx"),
    "3D.elastic": ("configuration_ci.3D.elastic.txt", "seismogram.3D.elastic.ref.vy.mtx"),
    "2D.visco": ("configuration_ci.2D.visco.txt", "seismogram.2D.visco.ref.vy.mtx"),
    "3D.visco": ("configuration_ci.3D.visco.txt", "seismogram.3D.visco.ref.vy.mtx"),
}


def load_case(name: str, dtype=np.float32, edge_order_reduction: int = 0):
    """The goldens were made with zero-padded sparse operators, hence the
    default edge_order_reduction=0 (see wave_config.edgeOrderReduction)."""
    cfg_file, golden = CASES[name]
    p = refcpu.read_parameter_file(os.path.join(CI, cfg_file))
    cfg = refcpu.config_from_parameters(p)
    cfg.edgeOrderReduction = edge_order_reduction
    nt = refcpu.nt_of(cfg)
    n = cfg.NX * cfg.NY * (1 if cfg.dimension == 2 else cfg.NZ)
    model_read = int(refcpu._num(p.get("modelread", "0"), int))
    if model_read:
        model = refcpu.two_layer(cfg, dtype)
    else:
        model = {}
        for key, name_ in (("velocityp", "vp"), ("velocitys", "vs"), ("rho", "rho"),
                           ("taup", "taup"), ("taus", "taus")):
            if key in p:
                model[name_] = np.full(n, refcpu._num(p[key], float), dtype=dtype)
    srcs = refcpu.read_sources(os.path.join(CI, os.path.basename(p["sourcefilename"].split()[0]) + ".txt"))
    recs = refcpu.read_receivers(os.path.join(CI, os.path.basename(p["receiverfilename"].split()[0]) + ".txt"))
    # only the first shot (Test_CompareSeismogram compares shot sourceSettings[0].sourceNo)
    shot = srcs[0]["no"]
    srcs = [s for s in srcs if s["no"] == shot]
    src_idx = np.array([refcpu.grid_index(cfg, s["x"], s["y"], s["z"]) for s in srcs], dtype=np.int64)
    src_type = np.array([s["type"] for s in srcs], dtype=np.int32)
    signals = np.stack([refcpu.ricker(nt, cfg.DT, s["fc"], s["amp"], s["tshift"], dtype) for s in srcs])
    rec_idx = np.array([refcpu.grid_index(cfg, r["x"], r["y"], r["z"]) for r in recs], dtype=np.int64)
    rec_type = np.array([r["type"] for r in recs], dtype=np.int32)
    ref = refcpu.read_mtx_array(os.path.join(CI, golden))
    return dict(cfg=cfg, nt=nt, model=model, src_idx=src_idx, src_type=src_type, signals=signals,
                rec_idx=rec_idx, rec_type=rec_type, golden=ref)


def run_oracle(case: dict, dtype=np.float32) -> np.ndarray:
    o = refcpu.Oracle(case["cfg"], case["model"], case["src_idx"], case["src_type"],
                      case["signals"].astype(dtype), case["rec_idx"], case["rec_type"], dtype=dtype)
    try:
        return o.run()
    finally:
        o.close()


# The variable-grid acoustic CI cases (par/ci/configuration_ci.{2D,3D}.acoustic.varGrid.txt
# with par/ci/gridConfig.txt): layers of spacing DH and 3 DH, FD orders 2 and 6,
# CPML and the mirror free surface.
VARGRID_CASES = {
    "2D.acoustic.varGrid": ("configuration_ci.2D.acoustic.varGrid.txt", "seismogram.2D.acoustic.varGrid.ref.p.mtx",
                            "sources_ci.2D.varGrid.txt", "receiver_ci.2D.varGrid.txt"),
    "3D.acoustic.varGrid": ("configuration_ci.3D.acoustic.varGrid.txt", "seismogram.3D.acoustic.varGrid.ref.p.mtx",
                            "sources_ci.3D.varGrid.txt", "receiver_ci.3D.varGrid.txt"),
}


def load_vargrid_case(name: str, dtype=np.float32, edge_order_reduction: int = 0):
    """Configuration, grid, acquisition (mapped with Coordinates::coordinate2index),
    homogeneous model on the grid's points and the golden seismogram. Like
    the regular-grid goldens, these were made with zero-padded operators."""
    from oracle import vargrid
    cfg_file, golden, src_file, rec_file = VARGRID_CASES[name]
    p = refcpu.read_parameter_file(os.path.join(CI, cfg_file))
    cfg = refcpu.config_from_parameters(p, base_dir=CI)
    cfg.edgeOrderReduction = edge_order_reduction
    iface = [cfg.gridInterface[i] for i in range(cfg.gridLayers)]
    dhf = [cfg.gridDHFactor[i] for i in range(cfg.gridLayers)]
    orders = [cfg.gridFDOrder[i] for i in range(cfg.gridLayers)]
    g = vargrid.VarGrid(cfg.NX, cfg.NY, cfg.NZ if cfg.dimension == 3 else 1, cfg.DH, iface, dhf)
    nt = refcpu.nt_of(cfg)
    srcs = refcpu.read_sources(os.path.join(CI, src_file))
    srcs = [s for s in srcs if s["no"] == srcs[0]["no"]]
    recs = refcpu.read_receivers(os.path.join(CI, rec_file))
    src_idx = g.coordinate2index([s["x"] for s in srcs], [s["y"] for s in srcs], [s["z"] for s in srcs])
    rec_idx = g.coordinate2index([r["x"] for r in recs], [r["y"] for r in recs], [r["z"] for r in recs])
    signals = np.stack([refcpu.ricker(nt, cfg.DT, s["fc"], s["amp"], s["tshift"], dtype) for s in srcs])
    model = dict(rho=np.full(g.N, refcpu._num(p["rho"], float), dtype=dtype),
                 vp=np.full(g.N, refcpu._num(p["velocityp"], float), dtype=dtype))
    return dict(cfg=cfg, grid=g, orders=orders, nt=nt, model=model,
                src_idx=np.asarray(src_idx, np.int64), src_type=np.array([s["type"] for s in srcs], np.int32),
                signals=signals, rec_idx=np.asarray(rec_idx, np.int64),
                rec_type=np.array([r["type"] for r in recs], np.int32),
                golden=refcpu.read_mtx_array(os.path.join(CI, golden)))


def run_vargrid_oracle(case: dict, dtype=np.float32) -> np.ndarray:
    from oracle import vargrid
    cfg, g = case["cfg"], case["grid"]
    cp = damp = None
    if cfg.DampingBoundary == 2:
        cp = vargrid.cpml_coefficients(g, cfg.BoundaryWidth, cfg.NPower, cfg.CenterFrequencyCPML, cfg.VMaxCPML,
                                       cfg.DT, cfg.FreeSurface != 0, dtype)
    elif cfg.DampingBoundary == 1:
        damp = vargrid.abs_damping(g, cfg.BoundaryWidth, cfg.DampingCoeff, cfg.FreeSurface != 0, dtype)
    sim = vargrid.AcousticVarGrid(g, case["orders"], cfg.DT, case["model"]["rho"], case["model"]["vp"], cfg.FreeSurface,
                                  cp, case["src_idx"], case["src_type"], case["signals"].astype(dtype),
                                  case["rec_idx"], case["rec_type"], dtype=dtype,
                                  var_order=bool(cfg.useVariableFDoperators), edge=bool(cfg.edgeOrderReduction),
                                  var_grid=bool(cfg.useVariableGrid), damping=damp)
    return sim.run(case["nt"])
