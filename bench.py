"""Benchmark of the forward time step on the 3-D elastic workload:
256^3 grid, DH = 2 m, 8th-order staggered FD, free surface on top and a
20-point CPML on the other faces, 8 depth layers (vp ~ U[1800,4500], seed 2,
vs = vp/1.73, rho = 310 vp^0.25) with a +-5% seeded random perturbation,
explosive Ricker source (10 Hz) at (128, 20, 128), 2,000 three-component
receivers on the surface, DT = 1.5e-4 s, NT = 3000. Synthetic inputs of those
shapes (there is no dataset); a "step" is one time step over the whole grid.

Prints one JSON line (rank 0). --impl reference times the reference
formulation (the CPU oracle, CSR operators + per-operation passes, FP32) on the
host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gpt-updates/s, %HBM roofline; shot-gradients/s batched vs plain @1e-4 L2 err"
UNIT = "Gpt-updates/s"
WORKLOAD = "3-D elastic 256^3, order 8, free surface + 20-pt CPML, DT=1.5e-4, NT=3000, 2000 3-C surface receivers"

NX = NY = NZ = 256
N = NX * NY * NZ


def set_grid(n: int):
    """Smaller cube with the same physics (used for profiling captures)."""
    global NX, NY, NZ, N
    NX = NY = NZ = n
    N = n ** 3
    CONFIG_KW.update(NX=n, NY=n, NZ=n)
BOUNDARY = 20
# algorithmic bytes per grid point and step (state arrays read+written once,
# base material arrays read once) and the CPML psi traffic per kernel
STATE_FIELDS = 9
MATERIAL_BASE = 3
ALG_BYTES_PER_PT = 4 * (2 * STATE_FIELDS + MATERIAL_BASE)           # 84 B
VEL_BYTES_PER_PT = 4 * (6 + 3 + 1 + 3)                             # 52 B: read 6 S, 3 v, rho; write 3 v
STR_BYTES_PER_PT = 4 * (3 + 6 + 2 + 6)                             # 68 B: read 3 v, 6 S, M, mu; write 6 S


def slab_points():
    w = BOUNDARY
    x = 2 * w * NY * NZ
    z = 2 * w * NX * NY
    y = w * NX * NZ            # free surface: no top slab
    return x, y, z


def psi_bytes_per_kernel():
    # 3 psi arrays per direction per kernel, each read + written (8 B)
    x, y, z = slab_points()
    return 3 * 8 * (x + y + z)


CONFIG_KW = dict(dimension=3, equation="elastic", NX=NX, NY=NY, NZ=NZ, DH=2.0, DT=1.5e-4, T=0.45,
                 spatialFDorder=8, FreeSurface=1, DampingBoundary=2, BoundaryWidth=BOUNDARY, NPower=4.0,
                 CenterFrequencyCPML=10.0, VMaxCPML=4725.0, useStencilMatrix=0, edgeOrderReduction=1)


def make_model():
    """8 layers of 32 cells along depth, vp_k ~ U[1800,4500] (seed 2), +-5% clipped
    Gaussian perturbation (seed 20260002), vs = vp/1.73, rho = 310 vp^0.25."""
    rng = np.random.default_rng(2)
    vpk = rng.uniform(1800.0, 4500.0, 8)
    vp = np.repeat(vpk, (NY + 7) // 8)[:NY, None, None] * np.ones((NY, NZ, NX))
    eps = 0.05 * np.clip(np.random.default_rng(20260002).standard_normal((NY, NZ, NX)), -1, 1)
    vp = (vp * (1 + eps)).astype(np.float32).reshape(-1)
    vs = (vp / 1.73).astype(np.float32)
    rho = (310.0 * vp.astype(np.float64) ** 0.25).astype(np.float32)
    return dict(rho=rho, vp=vp, vs=vs)


def make_acquisition(nt, dt):
    from oracle.refcpu import ricker  # plain host formula for the synthetic source signal
    sidx = np.array([NX // 2 + NX * (NZ // 2 + NZ * 20)], dtype=np.int64)
    stype = np.array([1], dtype=np.int32)
    sig = ricker(nt, dt, 10.0, 1.0, 0.0, np.float32)[None, :]
    xs = (30 + 5 * np.arange(40)) % NX
    zs = (30 + 4 * np.arange(50)) % NZ
    X, Z = np.meshgrid(xs, zs, indexing="ij")
    base = (X + NX * Z).reshape(-1).astype(np.int64)            # y = 0 (surface)
    ridx = np.concatenate([base, base, base])
    rtype = np.concatenate([np.full(base.size, t, np.int32) for t in (2, 3, 4)])
    return sidx, stype, sig, ridx, rtype


class ClockSampler:
    """nvidia-smi clocks + throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [v.strip() for v in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "elastic3d_o8_256_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_sample(steps: int, warm: int, budget_s: float = 60.0):
    """The reference formulation (oracle refcpu<float>, CSR operators and one
    pass per vector operation) on the full grid, all host threads, for at most
    `steps` steps or `budget_s` seconds of stepping; returns
    (Gpt/s, cores, seconds, steps timed)."""
    from oracle import refcpu
    cores = os.cpu_count() or 1
    refcpu.set_threads(cores)
    cfg = refcpu.make_config(**CONFIG_KW)
    nt = refcpu.nt_of(cfg)
    m = make_model()
    sidx, stype, sig, ridx, rtype = make_acquisition(nt, cfg.DT)
    o = refcpu.Oracle(cfg, m, sidx, stype, sig, ridx, rtype, dtype=np.float32)
    o.step(0, warm, copy_state=True)
    sec, done = 0.0, 0
    while done < steps and sec < budget_s:
        sec += o.step(warm + done, warm + done + 1, copy_state=True)
        done += 1
    o.close()
    return N * done / sec / 1e9, cores, sec, done


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    gpts, cores, sec, done = cpu_sample(args.steps, min(args.warmup, 1))
    line = {
        "impl": "reference", "metric": METRIC, "value": gpts, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3 / max(done, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded layered model, Ricker source)",
        "config": {"workload": WORKLOAD, "grid": [NX, NY, NZ], "order": 8, "steps_sampled": done},
        "cpu_baseline": {"value": gpts, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"1 warm-up + {done} timed steps of the full 256^3 grid (CSR operators, "
                                   f"one pass per vector operation, FP32; at most 60 s of stepping)"},
        "e2e": {"value": gpts, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args):
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__ as g
    wave = g.load_package()
    cfg = wave.WaveConfig.make(**CONFIG_KW)
    model = make_model()
    s = wave.Factory.Create("3D", "elastic").initForwardSolver(cfg)
    sidx, stype, sig, ridx, rtype = make_acquisition(s.nt, cfg.DT)
    dev_model = {k: torch.from_numpy(v).cuda() for k, v in model.items()}
    s.prepareForModelling(dev_model)
    s.setSources(sidx, stype, sig)
    s.setReceivers(ridx, rtype)
    assert args.warmup + args.steps <= s.nt

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # warm-up, then the timed region: K steps with per-kernel CUDA events on
    # the solver's stream (inputs resident in HBM, state 9 x 64 MiB >> L2)
    s.run(0, args.warmup)
    barrier()
    s.set_timing(True)
    launches0 = s.launch_count()
    stream = torch.cuda.ExternalStream(s.stream())
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        barrier()
        ev0.record(stream)
        s.run(args.warmup, args.warmup + args.steps)
        ev1.record(stream)
        barrier()
    launches = s.launch_count() - launches0
    ms_total = ev0.elapsed_time(ev1)
    vel_ms, str_ms, nsamp = s.kernel_times()
    passes = s.streaming_passes()
    s.set_timing(False)
    t_max = torch.tensor([ms_total], device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t_max, op=torch.distributed.ReduceOp.MAX)
    ms_total = float(t_max.item())
    ms_step = ms_total / args.steps
    value = world * N * args.steps / (ms_total * 1e-3) / 1e9
    finite = s.check_finite()
    s.close()

    # end-to-end through the public API with host buffers: model upload and
    # preparation, sources/receivers, K steps, seismogram read-back
    e2e = None
    if args.no_e2e:
        s2 = None
    else:
        s2 = wave.Factory.Create("3D", "elastic").initForwardSolver(cfg)
    if s2 is not None:
        barrier()
        t0 = time.perf_counter()
        s2.prepareForModelling(model)
        s2.setSources(sidx, stype, sig)
        s2.setReceivers(ridx, rtype)
        s2.run(0, args.steps)
        seis = s2.seismograms()
        t1 = time.perf_counter()
        s2.close()
        h2d = sum(v.nbytes for v in model.values()) + sig.nbytes + sidx.nbytes + stype.nbytes + ridx.nbytes + rtype.nbytes
        d2h = seis.nbytes
        e2e = {"value": world * N * args.steps / (t1 - t0) / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps}

    peak, peak_kind = load_peaks()
    psi_b = psi_bytes_per_kernel()
    str_bytes = STR_BYTES_PER_PT * N + psi_b
    vel_bytes = VEL_BYTES_PER_PT * N + psi_b
    dominant = "stress" if str_ms >= vel_ms else "velocity"
    dom_bytes, dom_ms = (str_bytes, str_ms) if dominant == "stress" else (vel_bytes, vel_ms)
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic = load_traffic()
    step_alg = ALG_BYTES_PER_PT * N + 2 * psi_b
    names = {"velocity": "el3d_vel<4> (TMA streaming)" if passes & 1 else "elastic_v<4> (generic)",
             "stress": "el3d_str<4> (TMA streaming)" if passes & 2 else "elastic_s<4> (generic)"}
    roof = {"bound": "hbm", "kernel": names[dominant], "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_kind": f"{peak_kind} copy bandwidth (burst)",
            "traffic": (traffic or {}).get(dominant),
            "alg_bytes_per_launch": dom_bytes,
            "step_pair": {"alg_bytes_per_step": step_alg, "ms": vel_ms + str_ms,
                          "achieved": step_alg / ((vel_ms + str_ms) * 1e-3) / 1e9,
                          "frac": step_alg / ((vel_ms + str_ms) * 1e-3) / 1e9 / peak},
            "kernel_ms": {"velocity": vel_ms, "stress": str_ms, "samples": nsamp}, "kernels": names}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded layered model, Ricker source)",
        "config": {"workload": WORKLOAD if NX == 256 else f"3-D elastic {NX}^3 (profiling size)", "grid": [NX, NY, NZ],
                   "order": 8, "l2": "inputs larger than L2 (state 9 x N x 4 B)",
                   "parallelism": f"shot replicas x{world}" if world > 1 else "1 GPU"},
        "roofline": roof, "e2e": e2e, "gpu_launches": launches, "finite": finite,
    }
    clocks = clk.summary()
    if clocks:
        line["clocks"] = clocks
    if rank == 0 and world == 1 and not args.no_cpu:
        gpts, cores, sec, done = cpu_sample(args.cpu_steps, 1, budget_s=30.0)
        line["cpu_baseline"] = {"value": gpts, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"1 warm-up + {done} timed steps of the full 256^3 grid "
                                          f"with the CPU oracle (reference formulation, FP32), {sec:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--grid", type=int, default=256, help="cube edge (profiling captures use a smaller cube)")
    args = ap.parse_args()
    if args.grid != 256:
        set_grid(args.grid)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
