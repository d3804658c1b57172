"""Benchmark of the forward time step on the 3-D elastic workload:
256^3 grid, DH = 2 m, 8th-order staggered FD, free surface on top and a
20-point CPML on the other faces, 8 depth layers (vp ~ U[1800,4500], seed 2,
vs = vp/1.73, rho = 310 vp^0.25) with a +-5% seeded random perturbation,
explosive Ricker source (10 Hz) at (128, 20, 128), 2,000 three-component
receivers on the surface, DT = 1.5e-4 s, NT = 3000. Synthetic inputs of those
shapes (there is no dataset); a "step" is one time step over the whole grid.
Sparse operators with zero-padded edge rows (edgeOrderReduction=0, the rule
the reference's CI goldens were made with): with the current edge-order
reduction this heterogeneous model grows without bound after ~2500 of the
3000 steps, in FP64 as in FP32, so a whole-shot run would not be a valid
simulation.

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
WORKLOAD = "3-D elastic 256^3, order 8, free surface + 20-pt CPML, DT=1.5e-4, NT=3000, 2000 3-C surface receivers, zero-padded edge rows"

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
                 CenterFrequencyCPML=10.0, VMaxCPML=4725.0, useStencilMatrix=0, edgeOrderReduction=0)


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


def make_acquisition(nt, dt, wavelet=None, shot=0):
    """Explosive source of shot `shot` (shots step 16 cells along x) and the
    2,000 three-component surface receivers. `wavelet(shape, nt, dt, fc, amp,
    tshift)` makes the source signal: the library's wave_wavelet on the GPU
    arm, the oracle's restatement on the CPU reference arm."""
    if wavelet is None:
        from oracle.refcpu import ricker
        wavelet = lambda shape, n, d, fc, amp, ts: ricker(n, d, fc, amp, ts, np.float32)
    sx = (NX // 2 + 16 * shot) % NX
    sidx = np.array([sx + NX * (NZ // 2 + NZ * 20)], dtype=np.int64)
    stype = np.array([1], dtype=np.int32)
    sig = np.asarray(wavelet(1, nt, dt, 10.0, 1.0, 0.0), dtype=np.float32)[None, :]
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


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The largest x over all ranks (all_reduce MAX on the initialised process
    group, NCCL with device "cuda" or gloo with "cpu"); x itself on one rank."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Whole-job throughput of N shot replicas: the units all ranks processed
    over the slowest rank's time (weak scaling: per-rank work is fixed)."""
    return world * units_per_rank / seconds_max


FIELDS_3D = ("vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz")


def cpu_sample(steps: int, warm: int, budget_s: float = 60.0, fields_out: dict | None = None):
    """The reference formulation (oracle refcpu<float>, CSR operators and one
    pass per vector operation) on the full grid, all host threads, for at most
    `steps` steps or `budget_s` seconds of stepping; returns
    (Gpt/s, cores, seconds, steps timed). With `fields_out`, the nine
    wavefields after the last step are stored there (float32)."""
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
    if fields_out is not None:
        for f in FIELDS_3D:
            fields_out[f] = o.field(f).astype(np.float32)
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


def step_roofline(vel_ms, str_ms, passes):
    """The 3-D elastic step against the HBM roofline. `achieved` is the step's
    algorithmic bytes (84 B per grid point + 8 B per CPML psi array and slab
    point: 1.724 GB at 256^3) over the CUDA-event time of the step kernels, so
    a kernel pair that moves more than the single-sweep figure reads lower;
    `traffic` is the step kernels' measured DRAM bytes (ncu) per step."""
    peak, peak_kind = load_peaks()
    psi_b = psi_bytes_per_kernel()
    step_alg = ALG_BYTES_PER_PT * N + 2 * psi_b
    step_ms = vel_ms + str_ms
    achieved = step_alg / (step_ms * 1e-3) / 1e9

    def kname(pass_bit, pair_bit, base):
        if passes & pair_bit:
            return f"el3dp_{base}<4> (TMA streaming, two points per thread)"
        return f"el3d_{base}<4> (TMA streaming)" if passes & pass_bit else f"elastic_{base[0]}<4> (generic)"
    names = {"velocity": kname(1, 4, "vel"), "stress": kname(2, 8, "str")}
    traffic = load_traffic() or {}
    t_v, t_s = (traffic.get(names[k].split("<")[0]) for k in ("velocity", "stress"))
    step_traffic = (t_v + t_s) if (t_v and t_s and NX == 256) else None
    vel_b = VEL_BYTES_PER_PT * N + psi_b
    str_b = STR_BYTES_PER_PT * N + psi_b
    return {"bound": "hbm", "kernel": f"{names['velocity'].split(' ')[0]} + {names['stress'].split(' ')[0]} (one time step)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": f"{peak_kind} copy bandwidth (burst)", "traffic": step_traffic,
            "traffic_note": "DRAM bytes per step: ncu dram__bytes_read.sum + dram__bytes_write.sum of the step kernels "
                            "at 256^3 (profiles/el3dp_*_streaming_256.md)",
            "alg_bytes_per_step": step_alg, "alg_bytes_note": "84 B/pt (9 state arrays read+written, 3 base materials "
                                                              "read) + 8 B per psi array per slab point",
            "step_ms": step_ms,
            "per_pass": {"velocity": {"kernel": names["velocity"], "ms": vel_ms, "alg_bytes": vel_b,
                                      "frac_of_own_bytes": vel_b / (vel_ms * 1e-3) / 1e9 / peak,
                                      "traffic": t_v if NX == 256 else None},
                         "stress": {"kernel": names["stress"], "ms": str_ms, "alg_bytes": str_b,
                                    "frac_of_own_bytes": str_b / (str_ms * 1e-3) / 1e9 / peak,
                                    "traffic": t_s if NX == 256 else None}}}


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
    # one shot per rank (disjoint shot lists, no data-path collective)
    sidx, stype, sig, ridx, rtype = make_acquisition(s.nt, cfg.DT, wave.wavelet, shot=rank)
    dev_model = {k: torch.from_numpy(v).cuda() for k, v in model.items()}
    s.prepareForModelling(dev_model)
    if args.kernel_path:
        s.set_kernel_path(args.kernel_path)
    s.setSources(sidx, stype, sig)
    s.setReceivers(ridx, rtype)
    assert args.warmup + args.steps + 8 <= s.nt, "warmup + steps must leave at least 8 steps for the kernel timing"

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # warm-up (it also captures the step graph), then the timed region: K
    # steps of the product path (graph replay of 16-step chunks with
    # programmatic dependent launch) between two CUDA events on the solver's
    # stream (inputs resident in HBM, state 9 x 64 MiB >> L2)
    s.run(0, args.warmup)
    barrier()
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
    # the step kernels' own durations (roofline): a few more steps with an
    # event pair around every kernel (no graph)
    t_k = args.warmup + args.steps
    n_k = min(32, s.nt - t_k)
    s.set_timing(True)
    s.run(t_k, t_k + n_k)
    vel_ms, str_ms, nsamp = s.kernel_times()
    passes = s.streaming_passes()
    s.set_timing(False)
    ms_total = max_over_ranks(ms_total, world)
    ms_step = ms_total / args.steps
    value = whole_job_rate(N * args.steps, ms_total * 1e-3, world) / 1e9
    finite = s.check_finite()
    s.close()

    # end to end through the public API with host buffers, one whole shot:
    # handle creation, model upload and preparation, acquisition, every time
    # step of the shot, seismogram read-back
    e2e = None
    if not args.no_e2e:
        e2e_steps = args.e2e_steps or s.nt
        barrier()
        t0 = time.perf_counter()
        s2 = wave.Factory.Create("3D", "elastic").initForwardSolver(cfg)
        s2.prepareForModelling(model)
        s2.setSources(sidx, stype, sig)
        s2.setReceivers(ridx, rtype)
        s2.run(0, e2e_steps)
        seis = s2.seismograms()
        t1 = time.perf_counter()
        s2.close()
        h2d = sum(v.nbytes for v in model.values()) + sig.nbytes + sidx.nbytes + stype.nbytes + ridx.nbytes + rtype.nbytes
        d2h = seis.nbytes
        e2e_s = max_over_ranks(t1 - t0, world)
        e2e = {"value": whole_job_rate(N * e2e_steps, e2e_s, world) / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": h2d / e2e_steps, "d2h_bytes_per_step": d2h / e2e_steps, "steps": e2e_steps,
               "what": "create + model upload/preparation + acquisition + all steps of one shot + seismogram read-back"}

    roof = step_roofline(vel_ms, str_ms, passes)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded layered model, Ricker source)",
        "config": {"workload": WORKLOAD if NX == 256 else f"3-D elastic {NX}^3 (profiling size)", "grid": [NX, NY, NZ],
                   "order": 8, "l2": "inputs larger than L2 (state 9 x N x 4 B)",
                   "parallelism": f"one shot per rank x{world}" if world > 1 else "1 GPU"},
        "roofline": roof, "e2e": e2e, "gpu_launches": launches, "finite": finite,
        "timed_path": "CUDA graph replay of 16-step chunks (the library's multi-step path); roofline kernel times "
                      "from further steps with per-kernel events",
    }
    clocks = clk.summary()
    if clocks:
        line["clocks"] = clocks
    if rank == 0 and world == 1 and not args.no_cpu:
        ref_fields = {}
        gpts, cores, sec, done = cpu_sample(args.cpu_steps, 1, budget_s=30.0, fields_out=ref_fields)
        line["cpu_baseline"] = {"value": gpts, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"1 warm-up + {done} timed steps of the full 256^3 grid "
                                          f"with the CPU oracle (reference formulation, FP32), {sec:.1f} s"}
        # parity on this workload: the same steps from rest on the GPU (same inputs), all nine wavefields
        s3 = wave.Factory.Create("3D", "elastic").initForwardSolver(cfg)
        s3.prepareForModelling(dev_model)
        acq = make_acquisition(s3.nt, cfg.DT)
        s3.setSources(*acq[:3])
        s3.setReceivers(*acq[3:])
        s3.run(0, 1 + done)
        num = den = 0.0
        for f in FIELDS_3D:
            a, b = s3.field(f).astype(np.float64), ref_fields[f].astype(np.float64)
            num += float(np.sum((a - b) ** 2))
            den += float(np.sum(b ** 2))
        s3.close()
        line["parity"] = {"rel_l2": (num / den) ** 0.5 if den > 0 else None, "steps": 1 + done,
                          "vs": "CPU oracle refcpu<float> (the reference formulation in FP32)",
                          "what": "all nine wavefields of the full 256^3 grid after the same steps from rest; "
                                  "the tests check the FP64 oracle on this configuration"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
# The other measured workloads (--workload): 2-D acoustic whole job, 3-D
# visco-elastic, 128-shot batched 2-D TMz EM. Each prints one JSON line of the
# same shape as the default 3-D elastic line.
# ---------------------------------------------------------------------------
EPS0, MU0 = 8.8541878176e-12, 1.2566370614e-6      # the reference's vacuum constants


def _clocked(fn, stream):
    """Runs fn() between two CUDA events on `stream` with nvidia-smi sampling; returns (ms, clocks)."""
    import torch
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        fn()
        ev1.record(stream)
        torch.cuda.synchronize()
    return ev0.elapsed_time(ev1), clk.summary()


def _timed(fn, stream):
    """fn() between two CUDA events on `stream`; returns ms."""
    import torch
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    fn()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1)


def _line(metric, value, steps, warmup, ms_step, config, roof, e2e, launches, clocks, cpu, extra=None):
    line = {"metric": metric, "value": value, "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded, shapes of the workload)", "config": config, "roofline": roof, "e2e": e2e,
            "gpu_launches": launches}
    if clocks:
        line["clocks"] = clocks
    if cpu:
        line["cpu_baseline"] = cpu
    if extra:
        line.update(extra)
    print(json.dumps(line), flush=True)


def _roof(alg_bytes_step, ms_step, kernel, note=None):
    peak, kind = load_peaks()
    ach = alg_bytes_step / (ms_step * 1e-3) / 1e9
    r = {"bound": "hbm", "kernel": kernel, "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
         "peak_kind": f"{kind} copy bandwidth (burst)", "traffic": None, "alg_bytes_per_step": alg_bytes_step}
    if note:
        r["note"] = note
    return r


def _oracle_rate(cfg_kw, model, acq, steps, budget_s=20.0):
    """Gpt/s of the CPU oracle (fp32, all host threads) over at most `steps` steps / `budget_s` s."""
    from oracle import refcpu
    cores = os.cpu_count() or 1
    refcpu.set_threads(cores)
    cfg = refcpu.make_config(**cfg_kw)
    n = cfg.NX * cfg.NY * (cfg.NZ if cfg.dimension == 3 else 1)
    sidx, stype, sig, ridx, rtype = acq
    o = refcpu.Oracle(cfg, model, sidx, stype, sig, ridx, rtype, dtype=np.float32)
    o.step(0, 1, copy_state=True)
    sec, done = 0.0, 0
    while done < steps and sec < budget_s:
        sec += o.step(1 + done, 2 + done, copy_state=True)
        done += 1
    o.close()
    return n * done / sec / 1e9, cores, done, sec


def _ricker(nt, dt, fc):
    """Ricker source signal from the library's own wave_wavelet (shape 1)."""
    import __graft_entry__ as g
    return g.load_package().wavelet(1, nt, dt, fc, 1.0, 0.0)


# ---- config 1: 2-D acoustic 400 x 200 -------------------------------------
AC2_KW = dict(dimension=2, equation="acoustic", NX=400, NY=200, NZ=1, DH=1.0, DT=2e-4, T=0.4, spatialFDorder=4,
              FreeSurface=0, DampingBoundary=2, BoundaryWidth=20, NPower=4.0, CenterFrequencyCPML=15.0,
              VMaxCPML=2500.0, useStencilMatrix=0, edgeOrderReduction=1)


def ac2_model():
    y = np.arange(200)[:, None] * np.ones((1, 400))
    vp = np.where(y < 100, 1500.0, 2500.0).astype(np.float32).reshape(-1)
    rho = np.where(y < 100, 1000.0, 2000.0).astype(np.float32).reshape(-1)
    return dict(rho=rho, vp=vp)


def ac2_acq(nt, dt):
    sidx = np.array([200 + 400 * 20], np.int64)
    sig = _ricker(nt, dt, 15.0)[None, :]
    ridx = (2 + 4 * np.arange(100) + 400 * 10).astype(np.int64)
    return sidx, np.array([1], np.int32), sig, ridx, np.ones(100, np.int32)


def run_acoustic2d(args, wave):
    import torch
    n = 400 * 200
    psi_pts = 2 * 20 * 200 + 2 * 20 * 400
    alg = 4 * (2 * 3 + 2) * n + 2 * 8 * psi_pts            # 32 B/pt + psi
    vals = {}
    for stencil in (0, 1):
        cfg = wave.WaveConfig.make(**dict(AC2_KW, useStencilMatrix=stencil))
        s = wave.Factory.Create("2D", "acoustic").initForwardSolver(cfg)
        acq = ac2_acq(s.nt, cfg.DT)
        s.prepareForModelling({k: torch.from_numpy(v).cuda() for k, v in ac2_model().items()})
        s.setSources(*acq[:3])
        s.setReceivers(*acq[3:])
        s.run(0, s.nt)                                        # warm-up job (graph capture)
        s.resetCPML()
        l0 = s.launch_count()
        ms, clocks = _clocked(lambda: s.run(0, s.nt), torch.cuda.ExternalStream(s.stream()))
        launches = s.launch_count() - l0
        nt = s.nt
        s.close()
        vals[stencil] = (n * nt / (ms * 1e-3) / 1e9, ms / nt, launches, clocks)
    value, ms_step, launches, clocks = vals[0]
    # end to end with host buffers: create, model, acquisition, whole job, seismograms
    t0 = time.perf_counter()
    cfg = wave.WaveConfig.make(**AC2_KW)
    s = wave.Factory.Create("2D", "acoustic").initForwardSolver(cfg)
    acq = ac2_acq(s.nt, cfg.DT)
    m = ac2_model()
    s.prepareForModelling(m)
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    s.run(0, s.nt)
    seis = s.seismograms()
    nt = s.nt
    s.close()
    e2e_s = time.perf_counter() - t0
    h2d = sum(v.nbytes for v in m.values()) + sum(a.nbytes for a in acq)
    e2e = {"value": n * nt / e2e_s / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d / nt, "d2h_bytes_per_step": seis.nbytes / nt}
    cpu = None
    if not args.no_cpu:
        g, cores, done, sec = _oracle_rate(AC2_KW, {k: v.astype(np.float64) for k, v in ac2_model().items()}, acq, nt, 20.0)
        cpu = {"value": g, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{done} steps of the 400x200 job with the CPU oracle (FP32), {sec:.1f} s"}
    cfgd = {"workload": "2-D acoustic 400x200, order 4, 20-pt CPML, NT=2000, whole job graph-captured",
            "grid": [400, 200], "order": 4, "l2": "L2-resident (state 0.96 MB): launch/latency bound",
            "stencil_mode_value": vals[1][0], "parallelism": "1 GPU"}
    _line(UNIT, value, nt, nt, ms_step, cfgd, _roof(alg, ms_step, "acoustic_v<2> + acoustic_p<2>",
          "whole state in L2: the HBM roofline is not the bound here"), e2e, launches, clocks, cpu)


# ---- variable grid: the reference's 3-D acoustic variable-grid CI case ------
def vg_case(wave):
    """Configuration, homogeneous model and acquisition of the 3-D variable-grid
    CI case (104 x 303 x 104 fine grid, layers of spacing 17 m / 51 m with FD
    orders 2 / 6, CPML 30, free surface, NT = 1000), from the committed fixtures."""
    ci = os.path.join(ROOT, "tests", "golden", "ci")
    cfg = wave.WaveConfig.from_file(os.path.join(ci, "configuration_ci.3D.acoustic.varGrid.txt"))
    cfg.edgeOrderReduction = 0
    n = wave.grid_num_points(cfg)
    model = dict(rho=np.full(n, 2000.0, np.float32), vp=np.full(n, 3500.0, np.float32))

    def rows(name):
        with open(os.path.join(ci, name)) as f:
            return [l.split() for l in f if l.strip() and not l.startswith("#")]
    nt = int(np.float32(np.float32(cfg.T) / np.float32(cfg.DT)) + np.float32(0.5))
    srcs = [r for r in rows("sources_ci.3D.varGrid.txt")]
    srcs = [r for r in srcs if r[0] == srcs[0][0]]
    sidx = np.array([wave.grid_index(cfg, int(r[1]), int(r[2]), int(r[3])) for r in srcs], np.int64)
    stype = np.array([int(r[4]) for r in srcs], np.int32)
    sig = np.stack([wave.wavelet(int(r[6]), nt, cfg.DT, float(r[7]), float(r[8]), float(r[9])) for r in srcs])
    recs = rows("receiver_ci.3D.varGrid.txt")
    ridx = np.array([wave.grid_index(cfg, int(r[0]), int(r[1]), int(r[2])) for r in recs], np.int64)
    rtype = np.array([int(r[3]) for r in recs], np.int32)
    return cfg, model, (sidx, stype, sig, ridx, rtype)


def vg_alg_bytes(wave, cfg):
    """Algorithmic bytes of one step: per point one 4 B stencil class per pass
    (the class and CPML tables, 1.7 MB, stay on chip), the fields and
    materials read or written once, a 2 B CPML coefficient code per axis and
    pass, and psi read and written where the per-layer CPML frame has
    coefficients."""
    x, y, z, (NX, NY, NZ) = wave.grid_coordinates(cfg)
    n = len(x)
    iface = [cfg.gridInterface[i] for i in range(cfg.gridLayers)] + [NY]
    dhf = np.ones(n, np.int64)
    for l in range(cfg.gridLayers):
        dhf[(y >= iface[l]) & (y < iface[l + 1])] = cfg.gridDHFactor[l]
    w = np.ceil(cfg.BoundaryWidth / dhf)
    frame = 0
    for c, ext, top in ((x, NX, True), (y, NY, cfg.FreeSurface == 0), (z, NZ, True)):
        d = np.minimum(c, ext - 1 - c) // dhf
        inside = d < w
        if not top:
            inside &= ~(c // dhf < w)
        frame += int(inside.sum())
    per_point = (4 + 4 + 24 + 12 + 6) + (4 + 12 + 4 + 8 + 6)
    return n * per_point + 2 * 8 * frame, n, per_point, frame


def run_vargrid3d(args, wave):
    import torch
    cfg, model, acq = vg_case(wave)
    alg, n, per_point, frame = vg_alg_bytes(wave, cfg)
    s = wave.Factory.Create("3D", "acoustic").initForwardSolver(cfg)
    s.prepareForModelling({k: torch.from_numpy(v).cuda() for k, v in model.items()})
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    nt = s.nt
    for _ in range(max(1, args.warmup // 20)):          # warm-up jobs (graph capture)
        s.run(0, nt)
        s.resetCPML()
    l0 = s.launch_count()
    ms, clocks = _clocked(lambda: s.run(0, nt), torch.cuda.ExternalStream(s.stream()))
    launches = s.launch_count() - l0
    s.close()
    value, ms_step = n * nt / (ms * 1e-3) / 1e9, ms / nt
    e2e = None
    if not args.no_e2e:
        t0 = time.perf_counter()
        s = wave.Factory.Create("3D", "acoustic").initForwardSolver(cfg)
        s.prepareForModelling(model)
        s.setSources(*acq[:3])
        s.setReceivers(*acq[3:])
        s.run(0, nt)
        seis = s.seismograms()
        s.close()
        e2e_s = time.perf_counter() - t0
        h2d = sum(v.nbytes for v in model.values()) + sum(a.nbytes for a in acq)
        e2e = {"value": n * nt / e2e_s / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d / nt,
               "d2h_bytes_per_step": seis.nbytes / nt,
               "note": "includes the host assembly of the grid's operators and their upload"}
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import ci_cases
        from oracle import vargrid
        case = ci_cases.load_vargrid_case("3D.acoustic.varGrid")
        c = case["cfg"]
        cp = vargrid.cpml_coefficients(case["grid"], c.BoundaryWidth, c.NPower, c.CenterFrequencyCPML, c.VMaxCPML,
                                       c.DT, c.FreeSurface != 0)
        sim = vargrid.AcousticVarGrid(case["grid"], case["orders"], c.DT, case["model"]["rho"], case["model"]["vp"],
                                      c.FreeSurface, cp, case["src_idx"], case["src_type"], case["signals"],
                                      case["rec_idx"], case["rec_type"], edge=False)
        sim.step(0)
        t0, done = time.perf_counter(), 0
        while done < nt - 1 and time.perf_counter() - t0 < 20.0:
            sim.step(1 + done)
            done += 1
        sec = time.perf_counter() - t0
        cpu = {"value": n * done / sec / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"{done} steps of the job with the variable-grid oracle (scipy.sparse CSR, FP32), {sec:.1f} s"}
    cfgd = {"workload": "3-D acoustic variable grid (the reference's CI case): 104x303x104 fine grid, "
                        f"{n} points in 4 layers (17 m / 51 m), orders 2/6, CPML 30, free surface, NT={nt}",
            "points": n, "parallelism": "1 GPU", "l2": "state ~0.4 GB > L2"}
    roof = _roof(alg, ms_step, "vg_vel + vg_interp + vg_pres (stencil classes)",
                 f"{per_point} B/pt + psi; the ELL blocks (kernel path 1) would add {6 * 6 * 8 - 8} B/pt")
    _line(UNIT, value, nt, nt, ms_step, cfgd, roof, e2e, launches, clocks, cpu)


# ---- config 3: 3-D visco-elastic 512 x 256 (depth) x 512 -------------------
def _tau_method(q, f0, freqs):
    w0 = 2 * np.pi * f0
    ts = [1.0 / (2 * np.pi * f) for f in freqs]
    return (1.0 / q) / sum(w0 * t / (1 + w0 * w0 * t * t) for t in ts)


VI3_FREQ = [10.0 / 3.0, 30.0]
VI3_KW = dict(dimension=3, equation="viscoelastic", NX=512, NY=256, NZ=512, DH=5.0, DT=5e-4, T=2.0, spatialFDorder=4,
              FreeSurface=0, DampingBoundary=2, BoundaryWidth=20, NPower=4.0, CenterFrequencyCPML=10.0, VMaxCPML=3600.0,
              numRelaxationMechanisms=2, relaxationFrequency=VI3_FREQ, useStencilMatrix=0, edgeOrderReduction=1)


def vi3_model(NX, NY, NZ, device):
    """vp 3000, vs 1700, rho 2200 times (1 + 0.05 n); n = white noise (seed 20260003)
    smoothed by a Gaussian of sigma = 10 cells (reflecting edges, separable, on
    the GPU), rescaled to unit std and clipped to +-3; tau from the tau-method
    at 10 Hz with Qp = 80, Qs = 50."""
    import torch
    g = np.random.default_rng(20260003).standard_normal((NY, NZ, NX), dtype=np.float32)
    t = torch.from_numpy(g).to(device)
    for dim in range(3):
        x = t.movedim(dim, -1)
        shp = x.shape
        r = min(40, shp[-1] - 1)                     # 4 sigma, or less on short axes
        k = torch.arange(-r, r + 1, device=device, dtype=torch.float32)
        w = torch.exp(-0.5 * (k / 10.0) ** 2)
        w = (w / w.sum()).view(1, 1, -1)
        x = x.reshape(-1, 1, shp[-1])
        x = torch.cat([x[..., 1:r + 1].flip(-1), x, x[..., -r - 1:-1].flip(-1)], dim=-1)   # reflecting edges
        out = torch.empty((x.shape[0], 1, shp[-1]), device=device, dtype=torch.float32)
        for c0 in range(0, x.shape[0], 16384):
            out[c0:c0 + 16384] = torch.nn.functional.conv1d(x[c0:c0 + 16384], w)
        t = out.reshape(shp).movedim(-1, dim)
    t = ((t - t.mean()) / t.std()).clamp_(-3, 3)
    f = (1 + 0.05 * t).reshape(-1).contiguous()
    tp, ts = _tau_method(80.0, 10.0, VI3_FREQ), _tau_method(50.0, 10.0, VI3_FREQ)
    return dict(vp=3000.0 * f, vs=1700.0 * f, rho=2200.0 * f, taup=torch.full_like(f, tp), taus=torch.full_like(f, ts))


def vi3_acq(NX, NY, NZ, nt, dt):
    sidx = np.array([NX // 2 + NX * (NZ // 2 + NZ * min(40, NY - 1))], np.int64)
    sig = _ricker(nt, dt, 10.0)[None, :]
    xs = (40 + 7 * np.arange(64)) % NX
    zs = (40 + 7 * np.arange(64)) % NZ
    X, Z = np.meshgrid(xs, zs, indexing="ij")
    ridx = (X + NX * (Z + NZ * min(20, NY - 1))).reshape(-1).astype(np.int64)
    return sidx, np.array([1], np.int32), sig, ridx, np.full(ridx.size, 3, np.int32)


def run_visco3d(args, wave):
    import torch
    kw = dict(VI3_KW)
    if args.grid != 256:
        kw.update(NX=2 * args.grid, NY=args.grid, NZ=2 * args.grid)
    NXv, NYv, NZv = kw["NX"], kw["NY"], kw["NZ"]
    n = NXv * NYv * NZv
    cfg = wave.WaveConfig.make(**kw)
    s = wave.Factory.Create("3D", "viscoelastic").initForwardSolver(cfg)
    model = vi3_model(NXv, NYv, NZv, "cuda")
    acq = vi3_acq(NXv, NYv, NZv, s.nt, cfg.DT)
    s.prepareForModelling(model)
    if args.kernel_path:
        s.set_kernel_path(args.kernel_path)
    s.setSources(*acq[:3])
    s.setReceivers(*acq[3:])
    s.run(0, args.warmup)
    l0 = s.launch_count()
    ms, clocks = _clocked(lambda: s.run(args.warmup, args.warmup + args.steps), torch.cuda.ExternalStream(s.stream()))
    launches = s.launch_count() - l0
    finite = s.check_finite()
    passes = s.streaming_passes()
    s.close()
    ms_step = ms / args.steps
    value = n * args.steps / (ms * 1e-3) / 1e9
    vel_kernel = ("el3dp_vel<2> (TMA streaming, two points per thread)" if passes & 4 else
                  "el3d_vel<2> (TMA streaming)" if passes & 1 else "elastic_v<2> (generic)")
    str_kernel = ("el3dp_vstr<2,2> (TMA streaming, two points per thread)" if passes & 8 else "visco_s<2> (generic)")
    w = 20
    psi_pts = 2 * w * NYv * NZv + 2 * w * NXv * NYv + 2 * w * NXv * NZv
    alg = 4 * (2 * (9 + 6 * 2) + 5) * n + 6 * 8 * psi_pts       # 188 B/pt + psi
    e2e = None
    if not args.no_e2e:
        host_model = {k: v.cpu().numpy() for k, v in model.items()}
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = wave.Factory.Create("3D", "viscoelastic").initForwardSolver(cfg)
        e2e_steps = args.e2e_steps or s2.nt
        s2.prepareForModelling(host_model)
        s2.setSources(*acq[:3])
        s2.setReceivers(*acq[3:])
        s2.run(0, e2e_steps)
        seis = s2.seismograms()
        s2.close()
        sec = time.perf_counter() - t0
        h2d = sum(v.nbytes for v in host_model.values()) + sum(a.nbytes for a in acq)
        e2e = {"value": n * e2e_steps / sec / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d / e2e_steps,
               "d2h_bytes_per_step": seis.nbytes / e2e_steps, "steps": e2e_steps,
               "what": "create + model upload/preparation + acquisition + all steps of one shot + seismogram read-back"}
    del model
    cpu = None
    if not args.no_cpu:
        sk = dict(kw, NX=128, NY=64, NZ=128)
        smodel = {k: v.cpu().numpy().astype(np.float64) for k, v in vi3_model(128, 64, 128, "cuda").items()}
        g, cores, done, sec = _oracle_rate(sk, smodel, vi3_acq(128, 64, 128, 4000, kw["DT"]), 10, 20.0)
        cpu = {"value": g, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{done} steps of the same physics on a 128x64x128 sub-grid with the CPU oracle (FP32), {sec:.1f} s"}
    cfgd = {"workload": f"3-D visco-elastic {NXv}x{NYv}(depth)x{NZv}, order 4, L=2, 20-pt CPML, DT=5e-4, NT=4000, 4096 receivers",
            "grid": [NXv, NYv, NZv], "order": 4, "L": 2, "l2": "inputs larger than L2 (state 21 x N x 4 B)",
            "parallelism": "1 GPU"}
    _line(UNIT, value, args.steps, args.warmup, ms_step, cfgd, _roof(alg, ms_step, vel_kernel + " + " + str_kernel),
          e2e, launches, clocks, cpu, {"finite": finite})


# ---- config 4: 128-shot batched 2-D TMz EM --------------------------------
C0 = 1.0 / np.sqrt(MU0 * EPS0)
TM_DT = 0.9 * 0.02 / ((7.0 / 6.0) * np.sqrt(2.0) * C0 / 2.0)


def tm_shots(nshots):
    rng = np.random.default_rng(20260004)
    shots = []
    for _ in range(nshots):
        nx, ny = int(rng.integers(300, 1201)), int(rng.integers(150, 501))
        K = int(rng.integers(3, 9))
        depths = np.sort(rng.integers(1, ny, K - 1))
        er_l = rng.uniform(4.0, 25.0, K)
        sg_l = 10 ** rng.uniform(-4.0, -2.0, K)
        layer = np.searchsorted(depths, np.arange(ny), side="right")
        er = np.repeat(er_l[layer][:, None], nx, axis=1)
        sg = np.repeat(sg_l[layer][:, None], nx, axis=1)
        for _r in range(int(rng.integers(0, 4))):
            x0, y0 = int(rng.integers(0, nx - 10)), int(rng.integers(0, ny - 10))
            w, h = int(rng.integers(10, max(11, nx // 4))), int(rng.integers(5, max(6, ny // 4)))
            er[y0:y0 + h, x0:x0 + w] = rng.uniform(4.0, 25.0)
            sg[y0:y0 + h, x0:x0 + w] = 10 ** rng.uniform(-4.0, -2.0)
        shots.append((nx, ny, dict(eps_r=er.astype(np.float32).reshape(-1), sigma=sg.astype(np.float32).reshape(-1),
                                   mu_r=np.ones(nx * ny, np.float32))))
    return shots


def tm_cfg_kw(nx, ny):
    return dict(dimension=2, equation="tmem", NX=nx, NY=ny, NZ=1, DH=0.02, DT=TM_DT, T=3000 * TM_DT, spatialFDorder=4,
                FreeSurface=0, DampingBoundary=2, BoundaryWidth=20, NPower=4.0, CenterFrequencyCPML=2e8, VMaxCPML=C0 / 2,
                useStencilMatrix=0, edgeOrderReduction=1)


def tm_acq(nx, nt):
    sidx = np.array([30 + nx * 25], np.int64)
    sig = _ricker(nt, TM_DT, 2e8)[None, :]
    ridx = (40 + 4 * np.arange(60) + nx * 25).astype(np.int64)
    return sidx, np.array([1], np.int32), sig, ridx, np.ones(60, np.int32)


def run_tmem_batch(args, wave):
    import torch
    nshots = args.shots
    shots = tm_shots(nshots)
    npts = sum(nx * ny for nx, ny, _ in shots)
    cfgs = [wave.WaveConfig.make(**tm_cfg_kw(nx, ny)) for nx, ny, _ in shots]
    # batched: all shots in each launch (schedule autotuned unless --schedule fixes it)
    b = wave.Batch(cfgs)
    if args.schedule:
        b.set_schedule(*(int(v) for v in args.schedule.split(",")))
    for shot, (nx, ny, m) in zip(b.shots, shots):
        shot.prepareForModelling({k: torch.from_numpy(v).cuda() for k, v in m.items()})
        acq = tm_acq(nx, shot.nt)
        shot.setSources(*acq[:3])
        shot.setReceivers(*acq[3:])
    b.run(0, args.warmup)
    sched = b.schedule()
    l0 = b.launch_count()
    ms, clocks = _clocked(lambda: b.run(args.warmup, args.warmup + args.steps), torch.cuda.ExternalStream(b.stream()))
    launches = b.launch_count() - l0
    b.close()
    value = npts * args.steps / (ms * 1e-3) / 1e9
    # plain: the same shots one at a time through single-shot handles
    plain_ms = 0.0
    for (nx, ny, m), cfg in zip(shots, cfgs):
        s = wave.Factory.Create("2D", "tmem").initForwardSolver(cfg)
        s.prepareForModelling({k: torch.from_numpy(v).cuda() for k, v in m.items()})
        acq = tm_acq(nx, s.nt)
        s.setSources(*acq[:3])
        s.setReceivers(*acq[3:])
        s.run(0, args.warmup)
        plain_ms += _timed(lambda: s.run(args.warmup, args.warmup + args.steps), torch.cuda.ExternalStream(s.stream()))
        s.close()
    plain = npts * args.steps / (plain_ms * 1e-3) / 1e9
    psi_b = sum(2 * 8 * 2 * 20 * (nx + ny) for nx, ny, _ in shots)
    alg = 36 * npts + psi_b
    e2e = None
    if not args.no_e2e:
        t0 = time.perf_counter()
        b2 = wave.Batch(cfgs)
        h2d = d2h = 0
        for shot, (nx, ny, m) in zip(b2.shots, shots):
            shot.prepareForModelling(m)
            acq = tm_acq(nx, shot.nt)
            shot.setSources(*acq[:3])
            shot.setReceivers(*acq[3:])
            h2d += sum(v.nbytes for v in m.values()) + sum(a.nbytes for a in acq)
        e2e_steps = args.e2e_steps or b2.nt
        b2.run(0, e2e_steps)
        for shot in b2.shots:
            d2h += shot.seismograms().nbytes
        b2.close()
        sec = time.perf_counter() - t0
        e2e = {"value": npts * e2e_steps / sec / 1e9, "unit": UNIT, "h2d_bytes_per_step": h2d / e2e_steps,
               "d2h_bytes_per_step": d2h / e2e_steps, "steps": e2e_steps,
               "what": "batch creation + models + acquisitions of all shots + all steps + seismogram read-back"}
    cpu = None
    if not args.no_cpu:
        rates = []
        done_tot, sec_tot, cores = 0, 0.0, 1
        for nx, ny, m in shots[:4]:
            g, cores, done, sec = _oracle_rate(tm_cfg_kw(nx, ny), {k: v.astype(np.float64) for k, v in m.items()},
                                               tm_acq(nx, 3000), 50, 5.0)
            rates.append(g)
            done_tot += done
            sec_tot += sec
        cpu = {"value": float(np.mean(rates)), "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"4 of the shots, {done_tot} shot-steps in {sec_tot:.1f} s with the CPU oracle (FP32)"}
    cfgd = {"workload": f"batched 2-D TMz EM, {nshots} shots, nx U[300,1200], ny U[150,500], order 4, 20-pt CPML, "
                        f"DT={TM_DT:.3e}, NT=3000, 60 Ez receivers per shot",
            "shots": nshots, "points_per_step": npts, "l2": "inputs larger than L2 (3 x 31 M x 4 B)", "parallelism": "1 GPU"}
    _line(UNIT, value, args.steps, args.warmup, ms / args.steps, cfgd,
          _roof(alg, ms / args.steps, "tm_h_batch<2> + tm_e_batch<2>"), e2e, launches, clocks, cpu,
          {"plain_value": plain, "batched_over_plain": value / plain, "schedule": sched})


# ---- config 5: 2-D elastic FWI gradient, 32 shots ---------------------------
FWI_KW = dict(dimension=2, equation="elastic", NX=600, NY=300, NZ=1, DH=5.0, DT=5e-4, T=2.0, spatialFDorder=4,
              FreeSurface=0, DampingBoundary=2, BoundaryWidth=20, NPower=4.0, CenterFrequencyCPML=10.0, VMaxCPML=4400.0,
              useStencilMatrix=0, edgeOrderReduction=1)


def fwi_models(NX, NY):
    """True model: 6 layers, vp 1800 -> 4000 with depth, vs = vp/1.73, rho = 310 vp^0.25,
    Gaussian anomalies +-10 % on vp and vs (sigma 15 cells) at (200, 120) and
    (400, 180); start model = true smoothed by a Gaussian of 10 cells."""
    from scipy.ndimage import gaussian_filter
    y, x = np.mgrid[0:NY, 0:NX]
    layer = np.minimum(y * 6 // NY, 5)
    vp = 1800.0 + (4000.0 - 1800.0) * layer / 5.0
    blob = lambda cx, cy: np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * 15.0 ** 2))
    pert = 0.10 * blob(200, 120) - 0.10 * blob(400, 180)
    vpt = vp * (1 + pert)
    vst = vp / 1.73 * (1 + pert)
    true = dict(vp=vpt, vs=vst, rho=310.0 * vpt ** 0.25)
    start = {k: gaussian_filter(v, 10.0, mode="nearest") for k, v in true.items()}
    f = lambda d: {k: v.astype(np.float32).reshape(-1) for k, v in d.items()}
    return f(true), f(start)


def fwi_acq(NX, k, nt, dt):
    sidx = np.array([30 + 17 * k + NX * 10], np.int64)
    sig = _ricker(nt, dt, 10.0)[None, :]
    xs = 30 + 4 * np.arange(136)
    ridx = np.concatenate([xs + NX * 10, xs + NX * 10]).astype(np.int64)
    rtype = np.concatenate([np.full(136, 2), np.full(136, 3)]).astype(np.int32)
    return sidx, np.array([1], np.int32), sig, ridx, rtype


def run_fwi2d(args, wave):
    import torch
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    nshots = min(args.shots, 32)
    cfg = wave.WaveConfig.make(**FWI_KW)
    NX, NY = 600, 300
    true, start = fwi_models(NX, NY)
    K = 50
    if world > 1:
        return run_fwi2d_shot_domains(args, wave, cfg, nshots, true, start, K, world, rank)
    # observed data: the FP32 forward on the true model, one shot at a time
    dobs, acqs = [], []
    for k in range(nshots):
        s = wave.Factory.Create("2D", "elastic").initForwardSolver(cfg)
        acq = fwi_acq(NX, k, s.nt, cfg.DT)
        s.prepareForModelling(true)
        s.setSources(*acq[:3])
        s.setReceivers(*acq[3:])
        s.run(0, s.nt)
        dobs.append(s.seismograms())
        acqs.append(acq)
        nt = s.nt
        s.close()
    # Both arms time the same work from the same starting point: handle
    # creation, model upload and preparation, acquisition, forward +
    # checkpointed adjoint of every shot, gradients back on the host.
    def plain_once():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        grad, J = None, 0.0
        for k in range(nshots):
            s = wave.Factory.Create("2D", "elastic").initForwardSolver(cfg)
            s.prepareForModelling(start)
            s.setSources(*acqs[k][:3])
            s.setReceivers(*acqs[k][3:])
            Jk, gvp, gvs, grho = s.adjoint_gradient(dobs[k], checkpoint_every=K)
            J += Jk
            grad = gvp.astype(np.float64) if grad is None else grad + gvp
            s.close()
        return time.perf_counter() - t0, J, grad

    def batched_once(count=False):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b = wave.Batch([cfg] * nshots)
        for shot, acq in zip(b.shots, acqs):
            shot.prepareForModelling(start)
            shot.setSources(*acq[:3])
            shot.setReceivers(*acq[3:])
        l0 = b.launch_count()
        mis, bvp, bvs, brho = b.adjoint_gradient(dobs, checkpoint_every=K, sum_shots=True)
        torch.cuda.synchronize()
        sec = time.perf_counter() - t0
        nl = b.launch_count() - l0
        b.close()
        return sec, mis, bvp, nl

    plain_runs = [plain_once() for _ in range(args.repeats)]
    with ClockSampler(torch.cuda.current_device()) as clk:
        batch_runs = [batched_once() for _ in range(args.repeats)]
    plain_s = statistics.median(r[0] for r in plain_runs)
    batch_s = statistics.median(r[0] for r in batch_runs)
    misfit_plain, plain_grad = plain_runs[-1][1], plain_runs[-1][2]
    mis, bvp = batch_runs[-1][1], batch_runs[-1][2]
    # forward steps counted by the batch plus the adjoint driver's own launches (per step: view copy,
    # residual injection, two adjoint kernels; per segment: two state copies; per shot: residual, chain rule)
    launches = batch_runs[-1][3] + 4 * nt + 2 * ((nt + K - 1) // K) + 2 * nshots
    rel = float(np.linalg.norm(bvp - plain_grad) / np.linalg.norm(plain_grad))
    value = nshots / batch_s
    plain = nshots / plain_s
    n = NX * NY
    # algorithmic bytes per shot-step: forward 52 + recompute 72 + adjoint/imaging 96 B/pt
    alg = 220 * n * nt * nshots
    h2d = sum(d.nbytes for d in dobs) + sum(a.nbytes for acq in acqs for a in acq)
    line_cfg = {"workload": f"2-D elastic FWI gradient 600x300 order 4, 20-pt CPML, DT=5e-4, NT={nt}, {nshots} shots, "
                            f"136 two-component receivers, checkpoints every {K} steps",
                "shots": nshots, "grid": [NX, NY], "order": 4, "checkpoint_every": K, "parallelism": "1 GPU",
                "l2": "inputs larger than L2 over a shot-gradient (recompute buffers 51 states x 32 shots)"}
    ms_grad = batch_s * 1e3 / nshots
    roof = _roof(alg / nshots, ms_grad, "elastic_v/s_batch<2> + adj_pass<2> (batched)",
                 "220 B/pt per shot-step (forward 52, recompute 72, adjoint+imaging 96)")
    _line("shot-gradients/s", value, nshots, 1, ms_grad, line_cfg, roof,
          {"value": value, "unit": "shot-gradients/s", "h2d_bytes_per_step": h2d / nshots, "d2h_bytes_per_step": 3 * n * 4},
          launches, clk.summary(), None,
          {"unit": "shot-gradients/s", "plain_value": plain, "batched_over_plain": value / plain,
           "repeats": args.repeats, "timing": "median of the repeats; both arms time handle creation, model, "
                                             "acquisition, forward + adjoint and the gradient read-back",
           "batched_s_all": [r[0] for r in batch_runs], "plain_s_all": [r[0] for r in plain_runs],
           "misfit": float(sum(mis)), "misfit_plain": misfit_plain, "batched_vs_plain_grad_rel_l2": rel})


def run_fwi2d_shot_domains(args, wave, cfg, nshots, true, start, K, world, rank):
    """--gpus N: the 32 shots split into contiguous blocks over the ranks (one
    GPU each), each block one batch, the gradients summed over the ranks
    (the only collective); rate = all shots over the slowest rank's time."""
    import torch
    import torch.distributed as dist
    lb, ub = wave.shot_range(nshots, rank, world)
    dobs, acqs = [None] * nshots, [None] * nshots
    for k in range(lb, ub):
        s = wave.Factory.Create("2D", "elastic").initForwardSolver(cfg)
        acqs[k] = fwi_acq(600, k, s.nt, cfg.DT)
        s.prepareForModelling(true)
        s.setSources(*acqs[k][:3])
        s.setReceivers(*acqs[k][3:])
        s.run(0, s.nt)
        dobs[k] = s.seismograms()
        s.close()
    times = []
    for _ in range(args.repeats):
        torch.cuda.synchronize()
        dist.barrier()
        t0 = time.perf_counter()
        mis, gvp, gvs, grho = wave.fwi_gradient_shot_domains(cfg, start, acqs, dobs, checkpoint_every=K)
        torch.cuda.synchronize()
        times.append(max_over_ranks(time.perf_counter() - t0, world))
    sec = statistics.median(times)
    if rank == 0:
        n = 600 * 300
        cfgd = {"workload": f"2-D elastic FWI gradient 600x300 order 4, {nshots} shots over {world} ranks",
                "shots": nshots, "parallelism": f"shot domains x{world} (gradient sum over ranks)"}
        _line("shot-gradients/s", nshots / sec, nshots, 0, sec * 1e3 / nshots, cfgd, None,
              {"value": nshots / sec, "unit": "shot-gradients/s", "h2d_bytes_per_step": None,
               "d2h_bytes_per_step": 3 * n * 4}, None, None, None,
              {"unit": "shot-gradients/s", "n_gpus": world, "misfit": mis, "repeats": args.repeats})
    dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=40, help="full-grid CPU oracle steps for cpu_baseline (at most 30 s)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=0, help="time steps of the end-to-end shot (0 = the whole shot, NT)")
    ap.add_argument("--grid", type=int, default=256, help="cube edge (profiling captures use a smaller cube)")
    ap.add_argument("--workload", default="elastic3d", choices=["elastic3d", "acoustic2d", "visco3d", "tmem_batch", "fwi2d", "vargrid3d"])
    ap.add_argument("--shots", type=int, default=128, help="shots of the batched EM workload")
    ap.add_argument("--repeats", type=int, default=3, help="repeats of the FWI-gradient arms (median reported)")
    ap.add_argument("--schedule", default="", help="tmem_batch: fix the batch schedule as 'cols,rows,blocks_per_sm' "
                                                  "(profiling; default: the autotuner)")
    ap.add_argument("--kernel-path", type=int, default=0, choices=[0, 1, 2, 3],
                    help="3-D elastic and visco-elastic kernels: 0 automatic, 1 generic, 2 one-point streaming, 3 two-point streaming (profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload != "elastic3d":
        import __graft_entry__ as g
        wave = g.load_package()
        {"acoustic2d": run_acoustic2d, "visco3d": run_visco3d, "tmem_batch": run_tmem_batch,
         "fwi2d": run_fwi2d, "vargrid3d": run_vargrid3d}[args.workload](args, wave)
        return
    if args.grid != 256:
        set_grid(args.grid)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
