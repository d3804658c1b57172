"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
seismograms and against the FP64 oracle.

Tolerance: relative L2 over all traces and samples <= 1e-4 (FP32 kernels vs the
FP64 oracle, and vs the reference's FP32 goldens); the reference's own gate
(average misfit per sample <= 5e-7) is applied to the goldens as well.
"""
import ctypes

import numpy as np
import pytest

import ci_cases

pytestmark = pytest.mark.gpu
TOL = 1e-4
GATE = 5e-7


def to_wave_cfg(wave, cfg):
    c = wave.WaveConfig()
    ctypes.memmove(ctypes.byref(c), ctypes.byref(cfg), ctypes.sizeof(c))
    return c


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", list(ci_cases.CASES))
def test_gpu_matches_reference_goldens(name, wave, refcpu):
    case = ci_cases.load_case(name)
    cfg = to_wave_cfg(wave, case["cfg"])
    seis = wave.simulate(cfg, case["model"], case["src_idx"], case["src_type"], case["signals"],
                         case["rec_idx"], case["rec_type"])
    g = case["golden"]
    assert refcpu.reference_misfit(seis.astype(np.float64), g) < GATE
    assert rel(seis, g) < TOL


# ----------------------------------------------------------------------------
# every equation x boundary x operator mode against the FP64 oracle
# ----------------------------------------------------------------------------
def make_case(refcpu, eq, dim, order, fs=0, boundary=2, stencil=0, reduce=1, L=2, seed=0, dims=None):
    rng = np.random.default_rng(seed)
    em = eq in ("tmem", "emem", "viscotmem", "viscoemem")
    if dims is not None:
        NX, NY, NZ = dims
    elif dim == 2:
        NX, NY, NZ = 90, 70, 1
    else:
        NX, NY, NZ = 44, 38, 36
    n = NX * NY * NZ
    if em:
        DH = 0.02
        eps_r = rng.uniform(4.0, 9.0, n)
        model = dict(eps_r=eps_r, sigma=10 ** rng.uniform(-4, -2, n), mu_r=np.ones(n))
        if eq.startswith("visco"):
            model.update(tau_eps=rng.uniform(0.05, 0.3, n), tau_sigma=rng.uniform(0.05, 0.3, n))
        vmax, vmin = 3e8 / 2.0, 3e8 / 3.0
        extra = dict(CenterFrequencyCPML=2e8, VMaxCPML=vmax)
    else:
        DH = 5.0
        vp = rng.uniform(2500.0, 3200.0, n)
        model = dict(vp=vp, vs=vp / 1.8, rho=310.0 * vp ** 0.25,
                     taup=rng.uniform(0.02, 0.06, n), taus=rng.uniform(0.02, 0.06, n))
        vmax, vmin = 3200.0, 2500.0 / 1.8 if eq not in ("acoustic",) else 2500.0
        extra = dict(CenterFrequencyCPML=12.0, VMaxCPML=vmax)
    DT = 0.35 * DH / (vmax * np.sqrt(dim) * (1.3 if order > 2 else 1.0))
    nt = 600
    cfg = refcpu.make_config(dimension=dim, equation=eq, NX=NX, NY=NY, NZ=NZ, DH=DH, DT=DT, T=nt * DT,
                             spatialFDorder=order, FreeSurface=fs, DampingBoundary=boundary,
                             BoundaryWidth=10 if boundary else 0, DampingCoeff=8.0, NPower=4.0,
                             numRelaxationMechanisms=L if eq.startswith("visco") else 0,
                             relaxationFrequency=[1e8, 6e8, 0.0, 0.0] if em else [8.0, 30.0, 0.0, 0.0],
                             useStencilMatrix=stencil,
                             edgeOrderReduction=reduce, **extra)
    nt = refcpu.nt_of(cfg)
    fc = vmin / (8 * DH)
    sx, sy, sz = NX // 2, (2 if fs else NY // 3), NZ // 2
    src_type = {"acoustic": 1, "elastic": 1, "viscoelastic": 1, "sh": 4, "viscosh": 4, "tmem": 1, "viscotmem": 1,
                "emem": 1 if dim == 3 else 4, "viscoemem": 1 if dim == 3 else 4}[eq]
    sidx = np.array([refcpu.grid_index(cfg, sx, sy, sz)])
    sig = refcpu.ricker(nt, DT, fc, 1.0, 0.0, np.float64)[None]
    if eq in ("sh", "viscosh"):
        rtypes = [4, 4, 4]
    elif eq in ("tmem", "viscotmem"):
        rtypes = [1, 1, 1]
    elif eq in ("emem", "viscoemem"):
        rtypes = [1, 2, 3, 4] if dim == 3 else [2, 3, 4]
    else:
        rtypes = [1, 2, 3] + ([4] if dim == 3 else [])
    ridx = [refcpu.grid_index(cfg, 3 + (7 * k) % (NX - 6), (k * 5) % NY if not fs else 0, (3 * k) % NZ)
            for k in range(len(rtypes))]
    ridx += [refcpu.grid_index(cfg, NX - 4, NY - 3, NZ - 1), refcpu.grid_index(cfg, 1, NY // 2, 0)]
    rtypes += [rtypes[0], rtypes[-1]]
    model = {k: v for k, v in model.items()}
    return cfg, model, sidx, np.array([src_type]), sig, np.array(ridx, dtype=np.int64), np.array(rtypes)


def run_both(wave, refcpu, case):
    cfg, model, sidx, stype, sig, ridx, rtype = case
    o = refcpu.Oracle(cfg, model, sidx, stype, sig, ridx, rtype, dtype=np.float64)
    ref = o.run()
    o.close()
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    gpu = wave.simulate(to_wave_cfg(wave, cfg), m32, sidx, stype, sig.astype(np.float32), ridx, rtype)
    return gpu, ref


SEISMIC = [
    # (eq, dim, order, fs, boundary, stencil, reduce)
    ("acoustic", 2, 4, 0, 2, 0, 1),
    ("acoustic", 2, 8, 1, 1, 1, 0),
    ("acoustic", 3, 6, 0, 2, 0, 1),
    ("acoustic", 3, 4, 1, 2, 0, 0),
    ("elastic", 2, 2, 0, 2, 0, 1),
    ("elastic", 2, 12, 1, 2, 0, 1),
    ("elastic", 2, 10, 1, 1, 0, 0),
    ("elastic", 3, 8, 1, 2, 0, 1),
    ("elastic", 3, 4, 0, 1, 1, 0),
    ("elastic", 3, 2, 0, 0, 0, 1),
    ("viscoelastic", 2, 6, 1, 2, 0, 1),
    ("viscoelastic", 2, 4, 0, 1, 1, 0),
    ("viscoelastic", 3, 4, 0, 2, 0, 1),
    ("viscoelastic", 3, 2, 1, 1, 0, 1),
    ("sh", 2, 4, 0, 2, 0, 1),
    ("sh", 2, 8, 1, 1, 0, 0),
    ("viscosh", 2, 6, 0, 2, 0, 1),
    ("tmem", 2, 4, 0, 2, 0, 1),
    ("tmem", 2, 6, 0, 1, 1, 0),
    ("emem", 2, 4, 0, 2, 0, 1),
    ("emem", 2, 2, 0, 1, 0, 0),
    ("viscotmem", 2, 4, 0, 2, 0, 1),
    ("viscotmem", 2, 8, 0, 1, 1, 0),
    ("viscoemem", 2, 6, 0, 2, 0, 1),
    ("viscoemem", 2, 2, 0, 0, 0, 1),
    ("emem", 3, 4, 0, 2, 0, 1),
    ("emem", 3, 2, 0, 1, 0, 0),
    ("viscoemem", 3, 6, 0, 2, 0, 1),
    ("viscoemem", 3, 4, 0, 1, 1, 0),
]


@pytest.mark.parametrize("eq,dim,order,fs,boundary,stencil,reduce", SEISMIC)
def test_gpu_matches_fp64_oracle(eq, dim, order, fs, boundary, stencil, reduce, wave, refcpu):
    case = make_case(refcpu, eq, dim, order, fs, boundary, stencil, reduce)
    gpu, ref = run_both(wave, refcpu, case)
    assert np.abs(ref).max() > 0
    assert rel(gpu, ref) < TOL, f"relative L2 {rel(gpu, ref):.3e}"


STREAMING = [
    # (order, fs, boundary, stencil, reduce, (NX, NY, NZ)): NX % 4 == 0 selects the TMA kernels
    (8, 1, 2, 0, 1, (64, 50, 48)),
    (2, 0, 1, 1, 0, (40, 33, 37)),
    (4, 1, 1, 0, 0, (44, 38, 36)),
    (12, 0, 2, 0, 1, (48, 45, 35)),
    (6, 1, 0, 0, 1, (36, 40, 33)),
    (10, 1, 2, 1, 0, (52, 41, 30)),
]


@pytest.mark.parametrize("order,fs,boundary,stencil,reduce,dims", STREAMING)
def test_streaming_elastic_kernels_match_oracle_and_generic(order, fs, boundary, stencil, reduce, dims, wave, refcpu):
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, "elastic", 3, order, fs, boundary, stencil, reduce,
                                                          dims=dims)
    o = refcpu.Oracle(cfg, model, sidx, stype, sig, ridx, rtype, dtype=np.float64)
    ref = o.run()
    o.close()
    wc = to_wave_cfg(wave, cfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    s32 = sig.astype(np.float32)
    fast = wave.simulate(wc, m32, sidx, stype, s32, ridx, rtype, kernel_path=2, expect_streaming=True)
    generic = wave.simulate(wc, m32, sidx, stype, s32, ridx, rtype, kernel_path=1, expect_streaming=False)
    auto = wave.simulate(wc, m32, sidx, stype, s32, ridx, rtype, kernel_path=0)
    assert rel(fast, ref) < TOL, f"streaming vs FP64 oracle {rel(fast, ref):.3e}"
    assert rel(generic, ref) < TOL
    assert rel(fast, generic) < 1e-5
    # the automatic path times both kernels per pass on the unstepped state and must leave it untouched
    assert rel(auto, generic) < 1e-5


PAIRS = [
    # (order, fs, boundary, stencil, reduce, (NX, NY, NZ)): 64-wide tiles meeting at most one x CPML slab
    (8, 1, 2, 0, 1, (128, 50, 48)),
    (2, 0, 1, 1, 0, (128, 33, 37)),
    (4, 1, 1, 0, 0, (132, 38, 36)),
    (12, 0, 2, 0, 1, (136, 45, 35)),
    (6, 1, 0, 0, 1, (128, 40, 33)),
    (10, 1, 2, 1, 0, (132, 41, 30)),
]


@pytest.mark.parametrize("order,fs,boundary,stencil,reduce,dims", PAIRS)
def test_two_point_streaming_kernels_match_oracle_and_generic(order, fs, boundary, stencil, reduce, dims, wave, refcpu):
    """The two-points-per-thread streaming kernels (path 3) against the FP64
    oracle and the generic kernels."""
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, "elastic", 3, order, fs, boundary, stencil, reduce,
                                                          dims=dims)
    o = refcpu.Oracle(cfg, model, sidx, stype, sig, ridx, rtype, dtype=np.float64)
    ref = o.run()
    o.close()
    wc = to_wave_cfg(wave, cfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    s32 = sig.astype(np.float32)
    pairs = wave.simulate(wc, m32, sidx, stype, s32, ridx, rtype, kernel_path=3, expect_streaming=True)
    generic = wave.simulate(wc, m32, sidx, stype, s32, ridx, rtype, kernel_path=1, expect_streaming=False)
    assert rel(pairs, ref) < TOL, f"two-point streaming vs FP64 oracle {rel(pairs, ref):.3e}"
    assert rel(pairs, generic) < 1e-5


@pytest.mark.parametrize("order,fs,boundary,dims,L", [(8, 1, 2, (128, 44, 40), 2), (4, 0, 1, (132, 40, 36), 2),
                                                    (4, 1, 2, (128, 40, 36), 2), (2, 0, 2, (96, 36, 32), 1),
                                                    (6, 0, 2, (100, 38, 34), 1)])
def test_visco_elastic_streaming_kernels(order, fs, boundary, dims, L, wave, refcpu):
    """3-D visco-elastic: path 2 runs the one-point streaming velocity kernel
    with the generic memory-variable stress kernel; path 3 runs the two-point
    streaming kernels for both passes (the memory-variable stress kernel
    el3dp_vstr: orders 2-8, one or two mechanisms). Against the FP64 oracle
    and the generic kernels."""
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, "viscoelastic", 3, order, fs, boundary, dims=dims, L=L)
    o = refcpu.Oracle(cfg, model, sidx, stype, sig, ridx, rtype, dtype=np.float64)
    ref = o.run()
    o.close()
    wc = to_wave_cfg(wave, cfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    s32 = sig.astype(np.float32)
    generic = wave.simulate(wc, m32, sidx, stype, s32, ridx, rtype, kernel_path=1, expect_streaming=False)
    assert rel(generic, ref) < TOL
    for path, bits in ((2, 0b0001), (3, 0b1111)):
        s = wave.Factory.Create("3D", "viscoelastic").initForwardSolver(wc)
        s.prepareForModelling(m32)
        s.set_kernel_path(path)
        assert s.streaming_passes() == bits
        s.setSources(sidx, stype, s32)
        s.setReceivers(ridx, rtype)
        s.run(0, s.nt)
        out = s.seismograms()
        s.close()
        assert rel(out, ref) < TOL, f"path {path} vs FP64 oracle {rel(out, ref):.3e}"
        assert rel(out, generic) < 1e-5, f"path {path} vs generic {rel(out, generic):.3e}"


def test_multi_step_graph_equals_single_steps(wave, refcpu):
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, "elastic", 2, 8, 1, 2)
    wc = to_wave_cfg(wave, cfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    outs = []
    for mode in ("graph", "single"):
        s = wave.Factory.Create("2D", "elastic").initForwardSolver(wc)
        s.prepareForModelling(m32)
        s.setSources(sidx, stype, sig.astype(np.float32))
        s.setReceivers(ridx, rtype)
        if mode == "graph":
            s.run(0, s.nt)
        else:
            for t in range(s.nt):
                s.run(t)
        outs.append(s.seismograms())
        s.close()
    assert np.array_equal(outs[0], outs[1])


DEPENDENT = [
    # (eq, dim, order, fs, boundary, dims, kernel_path): ABS and CPML, generic and streaming passes
    ("acoustic", 2, 4, 0, 1, None, 0),
    ("elastic", 2, 8, 1, 2, None, 0),
    ("viscoelastic", 3, 4, 0, 1, None, 0),
    ("tmem", 2, 6, 0, 2, None, 0),
    ("emem", 3, 4, 0, 2, None, 0),
    ("elastic", 3, 8, 1, 2, (64, 50, 48), 2),
]


@pytest.mark.parametrize("eq,dim,order,fs,boundary,dims,path", DEPENDENT)
def test_dependent_launch_is_bit_identical(eq, dim, order, fs, boundary, dims, path, wave, refcpu):
    """Programmatic dependent launch only changes when the kernels are
    scheduled: seismograms and final wavefields equal the serialised launches
    bit for bit, through the step graph and through single steps."""
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, eq, dim, order, fs, boundary, dims=dims)
    wc = to_wave_cfg(wave, cfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    outs = []
    for on in (True, False):
        s = wave.Factory.Create(f"{dim}D", eq).initForwardSolver(wc)
        s.prepareForModelling(m32)
        s.set_kernel_path(path)
        s.set_dependent_launch(on)
        s.setSources(sidx, stype, sig.astype(np.float32))
        s.setReceivers(ridx, rtype)
        s.run(0, s.nt - 5)
        for t in range(s.nt - 5, s.nt):
            s.run(t)
        outs.append((s.seismograms(), s.state()))
        s.close()
    assert np.abs(outs[0][0]).max() > 0
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])


def test_checkpoint_resume_is_bit_identical(wave, refcpu):
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, "viscoelastic", 3, 4, 0, 2)
    wc = to_wave_cfg(wave, cfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    s = wave.Factory.Create("3D", "viscoelastic").initForwardSolver(wc)
    s.prepareForModelling(m32)
    s.setSources(sidx, stype, sig.astype(np.float32))
    s.setReceivers(ridx, rtype)
    s.run(0, 100)
    blob = s.state()
    s.run(100, 200)
    a = s.seismograms()[:, 100:200].copy()
    s.set_state(blob)
    s.run(100, 200)
    b = s.seismograms()[:, 100:200].copy()
    s.close()
    assert np.array_equal(a, b)


def test_device_model_pointers_match_host(wave, refcpu):
    torch = pytest.importorskip("torch")
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, "acoustic", 2, 4, 0, 2)
    wc = to_wave_cfg(wave, cfg)
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    host = wave.simulate(wc, m32, sidx, stype, sig.astype(np.float32), ridx, rtype)
    dev = {k: torch.from_numpy(v).cuda() for k, v in m32.items()}
    devout = wave.simulate(wc, dev, sidx, stype, torch.from_numpy(sig.astype(np.float32)).cuda(), ridx, rtype)
    assert np.array_equal(host, devout)


def test_nonfinite_wavefield_is_reported(wave, refcpu):
    """A CFL violation blows the wavefield up; the device finite check reports
    it as WAVE_ERR_NONFINITE (Simulation.cpp:519) and nothing traps."""
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, "acoustic", 2, 4, 0, 0)
    wc = to_wave_cfg(wave, cfg)
    wc.DT = wc.DT * 20
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    with pytest.raises(wave.WaveError) as e:
        wave.simulate(wc, m32, sidx, stype, sig.astype(np.float32), ridx, rtype)
    assert e.value.code == wave.WAVE_ERR_NONFINITE


def test_launch_count_is_native(wave, refcpu):
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, "tmem", 2, 4, 0, 2)
    s = wave.Factory.Create("2D", "tmem").initForwardSolver(to_wave_cfg(wave, cfg))
    s.prepareForModelling({k: v.astype(np.float32) for k, v in model.items()})
    s.setSources(sidx, stype, sig.astype(np.float32))
    s.setReceivers(ridx, rtype)
    before = s.launch_count()
    s.run(0, 40)
    s.seismograms()
    assert s.launch_count() - before >= 40 * 3
    s.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_acoustic_fused_source_receiver_step_is_bit_identical(dim, wave, refcpu):
    """On small acoustic grids the pressure kernel adds the sources and records
    the receivers itself (one launch less per step); kernel path 1 keeps the
    separate source/receiver kernel. Same operations: same bits. Two sources,
    receivers of every component, two of them at one point."""
    cfg, model, sidx, stype, sig, ridx, rtype = make_case(refcpu, "acoustic", dim, 4, 1, 2)
    sidx = np.concatenate([sidx, sidx + 7])
    stype = np.concatenate([stype, stype])
    sig = np.concatenate([sig, 0.5 * sig])
    ridx = np.concatenate([ridx, ridx[:1]])
    rtype = np.concatenate([rtype, [2]])
    m32 = {k: v.astype(np.float32) for k, v in model.items()}
    wc = to_wave_cfg(wave, cfg)
    a = wave.simulate(wc, m32, sidx, stype, sig.astype(np.float32), ridx, rtype, kernel_path=0)
    b = wave.simulate(wc, m32, sidx, stype, sig.astype(np.float32), ridx, rtype, kernel_path=1)
    np.testing.assert_array_equal(a, b)
    o = refcpu.Oracle(cfg, model, sidx, stype, sig, ridx, rtype, dtype=np.float64)
    ref = o.run()
    o.close()
    assert rel(a, ref) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 4, 8])
def test_gpu_tez_equals_gpu_sh_under_the_te_sh_analogy(order, wave, refcpu):
    """The CUDA TEz step against the CUDA SH step (which passes the reference's
    2-D SH golden): under the TE/SH analogy of test_oracle_em.te_sh_pair the
    Hz traces equal the mapped vz traces to FP32 rounding (the material
    coefficients are formed differently: 1/rho from the host's rho = mu_r mu0
    against 1/(4-point average of mu) with mu = mu_r mu0 formed on the
    device), and both agree with the FP64 oracle."""
    from test_oracle_em import te_sh_pair
    (te, tm, ta), (sh, sm, sa) = te_sh_pair(refcpu, order)
    out = []
    for cfg, model, acq, key in ((te, tm, ta, "emem"), (sh, sm, sa, "sh")):
        s = wave.Factory.Create("2D", key).initForwardSolver(to_wave_cfg(wave, cfg))
        s.prepareForModelling({k: v.astype(np.float32) for k, v in model.items()})
        s.setSources(acq[0], acq[1], acq[2].astype(np.float32))
        s.setReceivers(acq[3], acq[4])
        s.run(0, s.nt)
        out.append(s.seismograms().astype(np.float64))
        s.close()
    o = refcpu.Oracle(sh, sm, *sa, dtype=np.float64)
    ref = o.run()
    o.close()
    d_te, d_sh = out
    print(f"TEz vs SH order {order}: rel {rel(d_te, d_sh):.2e}; TEz vs FP64 {rel(d_te, ref):.2e}; SH vs FP64 {rel(d_sh, ref):.2e}")
    assert rel(d_te, d_sh) <= 1e-5
    assert rel(d_te, ref) <= 1e-5 and rel(d_sh, ref) <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("order", [2, 4, 8])
def test_gpu_3d_em_splits_into_gpu_tmz_and_tez(order, wave, refcpu):
    """The CUDA 3-D EM step on z-invariant line sources against the CUDA TMz
    and TEz steps (test_oracle_em.em3_split_case): the middle slice's Ez and
    Hz traces agree to FP32 rounding."""
    from test_oracle_em import em3_split_case
    out = []
    for cfg, model, acq in em3_split_case(refcpu, order):
        s = wave.Factory.Create("3D" if cfg.dimension == 3 else "2D", "tmem" if cfg.equation == 5 else "emem")
        s = s.initForwardSolver(to_wave_cfg(wave, cfg))
        s.prepareForModelling({k: v.astype(np.float32) for k, v in model.items()})
        s.setSources(acq[0], acq[1], acq[2].astype(np.float32))
        s.setReceivers(acq[3], acq[4])
        s.run(0, s.nt)
        out.append(s.seismograms().astype(np.float64))
        s.close()
    d3, dtm, dte = out
    k = dtm.shape[0]
    e1, e2 = rel(d3[:k], dtm), rel(d3[k:], dte)
    print(f"3-D EM vs TMz / TEz order {order}: Ez {e1:.2e}, Hz {e2:.2e}")
    assert e1 <= 1e-5 and e2 <= 1e-5
