// solver.cu — the solver handle behind the C ABI of include/wave.h:
// device-resident SoA state, model preparation on the device, the per-step
// kernel sequence, CUDA-graph replay of multi-step calls, seismogram buffers,
// checkpoint blobs and the finite check.
//
// Reference interface replaced: ForwardSolver<ValueType> (ForwardSolver/ForwardSolver.hpp:25-70)
// created by ForwardSolver::Factory::Create (ForwardSolverFactory.cpp:4-67) and
// driven once per time step by Simulation.cpp:444-476.
#include <cmath>
#include <cstring>
#include <exception>
#include <stdexcept>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "el3d.h"
#include "wave_internal.h"

using namespace wave;

namespace {

thread_local std::string g_create_err;
constexpr int kGraphSteps = 16;

bool eq_visco(int eq) { return eq == WAVE_EQ_VISCOELASTIC || eq == WAVE_EQ_VISCOSH || eq == WAVE_EQ_VISCOTMEM || eq == WAVE_EQ_VISCOEMEM; }
bool eq_em(int eq) { return eq >= WAVE_EQ_TMEM; }

// psi slot -> axis (0 x, 1 y, 2 z)
int psi_axis(int s)
{
    switch (s) {
    case PS_P_X: case PS_VXX: case PS_SXX_X: case PS_SXY_X: case PS_SXZ_X: case PS_VYX: case PS_VZX:
    case PS_EZX: case PS_HYX: case PS_EYX: case PS_HZX: return 0;
    case PS_P_Z: case PS_VZZ: case PS_SXZ_Z: case PS_SYZ_Z: case PS_SZZ_Z: case PS_VXZ: case PS_VYZ:
    case PS_EYZ: case PS_EXZ: case PS_HYZ: case PS_HXZ: return 2;
    default: return 1;
    }
}

} // namespace

#include "handle.h"
#include "trace.h"

namespace {


} // namespace

void wave::set_global_error(const std::string& msg) { g_create_err = msg; }

namespace {

int fail(wave_handle* h, int code, const std::string& msg)
{
    if (h) h->err = msg;
    else g_create_err = msg;
    return code;
}

#define WAVE_TRY(h, ...)                                                    \
    try {                                                                   \
        __VA_ARGS__                                                         \
    } catch (std::exception & ex) {                                         \
        return fail(h, WAVE_ERR_CUDA, ex.what());                           \
    }

int nt_from(const wave_config& c)
{
    float T = static_cast<float>(c.T), DT = static_cast<float>(c.DT);
    return static_cast<int>(T / DT + 0.5f);
}

Op1D to_device(wave_handle* h, const OpHost& o, int slot)
{
    Op1D d;
    d.n = o.n; d.E = o.E; d.full = o.full;
    for (int k = 0; k < kTabW; ++k) d.w[k] = o.w[k];
    float* t = h->alloc<float>(o.tab.size());
    h->check(cudaMemcpy(t, o.tab.data(), o.tab.size() * sizeof(float), cudaMemcpyHostToDevice), "table upload");
    h->opTab[slot] = t;
    d.tab = t;
    return d;
}

Cpml1D cpml_to_device(wave_handle* h, const CpmlHost& c, int axis, int n, int w)
{
    Cpml1D d;
    d.n = n; d.w = w; d.ns = c.ns; d.lo = c.lo; d.on = 1;
    const std::vector<float>* src[4] = {&c.a_full, &c.b_full, &c.a_half, &c.b_half};
    for (int k = 0; k < 4; ++k) {
        float* p = h->alloc<float>(n);
        h->check(cudaMemcpy(p, src[k]->data(), n * sizeof(float), cudaMemcpyHostToDevice), "cpml upload");
        h->cpmlProf[axis][k] = p;
    }
    d.a_full = h->cpmlProf[axis][0]; d.b_full = h->cpmlProf[axis][1];
    d.a_half = h->cpmlProf[axis][2]; d.b_half = h->cpmlProf[axis][3];
    return d;
}

std::vector<int> field_list(int eq, bool is3d)
{
    switch (eq) {
    case WAVE_EQ_ACOUSTIC: return is3d ? std::vector<int>{F_VX, F_VY, F_VZ, F_P} : std::vector<int>{F_VX, F_VY, F_P};
    case WAVE_EQ_ELASTIC:
    case WAVE_EQ_VISCOELASTIC:
        return is3d ? std::vector<int>{F_VX, F_VY, F_VZ, F_SXX, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ}
                    : std::vector<int>{F_VX, F_VY, F_SXX, F_SYY, F_SXY};
    case WAVE_EQ_SH:
    case WAVE_EQ_VISCOSH: return {F_VZ, F_SXZ, F_SYZ};
    case WAVE_EQ_TMEM:
    case WAVE_EQ_VISCOTMEM: return {F_HX, F_HY, F_EZ};
    case WAVE_EQ_EMEM:
    case WAVE_EQ_VISCOEMEM: return is3d ? std::vector<int>{F_HX, F_HY, F_HZ, F_EX, F_EY, F_EZ} : std::vector<int>{F_HZ, F_EX, F_EY};
    default: return {};
    }
}

std::vector<int> pass1_list(int eq, bool is3d)
{
    switch (eq) {
    case WAVE_EQ_ACOUSTIC:
    case WAVE_EQ_ELASTIC:
    case WAVE_EQ_VISCOELASTIC: return is3d ? std::vector<int>{F_VX, F_VY, F_VZ} : std::vector<int>{F_VX, F_VY};
    case WAVE_EQ_SH:
    case WAVE_EQ_VISCOSH: return {F_VZ};
    case WAVE_EQ_TMEM:
    case WAVE_EQ_VISCOTMEM: return {F_HX, F_HY};
    case WAVE_EQ_EMEM:
    case WAVE_EQ_VISCOEMEM: return is3d ? std::vector<int>{F_HX, F_HY, F_HZ} : std::vector<int>{F_HZ};
    default: return {};
    }
}

std::vector<int> mem_list(int eq, bool is3d)
{
    if (eq == WAVE_EQ_VISCOELASTIC) return is3d ? std::vector<int>{R_XX, R_YY, R_ZZ, R_XY, R_XZ, R_YZ} : std::vector<int>{R_XX, R_YY, R_XY};
    if (eq == WAVE_EQ_VISCOSH) return {R_XZ, R_YZ};
    if (eq == WAVE_EQ_VISCOTMEM) return {R_EZ};
    if (eq == WAVE_EQ_VISCOEMEM) return is3d ? std::vector<int>{R_EX, R_EY, R_EZ} : std::vector<int>{R_EX, R_EY};
    return {};
}

std::vector<int> psi_list(int eq, bool is3d)
{
    switch (eq) {
    case WAVE_EQ_ACOUSTIC:
        return is3d ? std::vector<int>{PS_P_X, PS_P_Y, PS_P_Z, PS_VXX, PS_VYY, PS_VZZ} : std::vector<int>{PS_P_X, PS_P_Y, PS_VXX, PS_VYY};
    case WAVE_EQ_ELASTIC:
    case WAVE_EQ_VISCOELASTIC:
        if (is3d)
            return {PS_SXX_X, PS_SXY_Y, PS_SXZ_Z, PS_SXY_X, PS_SYY_Y, PS_SYZ_Z, PS_SXZ_X, PS_SYZ_Y, PS_SZZ_Z,
                    PS_VXX, PS_VYY, PS_VZZ, PS_VXY, PS_VYX, PS_VXZ, PS_VZX, PS_VYZ, PS_VZY};
        return {PS_SXX_X, PS_SXY_Y, PS_SXY_X, PS_SYY_Y, PS_VXX, PS_VYY, PS_VXY, PS_VYX};
    case WAVE_EQ_SH:
    case WAVE_EQ_VISCOSH: return {PS_SXZ_X, PS_SYZ_Y, PS_VZX, PS_VZY};
    case WAVE_EQ_TMEM:
    case WAVE_EQ_VISCOTMEM: return {PS_EZY, PS_EZX, PS_HYX, PS_HXY};
    case WAVE_EQ_EMEM:
    case WAVE_EQ_VISCOEMEM:
        if (is3d)
            return {PS_EZY, PS_EYZ, PS_EXZ, PS_EZX, PS_EYX, PS_EXY, PS_HZY, PS_HYZ, PS_HXZ, PS_HZX, PS_HYX, PS_HXY};
        return {PS_EYX, PS_EXY, PS_HZY, PS_HZX};
    default: return {};
    }
}

// component types the reference accepts per equation
// (SourceReceiverImpl/FDTD2Dsh.hpp:29-34, ForwardSolverEM/SourceReceiverImpl/FDTD2Dtmem.hpp:29-34, ...)
bool type_ok(int eq, bool is3d, int type, bool source)
{
    (void)source;
    switch (eq) {
    case WAVE_EQ_ACOUSTIC:
    case WAVE_EQ_ELASTIC:
    case WAVE_EQ_VISCOELASTIC: return type >= 1 && type <= (is3d ? 4 : 3);
    case WAVE_EQ_SH:
    case WAVE_EQ_VISCOSH: return type == WAVE_TYPE_VZ;
    case WAVE_EQ_TMEM:
    case WAVE_EQ_VISCOTMEM: return type == WAVE_TYPE_EZ;
    case WAVE_EQ_EMEM:
    case WAVE_EQ_VISCOEMEM:
        // SourceReceiverImplEM.cpp:95-110: EZ, EX, EY and HZ; the 2-D TE fields have no EZ
        return is3d ? (type >= WAVE_TYPE_EZ && type <= WAVE_TYPE_HZ) : (type == WAVE_TYPE_EX || type == WAVE_TYPE_EY || type == WAVE_TYPE_HZ);
    default: return false;
    }
}

// the kernel a pass runs: 0 generic, 1 one-point streaming, 2 pair streaming.
// The streaming kernels cover both elastic passes and the velocity pass of the
// visco-elastic step (the same update; its stress pass has memory variables).
int pass_kernel(const wave_handle* h, int pass)
{
    // the visco-elastic stress pass has a two-point streaming kernel only
    const bool viscoStress = pass == 1 && h->cfg.equation == WAVE_EQ_VISCOELASTIC;
    if (pass == 1 && h->cfg.equation != WAVE_EQ_ELASTIC && !viscoStress) return 0;
    if (viscoStress && h->el3dp.gridVisco < 1) return 0;
    switch (h->kernelPath) {
    case 1: return 0;
    case 2: return h->el3d.ready && !viscoStress ? 1 : 0;
    case 3: return h->el3dp.ready ? 2 : 0;
    default: {
        const int k = h->passStreaming[pass];
        return (k == 1 && h->el3d.ready) || (k == 2 && h->el3dp.ready) ? k : 0;
    }
    }
}

void launch_kernel_of(wave_handle* h, int kind, int pass, bool dep)
{
    if (kind == 1) {
        h->check(el3d_launch(h->el3d, h->sp, pass, h->stream), "streaming kernel launch");
    } else if (kind == 2) {
        h->check(el3d_launch_pairs(h->el3dp, h->sp, pass, h->stream), "streaming kernel launch");
    } else {
        StepKernel k = kernel_for(kernel_eq(h->cfg.equation, h->is3d()), pass, h->H);
        launch_step_kernel(k, h->grid, h->block, h->sp, dep && h->dependentLaunch, h->stream);
    }
}

void launch_pass(wave_handle* h, int pass, bool dep = true) { launch_kernel_of(h, pass_kernel(h, pass), pass, dep); }

// Sources and receivers inside the acoustic pressure kernel (SrFuse): on
// grids of at most 2^20 points (the point map, 4 B per point, stays in L2)
// with pressure sources only and no ABS (whose damping of the velocities
// runs after the pressure kernel), unless kernel path 1 asks for the separate
// source/receiver kernel. Saves one launch per step on small grids.
void update_fusion(wave_handle* h)
{
    wave::SrFuse& F = h->sp.sr;
    F = wave::SrFuse{};
    h->graphDirty = true;
    bool ok = h->cfg.equation == WAVE_EQ_ACOUSTIC && !h->vg && !h->sp.abs && h->kernelPath != 1 &&
              h->N <= (1LL << 20) && h->seis != nullptr && h->nrec > 0 && h->nsrc == static_cast<int>(h->hSrcIdx.size()) &&
              h->nrec == static_cast<int>(h->hRecIdx.size());
    for (int t : h->hSrcType) ok = ok && t == WAVE_TYPE_P;
    if (!ok) return;
    // one record per marked point; sources and receivers chained in index order
    std::unordered_map<long long, int> rec;
    std::vector<int> ptSrc, ptRec, lastS, lastR;
    std::vector<int> srcNext(h->nsrc, -1), recNext(h->nrec, -1);
    auto record = [&](long long i) {
        auto it = rec.find(i);
        if (it != rec.end()) return it->second;
        const int k = static_cast<int>(ptSrc.size());
        rec.emplace(i, k);
        ptSrc.push_back(-1); ptRec.push_back(-1); lastS.push_back(-1); lastR.push_back(-1);
        return k;
    };
    for (int s = 0; s < h->nsrc; ++s) {
        const int k = record(h->hSrcIdx[s]);
        if (lastS[k] < 0) ptSrc[k] = s; else srcNext[lastS[k]] = s;
        lastS[k] = s;
    }
    for (int r = 0; r < h->nrec; ++r) {
        const int k = record(h->hRecIdx[r]);
        if (lastR[k] < 0) ptRec[k] = r; else recNext[lastR[k]] = r;
        lastR[k] = r;
    }
    std::vector<int> map(h->N, -1);
    for (const auto& e : rec) map[e.first] = e.second;
    if (!h->srMap) h->srMap = h->alloc<int>(h->N);
    h->check(cudaMemcpy(h->srMap, map.data(), h->N * sizeof(int), cudaMemcpyHostToDevice), "upload");
    auto up = [&](int slot, const std::vector<int>& v) {
        int* d = h->reuse(h->srList[slot], h->srListCap[slot], v.size());
        if (!v.empty()) h->check(cudaMemcpy(d, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice), "upload");
        return static_cast<const int*>(d);
    };
    F.ptSrc = up(0, ptSrc);
    F.ptRec = up(1, ptRec);
    F.srcNext = up(2, srcNext);
    F.recNext = up(3, recNext);
    F.map = h->srMap;
    F.nt = h->NT;
    F.tcounter = h->tcounter;
    F.signals = h->signals;
    F.rtype = h->rtype;
    F.seis = h->seis;
    F.on = 1;
}

void launch_step(wave_handle* h)
{
    if (h->vg) {
        bool done = false;
        h->launches += wave::vargrid_launch_step(h, h->dependentLaunch, nullptr, &done);
        if (!done) {
            h->launches += launch_srcrec(h->sq, h->tcounter, h->stream, h->dependentLaunch);
        }
        return;
    }
    if (h->decompType) wave::decompose_before_step(h);
    launch_pass(h, 0);
    launch_pass(h, 1);
    h->launches += 2;
    if (h->sp.abs) {
        const auto& p1 = h->pass1Fields;
        launch_abs_frame(h->sp, h->grid, h->block, p1.size() > 0 ? p1[0] : -1, p1.size() > 1 ? p1[1] : -1,
                         p1.size() > 2 ? p1[2] : -1, h->stream, h->dependentLaunch);
        h->launches += 1;
    }
    if (!h->sp.sr.on) {
        h->launches += launch_srcrec(h->sq, h->tcounter, h->stream, h->dependentLaunch);
    }
    if (h->decompType) h->launches += wave::decompose_after_step(h);
}

void launch_step_timed(wave_handle* h, std::vector<cudaEvent_t>& ev)
{
    cudaEvent_t a, b, c;
    cudaEventCreate(&a); cudaEventCreate(&b); cudaEventCreate(&c);
    if (h->decompType) wave::decompose_before_step(h);
    cudaEventRecord(a, h->stream);
    if (h->vg) {
        bool done = false;
        h->launches += wave::vargrid_launch_step(h, false, &b, &done);
        cudaEventRecord(c, h->stream);
        ev.push_back(a); ev.push_back(b); ev.push_back(c);
        if (!done) {
            h->launches += launch_srcrec(h->sq, h->tcounter, h->stream);
        }
        return;
    }
    launch_pass(h, 0, false);
    cudaEventRecord(b, h->stream);
    launch_pass(h, 1, false);
    cudaEventRecord(c, h->stream);
    ev.push_back(a); ev.push_back(b); ev.push_back(c);
    h->launches += 2;
    if (h->sp.abs) {
        const auto& p1 = h->pass1Fields;
        launch_abs_frame(h->sp, h->grid, h->block, p1.size() > 0 ? p1[0] : -1, p1.size() > 1 ? p1[1] : -1,
                         p1.size() > 2 ? p1[2] : -1, h->stream);
        h->launches += 1;
    }
    if (!h->sp.sr.on) {
        h->launches += launch_srcrec(h->sq, h->tcounter, h->stream);
    }
    if (h->decompType) h->launches += wave::decompose_after_step(h);
}

// Automatic kernel choice: times each pass with the generic and the streaming
// kernels on the current state and keeps the faster one per pass. Runs only
// on a state that has not been stepped, which every pass leaves at zero (all
// updates are linear in the wavefields and there is no source term in them).
void tune_passes(wave_handle* h)
{
    h->passStreaming[0] = h->passStreaming[1] = h->el3dp.ready ? 2 : (h->el3d.ready ? 1 : 0);
    if ((!h->el3d.ready && !h->el3dp.ready) || h->stepsSinceReset != 0) return;
    cudaEvent_t e0, e1;
    h->check(cudaEventCreate(&e0), "event");
    h->check(cudaEventCreate(&e1), "event");
    // candidates: the generic kernels and the streaming kernels that apply
    // (the two-point ones where they apply: on GB300 they beat the one-point
    // ones on every measured grid)
    const bool ready[3] = {true, h->el3d.ready && !h->el3dp.ready, h->el3dp.ready};
    for (int pass = 0; pass < 2; ++pass) {
        float best = 0.0f;
        h->passStreaming[pass] = 0;
        for (int kind = 0; kind < 3; ++kind) {
            if (!ready[kind]) continue;
            if (kind > 0 && pass == 1 && h->cfg.equation != WAVE_EQ_ELASTIC &&
                !(kind == 2 && h->cfg.equation == WAVE_EQ_VISCOELASTIC && h->el3dp.gridVisco > 0))
                continue;
            launch_kernel_of(h, kind, pass, false);
            h->check(cudaEventRecord(e0, h->stream), "event");
            for (int k = 0; k < 2; ++k) launch_kernel_of(h, kind, pass, false);
            h->check(cudaEventRecord(e1, h->stream), "event");
            h->check(cudaEventSynchronize(e1), "tuning");
            float ms = 0.0f;
            h->check(cudaEventElapsedTime(&ms, e0, e1), "event");
            if (kind == 0 || ms <= best) {
                best = ms;
                h->passStreaming[pass] = kind;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    h->check(cudaGetLastError(), "tuning launch");
    // the state was zero and stays zero; clear it anyway so tuning leaves no trace
    for (int f : h->fields) h->check(cudaMemsetAsync(h->f[f], 0, h->N * sizeof(float), h->stream), "memset");
    for (int rr = 0; rr < R_COUNT; ++rr)
        for (int l = 0; l < kMaxL; ++l)
            if (h->r[rr][l]) h->check(cudaMemsetAsync(h->r[rr][l], 0, h->N * sizeof(float), h->stream), "memset");
    for (int s2 = 0; s2 < PS_COUNT; ++s2)
        if (h->psi[s2]) h->check(cudaMemsetAsync(h->psi[s2], 0, h->psiLen[s2] * sizeof(float), h->stream), "memset");
    h->check(cudaStreamSynchronize(h->stream), "tuning");
}

void build_graph(wave_handle* h)
{
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    cudaGraph_t g;
    h->check(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    long long before = h->launches;
    for (int s = 0; s < kGraphSteps; ++s) launch_step(h);
    h->graphLaunchesPerStep = (h->launches - before) / kGraphSteps;   // kernels per captured step
    h->launches = before;
    h->check(cudaStreamEndCapture(h->stream, &g), "end capture");
    h->check(cudaGraphInstantiate(&h->graph, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    h->graphDirty = false;
}

// Copies n floats from a host or device pointer into a fresh device buffer.
float* stage(wave_handle* h, const float* p, size_t n, int mem, std::vector<float*>& tmp)
{
    if (!p) return nullptr;
    float* d = nullptr;
    h->check(cudaMallocAsync(&d, n * sizeof(float), h->stream), "cudaMallocAsync");
    tmp.push_back(d);
    h->check(cudaMemcpyAsync(d, p, n * sizeof(float), mem == WAVE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream), "model upload");
    return d;
}

// state blob layout: fields (solver order), memory variables, psi slabs, the step counter
std::vector<std::pair<void*, size_t>> state_parts(wave_handle* h)
{
    std::vector<std::pair<void*, size_t>> parts;
    for (int f : h->fields) parts.push_back({h->f[f], h->N * sizeof(float)});
    for (int rr = 0; rr < R_COUNT; ++rr)
        for (int l = 0; l < kMaxL; ++l)
            if (h->r[rr][l]) parts.push_back({h->r[rr][l], h->N * sizeof(float)});
    for (int s = 0; s < PS_COUNT; ++s)
        if (h->psi[s]) parts.push_back({h->psi[s], h->psiLen[s] * sizeof(float)});
    parts.push_back({h->tcounter, sizeof(int)});
    return parts;
}

} // namespace

void wave::step_once(wave_handle* h) { launch_step(h); }

// sum_l w^2 ts_l^2 / (1 + w^2 ts_l^2) with w = 2 pi f_CPML, ts_l = 1 / (2 pi f_l):
// the visco modulus relaxation (Viscoelastic.cpp:650-715), M = rho vp^2 / (1 + sum tauP)
float wave::visco_modulus_sum(const wave_config& c, int L)
{
    float sum = 0.0f;
    const float w_ref = static_cast<float>(2.0 * M_PI * c.CenterFrequencyCPML);
    for (int l = 0; l < L; ++l) {
        const float ts = static_cast<float>(1.0 / (2.0 * M_PI * static_cast<float>(c.relaxationFrequency[l])));
        sum += w_ref * w_ref * ts * ts / (1.0 + w_ref * w_ref * ts * ts);
    }
    return sum;
}


extern "C" {

const char* wave_last_error(const wave_handle* h)
{
    if (!h) return g_create_err.c_str();
    return h->err.c_str();
}

int wave_config_nt(const wave_config* cfg, int* nt)
{
    if (!cfg || !nt || cfg->DT <= 0) return fail(nullptr, WAVE_ERR_ARG, "wave_config_nt: invalid argument");
    *nt = nt_from(*cfg);
    return WAVE_OK;
}

int wave_config_from_file(const char* path, wave_config* cfg)
{
    if (!path || !cfg) return fail(nullptr, WAVE_ERR_ARG, "wave_config_from_file: null argument");
    std::string err;
    int rc = parse_config_file(path, cfg, err);
    if (rc != WAVE_OK) return fail(nullptr, rc, err);
    return WAVE_OK;
}

int wave_wavelet(int shape, int nt, double dt, double fc, double amp, double tshift, float* out)
{
    int rc = make_wavelet(shape, nt, dt, fc, amp, tshift, out);
    if (rc != WAVE_OK) return fail(nullptr, rc, "wave_wavelet: invalid shape or parameter");
    return WAVE_OK;
}

int wave_grid_num_points(const wave_config* cfg, int64_t* n)
{
    if (!cfg || !n) return fail(nullptr, WAVE_ERR_ARG, "wave_grid_num_points: null argument");
    if (cfg->useVariableGrid || cfg->useVariableFDoperators) {
        wave::VarGridLayout L;
        std::string err;
        int rc = wave::vargrid_layout(*cfg, L, err);
        if (rc != WAVE_OK) return fail(nullptr, rc, err);
        *n = L.N;
    } else {
        *n = cfg->NX * cfg->NY * (cfg->dimension == 3 ? cfg->NZ : 1);
    }
    return WAVE_OK;
}

int wave_grid_index(const wave_config* cfg, int64_t x, int64_t y, int64_t z, int64_t* idx)
{
    if (!cfg || !idx) return fail(nullptr, WAVE_ERR_ARG, "wave_grid_index: null argument");
    const int64_t NZ = cfg->dimension == 3 ? cfg->NZ : 1;
    if (cfg->useVariableGrid || cfg->useVariableFDoperators) {
        wave::VarGridLayout L;
        std::string err;
        int rc = wave::vargrid_layout(*cfg, L, err);
        if (rc != WAVE_OK) return fail(nullptr, rc, err);
        const long long i = L.index(x, y, z);
        if (i < 0) return fail(nullptr, WAVE_ERR_ARG, "Could not map from coordinate to index!");
        *idx = i;
        return WAVE_OK;
    }
    if (x < 0 || x >= cfg->NX || y < 0 || y >= cfg->NY || z < 0 || z >= NZ)
        return fail(nullptr, WAVE_ERR_ARG, "Could not map from coordinate to index!");
    *idx = x + z * cfg->NX + y * cfg->NX * NZ;
    return WAVE_OK;
}

int wave_grid_coordinates(const wave_config* cfg, int64_t* x, int64_t* y, int64_t* z, int64_t n, int64_t* extents3)
{
    if (!cfg) return fail(nullptr, WAVE_ERR_ARG, "wave_grid_coordinates: null argument");
    const int64_t NZ = cfg->dimension == 3 ? cfg->NZ : 1;
    wave::VarGridLayout L;
    const bool vg = cfg->useVariableGrid || cfg->useVariableFDoperators;
    if (vg) {
        std::string err;
        int rc = wave::vargrid_layout(*cfg, L, err);
        if (rc != WAVE_OK) return fail(nullptr, rc, err);
    }
    const int64_t N = vg ? L.N : cfg->NX * cfg->NY * NZ;
    if (extents3) {
        extents3[0] = vg ? L.NX : cfg->NX;
        extents3[1] = vg ? L.NY : cfg->NY;
        extents3[2] = vg ? L.NZ : NZ;
    }
    if (!x && !y && !z) return WAVE_OK;
    if (!x || !y || !z || n != N) return fail(nullptr, WAVE_ERR_ARG, "wave_grid_coordinates: n != the number of grid points");
    for (int64_t i = 0; i < N; ++i) {
        if (vg) {
            int a, b, c;
            L.coord(i, a, b, c);
            x[i] = a; y[i] = b; z[i] = c;
        } else {
            x[i] = i % cfg->NX;
            z[i] = (i / cfg->NX) % NZ;
            y[i] = i / (cfg->NX * NZ);
        }
    }
    return WAVE_OK;
}

int wave_grid_operator(const wave_config* cfg, int op, int* width, int32_t* cols, float* vals, int64_t capacity)
{
    if (!cfg || !width || op < 0 || op > 13) return fail(nullptr, WAVE_ERR_ARG, "wave_grid_operator: invalid arguments");
    if (op > 10 && cfg->dimension != 3)
        return fail(nullptr, WAVE_ERR_UNSUPPORTED, "wave_grid_operator: the staggered-z operators and StaggeredXZ are 3-D");
    if (!(cfg->useVariableGrid || cfg->useVariableFDoperators))
        return fail(nullptr, WAVE_ERR_ARG, "wave_grid_operator: not a variable-grid configuration");
    wave::VarGridHost G;
    std::string err;
    int rc = wave::vargrid_build(*cfg, G, err, op > 8);
    if (rc != WAVE_OK) return fail(nullptr, rc, err);
    const long long N = G.L.N;
    if (op < 6 || (op > 8 && op < 13)) {
        const wave::EllHost* ops[13] = {&G.Dxf, &G.Dyf, &G.Dzf, &G.Dxb, &G.Dyb, &G.Dzb, nullptr, nullptr, nullptr,
                                        &G.DyfSX, &G.DybSX, &G.DyfSZ, &G.DybSZ};
        const wave::EllHost& E = *ops[op];
        *width = E.W;
        if (!cols) return WAVE_OK;
        if (!vals || capacity < static_cast<int64_t>(E.W) * N) return fail(nullptr, WAVE_ERR_ARG, "wave_grid_operator: capacity too small");
        std::memcpy(cols, E.col.data(), E.col.size() * sizeof(int32_t));
        std::memcpy(vals, E.val.data(), E.val.size() * sizeof(float));
        return WAVE_OK;
    }
    const wave::InterpHost* in[4] = {&G.full, &G.stagX, &G.stagZ, &G.stagXZ};
    const wave::InterpHost& I = *in[op == 13 ? 3 : op - 6];
    *width = 4;
    if (!cols) return WAVE_OK;
    if (!vals || capacity < 4 * N) return fail(nullptr, WAVE_ERR_ARG, "wave_grid_operator: capacity too small");
    for (long long i = 0; i < N; ++i)
        for (int k = 0; k < 4; ++k) {
            cols[k * N + i] = static_cast<int32_t>(i);
            vals[k * N + i] = k == 0 ? 1.0f : 0.0f;
        }
    for (size_t r = 0; r < I.row.size(); ++r)
        for (int k = 0; k < 4; ++k) {
            cols[k * N + I.row[r]] = I.col[4 * r + k];
            vals[k * N + I.row[r]] = I.w[4 * r + k];
        }
    return WAVE_OK;
}

int wave_solver_create(const wave_config* cfg, wave_handle** out)
{
    if (!cfg || !out) return fail(nullptr, WAVE_ERR_ARG, "wave_solver_create: null argument");
    *out = nullptr;
    const wave_config& c = *cfg;
    wave::TraceRange region(wave::trace_init_name(c.dimension, c.equation));
    if (c.dimension != 2 && c.dimension != 3) return fail(nullptr, WAVE_ERR_ARG, "Unkown dimension");
    if (c.equation < WAVE_EQ_ACOUSTIC || c.equation > WAVE_EQ_VISCOEMEM) return fail(nullptr, WAVE_ERR_ARG, "Unkown type");
    const bool is3d = c.dimension == 3;
    // the reference factory's combinations (ForwardSolverFactory.cpp:13-66)
    if (is3d && (c.equation == WAVE_EQ_SH || c.equation == WAVE_EQ_VISCOSH || c.equation == WAVE_EQ_TMEM || c.equation == WAVE_EQ_VISCOTMEM))
        return fail(nullptr, WAVE_ERR_UNSUPPORTED, "no 3-D solver for this equation type in the reference factory");
    std::vector<double> coef;
    if (!fd_coefficients(c.spatialFDorder, coef)) return fail(nullptr, WAVE_ERR_ARG, "spatialFDorder = " + std::to_string(c.spatialFDorder) + " Unsupported spatialFDorder value.");
    if (c.NX < 1 || c.NY < 1 || (is3d && c.NZ < 1) || c.DH <= 0 || c.DT <= 0 || c.T <= 0)
        return fail(nullptr, WAVE_ERR_ARG, "grid dimensions, DH, DT and T must be positive");
    const long long NZ = is3d ? c.NZ : 1;
    if (c.NX > (1 << 30) || (c.NY * NZ + 7) / 8 > 65535 || c.NX * c.NY * NZ > (1LL << 40))
        return fail(nullptr, WAVE_ERR_ARG, "grid too large");
    if (c.DampingBoundary < 0 || c.DampingBoundary > 2) return fail(nullptr, WAVE_ERR_ARG, "DampingBoundary must be 0, 1 or 2");
    if (c.DampingBoundary != 0 && c.BoundaryWidth <= 0) return fail(nullptr, WAVE_ERR_ARG, "BoundaryWidth must be positive");
    if (c.DampingBoundary == 1 && (c.DampingCoeff <= 0 || c.DampingCoeff >= 100)) return fail(nullptr, WAVE_ERR_ARG, "DampingCoeff must be in (0, 100)");
    if (c.FreeSurface != 0 && c.FreeSurface != 1 && c.FreeSurface != 2) return fail(nullptr, WAVE_ERR_ARG, "FreeSurface must be 0, 1 or 2");
    if (eq_visco(c.equation) && (c.numRelaxationMechanisms < 1 || c.numRelaxationMechanisms > kMaxL))
        return fail(nullptr, WAVE_ERR_ARG, "numRelaxationMechanisms must be 1..4 for visco equations");
    if (eq_visco(c.equation))
        for (int l = 0; l < c.numRelaxationMechanisms; ++l)
            if (c.relaxationFrequency[l] <= 0) return fail(nullptr, WAVE_ERR_ARG, "relaxationFrequency must be positive");
    // variable grid / variable FD orders (Coordinates.cpp:35-95, Derivatives.cpp:12-55)
    const bool vgrid = c.useVariableGrid != 0 || c.useVariableFDoperators != 0;
    wave::VarGridHost vgHost;
    if (vgrid) {
        const bool elastic = c.equation == WAVE_EQ_ELASTIC;
        if (c.equation != WAVE_EQ_ACOUSTIC && !elastic)
            return fail(nullptr, WAVE_ERR_UNSUPPORTED, "variable grids are built for the acoustic and elastic equations");
        if (elastic && c.FreeSurface == 2)
            return fail(nullptr, WAVE_ERR_UNSUPPORTED, "the elastic variable grid is built with the mirror free surface (FreeSurface=1)");
        if (c.useStencilMatrix)
            return fail(nullptr, WAVE_ERR_ARG, "Variable FD operators are not available for stencil matrices");
        std::string err;
        int rc = wave::vargrid_build(c, vgHost, err, elastic);
        if (rc != WAVE_OK) return fail(nullptr, rc, err);
    }

    auto h = std::make_unique<wave_handle>();
    try {
        h->cfg = c;
        h->cfg.NZ = NZ;
        h->NX = static_cast<int>(c.NX); h->NY = static_cast<int>(c.NY); h->NZ = static_cast<int>(NZ);
        h->N = (long long)h->NX * h->NY * h->NZ;
        if (vgrid) {
            h->NX = vgHost.L.NX; h->NY = vgHost.L.NY; h->NZ = vgHost.L.NZ;
            h->N = vgHost.L.N;
        }
        h->NT = nt_from(c);
        h->H = c.spatialFDorder / 2;
        h->L = eq_visco(c.equation) ? c.numRelaxationMechanisms : 0;
        h->check(cudaGetDevice(&h->device), "cudaGetDevice");
        h->check(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        const float DT = static_cast<float>(c.DT), DH = static_cast<float>(c.DH);
        const int stencil = c.useStencilMatrix ? 1 : 0, reduce = c.edgeOrderReduction ? 1 : 0;
        const int q = c.spatialFDorder;
        StepParams& P = h->sp;
        P = StepParams{};
        P.NX = h->NX; P.NY = h->NY; P.NZ = h->NZ; P.is3d = is3d; P.N = h->N;
        P.scale = DT / DH;
        if (!vgrid) {
        P.Dxf = to_device(h.get(), build_op(h->NX, q, OP_F, stencil, reduce, DH, DT), 0);
        P.Dxb = to_device(h.get(), build_op(h->NX, q, OP_B, stencil, reduce, DH, DT), 1);
        P.Dyf = to_device(h.get(), build_op(h->NY, q, OP_F, stencil, reduce, DH, DT), 2);
        P.Dyb = to_device(h.get(), build_op(h->NY, q, OP_B, stencil, reduce, DH, DT), 3);
        if (is3d) {
            P.Dzf = to_device(h.get(), build_op(h->NZ, q, OP_F, stencil, reduce, DH, DT), 4);
            P.Dzb = to_device(h.get(), build_op(h->NZ, q, OP_B, stencil, reduce, DH, DT), 5);
        }
        P.fs = c.FreeSurface == 1 ? 1 : 0;
        if (P.fs) {
            P.DyfS = to_device(h.get(), build_op(h->NY, q, OP_FS_F, stencil, reduce, DH, DT), 6);
            P.DybS = to_device(h.get(), build_op(h->NY, q, OP_FS_B, stencil, reduce, DH, DT), 7);
        }
        }
        // fields
        h->fields = field_list(c.equation, is3d);
        h->pass1Fields = pass1_list(c.equation, is3d);
        for (int f : h->fields) P.f[f] = h->f[f] = h->alloc<float>(h->N);
        for (int rr : mem_list(c.equation, is3d))
            for (int l = 0; l < h->L; ++l) P.r[rr][l] = h->r[rr][l] = h->alloc<float>(h->N);
        // boundaries (the variable grid keeps per-point CPML coefficients, vargrid.cu)
        if (vgrid) wave::vargrid_setup(h.get(), vgHost);
        P.useCpml = c.DampingBoundary == 2 && !vgrid;
        if (P.useCpml) {
            const float np = static_cast<float>(c.NPower), fc = static_cast<float>(c.CenterFrequencyCPML), vm = static_cast<float>(c.VMaxCPML);
            const int w = c.BoundaryWidth;
            P.cx = cpml_to_device(h.get(), build_cpml(h->NX, w, false, np, fc, vm, DT, DH), 0, h->NX, w);
            P.cy = cpml_to_device(h.get(), build_cpml(h->NY, w, c.FreeSurface != 0, np, fc, vm, DT, DH), 1, h->NY, w);
            if (is3d) P.cz = cpml_to_device(h.get(), build_cpml(h->NZ, w, false, np, fc, vm, DT, DH), 2, h->NZ, w);
            for (int s : psi_list(c.equation, is3d)) {
                const int ax = psi_axis(s);
                long long len = ax == 0 ? (long long)P.cx.ns * h->NZ * h->NY
                               : ax == 1 ? (long long)h->NX * h->NZ * P.cy.ns
                                         : (long long)h->NX * P.cz.ns * h->NY;
                P.psi[s] = h->psi[s] = h->alloc<float>(len);
                h->psiLen[s] = len;
            }
        }
        P.abs = c.DampingBoundary == 1;
        if (P.abs) {
            auto coeff = build_abs_coeff(c.BoundaryWidth, static_cast<float>(c.DampingCoeff));
            h->absCoeff = h->alloc<float>(coeff.size());
            h->check(cudaMemcpy(h->absCoeff, coeff.data(), coeff.size() * sizeof(float), cudaMemcpyHostToDevice), "abs upload");
            P.absW = c.BoundaryWidth;
            P.absCoeff = h->absCoeff;
        }
        // visco coefficients (ForwardSolver3Dviscoelastic.cpp:56-66)
        P.L = h->L;
        P.DThalf = static_cast<float>(DT / 2.0);
        P.DT = static_cast<float>(DT);
        for (int l = 0; l < h->L; ++l) {
            const float rt = static_cast<float>(1.0 / (2.0 * M_PI * static_cast<float>(c.relaxationFrequency[l])));
            P.relaxTime[l] = rt;
            P.invRelax[l] = static_cast<float>(1.0 / rt);
            P.c1[l] = static_cast<float>(1.0 - DT / (2.0 * rt));
            P.c2[l] = static_cast<float>(1.0 / (1.0 + DT / (2.0 * rt)));
        }
        h->tcounter = h->alloc<int>(1);
        h->flag = h->alloc<int>(1);
        h->errWord = h->alloc<int>(1);
        h->check(cudaMemset(h->errWord, 0, sizeof(int)), "memset");
        // launch shape: 32 x 8 threads over (x, z + NZ*y)
        h->block = dim3(32, 8, 1);
        h->grid = dim3((h->NX + 31) / 32, static_cast<unsigned>((static_cast<long long>(h->NY) * h->NZ + 7) / 8), 1);
        // source/receiver parameters
        SrcRecParams& Q = h->sq;
        Q = SrcRecParams{};
        Q.eq = c.equation; Q.is3d = is3d; Q.nt = h->NT;
        for (int f = 0; f < F_COUNT; ++f) Q.f[f] = h->f[f];
        int rc = wave_solver_reset(h.get());
        if (rc != WAVE_OK) return fail(nullptr, rc, h->err);
    } catch (std::exception& ex) {
        return fail(nullptr, WAVE_ERR_CUDA, ex.what());
    }
    *out = h.release();
    return WAVE_OK;
}

int wave_solver_destroy(wave_handle* h)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_solver_destroy: null handle");
    cudaStreamSynchronize(h->stream);
    delete h;
    return WAVE_OK;
}

int wave_set_model(wave_handle* h, const float* rho, const float* vp, const float* vs, const float* taup,
                   const float* taus, size_t n, int mem)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_set_model: null handle");
    wave::TraceRange region("WAVE-Simulation.initModel");
    const int eq = h->cfg.equation;
    if (eq_em(eq)) return fail(h, WAVE_ERR_ARG, "wave_set_model: EM equation, use wave_set_model_em");
    if (n != static_cast<size_t>(h->N)) return fail(h, WAVE_ERR_ARG, "wave_set_model: n != the number of grid points");
    const bool needVp = eq != WAVE_EQ_SH && eq != WAVE_EQ_VISCOSH;
    const bool needVs = eq != WAVE_EQ_ACOUSTIC;
    const bool visco = eq_visco(eq);
    if (!rho || (needVp && !vp) || (needVs && !vs) || (visco && !taus) || (eq == WAVE_EQ_VISCOELASTIC && !taup))
        return fail(h, WAVE_ERR_ARG, "wave_set_model: a parameter the equation needs is NULL");
    WAVE_TRY(h, {
        const bool is3d = h->sp.is3d;
        PrepParams G{h->NX, h->NY, h->NZ, h->N};
        cudaStream_t s = h->stream;
        std::vector<float*> tmp;
        float* dRho = stage(h, rho, n, mem, tmp);
        float* dVp = needVp ? stage(h, vp, n, mem, tmp) : nullptr;
        float* dVs = needVs ? stage(h, vs, n, mem, tmp) : nullptr;
        float* dTp = eq == WAVE_EQ_VISCOELASTIC ? stage(h, taup, n, mem, tmp) : nullptr;
        float* dTs = visco ? stage(h, taus, n, mem, tmp) : nullptr;
        if (h->vg) {
            wave::vargrid_set_model(h, dRho, dVp, dVs);
            // rho, vp [, vs] for the adjoint's chain rule
            for (auto [slot, src] : {std::pair<int, const float*>{M_RHO, dRho}, {M_VP, dVp}, {M_VS, dVs}})
                if (src) {
                    if (!h->m[slot]) h->m[slot] = h->alloc<float>(h->N);
                    h->check(cudaMemcpyAsync(h->m[slot], src, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
                }
            for (float* p : tmp) cudaFreeAsync(p, s);
            h->check(cudaStreamSynchronize(s), "model preparation");
            h->modelSet = true;
            h->graphDirty = true;
            return WAVE_OK;
        }
        auto mat = [&](int slot) {
            if (!h->m[slot]) h->m[slot] = h->alloc<float>(h->N);
            h->sp.m[slot] = h->m[slot];
            return h->m[slot];
        };
        const float sum = visco ? visco_modulus_sum(h->cfg, h->L) : 0.0f;
        h->check(cudaMemcpyAsync(mat(M_RHO), dRho, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
        if (eq == WAVE_EQ_ELASTIC || eq == WAVE_EQ_VISCOELASTIC) {
            h->check(cudaMemcpyAsync(mat(M_VP), dVp, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
            h->check(cudaMemcpyAsync(mat(M_VS), dVs, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
        }
        if (eq == WAVE_EQ_ACOUSTIC)   // the acoustic adjoint's chain rule reads vp
            h->check(cudaMemcpyAsync(mat(M_VP), dVp, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
        if ((eq == WAVE_EQ_SH || eq == WAVE_EQ_VISCOSH) && !is3d)   // the SH adjoint's chain rule reads vs
            h->check(cudaMemcpyAsync(mat(M_VS), dVs, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
        if (needVp) k_modulus(G, dRho, dVp, dTp, sum, 0, mat(M_M), s);
        if (needVs) k_modulus(G, dRho, dVs, visco ? dTs : nullptr, sum, 1, mat(M_MU), s);
        if (eq == WAVE_EQ_SH || eq == WAVE_EQ_VISCOSH) {
            k_inverse(G, dRho, mat(M_IR), s);
            float* inv = nullptr;
            h->check(cudaMallocAsync(&inv, n * sizeof(float), s), "cudaMallocAsync");
            tmp.push_back(inv);
            k_inverse(G, h->m[M_MU], inv, s);
            k_harmonic(G, inv, 3, mat(M_MUXZ), s);   // 2-point along x (SH.cpp:429)
            k_harmonic(G, inv, 4, mat(M_MUYZ), s);   // 2-point along y (SH.cpp:430)
            if (visco) {
                k_avg2(G, dTs, 0, mat(M_TAUSXZ), s);
                k_avg2(G, dTs, 1, mat(M_TAUSYZ), s);
                k_one_plus(G, dTs, static_cast<float>(h->L), mat(M_OPLTS), s);
                // tau_s itself, for the adjoint's chain rule (adjoint.cu)
                h->check(cudaMemcpyAsync(mat(M_TAUS), dTs, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
            }
        } else {
            k_inv_avg2(G, dRho, 0, mat(M_IRX), s);
            k_inv_avg2(G, dRho, 1, mat(M_IRY), s);
            if (is3d) k_inv_avg2(G, dRho, 2, mat(M_IRZ), s);
            if (needVs) {
                float* inv = nullptr;
                h->check(cudaMallocAsync(&inv, n * sizeof(float), s), "cudaMallocAsync");
                tmp.push_back(inv);
                k_inverse(G, h->m[M_MU], inv, s);
                k_harmonic(G, inv, 0, mat(M_MUXY), s);
                if (is3d) {
                    k_harmonic(G, inv, 1, mat(M_MUXZ), s);
                    k_harmonic(G, inv, 2, mat(M_MUYZ), s);
                }
            }
            if (eq == WAVE_EQ_VISCOELASTIC) {
                h->check(cudaMemcpyAsync(mat(M_TAUP), dTp, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
                h->check(cudaMemcpyAsync(mat(M_TAUS), dTs, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
                k_avg4(G, dTs, 0, mat(M_TAUSXY), s);
                if (is3d) {
                    k_avg4(G, dTs, 1, mat(M_TAUSXZ), s);
                    k_avg4(G, dTs, 2, mat(M_TAUSYZ), s);
                }
                k_one_plus(G, dTp, static_cast<float>(h->L), mat(M_OPLTP), s);
                k_one_plus(G, dTs, static_cast<float>(h->L), mat(M_OPLTS), s);
            }
        }
        h->check(cudaGetLastError(), "model preparation");
        for (float* p : tmp) cudaFreeAsync(p, s);
        h->check(cudaStreamSynchronize(s), "model preparation");
        if ((eq == WAVE_EQ_ELASTIC || eq == WAVE_EQ_VISCOELASTIC) && is3d) {
            el3d_prepare(h->el3d, h->sp, h->m[M_RHO], h->m[M_M], h->m[M_MU], h->H, h->errWord);
            el3d_prepare_pairs(h->el3dp, h->sp, h->m[M_RHO], h->m[M_M], h->m[M_MU], h->H, h->errWord,
                               eq == WAVE_EQ_VISCOELASTIC ? h->m[M_TAUS] : nullptr);
            tune_passes(h);
        }
        h->modelSet = true;
        h->graphDirty = true;
    })
    return WAVE_OK;
}

int wave_set_model_em(wave_handle* h, const float* eps_r, const float* sigma, const float* mu_r,
                      const float* tau_eps, const float* tau_sigma, size_t n, int mem)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_set_model_em: null handle");
    wave::TraceRange region("WAVE-Simulation.initModel");
    const int eq = h->cfg.equation;
    if (!eq_em(eq)) return fail(h, WAVE_ERR_ARG, "wave_set_model_em: seismic equation, use wave_set_model");
    if (n != static_cast<size_t>(h->N)) return fail(h, WAVE_ERR_ARG, "wave_set_model_em: n != NX*NY*NZ");
    if (!eps_r || !sigma || !mu_r) return fail(h, WAVE_ERR_ARG, "wave_set_model_em: eps_r, sigma and mu_r are required");
    if ((eq == WAVE_EQ_VISCOTMEM || eq == WAVE_EQ_VISCOEMEM) && (!tau_eps || !tau_sigma))
        return fail(h, WAVE_ERR_ARG, "wave_set_model_em: visco-EM needs tau_eps and tau_sigma");
    WAVE_TRY(h, {
        PrepParams G{h->NX, h->NY, h->NZ, h->N};
        cudaStream_t s = h->stream;
        std::vector<float*> tmp;
        float* dEr = stage(h, eps_r, n, mem, tmp);
        float* dSig = stage(h, sigma, n, mem, tmp);
        float* dMr = stage(h, mu_r, n, mem, tmp);
        auto mat = [&](int slot) {
            if (!h->m[slot]) h->m[slot] = h->alloc<float>(h->N);
            h->sp.m[slot] = h->m[slot];
            return h->m[slot];
        };
        auto scratch = [&]() {
            float* p = nullptr;
            h->check(cudaMallocAsync(&p, n * sizeof(float), s), "cudaMallocAsync");
            tmp.push_back(p);
            return p;
        };
        // absolute permittivity / permeability (TMEM.cpp:230-241, ViscoTMEM.cpp:274-292,
        // Modelparameter.hpp:359-360)
        const float eps0 = 8.8541878176e-12f;
        float* eps = scratch();
        float* mu = scratch();
        k_scale(G, dEr, eps0, eps, s);
        k_scale(G, dMr, 1.2566370614e-6f, mu, s);
        const bool visco = eq == WAVE_EQ_VISCOTMEM || eq == WAVE_EQ_VISCOEMEM;
        const bool is3d = h->is3d();
        const float DTf = static_cast<float>(h->cfg.DT);
        float *dTe = nullptr, *dTs = nullptr;
        ViscoEmCoef vc{};
        if (visco) {
            // tau_sigma relative to tau_ref = 1/(2 pi f_c) (ViscoTMEM.cpp:285-286); the
            // solver coefficients of ForwardSolverEM.cpp:68-133
            dTe = stage(h, tau_eps, n, mem, tmp);
            float* ts = stage(h, tau_sigma, n, mem, tmp);
            dTs = scratch();
            const float tauRef = static_cast<float>(1.0 / (2.0 * M_PI * static_cast<float>(h->cfg.CenterFrequencyCPML)));
            k_scale(G, ts, tauRef, dTs, s);
            vc.DT = DTf;
            vc.eps0 = eps0;
            vc.L = h->L;
            float sumInv = 0.0f;
            for (int l = 0; l < h->L; ++l) {
                const float rt = h->sp.relaxTime[l];
                sumInv = static_cast<float>(static_cast<double>(sumInv) + 1.0 / static_cast<double>(rt));
                const double r = rt;
                h->sp.Cc[l] = static_cast<float>((1 - 0.5 * static_cast<double>(DTf) / r) / (1 + 0.5 * static_cast<double>(DTf) / r));
                float tv = static_cast<float>(1 / (1 + 0.5 * static_cast<double>(DTf) / r));
                tv /= (static_cast<float>(h->L) * rt * rt);
                vc.cdScale[l] = tv;
            }
            vc.sumInv = sumInv / static_cast<float>(h->L);
        }
        // Ca/Cb (and C_d) of one E component from its material values
        auto coeffs = [&](const float* e, const float* sg, const float* te, const float* ts, int ca, int cb, int cd0) {
            if (!visco) {
                k_cacb(G, e, sg, DTf, mat(ca), mat(cb), s);
                return;
            }
            float* cd[kMaxL] = {};
            for (int l = 0; l < h->L; ++l) cd[l] = mat(cd0 + l);
            k_visco_em(G, e, sg, te, ts, vc, mat(ca), mat(cb), cd, s);
        };
        if (eq == WAVE_EQ_TMEM || eq == WAVE_EQ_VISCOTMEM) {
            // TMEM/ViscoTMEM::calculateAveraging (TMEM.cpp:366-374, ViscoTMEM.cpp:442-450),
            // FD2Dtmem/FD2Dviscotmem::prepareForModelling (ForwardSolver2Dtmem.cpp:77-106,
            // ForwardSolver2Dviscotmem.cpp:95-124)
            k_inv_avg2(G, mu, 0, mat(M_IMUXZ), s);
            k_inv_avg2(G, mu, 1, mat(M_IMUYZ), s);
            coeffs(eps, dSig, dTe, dTs, M_CAZ, M_CBZ, M_CDZ0);
            if (visco) {
                // tau_eps and the scaled tau_sigma with the coefficient constants, for the adjoint's chain rule
                h->check(cudaMemcpyAsync(mat(M_TAUP), dTe, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
                h->check(cudaMemcpyAsync(mat(M_TAUS), dTs, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
                h->vemc = vc;
            }
        } else {
            // EMEM/ViscoEMEM::calculateAveraging (EMEM.cpp:378-392, ViscoEMEM.cpp:409-432),
            // prepareForModelling of FD2Demem/FD2Dviscoemem/FD3Demem/FD3Dviscoemem
            k_inv_avg4(G, mu, 0, mat(M_IMUXY), s);
            if (is3d) {
                k_inv_avg4(G, mu, 1, mat(M_IMUXZ), s);
                k_inv_avg4(G, mu, 2, mat(M_IMUYZ), s);
            }
            const int naxes = is3d ? 3 : 2;
            const int caS[3] = {M_CAX, M_CAY, M_CAZ}, cbS[3] = {M_CBX, M_CBY, M_CBZ}, cdS[3] = {M_CDX0, M_CDY0, M_CDZ0};
            for (int a = 0; a < naxes; ++a) {
                float* ea = scratch();
                float* sa = scratch();
                k_avg2(G, eps, a, ea, s);
                k_avg2(G, dSig, a, sa, s);
                float *ta = nullptr, *tsa = nullptr;
                if (visco) {
                    ta = scratch();
                    tsa = scratch();
                    k_avg2(G, dTe, a, ta, s);
                    k_avg2(G, dTs, a, tsa, s);
                }
                coeffs(ea, sa, ta, tsa, caS[a], cbS[a], cdS[a]);
            }
            if (visco) {
                // tau_eps and the scaled tau_sigma with the coefficient constants, for the adjoint's chain rule
                h->check(cudaMemcpyAsync(mat(M_TAUP), dTe, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
                h->check(cudaMemcpyAsync(mat(M_TAUS), dTs, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
                h->vemc = vc;
            }
        }
        if (eq == WAVE_EQ_TMEM || eq == WAVE_EQ_EMEM || eq == WAVE_EQ_VISCOEMEM || (eq == WAVE_EQ_VISCOTMEM && !is3d)) {
            // the base parameters, for the adjoint's chain rule (adjoint.cu)
            h->check(cudaMemcpyAsync(mat(M_EPSR), dEr, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
            h->check(cudaMemcpyAsync(mat(M_SIG), dSig, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
            h->check(cudaMemcpyAsync(mat(M_MUR), dMr, n * sizeof(float), cudaMemcpyDeviceToDevice, s), "copy");
        }
        h->check(cudaGetLastError(), "model preparation");
        for (float* p : tmp) cudaFreeAsync(p, s);
        h->check(cudaStreamSynchronize(s), "model preparation");
        h->modelSet = true;
        h->graphDirty = true;
    })
    return WAVE_OK;
}

int wave_set_sources(wave_handle* h, int n, const int64_t* idx, const int* type, const float* signals, int mem)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_set_sources: null handle");
    if (n < 0 || (n > 0 && (!idx || !type || !signals))) return fail(h, WAVE_ERR_ARG, "wave_set_sources: invalid arguments");
    for (int i = 0; i < n; ++i) {
        if (idx[i] < 0 || idx[i] >= h->N) return fail(h, WAVE_ERR_ARG, "wave_set_sources: source index outside the grid");
        if (!type_ok(h->cfg.equation, h->sp.is3d, type[i], true))
            return fail(h, WAVE_ERR_UNSUPPORTED, "wave_set_sources: source type " + std::to_string(type[i]) + " can not be implemented for this equation");
    }
    WAVE_TRY(h, {
        h->check(cudaStreamSynchronize(h->stream), "sync");
        h->nsrc = n;
        if (n > 0) {
            h->reuse(h->sidx, h->capSidx, n);
            h->reuse(h->stype, h->capStype, n);
            h->reuse(h->signals, h->capSignals, static_cast<size_t>(n) * h->NT);
            h->check(cudaMemcpy(h->sidx, idx, n * sizeof(long long), cudaMemcpyHostToDevice), "upload");
            h->check(cudaMemcpy(h->stype, type, n * sizeof(int), cudaMemcpyHostToDevice), "upload");
            h->check(cudaMemcpy(h->signals, signals, static_cast<size_t>(n) * h->NT * sizeof(float),
                                mem == WAVE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice), "upload");
        }
        h->sq.nsrc = n; h->sq.sidx = h->sidx; h->sq.stype = h->stype; h->sq.signals = h->signals;
        h->hSrcIdx.assign(idx, idx + n);
        h->hSrcType.assign(type, type + n);
        update_fusion(h);
        h->graphDirty = true;
    })
    return WAVE_OK;
}

int wave_set_receivers(wave_handle* h, int n, const int64_t* idx, const int* type)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_set_receivers: null handle");
    if (n < 0 || (n > 0 && (!idx || !type))) return fail(h, WAVE_ERR_ARG, "wave_set_receivers: invalid arguments");
    for (int i = 0; i < n; ++i) {
        if (idx[i] < 0 || idx[i] >= h->N) return fail(h, WAVE_ERR_ARG, "wave_set_receivers: receiver index outside the grid");
        if (!type_ok(h->cfg.equation, h->sp.is3d, type[i], false))
            return fail(h, WAVE_ERR_UNSUPPORTED, "wave_set_receivers: receiver type " + std::to_string(type[i]) + " can not be implemented for this equation");
    }
    WAVE_TRY(h, {
        h->check(cudaStreamSynchronize(h->stream), "sync");
        h->nrec = n;
        if (n > 0) {
            h->reuse(h->ridx, h->capRidx, n);
            h->reuse(h->rtype, h->capRtype, n);
            h->check(cudaMemcpy(h->ridx, idx, n * sizeof(long long), cudaMemcpyHostToDevice), "upload");
            h->check(cudaMemcpy(h->rtype, type, n * sizeof(int), cudaMemcpyHostToDevice), "upload");
        }
        h->reuse(h->seis, h->capSeis, static_cast<size_t>(n > 0 ? n : 1) * h->NT);
        h->check(cudaMemset(h->seis, 0, static_cast<size_t>(n > 0 ? n : 1) * h->NT * sizeof(float)), "memset");
        h->sq.nrec = n; h->sq.ridx = h->ridx; h->sq.rtype = h->rtype; h->sq.seis = h->seis;
        h->hRecIdx.assign(idx, idx + n);
        h->hRecType.assign(type, type + n);
        update_fusion(h);
        h->graphDirty = true;
    })
    return WAVE_OK;
}

int wave_solver_step(wave_handle* h, int t_begin, int t_end)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_solver_step: null handle");
    if (t_begin < 0 || t_end < t_begin || t_end > h->NT) return fail(h, WAVE_ERR_ARG, "wave_solver_step: time range outside [0, NT]");
    if (!h->modelSet) return fail(h, WAVE_ERR_STATE, "wave_solver_step: call wave_set_model first");
    if (!h->seis) return fail(h, WAVE_ERR_STATE, "wave_solver_step: call wave_set_receivers first");
    wave::TraceRange region("WAVE-Simulation.timeLoop");
    const char* stepName = wave::trace_timestep_name(h->cfg.dimension, h->cfg.equation);
    WAVE_TRY(h, {
        launch_set_counter(h->tcounter, t_begin, h->stream);
        h->launches += 1;
        int t = t_begin;
        if (h->timing) {
            std::vector<cudaEvent_t> ev;
            for (; t < t_end; ++t) {
                wave::TraceRange step(stepName);
                launch_step_timed(h, ev);
            }
            h->check(cudaGetLastError(), "step launch");
            h->check(cudaStreamSynchronize(h->stream), "step");
            for (size_t k = 0; k + 2 < ev.size(); k += 3) {
                float a = 0, b = 0;
                cudaEventElapsedTime(&a, ev[k], ev[k + 1]);
                cudaEventElapsedTime(&b, ev[k + 1], ev[k + 2]);
                h->velMsSum += a;
                h->strMsSum += b;
                h->timedSteps += 1;
            }
            for (auto e : ev) cudaEventDestroy(e);
        } else {
            // the step graph is captured at the first call after any change
            // (capture only: the host records the launches), so that a later
            // multi-step call replays it without a capture in its way
            if (h->graphDirty || !h->graph) build_graph(h);
            if (t_end - t >= kGraphSteps) {
                for (; t + kGraphSteps <= t_end; t += kGraphSteps) {
                    wave::TraceRange steps(stepName);   // kGraphSteps steps in one graph launch
                    h->check(cudaGraphLaunch(h->graph, h->stream), "graph launch");
                    h->launches += h->graphLaunchesPerStep * kGraphSteps;
                }
            }
            for (; t < t_end; ++t) {
                wave::TraceRange step(stepName);
                launch_step(h);
            }
            h->check(cudaGetLastError(), "step launch");
        }
        h->stepsSinceReset += t_end - t_begin;
    })
    return WAVE_OK;
}

int wave_solver_reset(wave_handle* h)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_solver_reset: null handle");
    WAVE_TRY(h, {
        for (int f : h->fields) h->check(cudaMemsetAsync(h->f[f], 0, h->N * sizeof(float), h->stream), "memset");
        for (int rr = 0; rr < R_COUNT; ++rr)
            for (int l = 0; l < kMaxL; ++l)
                if (h->r[rr][l]) h->check(cudaMemsetAsync(h->r[rr][l], 0, h->N * sizeof(float), h->stream), "memset");
        for (int s = 0; s < PS_COUNT; ++s)
            if (h->psi[s]) h->check(cudaMemsetAsync(h->psi[s], 0, h->psiLen[s] * sizeof(float), h->stream), "memset");
        if (h->seis) h->check(cudaMemsetAsync(h->seis, 0, static_cast<size_t>(h->nrec > 0 ? h->nrec : 1) * h->NT * sizeof(float), h->stream), "memset");
        h->check(cudaStreamSynchronize(h->stream), "reset");
        h->stepsSinceReset = 0;
    })
    return WAVE_OK;
}

// Reads and clears the device error word of the bounded waits.
static int device_error(wave_handle* h)
{
    int e = 0;
    if (!h->errWord) return 0;
    if (cudaMemcpy(&e, h->errWord, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return WAVE_ERR_CUDA;
    if (e) cudaMemset(h->errWord, 0, sizeof(int));
    return e;
}

int wave_get_seismograms(wave_handle* h, float* out, size_t count, int mem)
{
    if (!h || !out) return fail(h, WAVE_ERR_ARG, "wave_get_seismograms: null argument");
    if (count != static_cast<size_t>(h->nrec) * h->NT) return fail(h, WAVE_ERR_ARG, "wave_get_seismograms: count != n_receivers*NT");
    if (count == 0) return WAVE_OK;
    WAVE_TRY(h, {
        h->check(cudaMemcpyAsync(out, h->seis, count * sizeof(float), mem == WAVE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream), "seismogram copy");
        h->check(cudaStreamSynchronize(h->stream), "seismogram copy");
    })
    if (int e = device_error(h)) return fail(h, e, "a bounded device wait ran out during the time steps");
    return WAVE_OK;
}

int wave_check_finite(wave_handle* h)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_check_finite: null handle");
    int flag = 0;
    WAVE_TRY(h, {
        h->check(cudaMemsetAsync(h->flag, 0, sizeof(int), h->stream), "memset");
        for (int f : h->fields) launch_finite(h->f[f], h->N, h->flag, h->stream);
        if (h->seis && h->nrec > 0) launch_finite(h->seis, static_cast<long long>(h->nrec) * h->NT, h->flag, h->stream);
        h->check(cudaMemcpyAsync(&flag, h->flag, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "flag copy");
        h->check(cudaStreamSynchronize(h->stream), "finite check");
    })
    if (int e = device_error(h)) return fail(h, e, "a bounded device wait ran out during the time steps");
    if (flag) return fail(h, WAVE_ERR_NONFINITE, "Infinite or NaN value in seismogram or/and velocity wavefield!");
    return WAVE_OK;
}

int wave_get_state_size(wave_handle* h, size_t* bytes)
{
    if (!h || !bytes) return fail(h, WAVE_ERR_ARG, "wave_get_state_size: null argument");
    size_t b = 0;
    for (auto& p : state_parts(h)) b += p.second;
    *bytes = b;
    return WAVE_OK;
}

int wave_get_state(wave_handle* h, void* out, size_t bytes, int mem)
{
    size_t need = 0;
    if (!h || !out) return fail(h, WAVE_ERR_ARG, "wave_get_state: null argument");
    wave_get_state_size(h, &need);
    if (bytes != need) return fail(h, WAVE_ERR_ARG, "wave_get_state: wrong blob size");
    WAVE_TRY(h, {
        char* o = static_cast<char*>(out);
        for (auto& p : state_parts(h)) {
            h->check(cudaMemcpyAsync(o, p.first, p.second, mem == WAVE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream), "state copy");
            o += p.second;
        }
        h->check(cudaStreamSynchronize(h->stream), "state copy");
        h->stepsSinceReset = 1;   // a restored state is not the zero state
    })
    return WAVE_OK;
}

int wave_set_state(wave_handle* h, const void* in, size_t bytes, int mem)
{
    size_t need = 0;
    if (!h || !in) return fail(h, WAVE_ERR_ARG, "wave_set_state: null argument");
    wave_get_state_size(h, &need);
    if (bytes != need) return fail(h, WAVE_ERR_ARG, "wave_set_state: wrong blob size");
    WAVE_TRY(h, {
        const char* o = static_cast<const char*>(in);
        for (auto& p : state_parts(h)) {
            h->check(cudaMemcpyAsync(p.first, o, p.second, mem == WAVE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream), "state copy");
            o += p.second;
        }
        h->check(cudaStreamSynchronize(h->stream), "state copy");
        h->stepsSinceReset = 1;   // a restored state is not the zero state
    })
    return WAVE_OK;
}

int wave_get_nt(wave_handle* h, int* nt)
{
    if (!h || !nt) return fail(h, WAVE_ERR_ARG, "wave_get_nt: null argument");
    *nt = h->NT;
    return WAVE_OK;
}

int wave_device_bytes(wave_handle* h, int64_t* bytes)
{
    if (!h || !bytes) return fail(h, WAVE_ERR_ARG, "wave_device_bytes: null argument");
    size_t b = 0;
    for (size_t x : h->allocBytes) b += x;
    *bytes = static_cast<int64_t>(b);
    return WAVE_OK;
}

int wave_get_num_receivers(wave_handle* h, int* n)
{
    if (!h || !n) return fail(h, WAVE_ERR_ARG, "wave_get_num_receivers: null argument");
    *n = h->nrec;
    return WAVE_OK;
}

int wave_get_stream(wave_handle* h, void** stream)
{
    if (!h || !stream) return fail(h, WAVE_ERR_ARG, "wave_get_stream: null argument");
    *stream = h->stream;
    return WAVE_OK;
}

int wave_get_launch_count(wave_handle* h, long long* count)
{
    if (!h || !count) return fail(h, WAVE_ERR_ARG, "wave_get_launch_count: null argument");
    *count = h->launches;
    return WAVE_OK;
}

int wave_set_kernel_path(wave_handle* h, int path)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_set_kernel_path: null handle");
    if (path < 0 || path > 3) return fail(h, WAVE_ERR_ARG, "wave_set_kernel_path: path must be 0, 1, 2 or 3");
    h->kernelPath = path;
    h->graphDirty = true;
    WAVE_TRY(h, { update_fusion(h); })
    return WAVE_OK;
}

int wave_set_dependent_launch(wave_handle* h, int on)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_set_dependent_launch: null handle");
    h->dependentLaunch = on != 0;
    h->graphDirty = true;
    return WAVE_OK;
}

int wave_get_kernel_path(wave_handle* h, int* streamingActive)
{
    if (!h || !streamingActive) return fail(h, WAVE_ERR_ARG, "wave_get_kernel_path: null argument");
    const int k0 = pass_kernel(h, 0), k1 = pass_kernel(h, 1);
    *streamingActive = (k0 ? 1 : 0) | (k1 ? 2 : 0) | (k0 == 2 ? 4 : 0) | (k1 == 2 ? 8 : 0);
    return WAVE_OK;
}

int wave_set_timing(wave_handle* h, int on)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_set_timing: null handle");
    h->timing = on != 0;
    h->velMsSum = h->strMsSum = 0;
    h->timedSteps = 0;
    return WAVE_OK;
}

int wave_get_kernel_times(wave_handle* h, double* velocity_ms, double* stress_ms, long long* samples)
{
    if (!h) return fail(nullptr, WAVE_ERR_ARG, "wave_get_kernel_times: null handle");
    const double n = h->timedSteps > 0 ? static_cast<double>(h->timedSteps) : 1.0;
    if (velocity_ms) *velocity_ms = h->velMsSum / n;
    if (stress_ms) *stress_ms = h->strMsSum / n;
    if (samples) *samples = h->timedSteps;
    return WAVE_OK;
}

} // extern "C"
