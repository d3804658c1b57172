// batch.cu — many shots with uneven grids stepped together.
//
// Each shot is an ordinary solver handle (its own device state, model,
// sources, receivers, seismograms); the batch fuses the time step of all
// shots into one launch per pass over a work list of (shot, 32x8 tile)
// blocks, followed by one source/receiver block per shot. Multi-step calls
// replay a captured CUDA graph of kGraphSteps steps. The shot-level parallelism
// of the reference (MPI shot domains, Simulation.cpp:116-121, 339-369) becomes
// one device-wide launch.
#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "handle.h"

using namespace wave;

struct wave_batch {
    std::vector<wave_handle*> shots;
    cudaStream_t stream = nullptr;
    std::string err;
    StepParams* dP = nullptr;
    SrcRecParams* dQ = nullptr;
    BatchTile* dTiles = nullptr;
    int ntiles = 0;
    int* counters = nullptr;
    int eq = 0, H = 1, NT = 0;
    bool abs = false;
    std::vector<int> pass1;
    cudaGraphExec_t graph = nullptr;
    bool dirty = true;
    long long launches = 0;

    ~wave_batch()
    {
        if (graph) cudaGraphExecDestroy(graph);
        cudaFree(dP);
        cudaFree(dQ);
        cudaFree(dTiles);
        cudaFree(counters);
        for (auto* h : shots) wave_solver_destroy(h);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

constexpr int kBatchGraphSteps = 16;
thread_local std::string g_batch_err;

int bfail(wave_batch* b, int code, const std::string& m)
{
    if (b) b->err = m;
    else g_batch_err = m;
    return code;
}

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// Uploads the shots' step and source/receiver parameters and the tile list.
void refresh(wave_batch* b)
{
    const int n = static_cast<int>(b->shots.size());
    std::vector<StepParams> P(n);
    std::vector<SrcRecParams> Q(n);
    std::vector<BatchTile> tiles;
    for (int s = 0; s < n; ++s) {
        wave_handle* h = b->shots[s];
        P[s] = h->sp;
        Q[s] = h->sq;
        const int rows = h->NY * h->NZ;
        for (int r0 = 0; r0 < rows; r0 += kTileRows)
            for (int x0 = 0; x0 < h->NX; x0 += 32) tiles.push_back({s, x0, r0, 0});
    }
    cudaFree(b->dP);
    cudaFree(b->dQ);
    cudaFree(b->dTiles);
    b->dP = nullptr; b->dQ = nullptr; b->dTiles = nullptr;
    ck(cudaMalloc(&b->dP, n * sizeof(StepParams)), "cudaMalloc");
    ck(cudaMalloc(&b->dQ, n * sizeof(SrcRecParams)), "cudaMalloc");
    ck(cudaMalloc(&b->dTiles, tiles.size() * sizeof(BatchTile)), "cudaMalloc");
    ck(cudaMemcpy(b->dP, P.data(), n * sizeof(StepParams), cudaMemcpyHostToDevice), "upload");
    ck(cudaMemcpy(b->dQ, Q.data(), n * sizeof(SrcRecParams), cudaMemcpyHostToDevice), "upload");
    ck(cudaMemcpy(b->dTiles, tiles.data(), tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice), "upload");
    b->ntiles = static_cast<int>(tiles.size());
}

void launch_batch_step(wave_batch* b)
{
    launch_batch_pass(b->eq, 0, b->H, b->dP, b->dTiles, b->ntiles, b->stream);
    launch_batch_pass(b->eq, 1, b->H, b->dP, b->dTiles, b->ntiles, b->stream);
    const auto& p1 = b->pass1;
    launch_batch_aux(b->dP, b->dTiles, b->ntiles, p1.size() > 0 ? p1[0] : -1, p1.size() > 1 ? p1[1] : -1,
                     p1.size() > 2 ? p1[2] : -1, b->dQ, b->counters, static_cast<int>(b->shots.size()), b->abs, b->stream);
    b->launches += b->abs ? 4 : 3;
}

} // namespace

extern "C" {

const char* wave_batch_last_error(const wave_batch* b) { return b ? b->err.c_str() : g_batch_err.c_str(); }

int wave_batch_create(const wave_config* cfgs, int nshots, wave_batch** out)
{
    if (!cfgs || !out || nshots < 1) return bfail(nullptr, WAVE_ERR_ARG, "wave_batch_create: invalid arguments");
    *out = nullptr;
    for (int s = 1; s < nshots; ++s) {
        const wave_config &a = cfgs[0], &c = cfgs[s];
        if (c.useVariableGrid || c.useVariableFDoperators)
            return bfail(nullptr, WAVE_ERR_UNSUPPORTED, "wave_batch_create: the batched launches run on regular grids only");
        if (c.dimension != a.dimension || c.equation != a.equation || c.spatialFDorder != a.spatialFDorder ||
            c.DT != a.DT || c.T != a.T || c.DampingBoundary != a.DampingBoundary || c.FreeSurface != a.FreeSurface ||
            c.numRelaxationMechanisms != a.numRelaxationMechanisms)
            return bfail(nullptr, WAVE_ERR_ARG, "wave_batch_create: shots must share dimension, equation, order, DT, T, boundary type, free surface and relaxation mechanisms");
    }
    auto b = std::make_unique<wave_batch>();
    for (int s = 0; s < nshots; ++s) {
        wave_handle* h = nullptr;
        int rc = wave_solver_create(&cfgs[s], &h);
        if (rc != WAVE_OK) return bfail(nullptr, rc, std::string("shot ") + std::to_string(s) + ": " + wave_last_error(nullptr));
        h->kernelPath = 1;     // batched launches use the generic kernel bodies
        b->shots.push_back(h);
    }
    try {
        ck(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        ck(cudaMalloc(&b->counters, nshots * sizeof(int)), "cudaMalloc");
        wave_handle* h0 = b->shots[0];
        b->eq = kernel_eq(h0->cfg.equation, h0->cfg.dimension == 3);
        b->H = h0->H;
        b->NT = h0->NT;
        b->abs = h0->sp.abs != 0;
        b->pass1 = h0->pass1Fields;
    } catch (std::exception& e) {
        return bfail(nullptr, WAVE_ERR_CUDA, e.what());
    }
    *out = b.release();
    return WAVE_OK;
}

int wave_batch_destroy(wave_batch* b)
{
    if (!b) return bfail(nullptr, WAVE_ERR_ARG, "wave_batch_destroy: null batch");
    cudaStreamSynchronize(b->stream);
    delete b;
    return WAVE_OK;
}

int wave_batch_shot(wave_batch* b, int shot, wave_handle** h)
{
    if (!b || !h || shot < 0 || shot >= static_cast<int>(b->shots.size())) return bfail(b, WAVE_ERR_ARG, "wave_batch_shot: invalid shot");
    *h = b->shots[shot];
    b->dirty = true;   // the caller may change the shot's model or acquisition
    return WAVE_OK;
}

int wave_batch_step(wave_batch* b, int t_begin, int t_end)
{
    if (!b) return bfail(nullptr, WAVE_ERR_ARG, "wave_batch_step: null batch");
    if (t_begin < 0 || t_end < t_begin || t_end > b->NT) return bfail(b, WAVE_ERR_ARG, "wave_batch_step: time range outside [0, NT]");
    for (size_t s = 0; s < b->shots.size(); ++s) {
        if (!b->shots[s]->modelSet) return bfail(b, WAVE_ERR_STATE, "wave_batch_step: shot " + std::to_string(s) + " has no model");
        if (!b->shots[s]->seis) return bfail(b, WAVE_ERR_STATE, "wave_batch_step: shot " + std::to_string(s) + " has no receivers");
    }
    try {
        // the shots' own streams may still run their model preparation
        for (auto* h : b->shots) ck(cudaStreamSynchronize(h->stream), "shot sync");
        if (b->dirty) {
            refresh(b);
            if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
            b->dirty = false;
        }
        launch_set_counters(b->counters, static_cast<int>(b->shots.size()), t_begin, b->stream);
        int t = t_begin;
        if (t_end - t >= kBatchGraphSteps) {
            if (!b->graph) {
                cudaGraph_t g;
                ck(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
                const long long before = b->launches;
                for (int k = 0; k < kBatchGraphSteps; ++k) launch_batch_step(b);
                b->launches = before;
                ck(cudaStreamEndCapture(b->stream, &g), "end capture");
                ck(cudaGraphInstantiate(&b->graph, g, 0), "graph instantiate");
                cudaGraphDestroy(g);
            }
            for (; t + kBatchGraphSteps <= t_end; t += kBatchGraphSteps) {
                ck(cudaGraphLaunch(b->graph, b->stream), "graph launch");
                b->launches += (b->abs ? 4 : 3) * kBatchGraphSteps;
            }
        }
        for (; t < t_end; ++t) launch_batch_step(b);
        ck(cudaGetLastError(), "batch step");
        // the shots' seismogram reads synchronise their own streams: order them after this batch
        ck(cudaStreamSynchronize(b->stream), "batch step");
    } catch (std::exception& e) {
        return bfail(b, WAVE_ERR_CUDA, e.what());
    }
    return WAVE_OK;
}

int wave_batch_adjoint_gradient(wave_batch* b, const float* const* dobs, int dobs_mem, int checkpoint_every, double* misfits,
                                float* const* grad_vp, float* const* grad_vs, float* const* grad_rho, int grad_mem, int sum_shots)
{
    if (!b) return bfail(nullptr, WAVE_ERR_ARG, "wave_batch_adjoint_gradient: null batch");
    const int ns = static_cast<int>(b->shots.size());
    if (!dobs || !misfits || !grad_vp || !grad_vs || !grad_rho || checkpoint_every < 1)
        return bfail(b, WAVE_ERR_ARG, "wave_batch_adjoint_gradient: invalid argument");
    for (int s = 0; s < ns; ++s) {
        const std::string why = adjoint_supported(b->shots[s]);
        if (!why.empty()) return bfail(b, WAVE_ERR_UNSUPPORTED, "wave_batch_adjoint_gradient: shot " + std::to_string(s) + ": " + why);
        if (!dobs[s]) return bfail(b, WAVE_ERR_ARG, "wave_batch_adjoint_gradient: missing observed data");
        if (sum_shots && b->shots[s]->N != b->shots[0]->N)
            return bfail(b, WAVE_ERR_ARG, "wave_batch_adjoint_gradient: summed gradients need shots of one grid");
    }
    std::vector<void*> tmp;
    auto dev = [&](size_t n) {
        void* p = nullptr;
        ck(cudaMalloc(&p, n * sizeof(float)), "cudaMalloc");
        tmp.push_back(p);
        return static_cast<float*>(p);
    };
    int rc = WAVE_OK;
    try {
        for (auto* h : b->shots) ck(cudaStreamSynchronize(h->stream), "shot sync");
        if (b->dirty) {
            refresh(b);
            if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
            b->dirty = false;
        }
        std::vector<const float*> dD(ns);
        for (int s = 0; s < ns; ++s) {
            const size_t nd = static_cast<size_t>(b->shots[s]->nrec) * b->NT;
            if (dobs_mem == WAVE_MEM_DEVICE) dD[s] = dobs[s];
            else {
                float* d = dev(nd);
                ck(cudaMemcpy(d, dobs[s], nd * sizeof(float), cudaMemcpyHostToDevice), "dobs upload");
                dD[s] = d;
            }
        }
        const int nout = sum_shots ? 1 : ns;
        std::vector<float*> g[3];
        float* const* outs[3] = {grad_vp, grad_vs, grad_rho};
        for (int k = 0; k < 3; ++k)
            for (int s = 0; s < nout; ++s) g[k].push_back(grad_mem == WAVE_MEM_DEVICE ? outs[k][s] : dev(b->shots[s]->N));
        AdjStepper S;
        S.stream = b->stream;
        S.set_counter = [b, ns](int n) { launch_set_counters(b->counters, ns, n, b->stream); };
        S.step = [b]() { launch_batch_step(b); };
        adjoint_run(b->shots, S, dD.data(), checkpoint_every, misfits, g[0].data(), g[1].data(), g[2].data(), sum_shots != 0);
        if (grad_mem != WAVE_MEM_DEVICE)
            for (int k = 0; k < 3; ++k)
                for (int s = 0; s < nout; ++s)
                    ck(cudaMemcpy(outs[k][s], g[k][s], b->shots[s]->N * sizeof(float), cudaMemcpyDeviceToHost), "gradient copy");
    } catch (std::exception& e) {
        rc = bfail(b, WAVE_ERR_CUDA, e.what());
    }
    for (void* p : tmp) cudaFree(p);
    return rc;
}

int wave_batch_get_stream(wave_batch* b, void** stream)
{
    if (!b || !stream) return bfail(b, WAVE_ERR_ARG, "wave_batch_get_stream: null argument");
    *stream = b->stream;
    return WAVE_OK;
}

int wave_batch_get_launch_count(wave_batch* b, long long* count)
{
    if (!b || !count) return bfail(b, WAVE_ERR_ARG, "wave_batch_get_launch_count: null argument");
    *count = b->launches;
    return WAVE_OK;
}

} // extern "C"
