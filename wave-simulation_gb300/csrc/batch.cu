// batch.cu — many shots with uneven grids stepped together.
//
// Each shot is an ordinary solver handle (its own device state, model,
// sources, receivers, seismograms); the batch fuses the time step of all
// shots into one launch per pass over a work list of (shot, tile) entries,
// followed by one source/receiver block per shot. The launches are
// persistent: their blocks walk the work list with a grid stride. Multi-step
// calls replay a captured CUDA graph of kBatchGraphSteps steps. The
// shot-level parallelism of the reference (MPI shot domains,
// Simulation.cpp:116-121, 339-369) becomes one device-wide launch.
//
// Schedule autotuner: the tile shape (32 or 64 points along x, 8 to 64 rows)
// and the resident blocks per SM (1, 2, 4 or 8 persistent blocks per SM, or
// one block per tile) are chosen by timing every candidate on the batch
// itself (one untimed and two timed steps each) the first time an unstepped
// batch is stepped; the state is reset afterwards. The choice is cached per
// (equation, FD order, size bucket: log2 of the mean points per shot and of
// the shot count) for the life of the process, so later batches of the same
// kind start with it.
#include <algorithm>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "handle.h"
#include "trace.h"

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
    // schedule: tile cols x rows, persistent blocks per SM (0 = one block per tile)
    int cols = 32, rows = kTileRows, perSM = 0;
    int grid = 0;
    BatchSched sched{};
    bool forced = false;      // set by wave_batch_set_schedule
    bool tuned = false;       // autotuned (or taken from the cache) once
    int tuneSource = 0;       // 0 default, 1 timed here, 2 from the cache, 3 forced

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

// (equation, order, log2 mean points per shot, log2 shot count) -> (cols, rows, blocks per SM)
using TuneKey = std::tuple<int, int, int, int>;
std::mutex g_tune_mutex;
std::map<TuneKey, std::tuple<int, int, int>> g_tune_cache;

TuneKey tune_key(const wave_batch* b)
{
    double pts = 0;
    for (auto* h : b->shots) pts += static_cast<double>(h->N);
    const int n = static_cast<int>(b->shots.size());
    return TuneKey{b->eq, b->H, static_cast<int>(std::lround(std::log2(std::max(1.0, pts / n)))),
                   static_cast<int>(std::lround(std::log2(static_cast<double>(n))))};
}

// Builds and uploads the work list for the batch's current tile shape and sets the grid.
} // namespace

bool wave::batch_tile_interior(const StepParams& P, int x0, int r0, int cols, int rows)
{
    if (P.is3d || P.NZ != 1 || P.L != 0) return false;
    const int x1 = x0 + cols, y1 = r0 + rows;   // exclusive ends
    if (x1 > P.NX || y1 > P.NY) return false;
    // interior rows of an operator: c in [E, n - E) (the edge band E > H keeps every tap inside the axis)
    auto interior = [](const Op1D& o, int c0, int c1) { return !o.full && c0 >= o.E && c1 <= o.n - o.E; };
    if (!interior(P.Dxf, x0, x1) || !interior(P.Dxb, x0, x1) || !interior(P.Dyf, r0, y1) || !interior(P.Dyb, r0, y1))
        return false;
    // outside both CPML slabs of each axis (slab() of the kernels returns -1)
    auto noSlab = [](const Cpml1D& c, int c0, int c1) { return c.w <= 0 || (c.n > 2 * c.w && c0 >= c.w && c1 <= c.n - c.w); };
    if (P.useCpml && (!noSlab(P.cx, x0, x1) || !noSlab(P.cy, r0, y1))) return false;
    // outside the ABS frame (damping factor 1)
    if (P.abs && (x0 < P.absW || x1 > P.NX - P.absW || r0 < P.absW || y1 > P.NY - P.absW)) return false;
    return true;
}

namespace {

void build_tiles(wave_batch* b)
{
    const int n = static_cast<int>(b->shots.size());
    std::vector<BatchTile> tiles;
    // interior tiles of the lossless 2-D TMz passes are staged in shared memory
    const int smem = batch_tile_smem(b->eq, b->H, b->cols, b->rows);
    int interior = 0;
    for (int s = 0; s < n; ++s) {
        wave_handle* h = b->shots[s];
        const int rows = h->NY * h->NZ;
        for (int r0 = 0; r0 < rows; r0 += b->rows)
            for (int x0 = 0; x0 < h->NX; x0 += b->cols) {
                const bool in = smem > 0 && batch_tile_interior(h->sp, x0, r0, b->cols, b->rows);
                interior += in ? 1 : 0;
                tiles.push_back({s, x0, r0, in ? kTileInterior : 0});
            }
    }
    cudaFree(b->dTiles);
    b->dTiles = nullptr;
    ck(cudaMalloc(&b->dTiles, tiles.size() * sizeof(BatchTile)), "cudaMalloc");
    ck(cudaMemcpy(b->dTiles, tiles.data(), tiles.size() * sizeof(BatchTile), cudaMemcpyHostToDevice), "upload");
    b->ntiles = static_cast<int>(tiles.size());
    b->sched = BatchSched{b->ntiles, b->cols, b->rows, interior > 0 ? smem : 0};
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int resident = std::max(1, batch_blocks_per_sm(b->eq, b->H, b->sched.smem));
    const int per = b->perSM > 0 ? std::min(b->perSM, resident) : 0;
    b->grid = per > 0 ? std::min(b->ntiles, per * sms) : b->ntiles;
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
}

// Uploads the shots' step and source/receiver parameters and the work list.
void refresh(wave_batch* b)
{
    const int n = static_cast<int>(b->shots.size());
    std::vector<StepParams> P(n);
    std::vector<SrcRecParams> Q(n);
    for (int s = 0; s < n; ++s) {
        P[s] = b->shots[s]->sp;
        Q[s] = b->shots[s]->sq;
    }
    cudaFree(b->dP);
    cudaFree(b->dQ);
    b->dP = nullptr; b->dQ = nullptr;
    ck(cudaMalloc(&b->dP, n * sizeof(StepParams)), "cudaMalloc");
    ck(cudaMalloc(&b->dQ, n * sizeof(SrcRecParams)), "cudaMalloc");
    ck(cudaMemcpy(b->dP, P.data(), n * sizeof(StepParams), cudaMemcpyHostToDevice), "upload");
    ck(cudaMemcpy(b->dQ, Q.data(), n * sizeof(SrcRecParams), cudaMemcpyHostToDevice), "upload");
    build_tiles(b);
}

void launch_batch_step(wave_batch* b)
{
    launch_batch_pass(b->eq, 0, b->H, b->dP, b->dTiles, b->sched, b->grid, b->stream);
    launch_batch_pass(b->eq, 1, b->H, b->dP, b->dTiles, b->sched, b->grid, b->stream);
    const auto& p1 = b->pass1;
    launch_batch_aux(b->dP, b->dTiles, b->sched, b->grid, p1.size() > 0 ? p1[0] : -1, p1.size() > 1 ? p1[1] : -1,
                     p1.size() > 2 ? p1[2] : -1, b->dQ, b->counters, static_cast<int>(b->shots.size()), b->abs, b->stream);
    b->launches += b->abs ? 4 : 3;
}

// Zeroes every shot's wavefields, memory variables and CPML state.
void reset_shots(wave_batch* b)
{
    for (auto* h : b->shots) {
        const int rc = wave_solver_reset(h);
        if (rc != WAVE_OK) throw std::runtime_error(std::string("reset after tuning: ") + wave_last_error(h));
        ck(cudaStreamSynchronize(h->stream), "reset");
    }
}

// The schedule autotuner (see the file comment). Runs on an unstepped batch
// at its first step call; leaves the state reset and the schedule set.
void autotune(wave_batch* b)
{
    const TuneKey key = tune_key(b);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            std::tie(b->cols, b->rows, b->perSM) = it->second;
            build_tiles(b);
            b->tuned = true;
            b->tuneSource = 2;
            return;
        }
    }
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    float best = 1e30f;
    std::tuple<int, int, int> pick{b->cols, b->rows, b->perSM};
    const long long launches0 = b->launches;
    for (int cols : {32, 64})
        for (int rows : {8, 16, 32, 64})
            for (int per : {0, 1, 2, 4, 8}) {
                b->cols = cols;
                b->rows = rows;
                b->perSM = per;
                build_tiles(b);
                launch_set_counters(b->counters, static_cast<int>(b->shots.size()), 0, b->stream);
                launch_batch_step(b);
                ck(cudaEventRecord(e0, b->stream), "event");
                launch_batch_step(b);
                launch_batch_step(b);
                ck(cudaEventRecord(e1, b->stream), "event");
                ck(cudaEventSynchronize(e1), "tuning step");
                float ms = 0;
                ck(cudaEventElapsedTime(&ms, e0, e1), "event");
                if (ms < best) { best = ms; pick = std::make_tuple(cols, rows, per); }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->launches = launches0;
    std::tie(b->cols, b->rows, b->perSM) = pick;
    build_tiles(b);
    reset_shots(b);
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache[key] = pick;
    }
    b->tuned = true;
    b->tuneSource = 1;
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
    wave::TraceRange region("WAVE-Simulation.timeLoop");
    const char* stepName = wave::trace_timestep_name(b->shots[0]->cfg.dimension, b->shots[0]->cfg.equation);
    try {
        // the shots' own streams may still run their model preparation
        for (auto* h : b->shots) ck(cudaStreamSynchronize(h->stream), "shot sync");
        if (b->dirty) {
            refresh(b);
            if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
            b->dirty = false;
        }
        if (!b->tuned && !b->forced && t_begin == 0) {
            bool fresh = true;
            for (auto* h : b->shots) fresh = fresh && h->stepsSinceReset == 0;
            if (fresh) autotune(b);
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
                wave::TraceRange steps(stepName);   // kBatchGraphSteps steps of every shot
                ck(cudaGraphLaunch(b->graph, b->stream), "graph launch");
                b->launches += (b->abs ? 4 : 3) * kBatchGraphSteps;
            }
        }
        for (; t < t_end; ++t) {
            wave::TraceRange step(stepName);
            launch_batch_step(b);
        }
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
    wave::TraceRange region("adjoint.gradient");
    try {
        for (auto* h : b->shots) ck(cudaStreamSynchronize(h->stream), "shot sync");
        if (b->dirty) {
            refresh(b);
            if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
            b->dirty = false;
        }
        // the forward steps of the gradient run on the tuned schedule too (the
        // adjoint starts from a zero state, so tuning on it changes nothing)
        if (!b->tuned && !b->forced) autotune(b);
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
        S.cols = b->cols;   // the tuned schedule
        S.rows = b->rows;
        S.blocks = b->grid < b->ntiles ? b->grid : 0;
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

int wave_batch_set_schedule(wave_batch* b, int tile_cols, int tile_rows, int blocks_per_sm)
{
    if (!b) return bfail(nullptr, WAVE_ERR_ARG, "wave_batch_set_schedule: null batch");
    if (tile_cols == 0 && tile_rows == 0) {   // back to the autotuner
        b->forced = false;
        b->tuned = false;
        return WAVE_OK;
    }
    if (tile_cols < 32 || tile_cols % 32 != 0 || tile_cols > 1024 || tile_rows < 8 || tile_rows % 8 != 0 || tile_rows > 1024 ||
        blocks_per_sm < 0 || blocks_per_sm > 64)
        return bfail(b, WAVE_ERR_ARG, "wave_batch_set_schedule: tile columns a multiple of 32, rows a multiple of 8 (up to 1024), "
                                      "0..64 blocks per SM");
    try {
        b->cols = tile_cols;
        b->rows = tile_rows;
        b->perSM = blocks_per_sm;
        b->forced = true;
        b->tuned = true;
        b->tuneSource = 3;
        if (!b->dirty) build_tiles(b);
    } catch (std::exception& e) {
        return bfail(b, WAVE_ERR_CUDA, e.what());
    }
    return WAVE_OK;
}

int wave_batch_get_schedule(wave_batch* b, int* tile_cols, int* tile_rows, int* blocks_per_sm, int* source)
{
    if (!b || !tile_cols || !tile_rows || !blocks_per_sm) return bfail(b, WAVE_ERR_ARG, "wave_batch_get_schedule: null argument");
    *tile_cols = b->cols;
    *tile_rows = b->rows;
    *blocks_per_sm = b->perSM;
    if (source) *source = b->tuneSource;
    return WAVE_OK;
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
