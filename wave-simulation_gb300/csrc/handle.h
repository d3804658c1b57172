// handle.h — the solver handle behind wave_handle* (solver.cu, batch.cu).
#pragma once

#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "el3d.h"
#include "vargrid.h"
#include "wave_internal.h"

using wave::StepParams;
using wave::SrcRecParams;
using wave::El3dPlan;
using wave::F_COUNT;
using wave::R_COUNT;
using wave::PS_COUNT;
using wave::M_COUNT;
using wave::kMaxL;

struct wave_handle {
    wave_config cfg{};
    int NT = 0, NX = 1, NY = 1, NZ = 1, H = 1, L = 0;
    long long N = 0;
    bool is3d() const { return cfg.dimension == 3; }
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;

    std::vector<void*> allocs;
    std::vector<size_t> allocBytes;   // the size of each entry of allocs
    float* f[F_COUNT] = {};
    float* r[R_COUNT][kMaxL] = {};
    float* psi[PS_COUNT] = {};
    long long psiLen[PS_COUNT] = {};
    float* m[M_COUNT] = {};
    float* opTab[8] = {};
    float* cpmlProf[3][4] = {};
    float* absCoeff = nullptr;
    int* tcounter = nullptr;
    int* flag = nullptr;

    long long* sidx = nullptr; int* stype = nullptr; float* signals = nullptr; int nsrc = 0;
    long long* ridx = nullptr; int* rtype = nullptr; float* seis = nullptr; int nrec = 0;
    // host copies of the acquisition and the point map of the fused acoustic
    // source/receiver step (solver.cu update_fusion)
    std::vector<long long> hSrcIdx, hRecIdx;
    std::vector<int> hSrcType, hRecType;
    int* srMap = nullptr;
    int* srList[4] = {};               // point records: first source, first receiver; source and receiver chains
    size_t srListCap[4] = {};
    size_t capSidx = 0, capStype = 0, capSignals = 0, capRidx = 0, capRtype = 0, capSeis = 0;

    StepParams sp{};
    SrcRecParams sq{};
    wave::ViscoEmCoef vemc{};          // visco-EM coefficient constants of the last model (the adjoint's chain rule)
    dim3 grid, block;
    bool modelSet = false;
    std::vector<int> fields;          // allocated field slots
    std::vector<int> pass1Fields;     // fields updated in pass 1 (ABS after pass 2)

    cudaGraphExec_t graph = nullptr;
    bool graphDirty = true;
    long long graphLaunchesPerStep = 0;   // kernels in one captured step

    // streaming 3-D elastic paths (kernels_el3d.cu: one point per thread;
    // kernels_el3d_pairs.cu: two x-adjacent points per thread)
    El3dPlan el3d, el3dp;
    // variable-grid operators (vargrid.cu); null on a regular grid
    std::shared_ptr<wave::VarGridDev> vg;
    // wavefield decomposition after every step (decompose.cu): 0 off, 1 up/down, 2 left/right
    int decompType = 0;
    float* decOld[3] = {};     // P, VX, VY before the step
    float* decS2[3] = {};      // Poynting estimates per field
    float* decOut[6] = {};     // P.up/left, P.down/right, VX.., VY..
    unsigned* decMax = nullptr;
    int kernelPath = 0;          // 0 automatic, 1 generic only, 2 one-point streaming, 3 pair streaming (where available)
    int passStreaming[2] = {0, 0};   // automatic path: timed choice per pass (0 generic, 1 one-point, 2 pair streaming)
    bool dependentLaunch = true;     // generic kernels launched with programmatic stream serialization
    long long stepsSinceReset = 0;   // steps run since creation or the last reset
    int* errWord = nullptr;      // device error word of the bounded waits

    bool timing = false;
    double velMsSum = 0, strMsSum = 0;
    long long timedSteps = 0;
    long long launches = 0;

    ~wave_handle()
    {
        if (graph) cudaGraphExecDestroy(graph);
        for (void* p : allocs) cudaFree(p);
        if (stream) cudaStreamDestroy(stream);
    }

    template <class T>
    T* alloc(size_t count)
    {
        void* p = nullptr;
        const size_t bytes = count * sizeof(T) > 0 ? count * sizeof(T) : 16;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) throw std::runtime_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        allocs.push_back(p);
        allocBytes.push_back(bytes);
        return static_cast<T*>(p);
    }
    // A device buffer of at least `need` elements in slot p (capacity cap):
    // kept when it is large enough, else freed and replaced, so repeated
    // calls (one per shot) do not accumulate allocations.
    template <class T>
    T* reuse(T*& p, size_t& cap, size_t need)
    {
        if (p && cap >= need) return p;
        if (p) {
            for (size_t k = 0; k < allocs.size(); ++k)
                if (allocs[k] == static_cast<void*>(p)) {
                    allocs.erase(allocs.begin() + k);
                    allocBytes.erase(allocBytes.begin() + k);
                    break;
                }
            cudaFree(p);
        }
        p = alloc<T>(need > 0 ? need : 1);
        cap = need > 0 ? need : 1;
        return p;
    }
    void check(cudaError_t e, const char* what)
    {
        if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }
};


namespace wave {
// one forward time step of a handle on its stream (solver.cu)
void step_once(wave_handle* h);
// the visco modulus relaxation sum of a configuration (solver.cu)
float visco_modulus_sum(const wave_config& c, int L);

// variable grid (vargrid.cu): upload of the host-built operators, model
// preparation, and the launches of one step (returns the kernel count;
// mid, if given, is recorded between the velocity and pressure halves)
void vargrid_setup(wave_handle* h, const VarGridHost& G);
// vs: the S-wave velocity of the 2-D elastic step (null for the acoustic step)
void vargrid_set_model(wave_handle* h, const float* rho, const float* vp, const float* vs);
int vargrid_launch_step(wave_handle* h, bool dep, cudaEvent_t* mid, bool* srcrecDone);
// the adjoint gradient of an acoustic or 2-D elastic variable-grid handle:
// forward with a checkpoint every K steps, residuals of dobs (device, nrec x
// NT), backward sweep; gvp, gvs, grho (device, N) receive dJ/dvp, dJ/dvs
// (zero for the acoustic step), dJ/drho
void vargrid_adjoint(wave_handle* h, const float* dobs, int K, double* misfit, float* gvp, float* gvs, float* grho);

// wavefield decomposition (decompose.cu): the copy of the fields before a
// step, and the two kernels after it (returns the kernel count)
void decompose_before_step(wave_handle* h);
int decompose_after_step(wave_handle* h);

// the adjoint gradient driver (adjoint.cu), shared by the single-handle and
// the batched entry points
struct AdjStepper {
    cudaStream_t stream;
    std::function<void(int)> set_counter;   // every shot's step counter to n
    std::function<void()> step;             // one forward step of every shot
    int cols = 32, rows = kTileRows;        // tile shape of the adjoint launches (points)
    int blocks = 0;                         // persistent blocks per launch (0: one per tile)
};
std::string adjoint_supported(const wave_handle* h);
void adjoint_run(const std::vector<wave_handle*>& shots, const AdjStepper& S, const float* const* dobs, int K, double* misfit,
                 float* const* gvp, float* const* gvs, float* const* grho, bool sum);
} // namespace wave
