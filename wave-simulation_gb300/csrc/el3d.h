// el3d.h — host interface of the streaming 3-D elastic kernels (kernels_el3d.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include "wave_internal.h"

namespace wave {

struct El3dMaps {
    CUtensorMap hSxx, hSxy, hSxz, hSyz, hSzz, hVx, hVy, hVz;           // halo boxes
    CUtensorMap cSxx, cSyy, cSzz, cSxy, cSxz, cSyz, cVx, cVy, cVz, cM;  // centre boxes
    CUtensorMap pRho, pMu, pTauS;                                       // (x,z)+1 boxes (tau_S: visco-elastic)
    CUtensorMap psV[9], psS[9];   // CPML memory variables of the velocity / stress pass (x-, y-, z-type, three each)
};

struct El3dSched {
    int ntx, ntz;   // column tiles along x and z
    int* err;       // device error word (WAVE_ERR_TIMEOUT when a bounded wait runs out)
};

struct El3dPlan {
    El3dMaps maps;
    El3dSched sched;
    int H = 0;
    int grid = 0;
    bool ready = false;
    // the visco-elastic stress kernel (two-point kernels only): its own grid
    // (its stage is larger), 0 when it does not apply
    int gridVisco = 0;
};

// Builds the tensor maps for the current field/material pointers; false when
// the streaming path does not apply (the generic kernels run instead).
bool el3d_prepare(El3dPlan& plan, const StepParams& P, const float* rho, const float* M, const float* mu, int H, int* errWord);
// pass 0 = velocity, 1 = stress
cudaError_t el3d_launch(const El3dPlan& plan, const StepParams& P, int pass, cudaStream_t s);
// the same for the two-points-per-thread kernels (kernels_el3d_pairs.cu)
bool el3d_prepare_pairs(El3dPlan& plan, const StepParams& P, const float* rho, const float* M, const float* mu, int H, int* errWord,
                        const float* tauS = nullptr);
cudaError_t el3d_launch_pairs(const El3dPlan& plan, const StepParams& P, int pass, cudaStream_t s);

} // namespace wave
