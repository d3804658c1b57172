// model_api.cu — model-preparation helpers exposed without a solver handle
// (the device side of Modelparameter::prepareForModelling, usable by FWI
// model updates between iterations).
#include <string>

#include <cuda_runtime.h>

#include "wave_internal.h"

namespace wave {
void set_global_error(const std::string& msg);
}

using namespace wave;

extern "C" int wave_average_shear_modulus(const float* mu, float* out, int64_t NX, int64_t NY, int64_t NZ, int mode, int mem)
{
    if (!mu || !out || NX < 1 || NY < 1 || NZ < 1 || mode < 0 || mode > 4) {
        set_global_error("wave_average_shear_modulus: invalid argument");
        return WAVE_ERR_ARG;
    }
    const long long n = NX * NY * NZ;
    PrepParams G{static_cast<int>(NX), static_cast<int>(NY), static_cast<int>(NZ), n};
    float *dMu = nullptr, *dOut = nullptr, *inv = nullptr;
    auto cleanup = [&]() {
        if (mem != WAVE_MEM_DEVICE) { cudaFree(dMu); cudaFree(dOut); }
        cudaFree(inv);
    };
    cudaError_t e = cudaSuccess;
    if (mem == WAVE_MEM_DEVICE) {
        dMu = const_cast<float*>(mu);
        dOut = out;
    } else {
        if ((e = cudaMalloc(&dMu, n * sizeof(float))) == cudaSuccess) e = cudaMalloc(&dOut, n * sizeof(float));
        if (e == cudaSuccess) e = cudaMemcpy(dMu, mu, n * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMalloc(&inv, n * sizeof(float));   // scratch: the inverse moduli
    if (e == cudaSuccess) {
        k_inv_clamped(G, dMu, inv, 0);
        k_harmonic(G, inv, mode, dOut, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess && mem != WAVE_MEM_DEVICE) e = cudaMemcpy(out, dOut, n * sizeof(float), cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) {
        set_global_error(std::string("wave_average_shear_modulus: ") + cudaGetErrorString(e));
        return WAVE_ERR_CUDA;
    }
    return WAVE_OK;
}
