// model_api.cu — model-preparation helpers exposed without a solver handle
// (the device side of Modelparameter::prepareForModelling, usable by FWI
// model updates between iterations).
#include <climits>
#include <mutex>
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

// ---------------------------------------------------------------------------
// Allocation-free variant of wave_average_shear_modulus.
//
// The inverse moduli that the harmonic average reads go to a fixed scratch
// array in device global memory instead of a cudaMalloc'd buffer, so the call
// allocates nothing. The scratch holds kNoAllocMaxPoints floats (16 MiB), which
// bounds the model size this entry point accepts.
constexpr long long kNoAllocMaxPoints = 1LL << 22;
static __device__ __align__(256) float g_invmu_scratch[kNoAllocMaxPoints];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
float* g_scratch_ptr[kMaxDevices] = {};

// One-time set-up per device (with that device current): the scratch array's
// device address. The address is cached for the life of the process, so this
// entry point must not be used on a device after cudaDeviceReset (the module
// is reloaded there and the array may move).
cudaError_t scratch_for_current_device(float** ptr)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_invmu_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = static_cast<float*>(p);
    }
    *ptr = g_scratch_ptr[dev];
    return cudaSuccess;
}

// Device memory of device `dev`, or managed memory. Called only when no CUDA
// error is pending (checked at entry), so clearing the query's own error for
// an unknown pointer drops nothing of the caller's.
bool on_device(const void* p, int dev)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}

} // namespace

extern "C" int wave_average_shear_modulus_noalloc(const float* mu, float* out, int64_t NX, int64_t NY, int64_t NZ, int mode,
                                                  void* stream)
{
    if (!mu || !out || NX < 1 || NY < 1 || NZ < 1 || mode < 0 || mode > 4 || NX > INT_MAX || NY > INT_MAX || NZ > INT_MAX) {
        set_global_error("wave_average_shear_modulus_noalloc: invalid argument");
        return WAVE_ERR_ARG;
    }
    const long long n = NX * NY * NZ;
    if (n > kNoAllocMaxPoints) {
        set_global_error("wave_average_shear_modulus_noalloc: NX*NY*NZ = " + std::to_string(n) + " exceeds the fixed scratch of " +
                         std::to_string(kNoAllocMaxPoints) + " points; use wave_average_shear_modulus");
        return WAVE_ERR_ARG;
    }
    // an error left pending by an earlier call would otherwise be reported (and cleared) as this call's
    cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) {
        set_global_error(std::string("wave_average_shear_modulus_noalloc: a CUDA error is pending from earlier work (") +
                         cudaGetErrorString(pending) + "); nothing was launched");
        return WAVE_ERR_CUDA;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || !on_device(mu, dev) || !on_device(out, dev)) {
        set_global_error("wave_average_shear_modulus_noalloc: mu and out must be device memory of the current device");
        return WAVE_ERR_ARG;
    }
    float* inv = nullptr;
    cudaError_t e = scratch_for_current_device(&inv);
    if (e == cudaSuccess) {
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        PrepParams G{static_cast<int>(NX), static_cast<int>(NY), static_cast<int>(NZ), n};
        k_inv_clamped(G, mu, inv, s);     // writes all n scratch values ...
        k_harmonic(G, inv, mode, out, s); // ... before any is read
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        set_global_error(std::string("wave_average_shear_modulus_noalloc: ") + cudaGetErrorString(e));
        return WAVE_ERR_CUDA;
    }
    return WAVE_OK;
}
