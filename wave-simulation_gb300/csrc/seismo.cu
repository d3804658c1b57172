// seismo.cu — the seismogram output path on the device: per-trace
// normalisation (Seismogram::normalizeTrace, Seismogram.cpp:215-240; AGC,
// Seismogram::calcInverseAGC, :323-387) and
// resampling to seismoDT (Seismogram::setSeismoDT + Common::calcResampleMat,
// Seismogram.cpp:610-618, Common.hpp:202-230; applied as data * resampleMat
// when a seismogram is written, Seismogram.cpp:109).
#include <cmath>
#include <string>

#include <cuda_runtime.h>

#include "wave_internal.h"

namespace wave {
void set_global_error(const std::string& msg);
cudaError_t envelope_device(float* d, long long ntr, long long nt, int mode);   // snapshot.cu
}

using namespace wave;

namespace {

// linear interpolation at k * coeff (coeff = seismoDT / DT in FP32): weight
// 1 - frac on sample floor(k coeff), frac on the next one, each only inside
// the trace
__global__ void resample_kernel(const float* __restrict__ in, long long ntr, long long nt, float coeff, long long ntOut,
                                float* __restrict__ out)
{
    const long long total = ntr * ntOut;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const long long tr = q / ntOut, k = q - tr * ntOut;
        const float rel = static_cast<float>(k) * coeff;
        const float fl = floorf(rel);
        const long long c0 = static_cast<long long>(fl);
        const float w1 = fmodf(rel, 1.0f);
        const float w0 = 1.0f - w1;
        const float* t = in + tr * nt;
        float s = 0.0f;
        if (c0 < nt) s += w0 * t[c0];
        if (c0 + 1 < nt) s += w1 * t[c0 + 1];
        out[q] = s;
    }
}

// one block per trace: max norm (mode 1) or l2 norm (mode >= 2); a zero norm divides by 1
__global__ void normalize_kernel(float* data, long long nt, int mode)
{
    __shared__ double part[32];
    float* t = data + blockIdx.x * nt;
    double acc = 0.0;
    for (long long k = threadIdx.x; k < nt; k += blockDim.x) {
        const double v = t[k];
        acc = mode == 1 ? fmax(acc, fabs(v)) : acc + v * v;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double w = __shfl_down_sync(0xffffffffu, acc, o);
        acc = mode == 1 ? fmax(acc, w) : acc + w;
    }
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = mode == 1 ? fmax(r, part[w]) : r + part[w];
        part[0] = mode == 1 ? r : sqrt(r);
    }
    __syncthreads();
    float norm = static_cast<float>(part[0]);
    if (norm == 0.0f) norm = 1.0f;
    for (long long k = threadIdx.x; k < nt; k += blockDim.x) t[k] /= norm;
}

// Inverse AGC of one trace per thread (Seismogram::calcInverseAGC,
// Seismogram.cpp:323-387) over the l2-normalised traces nd: a water level of
// 1e-3 x (the trace's squared l2 norm / nt) (wl0 for a zero trace), then a
// running sum of squares over the window [t - nagc, t + nagc] taken from the
// last sample backwards (the window ramps in over the last nagc samples and
// out over the first nagc, each sample adding its water level), inv[t] =
// 1 / sqrt(sum / window) or 0. FP32 throughout, no contraction, in the
// reference's order.
__global__ void agc_kernel(const float* __restrict__ nd, long long ntr, long long nt, long long nagc, float wl0,
                           float* __restrict__ inv)
{
    const long long tr = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tr >= ntr) return;
    const float* row = nd + tr * nt;
    float* out = inv + tr * nt;
    float ss = 0.0f;
    for (long long t = 0; t < nt; ++t) ss = __fadd_rn(ss, __fmul_rn(row[t], row[t]));
    const float l2 = sqrtf(ss);
    float wl = __fdiv_rn(__fmul_rn(l2, l2), static_cast<float>(nt));
    wl = wl != 0.0f ? static_cast<float>(static_cast<double>(wl) * 1e-3) : wl0;
    float sum = 0.0f, win = static_cast<float>(nagc);
    for (long long t = nt - nagc; t < nt; ++t) {
        sum = __fadd_rn(sum, __fmul_rn(row[t], row[t]));
        sum = __fadd_rn(sum, wl);
    }
    for (long long t = nt - 1; t >= 0; --t) {
        if (t >= nt - nagc) {
            const float v = row[t - nagc];
            sum = __fadd_rn(sum, __fmul_rn(v, v));
            sum = __fadd_rn(sum, wl);
            win = __fadd_rn(win, 1.0f);
        } else if (t >= nagc) {
            const float a = row[t - nagc], b = row[t + nagc];
            sum = __fadd_rn(sum, __fmul_rn(a, a));
            sum = __fsub_rn(sum, __fmul_rn(b, b));
        } else {
            const float b = row[t + nagc];
            sum = __fsub_rn(sum, __fmul_rn(b, b));
            sum = __fsub_rn(sum, wl);
            win = __fsub_rn(win, 1.0f);
        }
        float r = __fdiv_rn(sum, win);
        r = r > 0.0f ? __fdiv_rn(1.0f, sqrtf(r)) : 0.0f;
        out[t] = r;
    }
}

__global__ void mul_kernel(float* __restrict__ a, const float* __restrict__ b, long long n)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        a[q] = __fmul_rn(a[q], b[q]);
}

__global__ void sumsq_kernel(const float* __restrict__ a, long long n, double* out)
{
    double acc = 0.0;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        acc += static_cast<double>(a[q]) * a[q];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

int err(int code, const std::string& m)
{
    set_global_error(m);
    return code;
}

} // namespace

extern "C" int wave_resample_traces(const float* in, int64_t ntr, int64_t nt, double dt, double seismo_dt, float* out,
                                    int64_t* nt_out, int mem)
{
    if (!nt_out || ntr < 0 || nt < 1 || dt <= 0 || seismo_dt < 0) return err(WAVE_ERR_ARG, "wave_resample_traces: invalid argument");
    const float coeff = seismo_dt > 0 ? static_cast<float>(seismo_dt) / static_cast<float>(dt) : 1.0f;
    if (!(coeff > 0.0f)) return err(WAVE_ERR_ARG, "wave_resample_traces: invalid seismoDT");
    const long long ntNew = static_cast<long long>(std::floor(static_cast<float>(nt - 1) / coeff)) + 1;
    *nt_out = ntNew;
    if (!out || ntr == 0) return WAVE_OK;
    if (!in) return err(WAVE_ERR_ARG, "wave_resample_traces: null input");
    const float* dIn = in;
    float* dOut = out;
    float *tIn = nullptr, *tOut = nullptr;
    cudaError_t e = cudaSuccess;
    if (mem != WAVE_MEM_DEVICE) {
        e = cudaMalloc(&tIn, ntr * nt * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc(&tOut, ntr * ntNew * sizeof(float));
        if (e == cudaSuccess) e = cudaMemcpy(tIn, in, ntr * nt * sizeof(float), cudaMemcpyHostToDevice);
        dIn = tIn;
        dOut = tOut;
    }
    if (e == cudaSuccess) {
        resample_kernel<<<1216, 256>>>(dIn, ntr, nt, coeff, ntNew, dOut);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess && mem != WAVE_MEM_DEVICE) e = cudaMemcpy(out, tOut, ntr * ntNew * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(tIn);
    cudaFree(tOut);
    if (e != cudaSuccess) return err(WAVE_ERR_CUDA, std::string("wave_resample_traces: ") + cudaGetErrorString(e));
    return WAVE_OK;
}

extern "C" int wave_normalize_traces(float* data, int64_t ntr, int64_t nt, int mode, int mem)
{
    if (!data || ntr < 0 || nt < 1 || mode < 0 || mode > 4 || mode == 3 || (mode == 4 && nt < 2))
        return err(WAVE_ERR_ARG, "wave_normalize_traces: invalid argument (mode 0, 1, 2 or 4)");
    if (mode == 0 || ntr == 0) return WAVE_OK;
    float* d = data;
    float* t = nullptr;
    cudaError_t e = cudaSuccess;
    if (mem != WAVE_MEM_DEVICE) {
        e = cudaMalloc(&t, ntr * nt * sizeof(float));
        if (e == cudaSuccess) e = cudaMemcpy(t, data, ntr * nt * sizeof(float), cudaMemcpyHostToDevice);
        d = t;
    }
    if (e == cudaSuccess) {
        normalize_kernel<<<static_cast<unsigned>(ntr), 256>>>(d, nt, mode == 1 ? 1 : 2);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    // mode 4: after the l2 normalisation, divide by the water-levelled envelope
    if (e == cudaSuccess && mode == 4) e = envelope_device(d, ntr, nt, 1);
    if (e == cudaSuccess && mem != WAVE_MEM_DEVICE) e = cudaMemcpy(data, t, ntr * nt * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(t);
    if (e != cudaSuccess) return err(WAVE_ERR_CUDA, std::string("wave_normalize_traces: ") + cudaGetErrorString(e));
    return WAVE_OK;
}

extern "C" int wave_agc_normalize_traces(float* data, int64_t ntr, int64_t nt, double dt, double f_agc, float* inverse_agc, int mem)
{
    if (!data || ntr < 0 || nt < 1 || !(dt > 0) || !(f_agc > 0)) return err(WAVE_ERR_ARG, "wave_agc_normalize_traces: invalid argument");
    if (ntr == 0) return WAVE_OK;
    // NAGC = round(1 / (f DT)) with f DT formed in FP32, at most nt / 2 (Seismogram.cpp:333-335)
    const float prod = static_cast<float>(f_agc) * static_cast<float>(dt);
    long long nagc = std::llround(1.0 / static_cast<double>(prod));
    if (nagc > nt / 2) nagc = nt / 2;
    if (nagc < 0) nagc = 0;
    const size_t bytes = static_cast<size_t>(ntr) * nt * sizeof(float);
    float *d = data, *nd = nullptr, *inv = nullptr, *tmp = nullptr;
    double* acc = nullptr;
    cudaError_t e = cudaSuccess;
    if (mem != WAVE_MEM_DEVICE) {
        e = cudaMalloc(&tmp, bytes);
        if (e == cudaSuccess) e = cudaMemcpy(tmp, data, bytes, cudaMemcpyHostToDevice);
        d = tmp;
    }
    if (e == cudaSuccess) e = cudaMalloc(&nd, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&inv, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&acc, sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(acc, 0, sizeof(double));
    // the l2-normalised copy (normalizeTrace(2) before the AGC)
    if (e == cudaSuccess) e = cudaMemcpy(nd, d, bytes, cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess) {
        normalize_kernel<<<static_cast<unsigned>(ntr), 256>>>(nd, nt, 2);
        sumsq_kernel<<<1216, 256>>>(nd, static_cast<long long>(ntr) * nt, acc);
        e = cudaGetLastError();
    }
    double total = 0.0;
    if (e == cudaSuccess) e = cudaMemcpy(&total, acc, sizeof(double), cudaMemcpyDeviceToHost);
    // water level of a zero trace: 1e-3 x the l2 norm of all normalised traces / nt / ntr
    const float wl0 = static_cast<float>(1e-3 * static_cast<double>(static_cast<float>(std::sqrt(total))) / nt / ntr);
    if (e == cudaSuccess) {
        agc_kernel<<<static_cast<unsigned>((ntr + 127) / 128), 128>>>(nd, ntr, nt, nagc, wl0, inv);
        // normalizeTrace(3): the l2-normalised traces times the inverse AGC (Seismogram.cpp:235-237)
        mul_kernel<<<1216, 256>>>(nd, inv, static_cast<long long>(ntr) * nt);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(d, nd, bytes, cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess && mem != WAVE_MEM_DEVICE) e = cudaMemcpy(data, d, bytes, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && inverse_agc)
        e = cudaMemcpy(inverse_agc, inv, bytes, mem == WAVE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(tmp);
    cudaFree(nd);
    cudaFree(inv);
    cudaFree(acc);
    if (e != cudaSuccess) return err(WAVE_ERR_CUDA, std::string("wave_agc_normalize_traces: ") + cudaGetErrorString(e));
    return WAVE_OK;
}
