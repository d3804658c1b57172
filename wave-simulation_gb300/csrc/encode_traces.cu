// encode_traces.cu — receiver-side encoding of seismograms: the shots of a
// super-shot summed into the super-shot's receiver rows and split back out
// (Receivers::encode / Receivers::decode, Receivers.cpp:354-573), with the
// per-shot sign of the encoded amplitude and, for frequency-domain modelling,
// the single-frequency "ideal" band-pass at the shot's frequency
// (Filter::calcIdealBp with order 1 and Filter::apply, Filter.cpp:239-342).
//
// The filter projects a trace d(t_k), t_k = k DT, on exp(j w t) with
// w = 2 pi ceil(fc / df) df, df = 1 / (nFFT DT), nFFT the next power of two of
// NT - 1: out(t) = s Re(X exp(j w t)), X = sum_k d(t_k) exp(-j w t_k). For a
// block of traces (multi-offset data, the matrix apply) s = 2 / nFFT and the
// block is then divided by its largest magnitude; for a single trace
// (common-offset data, the vector apply) s = 1 / NT. One block per trace,
// the sums in FP64.
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "wave_internal.h"

namespace {

__global__ void project_rows(float* d, long long nt, double w, double DT, float scale, unsigned int* maxBits)
{
    float* row = d + blockIdx.x * nt;
    double xr = 0.0, xs = 0.0;
    for (long long k = threadIdx.x; k < nt; k += blockDim.x) {
        double s, c;
        sincos(w * (static_cast<double>(k) * DT), &s, &c);
        xr += row[k] * c;
        xs += row[k] * s;
    }
    __shared__ double rr[256], ss[256];
    rr[threadIdx.x] = xr;
    ss[threadIdx.x] = xs;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            rr[threadIdx.x] += rr[threadIdx.x + o];
            ss[threadIdx.x] += ss[threadIdx.x + o];
        }
        __syncthreads();
    }
    xr = rr[0];
    xs = ss[0];
    float m = 0.0f;
    for (long long k = threadIdx.x; k < nt; k += blockDim.x) {
        double s, c;
        sincos(w * (static_cast<double>(k) * DT), &s, &c);
        // Re((xr - j xs) (c + j s)) = xr c + xs s
        const float v = static_cast<float>((xr * c + xs * s) * scale);
        row[k] = v;
        m = fmaxf(m, fabsf(v));
    }
    if (maxBits) atomicMax(maxBits, __float_as_uint(m));   // non-negative floats order as their bits
}

__global__ void scale_by_max(float* d, long long n, const unsigned int* maxBits)
{
    const float m = __uint_as_float(*maxBits);
    if (!(m > 0.0f)) return;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) d[i] /= m;
}

// dst[dstRow[k]] (+)= sign src[srcRow[k]] for k < nrows
__global__ void move_rows(const float* src, float* dst, const int* srcRow, const int* dstRow, long long nt, float sign, int add)
{
    const float* s = src + srcRow[blockIdx.y] * nt;
    float* d = dst + dstRow[blockIdx.y] * nt;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < nt; k += (long long)gridDim.x * blockDim.x)
        d[k] = add ? d[k] + sign * s[k] : sign * s[k];
}

int next_pow2(long long n)
{
    float e = std::log(static_cast<float>(n));
    e /= std::log(2.0);
    return static_cast<int>(std::pow(2.0f, std::ceil(e)));
}

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

} // namespace

extern "C" int wave_encode_traces(int decode, int nshots, int nrec, int64_t nt, const int* mark, const int* super_mark,
                                  const float* amp, const float* fc, double DT, int common_offset, float* const* shot_data,
                                  float* super_data, int mem)
{
    if (nshots < 1 || nrec < 1 || nt < 2 || !mark || !super_mark || !amp || !shot_data || !super_data || (fc && DT <= 0.0) ||
        (common_offset && nshots != nrec)) {
        wave::set_global_error("wave_encode_traces: invalid arguments");
        return WAVE_ERR_ARG;
    }
    try {
        // super-shot rows, and each shot's rows (shot-local index, super-shot index)
        std::vector<int> superRow(common_offset ? nshots : nrec, -1);
        int nsup = 0;
        for (int r = 0; r < static_cast<int>(superRow.size()); ++r)
            if (super_mark[r]) superRow[r] = nsup++;
        std::vector<std::vector<int>> srcRows(nshots), dstRows(nshots);
        std::vector<int> shotRows(nshots, 0);
        for (int s = 0; s < nshots; ++s) {
            if (common_offset) {
                shotRows[s] = 1;
                if (super_mark[s] && mark[static_cast<long long>(s) * nrec + s]) { srcRows[s].push_back(0); dstRows[s].push_back(superRow[s]); }
                continue;
            }
            for (int r = 0; r < nrec; ++r)
                if (super_mark[r] && mark[static_cast<long long>(s) * nrec + r]) {
                    srcRows[s].push_back(shotRows[s]++);
                    dstRows[s].push_back(superRow[r]);
                }
        }
        cudaStream_t st = nullptr;
        ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
        std::vector<void*> tmp;
        struct Free {
            std::vector<void*>& v;
            cudaStream_t s;
            ~Free()
            {
                for (void* p : v) cudaFreeAsync(p, s);
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
        } freeAll{tmp, st};
        auto dev = [&](size_t bytes) {
            void* p = nullptr;
            ck(cudaMallocAsync(&p, bytes > 0 ? bytes : 4, st), "cudaMallocAsync");
            tmp.push_back(p);
            return p;
        };
        const size_t rowBytes = static_cast<size_t>(nt) * sizeof(float);
        const cudaMemcpyKind toDev = mem == WAVE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        const cudaMemcpyKind toOut = mem == WAVE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        float* dSup = static_cast<float*>(dev(nsup * rowBytes));
        unsigned int* dMax = static_cast<unsigned int*>(dev(sizeof(unsigned int)));
        if (decode) ck(cudaMemcpyAsync(dSup, super_data, nsup * rowBytes, toDev, st), "copy");
        else ck(cudaMemsetAsync(dSup, 0, nsup * rowBytes, st), "memset");
        const double df = 1.0 / (static_cast<double>(next_pow2(nt - 1)) * DT);
        for (int s = 0; s < nshots; ++s) {
            const int rows = shotRows[s], moved = static_cast<int>(srcRows[s].size());
            if (rows == 0) continue;
            const float sign = amp[s] < 0.0f ? -1.0f : 1.0f;
            float* dShot = static_cast<float*>(dev(rows * rowBytes));
            int* dSrc = static_cast<int*>(dev((moved + 1) * sizeof(int)));
            int* dDst = static_cast<int*>(dev((moved + 1) * sizeof(int)));
            if (moved > 0) {
                ck(cudaMemcpyAsync(dSrc, srcRows[s].data(), moved * sizeof(int), cudaMemcpyHostToDevice, st), "copy");
                ck(cudaMemcpyAsync(dDst, dstRows[s].data(), moved * sizeof(int), cudaMemcpyHostToDevice, st), "copy");
            }
            auto filter = [&]() {
                if (!fc) return;
                const double w = 2.0 * M_PI * std::ceil(static_cast<double>(static_cast<float>(fc[s]) / static_cast<float>(df))) * df;
                ck(cudaMemsetAsync(dMax, 0, sizeof(unsigned int), st), "memset");
                const float scale = common_offset ? 1.0f / static_cast<float>(nt) : 2.0f / static_cast<float>(next_pow2(nt - 1));
                project_rows<<<rows, 256, 0, st>>>(dShot, nt, w, DT, scale, common_offset ? nullptr : dMax);
                if (!common_offset) scale_by_max<<<64, 256, 0, st>>>(dShot, static_cast<long long>(rows) * nt, dMax);
            };
            if (!decode) {
                ck(cudaMemcpyAsync(dShot, shot_data[s], rows * rowBytes, toDev, st), "copy");
                filter();
                if (moved > 0) move_rows<<<dim3(8, moved), 256, 0, st>>>(dShot, dSup, dSrc, dDst, nt, sign, 1);
            } else {
                ck(cudaMemsetAsync(dShot, 0, rows * rowBytes, st), "memset");
                if (moved > 0) move_rows<<<dim3(8, moved), 256, 0, st>>>(dSup, dShot, dDst, dSrc, nt, sign, 0);
                filter();
                ck(cudaMemcpyAsync(shot_data[s], dShot, rows * rowBytes, toOut, st), "copy");
            }
            ck(cudaGetLastError(), "encode launch");
        }
        if (!decode) ck(cudaMemcpyAsync(super_data, dSup, nsup * rowBytes, toOut, st), "copy");
        ck(cudaStreamSynchronize(st), "encode");
    } catch (std::exception& e) {
        wave::set_global_error(std::string("wave_encode_traces: ") + e.what());
        return WAVE_ERR_CUDA;
    }
    return WAVE_OK;
}
