// snapshot.cu — outputs around the time loop: wavefield snapshots (the field
// getter used for Wavefields::write, e.g. Wavefields3Delastic.cpp:62-96), the
// energy snapshots of snapType 3 (curl and divergence,
// Wavefields2Delastic.cpp:218-250, Wavefields3Delastic.cpp:197-240), and the
// Hilbert transform of traces (Hilbert::HilbertFFT, HilbertFFT.cpp) with the
// envelope and instantaneous phase of Common.hpp:272-345.
#include <cctype>
#include <cmath>
#include <string>

#include <cuda_runtime.h>
#include <cufft.h>

#include "handle.h"
#include "stencil.cuh"

namespace wave {
void set_global_error(const std::string& msg);
}

using namespace wave;

namespace {

int herr(wave_handle* h, int code, const std::string& m)
{
    if (h) h->err = m;
    else set_global_error(m);
    return code;
}

// curl and divergence energies with the solver's own derivative operators
// (DT folded in, as the reference's Derivatives matrices):
//   2-D: curl = (Dyf vx - Dxf vy) sqrt(mu), div = (Dxb vx + Dyb vy) sqrt(M)
//   3-D: curl = sqrt(mu |curl v|^2),        div = sqrt(M (div v)^2)
template <int H>
__global__ void __launch_bounds__(256) curl_div_kernel(StepParams P, float* curl, float* div)
{
    Pt p;
    if (!point(P, p)) return;
    const long long i = p.i, sy = (long long)P.NX * P.NZ;
    const float *vx = P.f[F_VX], *vy = P.f[F_VY];
    const float M = P.m[M_M][i], mu = P.m[M_MU][i];
    if (!P.is3d) {
        float c = deriv<H, true>(vx, i, sy, p.y, P.Dyf);
        const float t = deriv<H, true>(vy, i, 1, p.x, P.Dxf);
        c -= t;
        c *= sqrtf(mu);
        float d = deriv<H, false>(vx, i, 1, p.x, P.Dxb);
        d += deriv<H, false>(vy, i, sy, p.y, P.Dyb);
        d *= sqrtf(M);
        curl[i] = c;
        div[i] = d;
        return;
    }
    const float* vz = P.f[F_VZ];
    float u = deriv<H, true>(vz, i, sy, p.y, P.Dyf);
    u -= deriv<H, true>(vy, i, P.NX, p.z, P.Dzf);
    float c = u * u;
    u = deriv<H, true>(vx, i, P.NX, p.z, P.Dzf);
    u -= deriv<H, true>(vz, i, 1, p.x, P.Dxf);
    c += u * u;
    u = deriv<H, true>(vy, i, 1, p.x, P.Dxf);
    u -= deriv<H, true>(vx, i, sy, p.y, P.Dyf);
    c += u * u;
    c *= mu;
    float d = deriv<H, false>(vx, i, 1, p.x, P.Dxb);
    d += deriv<H, false>(vy, i, sy, p.y, P.Dyb);
    d += deriv<H, false>(vz, i, P.NX, p.z, P.Dzb);
    d *= d;
    d *= M;
    curl[i] = sqrtf(c);
    div[i] = sqrtf(d);
}

// HilbertFFT::calcHilbertCoefficient: 1 at 0 (and N/2 for even N), 2 for the
// positive frequencies, 0 for the negative ones; with the 1/N of the inverse
__global__ void hilbert_weights(cufftComplex* f, long long ntr, int N)
{
    const long long total = ntr * N;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const int k = static_cast<int>(q % N);
        float w;
        if ((N & 1) == 0) w = (k == 0 || k == N / 2) ? 1.0f : (k < N / 2 ? 2.0f : 0.0f);
        else w = k == 0 ? 1.0f : (k < (N + 1) / 2 ? 2.0f : 0.0f);
        w *= 1.0f / static_cast<float>(N);
        f[q].x *= w;
        f[q].y *= w;
    }
}

__global__ void pad_traces(const float* __restrict__ in, long long ntr, long long nt, int N, cufftComplex* f)
{
    const long long total = ntr * N;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total; q += (long long)gridDim.x * blockDim.x) {
        const long long tr = q / N, k = q - tr * N;
        f[q].x = k < nt ? in[tr * nt + k] : 0.0f;
        f[q].y = 0.0f;
    }
}

// mode 0: envelope sqrt(x^2 + H(x)^2); mode 1: water-levelled envelope
// division of Seismogram::normalizeTrace mode 4 (envelope + 1e-3 max envelope)
__global__ void envelope_kernel(float* data, long long nt, int N, const cufftComplex* f, int mode)
{
    __shared__ float smax[32];
    float* t = data + blockIdx.x * nt;
    const cufftComplex* g = f + blockIdx.x * (long long)N;
    float mx = 0.0f;
    for (long long k = threadIdx.x; k < nt; k += blockDim.x) {
        float e = t[k] * t[k];
        e += g[k].y * g[k].y;
        mx = fmaxf(mx, sqrtf(e));
    }
    if (mode == 0) {
        __syncthreads();
        for (long long k = threadIdx.x; k < nt; k += blockDim.x) {
            float e = t[k] * t[k];
            e += g[k].y * g[k].y;
            t[k] = sqrtf(e);
        }
        return;
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmaxf(r, smax[w]);
        smax[0] = r;
    }
    __syncthreads();
    const float water = smax[0] != 0.0f ? 1e-3f * smax[0] : 1e-3f * 1e-3f;
    __syncthreads();
    for (long long k = threadIdx.x; k < nt; k += blockDim.x) {
        float e = t[k] * t[k];
        e += g[k].y * g[k].y;
        t[k] /= (sqrtf(e) + water);
    }
}

// instantaneous phase as Common::calcInstantaneousPhase (Common.hpp:297-345),
// whose imaginary part is -data (the Hilbert call there is commented out)
__global__ void phase_kernel(float* data, long long nt, int type)
{
    if (threadIdx.x != 0) return;
    float* t = data + blockIdx.x * nt;
    if (type == 1) {
        for (long long k = 0; k < nt; ++k) t[k] = atanf(-t[k] / t[k]);
        return;
    }
    float prevWrapped = 0.0f, prevOut = 0.0f;
    for (long long k = 0; k < nt; ++k) {
        const float x = t[k];
        const float ph = atan2f(-x, x);
        if (type == 2 || k == 0) {
            t[k] = ph;
            prevWrapped = ph;
            prevOut = ph;
            continue;
        }
        float d = ph - prevWrapped;
        d = d > static_cast<float>(M_PI) ? d - 2 * static_cast<float>(M_PI) : (d < -static_cast<float>(M_PI) ? d + 2 * static_cast<float>(M_PI) : d);
        prevWrapped = ph;
        prevOut = prevOut + d;
        t[k] = prevOut;
    }
}

// Common::calcNextPowTwo (Common.hpp:187-194) in FP32
int next_pow2(long long n)
{
    float temp = std::log(static_cast<float>(n));
    temp = static_cast<float>(temp / std::log(2.0));
    temp = std::ceil(temp);
    return static_cast<int>(std::pow(2.0f, temp));
}

// runs the Hilbert transform of ntr device traces; leaves the analytic signal in f
cudaError_t hilbert_device(const float* d, long long ntr, long long nt, int& N, cufftComplex*& f)
{
    N = next_pow2(nt - 1);
    if (N < nt) N = static_cast<int>(nt);   // the transform must cover the trace
    cudaError_t e = cudaMalloc(&f, ntr * N * sizeof(cufftComplex));
    if (e != cudaSuccess) return e;
    pad_traces<<<1216, 256>>>(d, ntr, nt, N, f);
    cufftHandle plan;
    if (cufftPlan1d(&plan, N, CUFFT_C2C, static_cast<int>(ntr)) != CUFFT_SUCCESS) return cudaErrorUnknown;
    cufftResult r = cufftExecC2C(plan, f, f, CUFFT_FORWARD);
    if (r == CUFFT_SUCCESS) {
        hilbert_weights<<<1216, 256>>>(f, ntr, N);
        r = cufftExecC2C(plan, f, f, CUFFT_INVERSE);
    }
    cufftDestroy(plan);
    if (r != CUFFT_SUCCESS) return cudaErrorUnknown;
    return cudaGetLastError();
}

} // namespace

namespace wave {
// envelope (mode 0) or envelope normalisation (mode 1) of device traces
cudaError_t envelope_device(float* d, long long ntr, long long nt, int mode)
{
    int N = 0;
    cufftComplex* f = nullptr;
    cudaError_t e = hilbert_device(d, ntr, nt, N, f);
    if (e == cudaSuccess) {
        envelope_kernel<<<static_cast<unsigned>(ntr), 256>>>(d, nt, N, f, mode);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(f);
    return e;
}
} // namespace wave

extern "C" {

int wave_get_field(wave_handle* h, const char* name, float* out, int mem)
{
    if (!h || !name || !out) return herr(h, WAVE_ERR_ARG, "wave_get_field: null argument");
    static const struct { const char* n; int f; } names[] = {
        {"vx", F_VX}, {"vy", F_VY}, {"vz", F_VZ}, {"p", F_P}, {"sxx", F_SXX}, {"syy", F_SYY}, {"szz", F_SZZ},
        {"sxy", F_SXY}, {"sxz", F_SXZ}, {"syz", F_SYZ}, {"hx", F_HX}, {"hy", F_HY}, {"hz", F_HZ},
        {"ex", F_EX}, {"ey", F_EY}, {"ez", F_EZ}};
    std::string s(name);
    for (auto& c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    int f = -1;
    for (auto& e : names)
        if (s == e.n) f = e.f;
    // decomposition parts (Wavefields2Dacoustic.cpp:86-107 file names): "p.up", "vx.down", "vy.left", ...
    const float* src = f >= 0 ? h->f[f] : nullptr;
    static const char* parts[2][6] = {{"p.up", "p.down", "vx.up", "vx.down", "vy.up", "vy.down"},
                                      {"p.left", "p.right", "vx.left", "vx.right", "vy.left", "vy.right"}};
    static const char* partsEz[2][6] = {{"ez.up", "ez.down", "", "", "", ""}, {"ez.left", "ez.right", "", "", "", ""}};
    const bool tm = h->cfg.equation == WAVE_EQ_TMEM;
    for (int t = 0; t < 2; ++t)
        for (int k = 0; k < 6; ++k)
            if (s == (tm ? partsEz : parts)[t][k]) {
                if (h->decompType != t + 1) return herr(h, WAVE_ERR_STATE, std::string("wave_get_field: ") + name + " needs wave_set_decomposition(h, " + std::to_string(t + 1) + ")");
                src = h->decOut[k];
            }
    if (!src) return herr(h, WAVE_ERR_ARG, std::string("wave_get_field: no wavefield ") + name + " for this equation");
    cudaError_t e = cudaMemcpyAsync(out, src, h->N * sizeof(float), mem == WAVE_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return herr(h, WAVE_ERR_CUDA, std::string("wave_get_field: ") + cudaGetErrorString(e));
    return WAVE_OK;
}

int wave_get_curl_div(wave_handle* h, float* curl, float* div, int mem)
{
    if (!h || !curl || !div) return herr(h, WAVE_ERR_ARG, "wave_get_curl_div: null argument");
    const int eq = h->cfg.equation;
    if (eq != WAVE_EQ_ELASTIC && eq != WAVE_EQ_VISCOELASTIC)
        return herr(h, WAVE_ERR_UNSUPPORTED, "wave_get_curl_div: curl and div energies exist for (visco-)elastic modelling only");
    if (!h->modelSet) return herr(h, WAVE_ERR_STATE, "wave_get_curl_div: set the model first");
    float *dc = curl, *dd = div, *tc = nullptr, *td = nullptr;
    cudaError_t e = cudaSuccess;
    if (mem != WAVE_MEM_DEVICE) {
        e = cudaMalloc(&tc, h->N * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc(&td, h->N * sizeof(float));
        dc = tc;
        dd = td;
    }
    if (e == cudaSuccess) {
        const StepParams& P = h->sp;
        switch (h->H) {
        case 1: curl_div_kernel<1><<<h->grid, h->block, 0, h->stream>>>(P, dc, dd); break;
        case 2: curl_div_kernel<2><<<h->grid, h->block, 0, h->stream>>>(P, dc, dd); break;
        case 3: curl_div_kernel<3><<<h->grid, h->block, 0, h->stream>>>(P, dc, dd); break;
        case 4: curl_div_kernel<4><<<h->grid, h->block, 0, h->stream>>>(P, dc, dd); break;
        case 5: curl_div_kernel<5><<<h->grid, h->block, 0, h->stream>>>(P, dc, dd); break;
        default: curl_div_kernel<6><<<h->grid, h->block, 0, h->stream>>>(P, dc, dd); break;
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e == cudaSuccess && mem != WAVE_MEM_DEVICE) {
        e = cudaMemcpy(curl, tc, h->N * sizeof(float), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(div, td, h->N * sizeof(float), cudaMemcpyDeviceToHost);
    }
    cudaFree(tc);
    cudaFree(td);
    if (e != cudaSuccess) return herr(h, WAVE_ERR_CUDA, std::string("wave_get_curl_div: ") + cudaGetErrorString(e));
    return WAVE_OK;
}

int wave_envelope(float* data, int64_t ntr, int64_t nt, int mem)
{
    if (!data || ntr < 0 || nt < 2) return herr(nullptr, WAVE_ERR_ARG, "wave_envelope: invalid argument (nt >= 2)");
    if (ntr == 0) return WAVE_OK;
    float* d = data;
    float* t = nullptr;
    cudaError_t e = cudaSuccess;
    if (mem != WAVE_MEM_DEVICE) {
        e = cudaMalloc(&t, ntr * nt * sizeof(float));
        if (e == cudaSuccess) e = cudaMemcpy(t, data, ntr * nt * sizeof(float), cudaMemcpyHostToDevice);
        d = t;
    }
    if (e == cudaSuccess) e = envelope_device(d, ntr, nt, 0);
    if (e == cudaSuccess && mem != WAVE_MEM_DEVICE) e = cudaMemcpy(data, t, ntr * nt * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(t);
    if (e != cudaSuccess) return herr(nullptr, WAVE_ERR_CUDA, std::string("wave_envelope: ") + cudaGetErrorString(e));
    return WAVE_OK;
}

int wave_instantaneous_phase(float* data, int64_t ntr, int64_t nt, int phase_type, int mem)
{
    if (!data || ntr < 0 || nt < 1 || phase_type < 1 || phase_type > 3)
        return herr(nullptr, WAVE_ERR_ARG, "wave_instantaneous_phase: invalid argument (phase type 1, 2 or 3)");
    if (ntr == 0) return WAVE_OK;
    float* d = data;
    float* t = nullptr;
    cudaError_t e = cudaSuccess;
    if (mem != WAVE_MEM_DEVICE) {
        e = cudaMalloc(&t, ntr * nt * sizeof(float));
        if (e == cudaSuccess) e = cudaMemcpy(t, data, ntr * nt * sizeof(float), cudaMemcpyHostToDevice);
        d = t;
    }
    if (e == cudaSuccess) {
        phase_kernel<<<static_cast<unsigned>(ntr), 32>>>(d, nt, phase_type);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess && mem != WAVE_MEM_DEVICE) e = cudaMemcpy(data, t, ntr * nt * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(t);
    if (e != cudaSuccess) return herr(nullptr, WAVE_ERR_CUDA, std::string("wave_instantaneous_phase: ") + cudaGetErrorString(e));
    return WAVE_OK;
}

} // extern "C"
