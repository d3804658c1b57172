// decompose.cu — wavefield decomposition of the 2-D acoustic and 2-D TMz
// wavefields into up/down-going (decomposeWavefieldType 1) or
// left/right-going (2) parts by the sign of a Poynting-vector estimate, after
// every time step: Simulation.cpp:450-461 (time derivative of the step:
// (new - old) / DT), FD2Dacoustic::decompose (Wavefields2Dacoustic.cpp:
// 119-300) and FD2Dtmem::decompose (Wavefields2Dtmem.cpp:109-160).
//
// Per field F (P, VX, VY; or EZ) and point:
//   S1  = -P * VY (type 1) or -P * VX (type 2); EZ * HX or -(EZ * HY)
//   S2F = -(D F) * dF/dt, D = Dyf (type 1) or Dxf (type 2), DT folded in
//   QF  = S2F * (max|S1| / max|S2F|) + S1
//   F.up / F.left  = F where QF <= 0, else 0
//   F.down / F.right = F where QF >= 0, else 0
// Two kernels per step: decomp_a computes S2F and the maxima (atomicMax on
// the bit patterns of non-negative floats), decomp_b the parts. The sign of
// NaN is taken as 0. All arithmetic uses rounding intrinsics in the
// reference's operation order.
#include <cuda_runtime.h>

#include "handle.h"
#include "stencil.cuh"

namespace wave {

namespace {

struct DecompParams {
    StepParams P;
    int type;
    int nf;                    // decomposed fields: 3 (P, VX, VY) or 1 (EZ)
    float negDTinv;            // -(1/DT) in single precision
    const float* s1a;          // S1 = s1sign * (s1a * s1b)
    const float* s1b;
    float s1sign;
    const float* cur[3];       // fields after the step
    const float* old[3];       // before the step
    float* s2[3];
    float* out[6];             // F.up/left, F.down/right for P, VX, VY
    unsigned* mx;              // max|S1|, max|S2P|, max|S2VX|, max|S2VY| as float bits
};

// the sign is applied exactly, so (-P)*VY = -(P*VY) and (EZ*HY)*(-1) are the same
__device__ __forceinline__ float s1_of(const DecompParams& D, long long i)
{
    return D.s1sign * __fmul_rn(D.s1a[i], D.s1b[i]);
}

template <int H>
__global__ void __launch_bounds__(256) decomp_a(DecompParams D)
{
    Pt p;
    if (!point(D.P, p)) return;
    const float s1 = s1_of(D, p.i);
    atomicMax(D.mx, __float_as_uint(fabsf(s1)));
    for (int q = 0; q < D.nf; ++q) {
        const float* f = D.cur[q];
        // wavefieldsTemp -= wavefields; wavefieldsTemp *= -DTinv
        const float dfdt = __fmul_rn(__fsub_rn(D.old[q][p.i], f[p.i]), D.negDTinv);
        const float d = D.type == 1 ? deriv<H, true>(f, p.i, static_cast<long long>(D.P.NX) * D.P.NZ, p.y, D.P.Dyf)
                                    : deriv<H, true>(f, p.i, 1, p.x, D.P.Dxf);
        const float s2 = -__fmul_rn(d, dfdt);
        D.s2[q][p.i] = s2;
        atomicMax(D.mx + 1 + q, __float_as_uint(fabsf(s2)));
    }
}

__global__ void __launch_bounds__(256) decomp_b(DecompParams D)
{
    Pt p;
    if (!point(D.P, p)) return;
    const float s1 = s1_of(D, p.i);
    const float m1 = __uint_as_float(D.mx[0]);
    for (int q = 0; q < D.nf; ++q) {
        const float ratio = __fdiv_rn(m1, __uint_as_float(D.mx[1 + q]));
        const float Q = __fadd_rn(__fmul_rn(D.s2[q][p.i], ratio), s1);
        const int sg = (Q > 0.0f) - (Q < 0.0f);
        const float f = D.cur[q][p.i];
        D.out[2 * q][p.i] = __fmul_rn(sg <= 0 ? 1.0f : 0.0f, f);
        D.out[2 * q + 1][p.i] = __fmul_rn(sg >= 0 ? 1.0f : 0.0f, f);
    }
}

DecompParams params_of(wave_handle* h)
{
    DecompParams D{};
    D.P = h->sp;
    D.type = h->decompType;
    const float DT = static_cast<float>(h->cfg.DT);
    D.negDTinv = -(1.0f / DT);
    const bool tm = h->cfg.equation == WAVE_EQ_TMEM;
    const int acoustic[3] = {F_P, F_VX, F_VY};
    D.nf = tm ? 1 : 3;
    for (int q = 0; q < D.nf; ++q) {
        D.cur[q] = h->f[tm ? F_EZ : acoustic[q]];
        D.old[q] = h->decOld[q];
        D.s2[q] = h->decS2[q];
    }
    if (tm) {   // EZ * HX, or -(EZ * HY)
        D.s1a = h->f[F_EZ];
        D.s1b = h->f[D.type == 1 ? F_HX : F_HY];
        D.s1sign = D.type == 1 ? 1.0f : -1.0f;
    } else {    // -P * VY, or -P * VX
        D.s1a = h->f[F_P];
        D.s1b = h->f[D.type == 1 ? F_VY : F_VX];
        D.s1sign = -1.0f;
    }
    for (int k = 0; k < 6; ++k) D.out[k] = h->decOut[k];
    D.mx = h->decMax;
    return D;
}

} // namespace

void decompose_before_step(wave_handle* h)
{
    const bool tm = h->cfg.equation == WAVE_EQ_TMEM;
    const int f[3] = {F_P, F_VX, F_VY};
    for (int q = 0; q < (tm ? 1 : 3); ++q)
        h->check(cudaMemcpyAsync(h->decOld[q], h->f[tm ? F_EZ : f[q]], h->N * sizeof(float), cudaMemcpyDeviceToDevice, h->stream),
                 "decomposition copy");
}

int decompose_after_step(wave_handle* h)
{
    const DecompParams D = params_of(h);
    h->check(cudaMemsetAsync(h->decMax, 0, 4 * sizeof(unsigned), h->stream), "decomposition reset");
    switch (h->H) {
    case 1: decomp_a<1><<<h->grid, h->block, 0, h->stream>>>(D); break;
    case 2: decomp_a<2><<<h->grid, h->block, 0, h->stream>>>(D); break;
    case 3: decomp_a<3><<<h->grid, h->block, 0, h->stream>>>(D); break;
    case 4: decomp_a<4><<<h->grid, h->block, 0, h->stream>>>(D); break;
    case 5: decomp_a<5><<<h->grid, h->block, 0, h->stream>>>(D); break;
    default: decomp_a<6><<<h->grid, h->block, 0, h->stream>>>(D); break;
    }
    decomp_b<<<h->grid, h->block, 0, h->stream>>>(D);
    h->check(cudaGetLastError(), "decomposition launch");
    return 2;
}

} // namespace wave

extern "C" int wave_set_decomposition(wave_handle* h, int type)
{
    if (!h) return WAVE_ERR_ARG;
    if (type < 0 || type > 2) {
        h->err = "wave_set_decomposition: decomposeWavefieldType must be 0, 1 or 2";
        return WAVE_ERR_ARG;
    }
    if (type != 0 && ((h->cfg.equation != WAVE_EQ_ACOUSTIC && h->cfg.equation != WAVE_EQ_TMEM) || h->is3d() || h->vg)) {
        h->err = "wave_set_decomposition: the decomposition exists for 2-D acoustic and 2-D TMz modelling on a regular grid";
        return WAVE_ERR_UNSUPPORTED;
    }
    try {
        if (type != 0 && !h->decMax) {
            for (int q = 0; q < 3; ++q) {
                h->decOld[q] = h->alloc<float>(h->N);
                h->decS2[q] = h->alloc<float>(h->N);
            }
            for (int k = 0; k < 6; ++k) {
                h->decOut[k] = h->alloc<float>(h->N);
                h->check(cudaMemset(h->decOut[k], 0, h->N * sizeof(float)), "memset");
            }
            h->decMax = h->alloc<unsigned>(4);
        }
    } catch (std::exception& ex) {
        h->err = ex.what();
        return WAVE_ERR_CUDA;
    }
    h->decompType = type;
    h->graphDirty = true;
    return WAVE_OK;
}
