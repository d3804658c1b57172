// kernels.cu — sm_103a kernels of the forward time step (one thread per grid
// point, all arithmetic FP32). Each equation is two fused passes, matching the
// two halves of the reference's ForwardSolver*::run:
//   pass 1 (velocity / H field): every derivative, its CPML psi update and the
//          field update in one kernel;
//   pass 2 (stress / pressure / E field): derivatives, CPML, memory variables,
//          free-surface exchange and ABS damping of the pass-2 fields.
// The ABS damping of the pass-1 fields runs in abs_frame_kernel after pass 2
// (pass 2 still needs their undamped values), then sources and receivers.
//
// Derivative operators are matrix-free: rows away from the grid edges use the
// interior weights held in the kernel parameters; the few edge rows (and the
// free-surface image rows) read a small per-axis table.
#include <cuda_runtime.h>

#include "stencil.cuh"

namespace wave {

#define LD(ptr) __ldg((ptr) + p.i)

// --------------------------------------------------------------------------
// acoustic: FD2Dacoustic::run (ForwardSolver2Dacoustic.cpp:121-190),
//           FD3Dacoustic::run (ForwardSolver3Dacoustic.cpp:122-230)
// --------------------------------------------------------------------------
template <int H>
__device__ __forceinline__ void acoustic_v_body(const StepParams& P, const Pt& p)
{
    const float* pr = P.f[F_P];
    float u = dX<H, true>(P, p, pr, P.Dxf, PS_P_X);
    u *= LD(P.m[M_IRX]);
    P.f[F_VX][p.i] += u;
    u = P.fs ? dY<H, true>(P, p, pr, P.DyfS, PS_P_Y) : dY<H, true>(P, p, pr, P.Dyf, PS_P_Y);
    u *= LD(P.m[M_IRY]);
    P.f[F_VY][p.i] += u;
    if (P.is3d) {
        u = dZ<H, true>(P, p, pr, P.Dzf, PS_P_Z);
        u *= LD(P.m[M_IRZ]);
        P.f[F_VZ][p.i] += u;
    }
}

template <int H>
__global__ void __launch_bounds__(256) acoustic_v(StepParams P)
{
    dependent_launch_prologue();
    // the pressure kernel of this step reads t = counter - 1
    if (P.sr.on && blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) *P.sr.tcounter += 1;
    Pt p;
    if (!point(P, p)) return;
    acoustic_v_body<H>(P, p);
}

template <int H>
__global__ void __launch_bounds__(256) acoustic_v_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { acoustic_v_body<H>(P, p); });
}

template <int H>
__device__ __forceinline__ void acoustic_p_body(const StepParams& P, const Pt& p)
{
    float u = dX<H, false>(P, p, P.f[F_VX], P.Dxb, PS_VXX);
    float ut = dY<H, false>(P, p, P.f[F_VY], P.Dyb, PS_VYY);
    u += ut;
    if (P.is3d) {
        ut = dZ<H, false>(P, p, P.f[F_VZ], P.Dzb, PS_VZZ);
        u += ut;
    }
    u *= LD(P.m[M_M]);
    float pv = P.f[F_P][p.i] + u;
    if (P.abs) pv *= absDamp(P, p);
    if (P.fs && p.y == 0) pv = 0.0f;   // FreeSurface::setSurfaceZero (FreeSurface.cpp:14-19)
    P.f[F_P][p.i] = pv;
}

// SourceReceiverImpl::applySource + gatherSeismogram (SourceReceiverImpl.cpp:
// 12-37, FDTDacoustic.cpp) at one marked point, after its pressure update:
// pressure sources in index order, then the receivers at the point
__device__ __forceinline__ void fused_srcrec(const StepParams& P, long long i)
{
    const int k = P.sr.map[i];
    if (k < 0) return;
    const int t = *P.sr.tcounter - 1;
    float pv = P.f[F_P][i];
    for (int s = P.sr.ptSrc[k]; s >= 0; s = P.sr.srcNext[s]) pv += P.sr.signals[(long long)s * P.sr.nt + t];
    P.f[F_P][i] = pv;
    for (int r = P.sr.ptRec[k]; r >= 0; r = P.sr.recNext[r]) {
        const int ty = P.sr.rtype[r];
        const float v = ty == WAVE_TYPE_P ? pv : ty == WAVE_TYPE_VX ? P.f[F_VX][i] : ty == WAVE_TYPE_VY ? P.f[F_VY][i] : P.f[F_VZ][i];
        P.sr.seis[(long long)r * P.sr.nt + t] = v;
    }
}

template <int H>
__global__ void __launch_bounds__(256) acoustic_p(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    acoustic_p_body<H>(P, p);
    if (P.sr.on) fused_srcrec(P, p.i);
}

template <int H>
__global__ void __launch_bounds__(256) acoustic_p_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { acoustic_p_body<H>(P, p); });
}

// --------------------------------------------------------------------------
// elastic + visco-elastic velocity: ForwardSolver2Delastic.cpp:150-205,
// ForwardSolver3Delastic.cpp:174-277, ForwardSolver3Dviscoelastic.cpp:186-268
// --------------------------------------------------------------------------
template <int H>
__device__ __forceinline__ void elastic_v_body(const StepParams& P, const Pt& p)
{
    const Op1D& DybS = P.fs ? P.DybS : P.Dyb;
    const Op1D& DyfS = P.fs ? P.DyfS : P.Dyf;
    const float *Sxx = P.f[F_SXX], *Syy = P.f[F_SYY], *Sxy = P.f[F_SXY];
    // vx
    float u = dX<H, true>(P, p, Sxx, P.Dxf, PS_SXX_X);
    float ut = dY<H, false>(P, p, Sxy, DybS, PS_SXY_Y);
    u += ut;
    if (P.is3d) {
        ut = dZ<H, false>(P, p, P.f[F_SXZ], P.Dzb, PS_SXZ_Z);
        u += ut;
    }
    u *= LD(P.m[M_IRX]);
    P.f[F_VX][p.i] += u;
    // vy
    u = dX<H, false>(P, p, Sxy, P.Dxb, PS_SXY_X);
    ut = dY<H, true>(P, p, Syy, DyfS, PS_SYY_Y);
    u += ut;
    if (P.is3d) {
        ut = dZ<H, false>(P, p, P.f[F_SYZ], P.Dzb, PS_SYZ_Z);
        u += ut;
    }
    u *= LD(P.m[M_IRY]);
    P.f[F_VY][p.i] += u;
    if (P.is3d) {
        // vz
        u = dX<H, false>(P, p, P.f[F_SXZ], P.Dxb, PS_SXZ_X);
        ut = dY<H, false>(P, p, P.f[F_SYZ], DybS, PS_SYZ_Y);
        u += ut;
        ut = dZ<H, true>(P, p, P.f[F_SZZ], P.Dzf, PS_SZZ_Z);
        u += ut;
        u *= LD(P.m[M_IRZ]);
        P.f[F_VZ][p.i] += u;
    }
}

template <int H>
__global__ void __launch_bounds__(256) elastic_v(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    elastic_v_body<H>(P, p);
}

template <int H>
__global__ void __launch_bounds__(256) elastic_v_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { elastic_v_body<H>(P, p); });
}

// elastic stress: ForwardSolver2Delastic.cpp:210-290, ForwardSolver3Delastic.cpp:283-409,
// free surface FreeSurface2Delastic.cpp:14-45 / FreeSurface3Delastic.cpp:15-47
template <int H>
__device__ __forceinline__ void elastic_s_body(const StepParams& P, const Pt& p)
{
    const float *vx = P.f[F_VX], *vy = P.f[F_VY];
    const float M = LD(P.m[M_M]), mu = LD(P.m[M_MU]);
    float vxx = dX<H, false>(P, p, vx, P.Dxb, PS_VXX);
    float vyy = dY<H, false>(P, p, vy, P.Dyb, PS_VYY);
    float vzz = 0.0f;
    if (P.is3d) vzz = dZ<H, false>(P, p, P.f[F_VZ], P.Dzb, PS_VZZ);
    float sxx = P.f[F_SXX][p.i], syy = P.f[F_SYY][p.i];
    float szz = P.is3d ? P.f[F_SZZ][p.i] : 0.0f;
    float u = vxx;
    u += vyy;
    if (P.is3d) u += vzz;
    u *= M;
    sxx += u; syy += u;
    if (P.is3d) {
        szz += u;
        u = vyy + vzz; u *= mu; sxx -= 2.0f * u;
        u = vxx + vzz; u *= mu; syy -= 2.0f * u;
        u = vxx + vyy; u *= mu; szz -= 2.0f * u;
    } else {
        u = vyy; u *= mu; sxx -= 2.0f * u;
        u = vxx; u *= mu; syy -= 2.0f * u;
    }
    // shear
    u = dY<H, true>(P, p, vx, P.Dyf, PS_VXY);
    float ut = dX<H, true>(P, p, vy, P.Dxf, PS_VYX);
    u += ut;
    u *= LD(P.m[M_MUXY]);
    float sxy = P.f[F_SXY][p.i] + u;
    float sxz = 0.0f, syz = 0.0f;
    if (P.is3d) {
        u = dZ<H, true>(P, p, vx, P.Dzf, PS_VXZ);
        ut = dX<H, true>(P, p, P.f[F_VZ], P.Dxf, PS_VZX);
        u += ut;
        u *= LD(P.m[M_MUXZ]);
        sxz = P.f[F_SXZ][p.i] + u;
        u = dZ<H, true>(P, p, vy, P.Dzf, PS_VYZ);
        ut = dY<H, true>(P, p, P.f[F_VZ], P.Dyf, PS_VZY);
        u += ut;
        u *= LD(P.m[M_MUYZ]);
        syz = P.f[F_SYZ][p.i] + u;
    }
    if (P.fs && p.y == 0) {
        // FreeSurfaceElastic::setModelparameter (FreeSurfaceElastic.cpp:11-47)
        float sv = M - 2.0f * mu;
        float sh = sv * sv;
        sh /= M;
        sh *= -1.0f;
        syy = 0.0f;
        const float hs = P.is3d ? vxx + vzz : vxx;
        float t = sh * hs;
        sxx += t;
        if (P.is3d) szz += t;
        t = sv * vyy;
        sxx -= t;
        if (P.is3d) szz -= t;
    }
    if (P.abs) {
        const float d = absDamp(P, p);
        sxx *= d; syy *= d; sxy *= d;
        if (P.is3d) { szz *= d; sxz *= d; syz *= d; }
    }
    P.f[F_SXX][p.i] = sxx;
    P.f[F_SYY][p.i] = syy;
    P.f[F_SXY][p.i] = sxy;
    if (P.is3d) {
        P.f[F_SZZ][p.i] = szz;
        P.f[F_SXZ][p.i] = sxz;
        P.f[F_SYZ][p.i] = syz;
    }
}

template <int H>
__global__ void __launch_bounds__(256) elastic_s(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    elastic_s_body<H>(P, p);
}

template <int H>
__global__ void __launch_bounds__(256) elastic_s_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { elastic_s_body<H>(P, p); });
}

// visco-elastic stress: ForwardSolver2Dviscoelastic.cpp:223-303,
// ForwardSolver3Dviscoelastic.cpp:270-446, free surface
// FreeSurface2Dviscoelastic.cpp / FreeSurface3Dviscoelastic.cpp:17-75
template <int H>
// The loops over stress components and relaxation mechanisms run to their
// compile-time bounds with run-time guards, so that S and R stay in registers.
__device__ __forceinline__ void visco_s_body(const StepParams& P, const Pt& p)
{
    const int L = P.L;
    const float DTh = P.DThalf;
    const float *vx = P.f[F_VX], *vy = P.f[F_VY];
    const float M = LD(P.m[M_M]), mu = LD(P.m[M_MU]);
    const float tauP = LD(P.m[M_TAUP]), tauS = LD(P.m[M_TAUS]);
    const float opP = LD(P.m[M_OPLTP]), opS = LD(P.m[M_OPLTS]);
    float vxx = dX<H, false>(P, p, vx, P.Dxb, PS_VXX);
    float vyy = dY<H, false>(P, p, vy, P.Dyb, PS_VYY);
    float vzz = 0.0f;
    if (P.is3d) vzz = dZ<H, false>(P, p, P.f[F_VZ], P.Dzb, PS_VZZ);
    const int nN = P.is3d ? 3 : 2;
    float S[3], R[3][kMaxL];
    const int slotS[3] = {F_SXX, F_SYY, F_SZZ};
    const int slotR[3] = {R_XX, R_YY, R_ZZ};
    #pragma unroll
    for (int k = 0; k < 3; ++k) if (k < nN) {
        S[k] = P.f[slotS[k]][p.i];
        #pragma unroll
        for (int l = 0; l < kMaxL; ++l) if (l < L) R[k][l] = P.r[slotR[k]][l][p.i];
    }
    float u = vxx;
    u += vyy;
    if (P.is3d) u += vzz;
    u *= M;
    #pragma unroll
    for (int l = 0; l < kMaxL; ++l) if (l < L) {
        float u2 = P.invRelax[l] * u;
        u2 *= tauP;
        #pragma unroll
        for (int k = 0; k < 3; ++k) if (k < nN) {
            S[k] += DTh * R[k][l];
            R[k][l] *= P.c1[l];
            R[k][l] -= u2;
        }
    }
    u *= opP;
    #pragma unroll
    for (int k = 0; k < 3; ++k) if (k < nN) S[k] += u;
    #pragma unroll
    for (int k = 0; k < 3; ++k) if (k < nN) {
        float sum;
        if (P.is3d) sum = k == 0 ? vyy + vzz : (k == 1 ? vxx + vzz : vxx + vyy);
        else sum = k == 0 ? vyy : vxx;
        u = sum;
        u *= mu;
        u *= 2.0f;
        #pragma unroll
        for (int l = 0; l < kMaxL; ++l) if (l < L) {
            float u2 = P.invRelax[l] * u;
            u2 *= tauS;
            R[k][l] += u2;
            R[k][l] *= P.c2[l];
            S[k] += DTh * R[k][l];
        }
        u *= opS;
        S[k] -= u;
    }
    // shear stresses
    const int nS = P.is3d ? 3 : 1;
    const int slotSh[3] = {F_SXY, F_SXZ, F_SYZ};
    const int slotRh[3] = {R_XY, R_XZ, R_YZ};
    const int matMu[3] = {M_MUXY, M_MUXZ, M_MUYZ};
    const int matTau[3] = {M_TAUSXY, M_TAUSXZ, M_TAUSYZ};
    float Sh[3];
    #pragma unroll
    for (int k = 0; k < 3; ++k) if (k < nS) {
        float ut;
        if (k == 0) { u = dY<H, true>(P, p, vx, P.Dyf, PS_VXY); ut = dX<H, true>(P, p, vy, P.Dxf, PS_VYX); }
        else if (k == 1) { u = dZ<H, true>(P, p, vx, P.Dzf, PS_VXZ); ut = dX<H, true>(P, p, P.f[F_VZ], P.Dxf, PS_VZX); }
        else { u = dZ<H, true>(P, p, vy, P.Dzf, PS_VYZ); ut = dY<H, true>(P, p, P.f[F_VZ], P.Dyf, PS_VZY); }
        u += ut;
        u *= LD(P.m[matMu[k]]);
        const float tauAv = LD(P.m[matTau[k]]);
        float s = P.f[slotSh[k]][p.i];
        #pragma unroll
        for (int l = 0; l < kMaxL; ++l) if (l < L) {
            float r = P.r[slotRh[k]][l][p.i];
            s += DTh * r;
            r *= P.c1[l];
            float u2 = P.invRelax[l] * u;
            u2 *= tauAv;
            r -= u2;
            r *= P.c2[l];
            s += DTh * r;
            P.r[slotRh[k]][l][p.i] = r;
        }
        u *= opS;
        Sh[k] = s + u;
    }
    if (P.fs && p.y == 0) {
        // FreeSurfaceViscoelastic::setModelparameter (FreeSurfaceViscoelastic.cpp:12-97)
        float temp = -2.0f * mu * opS;
        float temp2 = M * opP;
        temp += temp2;
        const float itemp2 = 1.0f / temp2;
        const float sV = temp;
        float sH = -1.0f * temp;
        sH *= temp;
        sH *= itemp2;
        const float hsum = P.is3d ? vxx + vzz : vxx;
        const int nx = P.is3d ? 2 : 1;
        const int kk[2] = {0, 2};
        #pragma unroll
        for (int l = 0; l < kMaxL; ++l) if (l < L)
            #pragma unroll
            for (int q = 0; q < 2; ++q) if (q < nx) S[kk[q]] -= DTh * R[kk[q]][l];
        #pragma unroll
        for (int q = 0; q < 2; ++q) if (q < nx) S[kk[q]] += sH * hsum;
        #pragma unroll
        for (int q = 0; q < 2; ++q) if (q < nx) S[kk[q]] -= sV * vyy;
        float t3 = 2.0f * mu * tauS;
        t3 -= M * tauP;
        float ratio = 2.0f * mu * opS;
        ratio /= M * opP;
        ratio -= 1.0f;
        #pragma unroll
        for (int l = 0; l < kMaxL; ++l) if (l < L) {
            float rv = t3; rv *= P.c2[l]; rv /= P.relaxTime[l];
            float rh = t3; rh *= ratio; rh *= P.c2[l]; rh /= P.relaxTime[l];
            #pragma unroll
            for (int q = 0; q < 2; ++q) if (q < nx) {
                R[kk[q]][l] += rh * hsum;
                R[kk[q]][l] -= rv * vyy;
                S[kk[q]] += DTh * R[kk[q]][l];
            }
        }
        S[1] = 0.0f;
        #pragma unroll
        for (int l = 0; l < kMaxL; ++l) if (l < L) R[1][l] = 0.0f;
    }
    if (P.abs) {
        const float d = absDamp(P, p);
        #pragma unroll
        for (int k = 0; k < 3; ++k) if (k < nN) S[k] *= d;
        #pragma unroll
        for (int k = 0; k < 3; ++k) if (k < nS) Sh[k] *= d;
    }
    #pragma unroll
    for (int k = 0; k < 3; ++k) if (k < nN) {
        P.f[slotS[k]][p.i] = S[k];
        #pragma unroll
        for (int l = 0; l < kMaxL; ++l) if (l < L) P.r[slotR[k]][l][p.i] = R[k][l];
    }
    #pragma unroll
    for (int k = 0; k < 3; ++k) if (k < nS) P.f[slotSh[k]][p.i] = Sh[k];
}

template <int H>
__global__ void __launch_bounds__(256, 5) visco_s(StepParams P)   // 48 registers: 5 blocks per SM (4.4 % faster than 64 at 4)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    visco_s_body<H>(P, p);
}

template <int H>
__global__ void __launch_bounds__(256) visco_s_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { visco_s_body<H>(P, p); });
}

// --------------------------------------------------------------------------
// SH / visco-SH: ForwardSolver2Dsh.cpp:137-190, ForwardSolver2Dviscosh.cpp:155-240
// --------------------------------------------------------------------------
template <int H>
__device__ __forceinline__ void sh_v_body(const StepParams& P, const Pt& p)
{
    float u = dX<H, false>(P, p, P.f[F_SXZ], P.Dxb, PS_SXZ_X);
    float ut = P.fs ? dY<H, false>(P, p, P.f[F_SYZ], P.DybS, PS_SYZ_Y) : dY<H, false>(P, p, P.f[F_SYZ], P.Dyb, PS_SYZ_Y);
    u += ut;
    u *= LD(P.m[M_IR]);
    P.f[F_VZ][p.i] += u;
}

template <int H>
__global__ void __launch_bounds__(256) sh_v(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    sh_v_body<H>(P, p);
}

template <int H>
__global__ void __launch_bounds__(256) sh_v_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { sh_v_body<H>(P, p); });
}

template <int H>
__device__ __forceinline__ void sh_s_body(const StepParams& P, const Pt& p)
{
    const float* vz = P.f[F_VZ];
    const float d = P.abs ? absDamp(P, p) : 1.0f;
    for (int k = 0; k < 2; ++k) {
        float u = k == 0 ? dX<H, true>(P, p, vz, P.Dxf, PS_VZX) : dY<H, true>(P, p, vz, P.Dyf, PS_VZY);
        u *= LD(P.m[k == 0 ? M_MUXZ : M_MUYZ]);
        float s = P.f[k == 0 ? F_SXZ : F_SYZ][p.i];
        if (P.L > 0) {
            const float tauAv = LD(P.m[k == 0 ? M_TAUSXZ : M_TAUSYZ]);
            const int rs = k == 0 ? R_XZ : R_YZ;
            for (int l = 0; l < P.L; ++l) {
                float r = P.r[rs][l][p.i];
                s += P.DThalf * r;
                r *= P.c1[l];
                float u2 = P.invRelax[l] * u;
                u2 *= tauAv;
                r -= u2;
                r *= P.c2[l];
                s += P.DThalf * r;
                P.r[rs][l][p.i] = r;
            }
            u *= LD(P.m[M_OPLTS]);
        }
        s += u;
        P.f[k == 0 ? F_SXZ : F_SYZ][p.i] = s * d;
    }
}

template <int H>
__global__ void __launch_bounds__(256) sh_s(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    sh_s_body<H>(P, p);
}

template <int H>
__global__ void __launch_bounds__(256) sh_s_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { sh_s_body<H>(P, p); });
}

// --------------------------------------------------------------------------
// ABS damping of the pass-1 fields (applied after pass 2 read them).
// --------------------------------------------------------------------------
__device__ __forceinline__ void abs_frame_body(const StepParams& P, const Pt& p, int f0, int f1, int f2)
{
    const float d = absDamp(P, p);
    if (d == 1.0f) return;
    if (f0 >= 0) P.f[f0][p.i] *= d;
    if (f1 >= 0) P.f[f1][p.i] *= d;
    if (f2 >= 0) P.f[f2][p.i] *= d;
}

__global__ void __launch_bounds__(256) abs_frame_kernel(StepParams P, int f0, int f1, int f2)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    abs_frame_body(P, p, f0, f1, f2);
}

__global__ void __launch_bounds__(256) abs_frame_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S,
                                                       int f0, int f1, int f2)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [=](const StepParams& P, const Pt& p, int) { abs_frame_body(P, p, f0, f1, f2); });
}

// --------------------------------------------------------------------------
// sources + receivers (SourceReceiverImpl.cpp:12-37 and the pressure variants
// FDTDacoustic.cpp, FDTD2Delastic.cpp:12-49, FDTD3Delastic.cpp:12-53,
// SourceReceiverImplEM.cpp): the raw sample of column t is added, then the
// receivers copy column t. One block; t read from a device counter so the
// same launch can be replayed from a CUDA graph.
// --------------------------------------------------------------------------
// field_of and srcrec_body: stencil.cuh (shared with the variable-grid step)

__global__ void __launch_bounds__(512) srcrec_kernel(SrcRecParams Q, int* tcounter)
{
    dependent_launch_prologue();
    srcrec_body(Q, tcounter);
}

// Many receivers: the sources (and the step counter) in one block, then the
// receivers over a grid, so the gather is not one block's serial loop of
// dependent loads. The receiver launch reads the step the source launch
// advanced the counter past.
__global__ void __launch_bounds__(512) sources_kernel(SrcRecParams Q, int* tcounter)
{
    dependent_launch_prologue();
    srcrec_body(Q, tcounter, false);
}

__global__ void __launch_bounds__(256) receivers_kernel(SrcRecParams Q, const int* tcounter)
{
    dependent_launch_prologue();
    receivers_body(Q, *tcounter - 1, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// one block per shot, each with its own step counter
__global__ void __launch_bounds__(512) srcrec_batch(const SrcRecParams* __restrict__ Qs, int* tcounters)
{
    srcrec_body(Qs[blockIdx.x], tcounters + blockIdx.x);
}

// --------------------------------------------------------------------------
// NaN/Inf status (Simulation.cpp:519, WavefieldsSeismic.cpp:12-40) over every
// point of a buffer; sets *flag when a non-finite value is found.
// --------------------------------------------------------------------------
__global__ void finite_kernel(const float* __restrict__ a, long long n, int* flag)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (!isfinite(a[i])) { *flag = 1; return; }
    }
}

// --------------------------------------------------------------------------
// model preparation (Modelparameter::prepareForModelling and the solvers'
// prepareForModelling), all on the device.
// --------------------------------------------------------------------------
__device__ __forceinline__ long long gidx(const PrepParams& G, int x, int y, int z) { return x + (long long)G.NX * (z + (long long)G.NZ * y); }

__device__ __forceinline__ void gcoord(const PrepParams& G, long long i, int& x, int& y, int& z)
{
    y = (int)(i / ((long long)G.NX * G.NZ));
    long long r = i - (long long)y * G.NX * G.NZ;
    z = (int)(r / G.NX);
    x = (int)(r - (long long)z * G.NX);
}

// 2-point average along an axis with the last point copied
// (Modelparameter::calcAverageMatrixX/Y/Z, Modelparameter.cpp:336-420)
__device__ __forceinline__ float avg2(const PrepParams& G, const float* a, long long i, int x, int y, int z, int axis)
{
    int nx = x, ny = y, nz = z;
    bool ok;
    if (axis == 0) { nx = x + 1; ok = nx < G.NX; }
    else if (axis == 1) { ny = y + 1; ok = ny < G.NY; }
    else { nz = z + 1; ok = nz < G.NZ; }
    if (!ok) return 1.0f * a[i];
    float s = 0.5f * a[i];
    s += 0.5f * a[gidx(G, nx, ny, nz)];
    return s;
}

// 4-point average in a plane with the edge fallbacks of
// calc4PointAverageMatrixRow (Modelparameter.cpp:448-527). plane 0=XY,1=XZ,2=YZ.
__device__ float avg4(const PrepParams& G, const float* a, long long i, int x, int y, int z, int plane)
{
    int p2x = x, p2y = y, p2z = z, p3x = x, p3y = y, p3z = z, p4x = x, p4y = y, p4z = z;
    if (plane == 0) { p2x = x + 1; p3y = y + 1; p4x = x + 1; p4y = y + 1; }
    else if (plane == 1) { p2x = x + 1; p3z = z + 1; p4x = x + 1; p4z = z + 1; }
    else { p2y = y + 1; p3z = z + 1; p4y = y + 1; p4z = z + 1; }
    const int maxX = max(x, max(p2x, max(p3x, p4x)));
    const int maxY = max(y, max(p2y, max(p3y, p4y)));
    const int maxZ = max(z, max(p2z, max(p3z, p4z)));
    const bool inX = maxX < G.NX, inY = maxY < G.NY, inZ = maxZ < G.NZ;
    if (inX && inY && inZ) {
        float s = 0.25f * a[i];
        s += 0.25f * a[gidx(G, p2x, p2y, p2z)];
        s += 0.25f * a[gidx(G, p3x, p3y, p3z)];
        s += 0.25f * a[gidx(G, p4x, p4y, p4z)];
        return s;
    }
    if (inX && !inY && inZ) { float s = 0.5f * a[gidx(G, maxX, y, maxZ)]; s += 0.5f * a[i]; return s; }
    if (!inX && inY && inZ) { float s = 0.5f * a[gidx(G, x, maxY, maxZ)]; s += 0.5f * a[i]; return s; }
    if (inX && inY && !inZ) { float s = 0.5f * a[gidx(G, maxX, maxY, z)]; s += 0.5f * a[i]; return s; }
    if ((!inX && !inY && inZ) || (inX && !inY && !inZ) || (!inX && inY && !inZ)) return 1.0f * a[i];
    return 0.0f;
}

__device__ __forceinline__ float inv_valid(float v)
{
    // calcInverseAveragedParameter + Common::replaceInvalid (Modelparameter.cpp:633-639)
    float r = 1.0f / v;
    return isfinite(r) ? r : 0.0f;
}

#define PREP_LOOP for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < G.N; i += (long long)gridDim.x * blockDim.x)

// modulus = rho * v * v, divided by (1 + sum*tau) for visco media
// (ModelparameterSeismic.cpp:131-136, Viscoelastic.cpp:650-715); optional clamp
// of values below 1 (ModelparameterSeismic.cpp:424).
__global__ void prep_modulus(PrepParams G, const float* rho, const float* v, const float* tau, float sum, int clamp, float* out)
{
    PREP_LOOP {
        float s = rho[i];
        s *= v[i];
        s *= v[i];
        if (tau) s = s / (1.0f + sum * tau[i]);
        if (clamp && s < 1.0f) s = 1.0f;
        out[i] = s;
    }
}

__global__ void prep_inverse(PrepParams G, const float* a, float* out)
{
    PREP_LOOP { out[i] = 1.0f / a[i]; }
}

__global__ void prep_inv_avg2(PrepParams G, const float* a, int axis, float* out)
{
    PREP_LOOP {
        int x, y, z;
        gcoord(G, i, x, y, z);
        out[i] = inv_valid(avg2(G, a, i, x, y, z, axis));
    }
}

__global__ void prep_inv_avg4(PrepParams G, const float* a, int plane, float* out)
{
    PREP_LOOP {
        int x, y, z;
        gcoord(G, i, x, y, z);
        out[i] = inv_valid(avg4(G, a, i, x, y, z, plane));
    }
}

__global__ void prep_avg2(PrepParams G, const float* a, int axis, float* out)
{
    PREP_LOOP {
        int x, y, z;
        gcoord(G, i, x, y, z);
        out[i] = avg2(G, a, i, x, y, z, axis);
    }
}

__global__ void prep_avg4(PrepParams G, const float* a, int plane, float* out)
{
    PREP_LOOP {
        int x, y, z;
        gcoord(G, i, x, y, z);
        out[i] = avg4(G, a, i, x, y, z, plane);
    }
}

// harmonic S-modulus average with the vacuum threshold
// (ModelparameterSeismic::calcAveragedSWaveModulus, ModelparameterSeismic.cpp:421-432):
// mu_av = 1 / A*(1/mu), values below 4 set to 0. mode: 0..2 = 4-point plane, 3+axis = 2-point
__global__ void prep_harmonic(PrepParams G, const float* invmu, int mode, float* out)
{
    PREP_LOOP {
        int x, y, z;
        gcoord(G, i, x, y, z);
        float av = mode < 3 ? avg4(G, invmu, i, x, y, z, mode) : avg2(G, invmu, i, x, y, z, mode - 3);
        float r = 1.0f / av;
        out[i] = r < 4.0f ? 0.0f : r;
    }
}

// 1/mu with moduli below 1 raised to 1 (ModelparameterSeismic.cpp:424-426)
__global__ void prep_inv_clamped(PrepParams G, const float* mu, float* out)
{
    PREP_LOOP {
        const float m = mu[i] < 1.0f ? 1.0f : mu[i];
        out[i] = 1.0f / m;
    }
}

__global__ void prep_one_plus(PrepParams G, const float* tau, float L, float* out)
{
    PREP_LOOP { out[i] = 1.0f + L * tau[i]; }
}

__global__ void prep_scale(PrepParams G, const float* a, float s, float* out)
{
    PREP_LOOP { out[i] = a[i] * s; }
}

// Ca, Cb (ForwardSolverEM.cpp:14-66)
__global__ void prep_cacb(PrepParams G, const float* eps, const float* sig, float DT, float* ca, float* cb)
{
    PREP_LOOP {
        float c = 0.5f / eps[i];
        c *= sig[i];
        c *= DT;
        c += 1.0f;
        const float cinv = 1.0f / c;
        float a = 0.5f / eps[i];
        a *= sig[i];
        a *= DT;
        a = 1.0f - a;
        ca[i] = a * cinv;
        float b = 1.0f / eps[i];
        cb[i] = b * cinv;
    }
}

// --------------------------------------------------------------------------
// launch table
// --------------------------------------------------------------------------
#define WAVE_KTAB(name) { name<1>, name<2>, name<3>, name<4>, name<5>, name<6> }

StepKernel kernel_for(int eq, int pass, int H)
{
    static const StepKernel ac_v[6] = WAVE_KTAB(acoustic_v), ac_p[6] = WAVE_KTAB(acoustic_p);
    static const StepKernel el_v[6] = WAVE_KTAB(elastic_v), el_s[6] = WAVE_KTAB(elastic_s), vi_s[6] = WAVE_KTAB(visco_s);
    static const StepKernel s_v[6] = WAVE_KTAB(sh_v), s_s[6] = WAVE_KTAB(sh_s);
    if (H < 1 || H > 6) return nullptr;
    if (eq >= WAVE_EQ_TMEM) return em_kernel_for(eq, pass, H);   // kernels_em.cu
    const int k = H - 1;
    switch (eq) {
    case WAVE_EQ_ACOUSTIC: return pass == 0 ? ac_v[k] : ac_p[k];
    case WAVE_EQ_ELASTIC: return pass == 0 ? el_v[k] : el_s[k];
    case WAVE_EQ_VISCOELASTIC: return pass == 0 ? el_v[k] : vi_s[k];
    case WAVE_EQ_SH:
    case WAVE_EQ_VISCOSH: return pass == 0 ? s_v[k] : s_s[k];
    default: return nullptr;
    }
}

__global__ void set_counter_kernel(int* c, int v) { *c = v; }

void launch_set_counter(int* c, int v, cudaStream_t s) { set_counter_kernel<<<1, 1, 0, s>>>(c, v); }

BatchKernel batch_kernel_for(int eq, int pass, int H)
{
    static const BatchKernel ac_v[6] = WAVE_KTAB(acoustic_v_batch), ac_p[6] = WAVE_KTAB(acoustic_p_batch);
    static const BatchKernel el_v[6] = WAVE_KTAB(elastic_v_batch), el_s[6] = WAVE_KTAB(elastic_s_batch), vi_s[6] = WAVE_KTAB(visco_s_batch);
    static const BatchKernel s_v[6] = WAVE_KTAB(sh_v_batch), s_s[6] = WAVE_KTAB(sh_s_batch);
    if (H < 1 || H > 6) return nullptr;
    if (eq >= WAVE_EQ_TMEM) return em_batch_kernel_for(eq, pass, H);   // kernels_em.cu
    const int k = H - 1;
    switch (eq) {
    case WAVE_EQ_ACOUSTIC: return pass == 0 ? ac_v[k] : ac_p[k];
    case WAVE_EQ_ELASTIC: return pass == 0 ? el_v[k] : el_s[k];
    case WAVE_EQ_VISCOELASTIC: return pass == 0 ? el_v[k] : vi_s[k];
    case WAVE_EQ_SH:
    case WAVE_EQ_VISCOSH: return pass == 0 ? s_v[k] : s_s[k];
    default: return nullptr;
    }
}

void launch_batch_pass(int eq, int pass, int H, const StepParams* Ps, const BatchTile* tiles, const BatchSched& S, int grid,
                       cudaStream_t s)
{
    BatchKernel k = batch_kernel_for(eq, pass, H);
    if (k && S.ntiles > 0) k<<<grid, dim3(32, 8, 1), S.smem, s>>>(Ps, tiles, S);
}

void launch_batch_aux(const StepParams* Ps, const BatchTile* tiles, const BatchSched& S, int grid, int f0, int f1, int f2,
                      const SrcRecParams* Qs, int* counters, int nshots, bool abs, cudaStream_t s)
{
    if (abs && S.ntiles > 0) abs_frame_batch<<<grid, dim3(32, 8, 1), 0, s>>>(Ps, tiles, S, f0, f1, f2);
    if (nshots > 0) srcrec_batch<<<nshots, 512, 0, s>>>(Qs, counters);
}

int batch_blocks_per_sm(int eq, int H, int smem)
{
    BatchKernel k = batch_kernel_for(eq, 0, H), k2 = batch_kernel_for(eq, 1, H);
    int a = 0, b = 0;
    if (!k || !k2) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k, 256, smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k2, 256, smem) != cudaSuccess) return 0;
    return a < b ? a : b;
}

// the largest staging area of an interior tile (two blocks still fit an SM)
constexpr long long kTileSmemMax = 96 * 1024;

int batch_tile_smem(int eq, int H, int cols, int rows)
{
    if (eq != WAVE_EQ_TMEM || H < 1 || H > 6 || cols < 1 || rows < 1 || cols > 1024 || rows > 1024) return 0;
    const long long C = cols, R = rows, h = 2 * H - 1;
    const long long hPass = (C + h) * (R + h) + 4 * C * R;           // Ez with halo; 1/mu x 2; Hx; Hy
    const long long ePass = (C + h) * R + C * (R + h) + 3 * C * R;   // Hy, Hx with halos; Ez; Ca; Cb
    const long long bytes = 4 * (hPass > ePass ? hPass : ePass);
    if (bytes > kTileSmemMax) return 0;
    BatchKernel k0 = batch_kernel_for(eq, 0, H), k1 = batch_kernel_for(eq, 1, H);
    if (cudaFuncSetAttribute(k0, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)) != cudaSuccess ||
        cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return static_cast<int>(bytes);
}

__global__ void set_counters_kernel(int* c, int n, int v)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x) c[i] = v;
}

void launch_set_counters(int* c, int n, int v, cudaStream_t s) { set_counters_kernel<<<1, 256, 0, s>>>(c, n, v); }

// Launch with programmatic stream serialization when dep is set: the kernel's
// blocks may be scheduled before its predecessor in the stream completes and
// wait in dependent_launch_prologue (kernel launch latency hidden on small grids).
template <typename... Args>
cudaError_t launch_maybe_dependent(void (*k)(Args...), dim3 grid, dim3 block, bool dep, cudaStream_t s, Args... args)
{
    cudaLaunchConfig_t c{};
    c.gridDim = grid;
    c.blockDim = block;
    c.stream = s;
    cudaLaunchAttribute a[1];
    a[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    a[0].val.programmaticStreamSerializationAllowed = 1;
    c.attrs = a;
    c.numAttrs = dep ? 1 : 0;
    return cudaLaunchKernelEx(&c, k, args...);
}

cudaError_t launch_step_kernel(StepKernel k, dim3 grid, dim3 block, const StepParams& P, bool dep, cudaStream_t s)
{
    return launch_maybe_dependent(k, grid, block, dep, s, P);
}

int launch_srcrec(const SrcRecParams& Q, int* tcounter, cudaStream_t s, bool dep)
{
    if (Q.nrec > kSplitReceivers) {
        launch_maybe_dependent(sources_kernel, dim3(1), dim3(512), dep, s, Q, tcounter);
        const int blocks = (Q.nrec + 255) / 256;
        launch_maybe_dependent(receivers_kernel, dim3(blocks), dim3(256), dep, s, Q, static_cast<const int*>(tcounter));
        return 2;
    }
    launch_maybe_dependent(srcrec_kernel, dim3(1), dim3(512), dep, s, Q, tcounter);
    return 1;
}

void launch_abs_frame(const StepParams& P, dim3 grid, dim3 block, int f0, int f1, int f2, cudaStream_t s, bool dep)
{
    launch_maybe_dependent(abs_frame_kernel, grid, block, dep, s, P, f0, f1, f2);
}

void launch_finite(const float* a, long long n, int* flag, cudaStream_t s)
{
    finite_kernel<<<1216, 256, 0, s>>>(a, n, flag);
}

// model preparation launchers
#define PREP_GRID 1216, 256, 0, s
void k_modulus(PrepParams G, const float* rho, const float* v, const float* tau, float sum, int clamp, float* out, cudaStream_t s) { prep_modulus<<<PREP_GRID>>>(G, rho, v, tau, sum, clamp, out); }
void k_inverse(PrepParams G, const float* a, float* out, cudaStream_t s) { prep_inverse<<<PREP_GRID>>>(G, a, out); }
void k_inv_avg2(PrepParams G, const float* a, int axis, float* out, cudaStream_t s) { prep_inv_avg2<<<PREP_GRID>>>(G, a, axis, out); }
void k_inv_avg4(PrepParams G, const float* a, int plane, float* out, cudaStream_t s) { prep_inv_avg4<<<PREP_GRID>>>(G, a, plane, out); }
void k_avg2(PrepParams G, const float* a, int axis, float* out, cudaStream_t s) { prep_avg2<<<PREP_GRID>>>(G, a, axis, out); }
void k_avg4(PrepParams G, const float* a, int plane, float* out, cudaStream_t s) { prep_avg4<<<PREP_GRID>>>(G, a, plane, out); }
void k_harmonic(PrepParams G, const float* invmu, int mode, float* out, cudaStream_t s) { prep_harmonic<<<PREP_GRID>>>(G, invmu, mode, out); }
void k_inv_clamped(PrepParams G, const float* mu, float* out, cudaStream_t s) { prep_inv_clamped<<<PREP_GRID>>>(G, mu, out); }
void k_one_plus(PrepParams G, const float* tau, float L, float* out, cudaStream_t s) { prep_one_plus<<<PREP_GRID>>>(G, tau, L, out); }
void k_scale(PrepParams G, const float* a, float sc, float* out, cudaStream_t s) { prep_scale<<<PREP_GRID>>>(G, a, sc, out); }
void k_cacb(PrepParams G, const float* eps, const float* sig, float DT, float* ca, float* cb, cudaStream_t s) { prep_cacb<<<PREP_GRID>>>(G, eps, sig, DT, ca, cb); }

struct CdOut {
    float* p[kMaxL];
};

// Visco-EM coefficients of one E component from its (averaged) static
// permittivity, conductivity and relaxation parameters: effective optical
// permittivity (clamped below at eps0) and conductivity, Ca/Cb, and C_d per
// mechanism (ForwardSolverEM.cpp:14-152).
__global__ void prep_visco_em(PrepParams G, const float* eps, const float* sig, const float* te, const float* ts, ViscoEmCoef c,
                              float* ca, float* cb, CdOut cd)
{
    PREP_LOOP {
        float eo = 1.0f - te[i];
        eo *= eps[i];
        const float tmp = sig[i] * ts[i];
        eo += tmp;
        if (eo < c.eps0) eo = c.eps0;
        float so = te[i] * c.sumInv;
        so *= eps[i];
        so += sig[i];
        float q = 0.5f / eo;
        q *= so;
        q *= c.DT;
        q += 1.0f;
        const float cinv = 1.0f / q;
        float a = 0.5f / eo;
        a *= so;
        a *= c.DT;
        a = 1.0f - a;
        ca[i] = a * cinv;
        const float b = 1.0f / eo;
        cb[i] = b * cinv;
        for (int l = 0; l < c.L; ++l) {
            float v = te[i] * c.cdScale[l];
            v *= eps[i];
            v *= -c.DT;
            cd.p[l][i] = v;
        }
    }
}

void k_visco_em(PrepParams G, const float* eps, const float* sig, const float* te, const float* ts, const ViscoEmCoef& c,
                float* ca, float* cb, float* const* cd, cudaStream_t s)
{
    CdOut o{};
    for (int l = 0; l < c.L && l < kMaxL; ++l) o.p[l] = cd[l];
    prep_visco_em<<<PREP_GRID>>>(G, eps, sig, te, ts, c, ca, cb, o);
}

} // namespace wave
