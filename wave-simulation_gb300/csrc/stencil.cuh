// stencil.cuh — device helpers shared by the step kernels (kernels.cu) and the
// adjoint kernels (adjoint.cu): matrix-free derivative rows, slab-compacted
// CPML psi indexing, point mapping of the one-thread-per-point launches, ABS
// taper.
#pragma once

#include <cuda_runtime.h>

#include "wave_internal.h"

namespace wave {

// --------------------------------------------------------------------------
// device helpers
// --------------------------------------------------------------------------
// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may be scheduled while its predecessor in the stream still
// runs. It first lets its own dependent launch be scheduled, then waits until
// the predecessor has completed and its writes are visible; no global memory
// is touched before the wait. Both instructions are no-ops in a normal launch.
__device__ __forceinline__ void dependent_launch_prologue()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// 1-D derivative along an axis with stride `st`; c = coordinate along the axis.
// FWD: taps at offsets -H+1..H, else -H..H-1 (Derivatives.cpp:149, 728).
template <int H, bool FWD>
__device__ __forceinline__ float deriv(const float* __restrict__ u, long long i, long long st, int c, const Op1D& op)
{
    float s = 0.0f;
    if (!op.full && c >= op.E && c < op.n - op.E) {
#pragma unroll
        for (int k = (FWD ? -H + 1 : -H); k <= (FWD ? H : H - 1); ++k)
            s += op.w[kMaxHalf + k] * __ldg(u + i + k * st);
    } else {
        const int slot = op.full ? c : (c < op.E ? c : op.E + c - (op.n - op.E));
        const float* t = op.tab + slot * kTabW + kMaxHalf;
#pragma unroll
        for (int k = -H; k <= H; ++k) {
            const int cc = c + k;
            const float wk = __ldg(t + k);
            if (cc >= 0 && cc < op.n && wk != 0.0f) s += wk * __ldg(u + i + k * st);
        }
    }
    return s;
}

// index into a slab-compacted psi array along an axis (-1: outside the slabs)
__device__ __forceinline__ int slab(int c, const Cpml1D& p)
{
    if (p.n <= 2 * p.w) return c;
    if (c < p.w) return p.lo ? c : -1;
    if (c >= p.n - p.w) return c - (p.n - p.ns);
    return -1;
}

// CPML::applyCPML (CPML.cpp:84-95): psi = b*psi + a*d; d += psi
__device__ __forceinline__ void cpml(float& d, float* __restrict__ psi, long long pidx, float a, float b)
{
    float ps = psi[pidx] * b;
    ps += a * d;
    psi[pidx] = ps;
    d += ps;
}

struct Pt {
    int x, y, z;
    long long i;
};

__device__ __forceinline__ bool point(const StepParams& P, Pt& p)
{
    p.x = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y * blockDim.y + threadIdx.y;
    if (p.x >= P.NX || r >= P.NY * P.NZ) return false;
    if (P.NZ == 1) {   // 2-D: no division
        p.y = r;
        p.z = 0;
    } else {
        p.y = r / P.NZ;
        p.z = r - p.y * P.NZ;
    }
    p.i = p.x + (long long)P.NX * (p.z + (long long)P.NZ * p.y);
    return true;
}

// batched launches: one block per (shot, 32 x kTileRows tile); the shot's
// parameters are staged in shared memory once per block
__device__ __forceinline__ void load_params(StepParams& dst, const StepParams* src)
{
    const int n = sizeof(StepParams) / sizeof(int);
    int* d = reinterpret_cast<int*>(&dst);
    const int* sp = reinterpret_cast<const int*>(src);
    for (int k = threadIdx.y * blockDim.x + threadIdx.x; k < n; k += blockDim.x * blockDim.y) d[k] = sp[k];
    __syncthreads();
}

// Shared-memory copy of a shot's StepParams in a batched kernel (raw storage:
// StepParams has default member initialisers, which a __shared__ object
// cannot run; load_params fills every byte).
#define BATCH_SHARED_PARAMS(name)                                                  \
    __shared__ __align__(16) unsigned char name##_mem[sizeof(StepParams)];          \
    StepParams& name = *reinterpret_cast<StepParams*>(name##_mem)

// The points of one tile of a batched launch: the 32 x 8 block covers
// S.cols x S.rows points in column groups of 32 and row groups of 8.
// body(params, point).
template <class Body>
__device__ __forceinline__ void tile_points(const StepParams& sP, const BatchTile& w, const BatchSched& S, Body body)
{
    for (int xg = 0; xg < S.cols; xg += 32) {
        const int x = w.x0 + xg + static_cast<int>(threadIdx.x);
        // four row groups per pass, unrolled, so that their (read-only
        // path) loads overlap: these kernels are bound by load latency
        for (int r0 = 0; r0 < S.rows; r0 += 32) {
#pragma unroll
            for (int g = 0; g < 4; ++g) {
                const int rr = r0 + 8 * g;
                const int r = w.r0 + rr + static_cast<int>(threadIdx.y);
                if (rr >= S.rows || x >= sP.NX || r >= sP.NY * sP.NZ) continue;
                Pt p;
                p.x = x;
                if (sP.NZ == 1) {   // 2-D: no division
                    p.y = r;
                    p.z = 0;
                } else {
                    p.y = r / sP.NZ;
                    p.z = r - p.y * sP.NZ;
                }
                p.i = p.x + (long long)sP.NX * (p.z + (long long)sP.NZ * p.y);
                body(sP, p);
            }
        }
    }
}

// Persistent batched launches: the block walks the work list with a grid
// stride; the parameters of a tile's shot are staged in shared memory when
// the shot changes (every thread first leaves the previous shot's).
// body(params, point, shot index).
template <class Body>
__device__ __forceinline__ void batch_loop(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, const BatchSched& S,
                                           StepParams& sP, Body body)
{
    int shot = -1;
    for (int t = blockIdx.x; t < S.ntiles; t += gridDim.x) {
        const BatchTile w = W[t];
        if (w.shot != shot) {
            __syncthreads();
            load_params(sP, Ps + w.shot);
            shot = w.shot;
        }
        tile_points(sP, w, S, [&](const StepParams& P, const Pt& p) { body(P, p, w.shot); });
    }
}

// psi indices along x / y / z for point p
__device__ __forceinline__ long long pix(const StepParams& P, const Pt& p, int s) { return s + (long long)P.cx.ns * (p.z + (long long)P.NZ * p.y); }
__device__ __forceinline__ long long piy(const StepParams& P, const Pt& p, int s) { return p.x + (long long)P.NX * (p.z + (long long)P.NZ * s); }
__device__ __forceinline__ long long piz(const StepParams& P, const Pt& p, int s) { return p.x + (long long)P.NX * (s + (long long)P.cz.ns * p.y); }

// derivative + CPML along x / y / z. HALF: the half-grid profile, by default
// for forward-type derivatives (CPML3D.cpp:31-153).
template <int H, bool FWD, bool HALF = FWD>
__device__ __forceinline__ float dX(const StepParams& P, const Pt& p, const float* u, const Op1D& op, int psiSlot)
{
    float d = deriv<H, FWD>(u, p.i, 1, p.x, op);
    if (P.useCpml) {
        int s = slab(p.x, P.cx);
        if (s >= 0) {
            const float a = HALF ? P.cx.a_half[p.x] : P.cx.a_full[p.x];
            const float b = HALF ? P.cx.b_half[p.x] : P.cx.b_full[p.x];
            cpml(d, P.psi[psiSlot], pix(P, p, s), a, b);
        }
    }
    return d;
}
template <int H, bool FWD, bool HALF = FWD>
__device__ __forceinline__ float dY(const StepParams& P, const Pt& p, const float* u, const Op1D& op, int psiSlot)
{
    float d = deriv<H, FWD>(u, p.i, (long long)P.NX * P.NZ, p.y, op);
    if (P.useCpml) {
        int s = slab(p.y, P.cy);
        if (s >= 0) {
            const float a = HALF ? P.cy.a_half[p.y] : P.cy.a_full[p.y];
            const float b = HALF ? P.cy.b_half[p.y] : P.cy.b_full[p.y];
            cpml(d, P.psi[psiSlot], piy(P, p, s), a, b);
        }
    }
    return d;
}
template <int H, bool FWD, bool HALF = FWD>
__device__ __forceinline__ float dZ(const StepParams& P, const Pt& p, const float* u, const Op1D& op, int psiSlot)
{
    float d = deriv<H, FWD>(u, p.i, P.NX, p.z, op);
    if (P.useCpml) {
        int s = slab(p.z, P.cz);
        if (s >= 0) {
            const float a = HALF ? P.cz.a_half[p.z] : P.cz.a_full[p.z];
            const float b = HALF ? P.cz.b_half[p.z] : P.cz.b_full[p.z];
            cpml(d, P.psi[psiSlot], piz(P, p, s), a, b);
        }
    }
    return d;
}

// ABS taper at a point (ABS2D.cpp:110-180, ABS3D.cpp:154-220); 1 outside the frame.
__device__ __forceinline__ float absDamp(const StepParams& P, const Pt& p)
{
    const int w = P.absW;
    auto edge = [](int c, int n) { return !((n - 1 - c) < c) ? c : (n - 1 - c); };
    const int dx = edge(p.x, P.NX), dy = edge(p.y, P.NY), dz = edge(p.z, P.NZ);
    int m;
    if (!P.is3d) {
        m = dx < dy ? dx : dy;
        if (P.fs && p.y < w) return dx < w ? P.absCoeff[dx] : 1.0f;
    } else {
        m = dx < dy ? dx : dy;
        m = m < dz ? m : dz;
        if (P.fs && p.y < w) {
            const int xz = !(dx < dz) ? dz : dx;
            return (dz < w || dx < w) ? P.absCoeff[xz] : 1.0f;
        }
    }
    return m < w ? P.absCoeff[m] : 1.0f;
}


// Sources then receivers of step t = *tcounter (SourceReceiverImpl.cpp:12-37,
// FDTD*.cpp pressure variants), one block; the counter is advanced at the end
// so the same launch can be replayed from a CUDA graph.
__device__ __forceinline__ float* field_of(const SrcRecParams& Q, int type)
{
    if (Q.eq >= WAVE_EQ_TMEM) {
        switch (type) {
        case WAVE_TYPE_EZ: return Q.f[F_EZ];
        case WAVE_TYPE_EX: return Q.f[F_EX];
        case WAVE_TYPE_EY: return Q.f[F_EY];
        default: return Q.f[F_HZ];
        }
    }
    switch (type) {
    case WAVE_TYPE_VX: return Q.f[F_VX];
    case WAVE_TYPE_VY: return Q.f[F_VY];
    case WAVE_TYPE_VZ: return Q.f[F_VZ];
    default: return Q.f[F_P];
    }
}

// receivers of step t, threads [first, first + stride) ... (SourceReceiverImpl.cpp:12-19)
__device__ __forceinline__ void receivers_body(const SrcRecParams& Q, int t, int first, int stride)
{
    const bool elasticP = (Q.eq == WAVE_EQ_ELASTIC || Q.eq == WAVE_EQ_VISCOELASTIC);
    for (int r = first; r < Q.nrec; r += stride) {
        const long long i = Q.ridx[r];
        const int type = Q.rtype[r];
        float v;
        if (Q.eq < WAVE_EQ_TMEM && type == WAVE_TYPE_P && elasticP) {
            v = Q.f[F_SXX][i];
            v += Q.f[F_SYY][i];
            if (Q.is3d) { v += Q.f[F_SZZ][i]; v /= 3.0f; }
            else v *= 0.5f;
        } else {
            v = field_of(Q, type)[i];
        }
        Q.seis[(long long)r * Q.nt + t] = v;
    }
}

__device__ __forceinline__ void srcrec_body(const SrcRecParams& Q, int* tcounter, bool withReceivers = true)
{
    const int t = *tcounter;
    const bool elasticP = (Q.eq == WAVE_EQ_ELASTIC || Q.eq == WAVE_EQ_VISCOELASTIC);
    for (int type = 1; type <= 4; ++type) {
        for (int s = threadIdx.x; s < Q.nsrc; s += blockDim.x) {
            if (Q.stype[s] != type) continue;
            const float v = Q.signals[(long long)s * Q.nt + t];
            const long long i = Q.sidx[s];
            if (Q.eq < WAVE_EQ_TMEM && type == WAVE_TYPE_P && elasticP) {
                atomicAdd(Q.f[F_SXX] + i, v);
                atomicAdd(Q.f[F_SYY] + i, v);
                if (Q.is3d) atomicAdd(Q.f[F_SZZ] + i, v);
            } else {
                atomicAdd(field_of(Q, type) + i, v);
            }
        }
        __syncthreads();
    }
    if (withReceivers) receivers_body(Q, t, threadIdx.x, blockDim.x);
    __syncthreads();
    if (threadIdx.x == 0) *tcounter = t + 1;
}

} // namespace wave
