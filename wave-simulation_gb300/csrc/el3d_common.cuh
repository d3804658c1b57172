// el3d_common.cuh — pieces shared by the streaming 3-D elastic kernels
// (kernels_el3d.cu: one point per thread, 32x8 tiles; kernels_el3d_pairs.cu:
// two x-adjacent points per thread, 64x8 tiles): FD coefficients, mbarrier /
// TMA wrappers, the (tile, plane) work schedule, the stage ring control,
// per-plane CPML state, the in-kernel material averages and the host-side
// tensor-map encoder.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "el3d.h"

namespace wave {
namespace el3d {

constexpr int MAXSEG = 64;   // work segments per CTA
constexpr int NCWARP = 8;    // warps of a CTA, one per z row of the tile

// Staggered FD coefficients (Derivatives::setFDCoef, Derivatives.cpp:2000-2042)
// as compile-time constants, so that the interior taps are FFMAs with
// immediates.
__host__ __device__ constexpr float fdc(int q, int j)
{
    switch (q) {
    case 2: return j == 0 ? -1.0f : 1.0f;
    case 4: { constexpr double c[2] = {1.0 / 24.0, -9.0 / 8.0}; return static_cast<float>(j < 2 ? c[j] : -c[3 - j]); }
    case 6: { constexpr double c[3] = {-3.0 / 640.0, 25.0 / 384.0, -75.0 / 64.0}; return static_cast<float>(j < 3 ? c[j] : -c[5 - j]); }
    case 8: {
        constexpr double c[4] = {5.0 / 7168.0, -49.0 / 5120.0, 245.0 / 3072.0, -1225.0 / 1024.0};
        return static_cast<float>(j < 4 ? c[j] : -c[7 - j]);
    }
    case 10: {
        constexpr double c[5] = {-8756999275442633.0 / 73786976294838206464.0, 8142668969129685.0 / 4611686018427387904.0,
                                 -567.0 / 40960.0, 735.0 / 8192.0, -19845.0 / 16384.0};
        return static_cast<float>(j < 5 ? c[j] : -c[9 - j]);
    }
    default: {
        constexpr double c[6] = {6448335830095439.0 / 295147905179352825856.0, -1655620175512543.0 / 4611686018427387904.0,
                                 6842103786556949.0 / 2305843009213693952.0, -628618285389933.0 / 36028797018963968.0,
                                 436540475965291.0 / 4503599627370496.0, -2750204998582123.0 / 2251799813685248.0};
        return static_cast<float>(j < 6 ? c[j] : -c[11 - j]);
    }
    }
}

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t saddr(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// try_wait with a suspend-time hint: a thread whose phase is not complete
// sleeps until it completes or `ns` nanoseconds pass, instead of returning at
// once, so waiting warps do not spin through the issue slots of the warps
// that compute.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t ns)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity), "r"(ns)
        : "memory");
    return ok != 0;
}
// bounded wait: gives up after `limit` sleeps of at most 1 us (2^17: about
// 0.13 s of waiting for copies that take microseconds); the caller reports it
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = 1u << 17)
{
    for (uint32_t i = 0; i < limit; ++i)
        if (mbar_try_wait_sleep(bar, parity, 1000u)) return true;
    return false;
}
__device__ __forceinline__ void tma_load(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int z, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(saddr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(z), "r"(y), "r"(saddr(bar))
        : "memory");
}
__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// ------------------------------------------------------------- work schedule
// The CTA's work is the contiguous range [g0, g1) of the (tile, plane) space
// (plane fastest). A run of planes of one tile is a segment; a segment of
// length L takes L + 2H iterations: 2H to fill the depth queues, then one
// compute plane per iteration. Iteration k of a segment starting at plane ya
// fetches queue plane q = ya - H + k and computes plane c = ya - 2H + k.
struct Segs {
    int n;
    int tile[MAXSEG], ya[MAXSEG], len[MAXSEG];
};

__device__ __forceinline__ int build_segments(Segs& S, long long g0, long long g1, int NY, int H)
{
    int n = 0, total = 0;
    long long g = g0;
    while (g < g1 && n < MAXSEG) {
        const long long t = g / NY;
        const long long gend = g1 < (t + 1) * NY ? g1 : (t + 1) * NY;
        S.tile[n] = static_cast<int>(t);
        S.ya[n] = static_cast<int>(g - t * NY);
        S.len[n] = static_cast<int>(gend - g) + 2 * H;
        total += S.len[n];
        ++n;
        g = gend;
    }
    S.n = n;
    return total;
}

// cursor over the iterations of the CTA's segments
struct Cursor {
    int seg, k;
    __device__ __forceinline__ void advance(const Segs& S)
    {
        if (++k == S.len[seg]) { ++seg; k = 0; }
    }
};

__device__ __forceinline__ int slab_of(int c, const Cpml1D& p)
{
    if (!p.on) return -1;
    if (p.n <= 2 * p.w) return c;
    if (c < p.w) return p.lo ? c : -1;
    if (c >= p.n - p.w) return c - (p.n - p.ns);
    return -1;
}

// table row for coordinate c of an operator (edge rows only)
__device__ __forceinline__ const float* row_of(const Op1D& op, int c)
{
    const int slot = op.full ? c : (c < op.E ? c : op.E + c - (op.n - op.E));
    return op.tab + slot * kTabW + kMaxHalf;
}
__device__ __forceinline__ bool interior_of(const Op1D& op, int c) { return !op.full && c >= op.E && c < op.n - op.E; }

__device__ __forceinline__ float abs_damp(const StepParams& P, int x, int y, int z)
{
    const int w = P.absW;
    auto edge = [](int c, int n) { return !((n - 1 - c) < c) ? c : (n - 1 - c); };
    const int dx = edge(x, P.NX), dy = edge(y, P.NY), dz = edge(z, P.NZ);
    int m = dx < dy ? dx : dy;
    m = m < dz ? m : dz;
    if (P.fs && y < w) {
        const int xz = !(dx < dz) ? dz : dx;
        return (dz < w || dx < w) ? P.absCoeff[xz] : 1.0f;
    }
    return m < w ? P.absCoeff[m] : 1.0f;
}

// per-plane (CTA-uniform) state along y
struct Plane {
    int y;
    bool yi;
    int sy;
    float ayf, byf, ayh, byh;
};

__device__ __forceinline__ void plane_setup(Plane& L, const StepParams& P, int y)
{
    L.y = y;
    L.yi = interior_of(P.Dyf, y);
    L.sy = P.useCpml ? slab_of(y, P.cy) : -1;
    L.ayf = L.byf = L.ayh = L.byh = 0.0f;
    if (L.sy >= 0) { L.ayf = P.cy.a_full[y]; L.byf = P.cy.b_full[y]; L.ayh = P.cy.a_half[y]; L.byh = P.cy.b_half[y]; }
}

__device__ __forceinline__ void report(int* err, int code)
{
    if (err) atomicExch(err, code);
}


// Box coordinate (along x or z) of a tile's CPML memory-variable box in the
// compact slab layout, or kNoBox when the tile lies outside both slabs. The
// host checks that no tile meets both slabs of an axis.
constexpr int kNoBox = -(1 << 30);

__device__ __forceinline__ int slab_box(const Cpml1D& p, int c0, int T)
{
    if (!p.on) return kNoBox;
    if (p.n <= 2 * p.w) return c0;
    if (p.lo && c0 < p.w) return c0;
    if (c0 + T > p.n - p.w) return c0 - (p.n - p.ns);
    return kNoBox;
}

// reciprocal by the hardware approximation (rcp.approx, 1 ulp)
__device__ __forceinline__ float rcp_fast(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// calcInverseAveragedParameter on a 2-point average (Modelparameter.cpp:336-420, 633-639)
__device__ __forceinline__ float inv_avg2f(float a, float b, bool in)
{
    float s;
    if (in) { s = 0.5f * a; s += 0.5f * b; }
    else s = a;
    const float r = rcp_fast(s);
    return isfinite(r) ? r : 0.0f;
}

// harmonic 4-point modulus average with the edge fallbacks of
// calc4PointAverageMatrixRow (Modelparameter.cpp:448-527) and the vacuum rule
// of calcAveragedSWaveModulus (ModelparameterSeismic.cpp:421-432). i1..i4 are
// the inverse moduli at the row point and its 2nd/3rd/4th neighbours; inA /
// inB say whether the two axes of the plane stay inside the grid.
__device__ __forceinline__ float harm4f(float i1, float i2, float i3, float i4, bool inA, bool inB)
{
    float s;
    if (inA && inB) {
        s = 0.25f * i1; s += 0.25f * i2; s += 0.25f * i3; s += 0.25f * i4;
    } else if (inA) {
        s = 0.5f * i2; s += 0.5f * i1;
    } else if (inB) {
        s = 0.5f * i3; s += 0.5f * i1;
    } else {
        s = i1;
    }
    const float r = rcp_fast(s);
    return r < 4.0f ? 0.0f : r;
}

__device__ __forceinline__ float inv_clampedf(float mu) { return rcp_fast(mu < 1.0f ? 1.0f : mu); }

// Ring control. Every stage has a release counter in shared memory that only
// grows: the warp whose release brings stage s to NCWARP x (round + 1) is the
// last reader of that round, and its lane 0 refills the stage at once with
// iteration it + NST. The copies so lead the compute by NST - 1 iterations
// and no warp ever waits for another one.
template <int NST, class IssueFn>
__device__ __forceinline__ void start_feed(const Segs& G, int total, int* issued, IssueFn issue)
{
    Cursor c{0, 0};
    int i = 0;
    for (; i < NST && i < total; ++i) {
        issue(i, c);
        c.advance(G);
    }
    *issued = i;
}

// End of iteration `it` for the calling warp: release its stage; the last
// warp to release it issues iteration it + NST into it (cursor `cur` is the
// iteration's own).
template <int NST, class IssueFn>
__device__ __forceinline__ void release_and_refill(int it, int total, const Cursor& cur, const Segs& G, unsigned* rel,
                                                   int* issued, volatile int* failed, IssueFn issue)
{
    __syncwarp();
    if ((threadIdx.x & 31) == 0) {
        const int s = it % NST;
        __threadfence_block();
        const unsigned old = atomicAdd(rel + s, 1u);
        if (old == NCWARP * static_cast<unsigned>(it / NST + 1) - 1u && it + NST < total && !*failed) {
            __threadfence_block();
            fence_proxy_async();
            Cursor c = cur;
#pragma unroll
            for (int k = 0; k < NST; ++k) c.advance(G);
            issue(s, c);
            atomicMax(issued, it + NST + 1);
        }
    }
}

// After the loop (every thread arrives): on a failed wait, thread 0 waits
// (bounded) for the copies that may still be in flight before the CTA exits.
template <int NST>
__device__ __forceinline__ void finish_ring(uint64_t* full, const int* issued, volatile int* failed)
{
    __syncthreads();
    if (threadIdx.x == 0 && *failed) {
        const int n = *reinterpret_cast<const volatile int*>(issued);
        for (int k = n > NST ? n - NST : 0; k < n; ++k) mbar_wait(full + k % NST, (k / NST) & 1);
    }
}

// common prologue: barrier init, schedule, abort check, tensor-map prefetch.
// Returns the CTA's iteration count.
template <int NST>
__device__ __forceinline__ int prologue(Segs& G, uint64_t* full, unsigned* rel, int* abortRun, volatile int* failed,
                                        const StepParams& P, const El3dSched& S, int H, const El3dMaps& T)
{
    if (threadIdx.x < sizeof(El3dMaps) / sizeof(CUtensorMap)) {
        const CUtensorMap* m = reinterpret_cast<const CUtensorMap*>(&T) + threadIdx.x;
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(m)) : "memory");
    }
    const long long GT = (long long)S.ntx * S.ntz * P.NY;
    const long long g0 = GT * blockIdx.x / gridDim.x, g1 = GT * (blockIdx.x + 1) / gridDim.x;
    if (threadIdx.x == 0) {
        // a failed wait in an earlier launch leaves the error word set: skip the work
        *abortRun = (S.err && *reinterpret_cast<volatile int*>(S.err) != 0) ? 1 : 0;
        *failed = 0;
        for (int s = 0; s < NST; ++s) {
            mbar_init(full + s, 1);
            rel[s] = 0;
        }
        fence_barrier_init();
        build_segments(G, g0, g1, P.NY, H);
    }
    __syncthreads();
    int total = 0;
    for (int k = 0; k < G.n; ++k) total += G.len[k];
    return *abortRun ? 0 : total;
}

} // namespace el3d

// ------------------------------------------------------------------------
// host side: tensor-map encoding
// ------------------------------------------------------------------------
namespace el3d_host {

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                              const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeFn encoder()
{
    static EncodeFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
    }
    return fn;
}

// 3-D fp32 map over a (d0 fastest, d1, d2) array with box (bx, bz, 1)
inline bool make_map_dims(CUtensorMap* m, const float* base, int d0, int d1, int d2, int bx, int bz)
{
    EncodeFn enc = encoder();
    if (!enc || d0 < 1 || d1 < 1 || d2 < 1) return false;
    cuuint64_t dims[3] = {(cuuint64_t)d0, (cuuint64_t)d1, (cuuint64_t)d2};
    cuuint64_t strides[2] = {(cuuint64_t)d0 * 4, (cuuint64_t)d0 * d1 * 4};
    cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)bz, 1};
    cuuint32_t es[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

inline bool make_map(CUtensorMap* m, const float* base, int NX, int NZ, int NY, int bx, int bz)
{
    EncodeFn enc = encoder();
    if (!enc) return false;
    cuuint64_t dims[3] = {(cuuint64_t)NX, (cuuint64_t)NZ, (cuuint64_t)NY};
    cuuint64_t strides[2] = {(cuuint64_t)NX * 4, (cuuint64_t)NX * NZ * 4};
    cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)bz, 1};
    cuuint32_t es[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

} // namespace el3d_host
} // namespace wave
