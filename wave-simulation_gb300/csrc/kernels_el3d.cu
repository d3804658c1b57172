// kernels_el3d.cu — streaming sm_103a kernels for the 3-D elastic time step
// (FD3Delastic::run, ForwardSolver3Delastic.cpp:120-414) on large grids.
//
// Each CTA owns a 32 (x) x 16 (z) column tile and marches it down the depth
// axis y (the slowest axis, reference layout idx = x + z*NX + y*NX*NZ). The
// CTAs are persistent: the grid is one CTA per SM and each CTA takes a
// contiguous run of (tile, plane) work, so every field plane is fetched from
// HBM once. Planes arrive through TMA bulk-tensor copies
// (cp.async.bulk.tensor.3d) into a 4-stage shared-memory ring tracked by
// mbarriers; one thread issues the copies four planes ahead of the compute.
// Depth derivatives come from per-thread register queues (2H+1 planes),
// x- and z-derivatives from the halo tiles in shared memory. The averaged
// material terms (1/rho averages, harmonic mu averages with the vacuum rules)
// are formed in-kernel from rho and mu, so the kernels read only the base
// material arrays. All waits are bounded: a wait that runs out sets the
// handle's error word and the CTA returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include "el3d.h"

namespace wave {

namespace el3d {

constexpr int TX = 32, TZ = 16, NTHR = TX * TZ, NSTAGE = 4;
constexpr int CB = TX * TZ * 4;                 // centre box bytes
constexpr int PW = TX + 4, PH = TZ + 1;          // "+1" box (x0..x0+35, z0..z0+16)
constexpr int PBYTES = PW * PH * 4;              // bytes one "+1" box copy delivers
constexpr int PB = ((PBYTES + 127) / 128) * 128; // its slot in the stage layout

__host__ __device__ constexpr int hx_of(int H) { return H <= 4 ? 4 : 8; }
__host__ __device__ constexpr int bw_of(int H) { return TX + 2 * hx_of(H); }
__host__ __device__ constexpr int bh_of(int H) { return TZ + 2 * H; }
__host__ __device__ constexpr int hbytes_of(int H) { return bw_of(H) * bh_of(H) * 4; }          // delivered
__host__ __device__ constexpr int hb_of(int H) { return ((hbytes_of(H) + 127) / 128) * 128; }  // layout slot
__host__ __device__ constexpr int vel_stage(int H) { return 5 * hb_of(H) + 6 * CB + PB; }
__host__ __device__ constexpr int str_stage(int H) { return 3 * hb_of(H) + 10 * CB + PB; }

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
// bounded wait: gives up after 2^20 polls (well under a second of waiting for
// copies that take microseconds); the caller reports it
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity)
{
    for (uint32_t i = 0; i < (1u << 20); ++i)
        if (mbar_try_wait(bar, parity)) return true;
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
struct Iter {
    int tile, q, c, ya;
    bool compute;
};

__device__ __forceinline__ bool iter_at(int it, long long g0, long long g1, int NY, int H, Iter& out)
{
    long long g = g0;
    while (g < g1) {
        const int t = static_cast<int>(g / NY);
        const int ya = static_cast<int>(g - (long long)t * NY);
        const long long gend = g1 < (long long)(t + 1) * NY ? g1 : (long long)(t + 1) * NY;
        const int len = static_cast<int>(gend - g) + 2 * H;
        if (it < len) {
            out.tile = t;
            out.ya = ya;
            out.q = ya - H + it;
            out.c = ya - 2 * H + it;
            out.compute = out.c >= ya;
            return true;
        }
        it -= len;
        g = gend;
    }
    return false;
}

__device__ __forceinline__ int total_iters(long long g0, long long g1, int NY, int H)
{
    int n = 0;
    long long g = g0;
    while (g < g1) {
        const long long t = g / NY;
        const long long gend = g1 < (t + 1) * NY ? g1 : (t + 1) * NY;
        n += static_cast<int>(gend - g) + 2 * H;
        g = gend;
    }
    return n;
}

// ------------------------------------------------------------ derivatives
// x from a halo tile (centre index ci), z from a halo tile (row stride BW),
// y from a register queue q[0..2H] holding planes c-H..c+H. Interior rows use
// the operator's interior weights; edge rows use the edge table (zero-filled
// neighbours outside the grid carry zero weight there).
template <int H, bool FWD>
__device__ __forceinline__ float d_line(const float* __restrict__ s, int ci, int stride, int c, const Op1D& op)
{
    float acc = 0.0f;
    if (!op.full && c >= op.E && c < op.n - op.E) {
#pragma unroll
        for (int k = (FWD ? -H + 1 : -H); k <= (FWD ? H : H - 1); ++k) acc += op.w[kMaxHalf + k] * s[ci + k * stride];
    } else {
        const int slot = op.full ? c : (c < op.E ? c : op.E + c - (op.n - op.E));
        const float* t = op.tab + slot * kTabW + kMaxHalf;
#pragma unroll
        for (int k = -H; k <= H; ++k) {
            const float wk = __ldg(t + k);
            if (wk != 0.0f) acc += wk * s[ci + k * stride];
        }
    }
    return acc;
}

template <int H, bool FWD>
__device__ __forceinline__ float d_queue(const float (&q)[2 * H + 1], int c, const Op1D& op)
{
    float acc = 0.0f;
    if (!op.full && c >= op.E && c < op.n - op.E) {
#pragma unroll
        for (int k = (FWD ? -H + 1 : -H); k <= (FWD ? H : H - 1); ++k) acc += op.w[kMaxHalf + k] * q[H + k];
    } else {
        const int slot = op.full ? c : (c < op.E ? c : op.E + c - (op.n - op.E));
        const float* t = op.tab + slot * kTabW + kMaxHalf;
#pragma unroll
        for (int k = -H; k <= H; ++k) {
            const float wk = __ldg(t + k);
            if (wk != 0.0f) acc += wk * q[H + k];
        }
    }
    return acc;
}

__device__ __forceinline__ int slab_of(int c, const Cpml1D& p)
{
    if (p.n <= 2 * p.w) return c;
    if (c < p.w) return p.lo ? c : -1;
    if (c >= p.n - p.w) return c - (p.n - p.ns);
    return -1;
}

__device__ __forceinline__ void cpml_x(const StepParams& P, float& d, int x, int y, int z, bool half, int slot)
{
    const int s = slab_of(x, P.cx);
    if (s < 0) return;
    float* psi = P.psi[slot] + s + (long long)P.cx.ns * (z + (long long)P.NZ * y);
    float ps = *psi * (half ? P.cx.b_half[x] : P.cx.b_full[x]);
    ps += (half ? P.cx.a_half[x] : P.cx.a_full[x]) * d;
    *psi = ps;
    d += ps;
}
__device__ __forceinline__ void cpml_y(const StepParams& P, float& d, int x, int y, int z, bool half, int slot)
{
    const int s = slab_of(y, P.cy);
    if (s < 0) return;
    float* psi = P.psi[slot] + x + (long long)P.NX * (z + (long long)P.NZ * s);
    float ps = *psi * (half ? P.cy.b_half[y] : P.cy.b_full[y]);
    ps += (half ? P.cy.a_half[y] : P.cy.a_full[y]) * d;
    *psi = ps;
    d += ps;
}
__device__ __forceinline__ void cpml_z(const StepParams& P, float& d, int x, int y, int z, bool half, int slot)
{
    const int s = slab_of(z, P.cz);
    if (s < 0) return;
    float* psi = P.psi[slot] + x + (long long)P.NX * (s + (long long)P.cz.ns * y);
    float ps = *psi * (half ? P.cz.b_half[z] : P.cz.b_full[z]);
    ps += (half ? P.cz.a_half[z] : P.cz.a_full[z]) * d;
    *psi = ps;
    d += ps;
}

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

// calcInverseAveragedParameter on a 2-point average (Modelparameter.cpp:336-420, 633-639)
__device__ __forceinline__ float inv_avg2(float a, float b, bool in)
{
    float s;
    if (in) { s = 0.5f * a; s += 0.5f * b; }
    else s = 1.0f * a;
    const float r = 1.0f / s;
    return isfinite(r) ? r : 0.0f;
}

// harmonic 4-point modulus average with the edge fallbacks of
// calc4PointAverageMatrixRow (Modelparameter.cpp:448-527) and the vacuum rule
// of calcAveragedSWaveModulus (ModelparameterSeismic.cpp:421-432). i1..i4 are
// the inverse moduli at the row point and its 2nd/3rd/4th neighbours; in2 /
// in3 say whether the two axes of the plane stay inside the grid.
__device__ __forceinline__ float harm4(float i1, float i2, float i3, float i4, bool inA, bool inB)
{
    float s;
    if (inA && inB) {
        s = 0.25f * i1; s += 0.25f * i2; s += 0.25f * i3; s += 0.25f * i4;
    } else if (inA) {       // second axis out: 2-point along the first axis
        s = 0.5f * i2; s += 0.5f * i1;
    } else if (inB) {       // first axis out: 2-point along the second axis
        s = 0.5f * i3; s += 0.5f * i1;
    } else {
        s = 1.0f * i1;
    }
    const float r = 1.0f / s;
    return r < 4.0f ? 0.0f : r;
}

__device__ __forceinline__ float inv_clamped(float mu) { return 1.0f / (mu < 1.0f ? 1.0f : mu); }

__device__ __forceinline__ void report(int* err, int code)
{
    if (err) atomicExch(err, code);
}

} // namespace el3d

using namespace el3d;

// ------------------------------------------------------------------------
// velocity pass (ForwardSolver3Delastic.cpp:174-277)
// ------------------------------------------------------------------------
template <int H>
__device__ __forceinline__ void vel_issue(const El3dMaps& T, const StepParams& P, const El3dSched& S, unsigned char* smem,
                                          uint64_t* bars, int it, long long g0, long long g1)
{
    Iter I;
    if (!iter_at(it, g0, g1, P.NY, H, I)) return;
    constexpr int HB = hb_of(H), HX = hx_of(H);
    const int s = it % NSTAGE;
    unsigned char* st = smem + s * vel_stage(H);
    uint64_t* bar = bars + s;
    const int x0 = (I.tile % S.ntx) * TX, z0 = (I.tile / S.ntx) * TZ;
    uint32_t bytes = 3 * CB + PBYTES;
    if (I.compute) bytes += 5 * hbytes_of(H) + 3 * CB;
    mbar_expect_tx(bar, bytes);
    unsigned char* c = st + 5 * HB;
    tma_load(c + 0 * CB, &T.cSxy, bar, x0, z0, I.q);
    tma_load(c + 1 * CB, &T.cSyy, bar, x0, z0, I.q);
    tma_load(c + 2 * CB, &T.cSyz, bar, x0, z0, I.q);
    tma_load(st + 5 * HB + 6 * CB, &T.pRho, bar, x0, z0, I.c + 1);
    if (I.compute) {
        tma_load(st + 0 * HB, &T.hSxx, bar, x0 - HX, z0 - H, I.c);
        tma_load(st + 1 * HB, &T.hSxy, bar, x0 - HX, z0 - H, I.c);
        tma_load(st + 2 * HB, &T.hSxz, bar, x0 - HX, z0 - H, I.c);
        tma_load(st + 3 * HB, &T.hSyz, bar, x0 - HX, z0 - H, I.c);
        tma_load(st + 4 * HB, &T.hSzz, bar, x0 - HX, z0 - H, I.c);
        tma_load(c + 3 * CB, &T.cVx, bar, x0, z0, I.c);
        tma_load(c + 4 * CB, &T.cVy, bar, x0, z0, I.c);
        tma_load(c + 5 * CB, &T.cVz, bar, x0, z0, I.c);
    }
}

template <int H>
__global__ void __launch_bounds__(NTHR, 1) el3d_vel(const __grid_constant__ El3dMaps T, const StepParams P, const El3dSched S)
{
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int HB = hb_of(H), HX = hx_of(H), BW = bw_of(H), ST = vel_stage(H);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + NSTAGE * ST);
    const int tx = threadIdx.x, tz = threadIdx.y, tid = tz * TX + tx;
    const long long G = (long long)S.ntx * S.ntz * P.NY;
    const long long g0 = G * blockIdx.x / gridDim.x, g1 = G * (blockIdx.x + 1) / gridDim.x;
    __shared__ int abortRun;
    if (tid == 0) {
        // a failed wait in an earlier launch leaves the error word set: skip the work
        abortRun = (S.err && *reinterpret_cast<volatile int*>(S.err) != 0) ? 1 : 0;
        for (int s = 0; s < NSTAGE; ++s) mbar_init(bars + s, 1);
        fence_barrier_init();
    }
    __syncthreads();
    const int total = abortRun ? 0 : total_iters(g0, g1, P.NY, H);
    if (tid == 0)
        for (int i = 0; i < NSTAGE && i < total; ++i) vel_issue<H>(T, P, S, smem, bars, i, g0, g1);

    float qxy[2 * H + 1], qyy[2 * H + 1], qyz[2 * H + 1];
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) qxy[k] = qyy[k] = qyz[k] = 0.0f;
    float r0 = 0.0f, rx = 0.0f, rz = 0.0f;   // rho at the compute plane: (x,z), (x+1,z), (x,z+1)
    const Op1D& DybS = P.fs ? P.DybS : P.Dyb;
    const Op1D& DyfS = P.fs ? P.DyfS : P.Dyf;
    const int ci = (tz + H) * BW + (tx + HX);
    bool failed = false;

    for (int it = 0; it < total; ++it) {
        const int s = it % NSTAGE;
        Iter I;
        iter_at(it, g0, g1, P.NY, H, I);
        if (!mbar_wait(bars + s, (it / NSTAGE) & 1)) failed = true;
        if (__syncthreads_or(failed)) {
            if (tid == 0) report(S.err, WAVE_ERR_TIMEOUT);
            return;
        }
        const unsigned char* st = smem + s * ST;
        const float* cen = reinterpret_cast<const float*>(st + 5 * HB);
#pragma unroll
        for (int k = 0; k < 2 * H; ++k) { qxy[k] = qxy[k + 1]; qyy[k] = qyy[k + 1]; qyz[k] = qyz[k + 1]; }
        qxy[2 * H] = cen[0 * TX * TZ + tid];
        qyy[2 * H] = cen[1 * TX * TZ + tid];
        qyz[2 * H] = cen[2 * TX * TZ + tid];
        const float* rb = reinterpret_cast<const float*>(st + 5 * HB + 6 * CB);
        const float rn = rb[tz * PW + tx];      // rho at (x, z, c+1)
        const int x = (I.tile % S.ntx) * TX + tx, z = (I.tile / S.ntx) * TZ + tz, y = I.c;
        if (I.compute && x < P.NX && z < P.NZ) {
            const float* hSxx = reinterpret_cast<const float*>(st + 0 * HB);
            const float* hSxy = reinterpret_cast<const float*>(st + 1 * HB);
            const float* hSxz = reinterpret_cast<const float*>(st + 2 * HB);
            const float* hSyz = reinterpret_cast<const float*>(st + 3 * HB);
            const float* hSzz = reinterpret_cast<const float*>(st + 4 * HB);
            const long long i = x + (long long)P.NX * (z + (long long)P.NZ * y);
            // vx
            float u = d_line<H, true>(hSxx, ci, 1, x, P.Dxf);
            if (P.useCpml) cpml_x(P, u, x, y, z, true, PS_SXX_X);
            float ut = d_queue<H, false>(qxy, y, DybS);
            if (P.useCpml) cpml_y(P, ut, x, y, z, false, PS_SXY_Y);
            u += ut;
            ut = d_line<H, false>(hSxz, ci, BW, z, P.Dzb);
            if (P.useCpml) cpml_z(P, ut, x, y, z, false, PS_SXZ_Z);
            u += ut;
            u *= inv_avg2(r0, rx, x + 1 < P.NX);
            P.f[F_VX][i] = cen[3 * TX * TZ + tid] + u;
            // vy
            u = d_line<H, false>(hSxy, ci, 1, x, P.Dxb);
            if (P.useCpml) cpml_x(P, u, x, y, z, false, PS_SXY_X);
            ut = d_queue<H, true>(qyy, y, DyfS);
            if (P.useCpml) cpml_y(P, ut, x, y, z, true, PS_SYY_Y);
            u += ut;
            ut = d_line<H, false>(hSyz, ci, BW, z, P.Dzb);
            if (P.useCpml) cpml_z(P, ut, x, y, z, false, PS_SYZ_Z);
            u += ut;
            u *= inv_avg2(r0, rn, y + 1 < P.NY);
            P.f[F_VY][i] = cen[4 * TX * TZ + tid] + u;
            // vz
            u = d_line<H, false>(hSxz, ci, 1, x, P.Dxb);
            if (P.useCpml) cpml_x(P, u, x, y, z, false, PS_SXZ_X);
            ut = d_queue<H, false>(qyz, y, DybS);
            if (P.useCpml) cpml_y(P, ut, x, y, z, false, PS_SYZ_Y);
            u += ut;
            ut = d_line<H, true>(hSzz, ci, BW, z, P.Dzf);
            if (P.useCpml) cpml_z(P, ut, x, y, z, true, PS_SZZ_Z);
            u += ut;
            u *= inv_avg2(r0, rz, z + 1 < P.NZ);
            P.f[F_VZ][i] = cen[5 * TX * TZ + tid] + u;
        }
        // carry rho of plane c+1 into the next iteration
        r0 = rn;
        rx = rb[tz * PW + tx + 1];
        rz = rb[(tz + 1) * PW + tx];
        __syncthreads();
        if (tid == 0 && it + NSTAGE < total) {
            fence_proxy_async();
            vel_issue<H>(T, P, S, smem, bars, it + NSTAGE, g0, g1);
        }
    }
}

// ------------------------------------------------------------------------
// stress pass (ForwardSolver3Delastic.cpp:283-409, FreeSurface3Delastic.cpp:15-47)
// ------------------------------------------------------------------------
template <int H>
__device__ __forceinline__ void str_issue(const El3dMaps& T, const StepParams& P, const El3dSched& S, unsigned char* smem,
                                          uint64_t* bars, int it, long long g0, long long g1)
{
    Iter I;
    if (!iter_at(it, g0, g1, P.NY, H, I)) return;
    constexpr int HB = hb_of(H), HX = hx_of(H);
    const int s = it % NSTAGE;
    unsigned char* st = smem + s * str_stage(H);
    uint64_t* bar = bars + s;
    const int x0 = (I.tile % S.ntx) * TX, z0 = (I.tile / S.ntx) * TZ;
    uint32_t bytes = 3 * CB + PBYTES;
    if (I.compute) bytes += 3 * hbytes_of(H) + 7 * CB;
    mbar_expect_tx(bar, bytes);
    unsigned char* c = st + 3 * HB;
    tma_load(c + 0 * CB, &T.cVx, bar, x0, z0, I.q);
    tma_load(c + 1 * CB, &T.cVy, bar, x0, z0, I.q);
    tma_load(c + 2 * CB, &T.cVz, bar, x0, z0, I.q);
    tma_load(st + 3 * HB + 10 * CB, &T.pMu, bar, x0, z0, I.c + 1);
    if (I.compute) {
        tma_load(st + 0 * HB, &T.hVx, bar, x0 - HX, z0 - H, I.c);
        tma_load(st + 1 * HB, &T.hVy, bar, x0 - HX, z0 - H, I.c);
        tma_load(st + 2 * HB, &T.hVz, bar, x0 - HX, z0 - H, I.c);
        tma_load(c + 3 * CB, &T.cSxx, bar, x0, z0, I.c);
        tma_load(c + 4 * CB, &T.cSyy, bar, x0, z0, I.c);
        tma_load(c + 5 * CB, &T.cSzz, bar, x0, z0, I.c);
        tma_load(c + 6 * CB, &T.cSxy, bar, x0, z0, I.c);
        tma_load(c + 7 * CB, &T.cSxz, bar, x0, z0, I.c);
        tma_load(c + 8 * CB, &T.cSyz, bar, x0, z0, I.c);
        tma_load(c + 9 * CB, &T.cM, bar, x0, z0, I.c);
    }
}

template <int H>
__global__ void __launch_bounds__(NTHR, 1) el3d_str(const __grid_constant__ El3dMaps T, const StepParams P, const El3dSched S)
{
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int HB = hb_of(H), HX = hx_of(H), BW = bw_of(H), ST = str_stage(H);
    constexpr int TT = TX * TZ;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + NSTAGE * ST);
    const int tx = threadIdx.x, tz = threadIdx.y, tid = tz * TX + tx;
    const long long G = (long long)S.ntx * S.ntz * P.NY;
    const long long g0 = G * blockIdx.x / gridDim.x, g1 = G * (blockIdx.x + 1) / gridDim.x;
    __shared__ int abortRun;
    if (tid == 0) {
        // a failed wait in an earlier launch leaves the error word set: skip the work
        abortRun = (S.err && *reinterpret_cast<volatile int*>(S.err) != 0) ? 1 : 0;
        for (int s = 0; s < NSTAGE; ++s) mbar_init(bars + s, 1);
        fence_barrier_init();
    }
    __syncthreads();
    const int total = abortRun ? 0 : total_iters(g0, g1, P.NY, H);
    if (tid == 0)
        for (int i = 0; i < NSTAGE && i < total; ++i) str_issue<H>(T, P, S, smem, bars, i, g0, g1);

    float qx[2 * H + 1], qy[2 * H + 1], qz[2 * H + 1];
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) qx[k] = qy[k] = qz[k] = 0.0f;
    // mu at the compute plane: (x,z), (x+1,z), (x,z+1), (x+1,z+1)
    float m00 = 1.0f, m10 = 1.0f, m01 = 1.0f, m11 = 1.0f;
    const int ci = (tz + H) * BW + (tx + HX);
    bool failed = false;

    for (int it = 0; it < total; ++it) {
        const int s = it % NSTAGE;
        Iter I;
        iter_at(it, g0, g1, P.NY, H, I);
        if (!mbar_wait(bars + s, (it / NSTAGE) & 1)) failed = true;
        if (__syncthreads_or(failed)) {
            if (tid == 0) report(S.err, WAVE_ERR_TIMEOUT);
            return;
        }
        const unsigned char* st = smem + s * ST;
        const float* cen = reinterpret_cast<const float*>(st + 3 * HB);
#pragma unroll
        for (int k = 0; k < 2 * H; ++k) { qx[k] = qx[k + 1]; qy[k] = qy[k + 1]; qz[k] = qz[k + 1]; }
        qx[2 * H] = cen[0 * TT + tid];
        qy[2 * H] = cen[1 * TT + tid];
        qz[2 * H] = cen[2 * TT + tid];
        const float* mb = reinterpret_cast<const float*>(st + 3 * HB + 10 * CB);
        const float n00 = mb[tz * PW + tx], n10 = mb[tz * PW + tx + 1], n01 = mb[(tz + 1) * PW + tx];
        const int x = (I.tile % S.ntx) * TX + tx, z = (I.tile / S.ntx) * TZ + tz, y = I.c;
        if (I.compute && x < P.NX && z < P.NZ) {
            const float* hVx = reinterpret_cast<const float*>(st + 0 * HB);
            const float* hVy = reinterpret_cast<const float*>(st + 1 * HB);
            const float* hVz = reinterpret_cast<const float*>(st + 2 * HB);
            const long long i = x + (long long)P.NX * (z + (long long)P.NZ * y);
            const bool inX = x + 1 < P.NX, inY = y + 1 < P.NY, inZ = z + 1 < P.NZ;
            const float M = cen[9 * TT + tid];
            const float mu = m00 < 1.0f ? 1.0f : m00;
            const float i00 = inv_clamped(m00), i10 = inv_clamped(m10), i01 = inv_clamped(m01), i11 = inv_clamped(m11);
            const float j00 = inv_clamped(n00), j10 = inv_clamped(n10), j01 = inv_clamped(n01);
            // XY: (x,y) (x+1,y) (x,y+1) (x+1,y+1); XZ: (x,z) (x+1,z) (x,z+1) (x+1,z+1);
            // YZ: (y,z) (y+1,z) (y,z+1) (y+1,z+1)  (calcAverageMatrixXY/XZ/YZ, Modelparameter.cpp:533-624)
            const float muXY = harm4(i00, i10, j00, j10, inX, inY);
            const float muXZ = harm4(i00, i10, i01, i11, inX, inZ);
            const float muYZ = harm4(i00, j00, i01, j01, inY, inZ);

            float vxx = d_line<H, false>(hVx, ci, 1, x, P.Dxb);
            if (P.useCpml) cpml_x(P, vxx, x, y, z, false, PS_VXX);
            float vyy = d_queue<H, false>(qy, y, P.Dyb);
            if (P.useCpml) cpml_y(P, vyy, x, y, z, false, PS_VYY);
            float vzz = d_line<H, false>(hVz, ci, BW, z, P.Dzb);
            if (P.useCpml) cpml_z(P, vzz, x, y, z, false, PS_VZZ);
            float sxx = cen[3 * TT + tid], syy = cen[4 * TT + tid], szz = cen[5 * TT + tid];
            float u = vxx;
            u += vyy;
            u += vzz;
            u *= M;
            sxx += u; syy += u; szz += u;
            u = vyy + vzz; u *= mu; sxx -= 2.0f * u;
            u = vxx + vzz; u *= mu; syy -= 2.0f * u;
            u = vxx + vyy; u *= mu; szz -= 2.0f * u;
            // shear
            u = d_queue<H, true>(qx, y, P.Dyf);
            if (P.useCpml) cpml_y(P, u, x, y, z, true, PS_VXY);
            float ut = d_line<H, true>(hVy, ci, 1, x, P.Dxf);
            if (P.useCpml) cpml_x(P, ut, x, y, z, true, PS_VYX);
            u += ut;
            u *= muXY;
            float sxy = cen[6 * TT + tid] + u;
            u = d_line<H, true>(hVx, ci, BW, z, P.Dzf);
            if (P.useCpml) cpml_z(P, u, x, y, z, true, PS_VXZ);
            ut = d_line<H, true>(hVz, ci, 1, x, P.Dxf);
            if (P.useCpml) cpml_x(P, ut, x, y, z, true, PS_VZX);
            u += ut;
            u *= muXZ;
            float sxz = cen[7 * TT + tid] + u;
            u = d_line<H, true>(hVy, ci, BW, z, P.Dzf);
            if (P.useCpml) cpml_z(P, u, x, y, z, true, PS_VYZ);
            ut = d_queue<H, true>(qz, y, P.Dyf);
            if (P.useCpml) cpml_y(P, ut, x, y, z, true, PS_VZY);
            u += ut;
            u *= muYZ;
            float syz = cen[8 * TT + tid] + u;
            if (P.fs && y == 0) {
                float sv = M - 2.0f * mu;
                float sh = sv * sv;
                sh /= M;
                sh *= -1.0f;
                syy = 0.0f;
                float t = sh * (vxx + vzz);
                sxx += t; szz += t;
                t = sv * vyy;
                sxx -= t; szz -= t;
            }
            if (P.abs) {
                const float d = abs_damp(P, x, y, z);
                sxx *= d; syy *= d; szz *= d; sxy *= d; sxz *= d; syz *= d;
            }
            P.f[F_SXX][i] = sxx;
            P.f[F_SYY][i] = syy;
            P.f[F_SZZ][i] = szz;
            P.f[F_SXY][i] = sxy;
            P.f[F_SXZ][i] = sxz;
            P.f[F_SYZ][i] = syz;
        }
        // carry mu of plane c+1 into the next iteration
        m00 = n00; m10 = n10; m01 = n01;
        m11 = mb[(tz + 1) * PW + tx + 1];
        __syncthreads();
        if (tid == 0 && it + NSTAGE < total) {
            fence_proxy_async();
            str_issue<H>(T, P, S, smem, bars, it + NSTAGE, g0, g1);
        }
    }
}

// ------------------------------------------------------------------------
// host side: tensor maps and launches
// ------------------------------------------------------------------------
namespace {

using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                              const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                              CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encoder()
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

bool make_map(CUtensorMap* m, const float* base, int NX, int NZ, int NY, int bx, int bz)
{
    EncodeFn enc = encoder();
    if (!enc) return false;
    cuuint64_t dims[3] = {(cuuint64_t)NX, (cuuint64_t)NZ, (cuuint64_t)NY};
    cuuint64_t strides[2] = {(cuuint64_t)NX * 4, (cuuint64_t)NX * NZ * 4};
    cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)bz, 1};
    cuuint32_t es[3] = {1, 1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int H>
size_t vel_smem() { return NSTAGE * vel_stage(H) + NSTAGE * sizeof(uint64_t); }
template <int H>
size_t str_smem() { return NSTAGE * str_stage(H) + NSTAGE * sizeof(uint64_t); }

} // namespace

template <int H>
static cudaError_t configure_h()
{
    cudaError_t e = cudaFuncSetAttribute(el3d_vel<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vel_smem<H>());
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(el3d_str<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)str_smem<H>());
}

template <int H>
static cudaError_t launch_h(const El3dPlan& plan, const StepParams& P, int pass, cudaStream_t s)
{
    const dim3 block(TX, TZ, 1);
    if (pass == 0) el3d_vel<H><<<plan.grid, block, vel_smem<H>(), s>>>(plan.maps, P, plan.sched);
    else el3d_str<H><<<plan.grid, block, str_smem<H>(), s>>>(plan.maps, P, plan.sched);
    return cudaGetLastError();
}

static cudaError_t configure(int H)
{
    switch (H) {
    case 1: return configure_h<1>();
    case 2: return configure_h<2>();
    case 3: return configure_h<3>();
    case 4: return configure_h<4>();
    case 5: return configure_h<5>();
    case 6: return configure_h<6>();
    default: return cudaErrorInvalidValue;
    }
}

// Builds the tensor maps for the current field/material pointers. Returns
// false when the streaming path does not apply (then the generic kernels run).
bool el3d_prepare(El3dPlan& plan, const StepParams& P, const float* rho, const float* M, const float* mu, int H, int* errWord)
{
    plan.ready = false;
    if (!P.is3d || H < 1 || H > 6 || (P.NX % 4) != 0 || P.NX < 8 || P.NZ < 2) return false;
    if (!rho || !M || !mu) return false;
    const int bx = bw_of(H), bz = bh_of(H);
    El3dMaps& T = plan.maps;
    bool ok = true;
    ok &= make_map(&T.hSxx, P.f[F_SXX], P.NX, P.NZ, P.NY, bx, bz);
    ok &= make_map(&T.hSxy, P.f[F_SXY], P.NX, P.NZ, P.NY, bx, bz);
    ok &= make_map(&T.hSxz, P.f[F_SXZ], P.NX, P.NZ, P.NY, bx, bz);
    ok &= make_map(&T.hSyz, P.f[F_SYZ], P.NX, P.NZ, P.NY, bx, bz);
    ok &= make_map(&T.hSzz, P.f[F_SZZ], P.NX, P.NZ, P.NY, bx, bz);
    ok &= make_map(&T.hVx, P.f[F_VX], P.NX, P.NZ, P.NY, bx, bz);
    ok &= make_map(&T.hVy, P.f[F_VY], P.NX, P.NZ, P.NY, bx, bz);
    ok &= make_map(&T.hVz, P.f[F_VZ], P.NX, P.NZ, P.NY, bx, bz);
    ok &= make_map(&T.cSxx, P.f[F_SXX], P.NX, P.NZ, P.NY, TX, TZ);
    ok &= make_map(&T.cSyy, P.f[F_SYY], P.NX, P.NZ, P.NY, TX, TZ);
    ok &= make_map(&T.cSzz, P.f[F_SZZ], P.NX, P.NZ, P.NY, TX, TZ);
    ok &= make_map(&T.cSxy, P.f[F_SXY], P.NX, P.NZ, P.NY, TX, TZ);
    ok &= make_map(&T.cSxz, P.f[F_SXZ], P.NX, P.NZ, P.NY, TX, TZ);
    ok &= make_map(&T.cSyz, P.f[F_SYZ], P.NX, P.NZ, P.NY, TX, TZ);
    ok &= make_map(&T.cVx, P.f[F_VX], P.NX, P.NZ, P.NY, TX, TZ);
    ok &= make_map(&T.cVy, P.f[F_VY], P.NX, P.NZ, P.NY, TX, TZ);
    ok &= make_map(&T.cVz, P.f[F_VZ], P.NX, P.NZ, P.NY, TX, TZ);
    ok &= make_map(&T.cM, M, P.NX, P.NZ, P.NY, TX, TZ);
    ok &= make_map(&T.pRho, rho, P.NX, P.NZ, P.NY, PW, PH);
    ok &= make_map(&T.pMu, mu, P.NX, P.NZ, P.NY, PW, PH);
    if (!ok) return false;
    plan.sched.ntx = (P.NX + TX - 1) / TX;
    plan.sched.ntz = (P.NZ + TZ - 1) / TZ;
    plan.sched.err = errWord;
    plan.H = H;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long work = (long long)plan.sched.ntx * plan.sched.ntz * P.NY;
    plan.grid = static_cast<int>(work < sms ? work : sms);
    if (configure(H) != cudaSuccess) return false;
    plan.ready = plan.grid > 0;
    return plan.ready;
}

cudaError_t el3d_launch(const El3dPlan& plan, const StepParams& P, int pass, cudaStream_t s)
{
    switch (plan.H) {
    case 1: return launch_h<1>(plan, P, pass, s);
    case 2: return launch_h<2>(plan, P, pass, s);
    case 3: return launch_h<3>(plan, P, pass, s);
    case 4: return launch_h<4>(plan, P, pass, s);
    case 5: return launch_h<5>(plan, P, pass, s);
    case 6: return launch_h<6>(plan, P, pass, s);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace wave
