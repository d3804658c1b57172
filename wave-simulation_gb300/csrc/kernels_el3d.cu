// kernels_el3d.cu — streaming sm_103a kernels for the 3-D elastic time step
// (FD3Delastic::run, ForwardSolver3Delastic.cpp:120-414) on large grids.
//
// Each CTA owns a 32 (x) x 8 (z) column tile and marches it down the depth
// axis y (the slowest axis, reference layout idx = x + z*NX + y*NX*NZ). The
// CTAs are persistent (two per SM); each takes a contiguous run of the
// (tile, plane) work, so every field plane is fetched from HBM once. Planes
// arrive through TMA bulk-tensor copies (cp.async.bulk.tensor.3d) into a
// 3-stage shared-memory ring ("full" mbarriers carry the transaction
// bytes). Each of the 8 warps computes one z row of the tile and releases a
// stage by a shared-memory counter; the warp that releases a stage last
// refills it at once, so copies lead the compute by two iterations. Warps
// never meet at a block barrier, so they run up to a ring's length apart and
// hide each other's latency. Depth derivatives come from
// per-thread register queues (2H+1 planes), x- and z-derivatives from the
// halo tiles in shared memory. Interior rows multiply compile-time FD
// coefficients and scale once by DT/DH; edge rows (order reduction, zero
// padding, free-surface image rows) use the operator's edge table. The
// averaged material terms (1/rho averages, harmonic mu averages with the
// vacuum rules and edge fallbacks) are formed in-kernel from rho and mu, so
// the kernels read only base material arrays. Every wait is bounded: a wait
// that runs out sets the handle's error word and the CTA returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <type_traits>

#include "el3d.h"
#include "el3d_common.cuh"

namespace wave {

namespace el3d {

constexpr int TX = 32, TZ = 8, NTHR = TX * TZ;
static_assert(NTHR / 32 == NCWARP, "one warp per z row of the tile");
constexpr int CB = TX * TZ * 4;                  // centre box bytes
constexpr int PW = TX + 4, PH = TZ + 1;          // "+1" box (x0..x0+35, z0..z0+8)
constexpr int PBYTES = PW * PH * 4;              // bytes one "+1" box copy delivers
constexpr int PB = ((PBYTES + 127) / 128) * 128; // its slot in the stage layout

__host__ __device__ constexpr int hx_of(int H) { return H <= 4 ? 4 : 8; }
__host__ __device__ constexpr int bw_of(int H) { return TX + 2 * hx_of(H); }
__host__ __device__ constexpr int bh_of(int H) { return TZ + 2 * H; }
__host__ __device__ constexpr int hbytes_of(int H) { return bw_of(H) * bh_of(H) * 4; }          // delivered
__host__ __device__ constexpr int hb_of(int H) { return ((hbytes_of(H) + 127) / 128) * 128; }  // layout slot

// ------------------------------------------------------------ derivatives
// Interior rows: compile-time coefficients, two interleaved partial sums (even
// and odd taps) to halve the dependent FMA chain; DT/DH is applied once after.
template <int H, bool FWD>
__device__ __forceinline__ float dsum(const float* __restrict__ s, int ci, int stride)
{
    float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
    for (int j = 0; j < 2 * H; j += 2) {
        a0 += fdc(2 * H, j) * s[ci + (FWD ? j - H + 1 : j - H) * stride];
        a1 += fdc(2 * H, j + 1) * s[ci + (FWD ? j - H + 2 : j - H + 1) * stride];
    }
    return a0 + a1;
}

// Edge rows (order reduction, zero padding, free-surface images): weights
// from the operator's edge table, offsets -H..H, branch-free (every offset is
// inside the staged halo, dropped columns carry weight zero).
template <int H>
__device__ __forceinline__ float dtab(const float* __restrict__ s, int ci, int stride, const float* __restrict__ t)
{
    float w[2 * H + 1];
#pragma unroll
    for (int k = -H; k <= H; ++k) w[k + H] = __ldg(t + k);
    float acc = 0.0f;
#pragma unroll
    for (int k = -H; k <= H; ++k) acc += w[k + H] * s[ci + k * stride];
    return acc;
}

// derivative along a line of a smem tile; INT: the whole warp is on interior rows
template <int H, bool FWD, bool INT>
__device__ __forceinline__ float dline(const float* __restrict__ s, int ci, int stride, bool interior, const float* row, float scale)
{
    if constexpr (INT) {
        return dsum<H, FWD>(s, ci, stride) * scale;
    } else {
        if (interior) return dsum<H, FWD>(s, ci, stride) * scale;
        return dtab<H>(s, ci, stride, row);
    }
}

template <int H, bool FWD, bool INT>
__device__ __forceinline__ float dqueue(const float (&q)[2 * H + 1], bool interior, const float* row, float scale)
{
    float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
    for (int j = 0; j < 2 * H; j += 2) {
        a0 += fdc(2 * H, j) * q[H + (FWD ? j - H + 1 : j - H)];
        a1 += fdc(2 * H, j + 1) * q[H + (FWD ? j - H + 2 : j - H + 1)];
    }
    if constexpr (INT) return (a0 + a1) * scale;
    if (interior) return (a0 + a1) * scale;
    float w[2 * H + 1];
#pragma unroll
    for (int k = -H; k <= H; ++k) w[k + H] = __ldg(row + k);
    float acc = 0.0f;
#pragma unroll
    for (int k = -H; k <= H; ++k) acc += w[k + H] * q[H + k];
    return acc;
}

// per-thread state of the current column: coordinates, edge flags, CPML
// coefficients and psi offsets along x and z (fixed while the CTA marches
// down one tile)
struct Column {
    int x, z;
    bool ok;                 // inside the grid
    bool xi, zi;             // interior rows along x / z
    int sx, sz;              // CPML slab indices (-1 outside)
    float axf, bxf, axh, bxh, azf, bzf, azh, bzh;
    long long px, pz;        // psi offsets without the y term
    const float *rxf, *rxb, *rzf, *rzb;   // edge-table rows (edge columns only)
    bool wint;               // every lane of the warp is on interior x and z rows
};

__device__ __forceinline__ void column_setup(Column& C, const StepParams& P, int x0, int z0)
{
    C.x = x0 + (threadIdx.x & 31);
    C.z = z0 + (threadIdx.x >> 5);
    C.ok = C.x < P.NX && C.z < P.NZ;
    C.xi = interior_of(P.Dxf, C.x);
    C.zi = interior_of(P.Dzf, C.z);
    C.sx = P.useCpml && C.ok ? slab_of(C.x, P.cx) : -1;
    C.sz = P.useCpml && C.ok ? slab_of(C.z, P.cz) : -1;
    C.axf = C.bxf = C.axh = C.bxh = C.azf = C.bzf = C.azh = C.bzh = 0.0f;
    if (C.sx >= 0) { C.axf = P.cx.a_full[C.x]; C.bxf = P.cx.b_full[C.x]; C.axh = P.cx.a_half[C.x]; C.bxh = P.cx.b_half[C.x]; }
    if (C.sz >= 0) { C.azf = P.cz.a_full[C.z]; C.bzf = P.cz.b_full[C.z]; C.azh = P.cz.a_half[C.z]; C.bzh = P.cz.b_half[C.z]; }
    C.px = C.sx + (long long)P.cx.ns * C.z;            // + ns*NZ*y
    C.pz = C.x + (long long)P.NX * C.sz;               // + NX*nsz*y
    C.rxf = C.xi || !C.ok ? nullptr : row_of(P.Dxf, C.x);
    C.rxb = C.xi || !C.ok ? nullptr : row_of(P.Dxb, C.x);
    C.rzf = C.zi || !C.ok ? nullptr : row_of(P.Dzf, C.z);
    C.rzb = C.zi || !C.ok ? nullptr : row_of(P.Dzb, C.z);
    C.wint = __all_sync(0xffffffffu, (C.xi && C.zi) || !C.ok);
}

__device__ __forceinline__ float* psi_x(const StepParams& P, int slot, const Column& C, int y)
{
    return P.psi[slot] + C.px + (long long)P.cx.ns * P.NZ * y;
}
__device__ __forceinline__ float* psi_z(const StepParams& P, int slot, const Column& C, int y)
{
    return P.psi[slot] + C.pz + (long long)P.NX * P.cz.ns * y;
}
__device__ __forceinline__ float* psi_y(const StepParams& P, int slot, const Column& C, const Plane& L)
{
    return P.psi[slot] + C.x + (long long)P.NX * (C.z + (long long)P.NZ * L.sy);
}

} // namespace el3d

using namespace el3d;

// ------------------------------------------------------------------------
// pipeline skeleton shared by the two passes
// ------------------------------------------------------------------------
// CPML::applyCPML (CPML.cpp:84-95): psi = b*psi + a*d; d += psi, with the old
// psi staged in shared memory by the producer and the new one written to HBM
__device__ __forceinline__ void cpml_s(float& d, float ps, float* gpsi, float a, float b)
{
    ps *= b;
    ps += a * d;
    *gpsi = ps;
    d += ps;
}

// Layout of one pipeline stage; psi boxes are x-type [0,3), y-type [3,6), z-type [6,9).
template <int H, int NHALO, int NCEN>
struct Stage {
    static constexpr int HB = hb_of(H);
    static constexpr int HALO = 0;
    static constexpr int CEN = NHALO * HB;
    static constexpr int PLUS = CEN + NCEN * CB;
    static constexpr int PSI = PLUS + PB;
    static constexpr int BYTES = PSI + 9 * CB;
    static constexpr int NST = 3;   // measured faster than 4 (more L1 left beside the ring)
};

template <int H> using VelStage = Stage<H, 5, 6>;
template <int H> using StrStage = Stage<H, 3, 10>;

// The CPML memory-variable boxes a (tile, plane c) iteration needs.
struct PsiBoxes {
    int bx, bz, sy;   // x-type / z-type box coordinates (kNoBox: none), y slab plane (-1: none)
    __device__ __forceinline__ uint32_t bytes() const
    {
        return ((bx != kNoBox) + (sy >= 0) + (bz != kNoBox)) * 3u * CB;
    }
};

__device__ __forceinline__ PsiBoxes psi_boxes(const StepParams& P, int x0, int z0, int c)
{
    if (!P.useCpml) return {kNoBox, kNoBox, -1};
    return {slab_box(P.cx, x0, TX), slab_box(P.cz, z0, TZ), slab_of(c, P.cy)};
}

// issues the psi boxes of one iteration into the stage's psi slots
__device__ __forceinline__ void issue_psi(const PsiBoxes& B, const CUtensorMap* m, unsigned char* ps, uint64_t* bar,
                                          int x0, int z0, int c)
{
    if (B.bx != kNoBox)
        for (int j = 0; j < 3; ++j) tma_load(ps + j * CB, m + j, bar, B.bx, z0, c);
    if (B.sy >= 0)
        for (int j = 3; j < 6; ++j) tma_load(ps + j * CB, m + j, bar, x0, z0, B.sy);
    if (B.bz != kNoBox)
        for (int j = 6; j < 9; ++j) tma_load(ps + j * CB, m + j, bar, x0, B.bz, c);
}

// ------------------------------------------------------------------------
// velocity pass (ForwardSolver3Delastic.cpp:174-277)
// ------------------------------------------------------------------------
template <int H>
__global__ void __launch_bounds__(NTHR, 2) el3d_vel(const __grid_constant__ El3dMaps T, const StepParams P, const El3dSched S)
{
    using L = VelStage<H>;
    constexpr int NST = L::NST, HX = hx_of(H), BW = bw_of(H), TT = TX * TZ;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * L::BYTES);
    unsigned* rel = reinterpret_cast<unsigned*>(full + NST);   // per-stage release counters
    __shared__ Segs G;
    __shared__ int abortRun;
    __shared__ volatile int failed;
    __shared__ int issued;
    const int total = prologue<NST>(G, full, rel, &abortRun, &failed, P, S, H, T);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    auto issue = [&](int s, const Cursor& cur) {
        unsigned char* st = smem + s * L::BYTES;
        uint64_t* bar = full + s;
        const int tile = G.tile[cur.seg], ya = G.ya[cur.seg];
        const int q = ya - H + cur.k, c = ya - 2 * H + cur.k;
        const bool compute = c >= ya;
        const int x0 = (tile % S.ntx) * TX, z0 = (tile / S.ntx) * TZ;
        const PsiBoxes B = compute ? psi_boxes(P, x0, z0, c) : PsiBoxes{kNoBox, kNoBox, -1};
        uint32_t bytes = 3 * CB + PBYTES + B.bytes();
        if (compute) bytes += 5 * hbytes_of(H) + 3 * CB;
        mbar_expect_tx(bar, bytes);
        issue_psi(B, T.psV, st + L::PSI, bar, x0, z0, c);
        unsigned char* cen = st + L::CEN;
        tma_load(cen + 0 * CB, &T.cSxy, bar, x0, z0, q);
        tma_load(cen + 1 * CB, &T.cSyy, bar, x0, z0, q);
        tma_load(cen + 2 * CB, &T.cSyz, bar, x0, z0, q);
        tma_load(st + L::PLUS, &T.pRho, bar, x0, z0, c + 1);
        if (compute) {
            tma_load(st + 0 * L::HB, &T.hSxx, bar, x0 - HX, z0 - H, c);
            tma_load(st + 1 * L::HB, &T.hSxy, bar, x0 - HX, z0 - H, c);
            tma_load(st + 2 * L::HB, &T.hSxz, bar, x0 - HX, z0 - H, c);
            tma_load(st + 3 * L::HB, &T.hSyz, bar, x0 - HX, z0 - H, c);
            tma_load(st + 4 * L::HB, &T.hSzz, bar, x0 - HX, z0 - H, c);
            tma_load(cen + 3 * CB, &T.cVx, bar, x0, z0, c);
            tma_load(cen + 4 * CB, &T.cVy, bar, x0, z0, c);
            tma_load(cen + 5 * CB, &T.cVz, bar, x0, z0, c);
        }
    };
    if (threadIdx.x == 0) start_feed<NST>(G, total, &issued, issue);

    const int tid = threadIdx.x;    // x = x0 + lane, z = z0 + warp
    float qxy[2 * H + 1], qyy[2 * H + 1], qyz[2 * H + 1];
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) qxy[k] = qyy[k] = qyz[k] = 0.0f;
    float r0 = 0.0f, rx = 0.0f, rz = 0.0f;   // rho at the compute plane: (x,z), (x+1,z), (x,z+1)
    const Op1D& DybS = P.fs ? P.DybS : P.Dyb;
    const Op1D& DyfS = P.fs ? P.DyfS : P.Dyf;
    const float scale = P.scale;
    const int ci = (warp + H) * BW + (lane + HX);
    Cursor cur{0, 0};
    Column C;

    for (int it = 0; it < total; ++it) {
        const int s = it % NST;
        const int tile = G.tile[cur.seg], ya = G.ya[cur.seg];
        if (cur.k == 0) column_setup(C, P, (tile % S.ntx) * TX, (tile / S.ntx) * TZ);
        const int y = ya - 2 * H + cur.k;
        const bool compute = y >= ya;
        if (!__all_sync(0xffffffffu, mbar_wait(full + s, (it / NST) & 1))) {
            failed = 1;
            report(S.err, WAVE_ERR_TIMEOUT);
            break;
        }
        const unsigned char* st = smem + s * L::BYTES;
        const float* cen = reinterpret_cast<const float*>(st + L::CEN);
#pragma unroll
        for (int k = 0; k < 2 * H; ++k) { qxy[k] = qxy[k + 1]; qyy[k] = qyy[k + 1]; qyz[k] = qyz[k + 1]; }
        qxy[2 * H] = cen[0 * TT + tid];
        qyy[2 * H] = cen[1 * TT + tid];
        qyz[2 * H] = cen[2 * TT + tid];
        const float* rb = reinterpret_cast<const float*>(st + L::PLUS);
        const float rn = rb[warp * PW + lane];      // rho at (x, z, y+1)
        if (compute && C.ok) {
            Plane Y;
            plane_setup(Y, P, y);
            const float* hSxx = reinterpret_cast<const float*>(st + 0 * L::HB);
            const float* hSxy = reinterpret_cast<const float*>(st + 1 * L::HB);
            const float* hSxz = reinterpret_cast<const float*>(st + 2 * L::HB);
            const float* hSyz = reinterpret_cast<const float*>(st + 3 * L::HB);
            const float* hSzz = reinterpret_cast<const float*>(st + 4 * L::HB);
            const float* ps = reinterpret_cast<const float*>(st + L::PSI) + tid;
            const float* ryb = Y.yi ? nullptr : row_of(DybS, y);
            const float* ryf = Y.yi ? nullptr : row_of(DyfS, y);
            const long long i = C.x + (long long)P.NX * (C.z + (long long)P.NZ * y);
            auto body = [&](auto interior) {
                constexpr bool INT = decltype(interior)::value;
                // the nine stress derivatives first (independent FMA chains), then CPML
                float dSxx_x = dline<H, true, INT>(hSxx, ci, 1, C.xi, C.rxf, scale);
                float dSxy_x = dline<H, false, INT>(hSxy, ci, 1, C.xi, C.rxb, scale);
                float dSxz_x = dline<H, false, INT>(hSxz, ci, 1, C.xi, C.rxb, scale);
                float dSxy_y = dqueue<H, false, INT>(qxy, Y.yi, ryb, scale);
                float dSyy_y = dqueue<H, true, INT>(qyy, Y.yi, ryf, scale);
                float dSyz_y = dqueue<H, false, INT>(qyz, Y.yi, ryb, scale);
                float dSxz_z = dline<H, false, INT>(hSxz, ci, BW, C.zi, C.rzb, scale);
                float dSyz_z = dline<H, false, INT>(hSyz, ci, BW, C.zi, C.rzb, scale);
                float dSzz_z = dline<H, true, INT>(hSzz, ci, BW, C.zi, C.rzf, scale);
                if (C.sx >= 0) {
                    cpml_s(dSxx_x, ps[0 * TT], psi_x(P, PS_SXX_X, C, y), C.axh, C.bxh);
                    cpml_s(dSxy_x, ps[1 * TT], psi_x(P, PS_SXY_X, C, y), C.axf, C.bxf);
                    cpml_s(dSxz_x, ps[2 * TT], psi_x(P, PS_SXZ_X, C, y), C.axf, C.bxf);
                }
                if (Y.sy >= 0) {
                    cpml_s(dSxy_y, ps[3 * TT], psi_y(P, PS_SXY_Y, C, Y), Y.ayf, Y.byf);
                    cpml_s(dSyy_y, ps[4 * TT], psi_y(P, PS_SYY_Y, C, Y), Y.ayh, Y.byh);
                    cpml_s(dSyz_y, ps[5 * TT], psi_y(P, PS_SYZ_Y, C, Y), Y.ayf, Y.byf);
                }
                if (C.sz >= 0) {
                    cpml_s(dSxz_z, ps[6 * TT], psi_z(P, PS_SXZ_Z, C, y), C.azf, C.bzf);
                    cpml_s(dSyz_z, ps[7 * TT], psi_z(P, PS_SYZ_Z, C, y), C.azf, C.bzf);
                    cpml_s(dSzz_z, ps[8 * TT], psi_z(P, PS_SZZ_Z, C, y), C.azh, C.bzh);
                }
                float u = dSxx_x;
                u += dSxy_y;
                u += dSxz_z;
                u *= inv_avg2f(r0, rx, C.x + 1 < P.NX);
                P.f[F_VX][i] = cen[3 * TT + tid] + u;
                u = dSxy_x;
                u += dSyy_y;
                u += dSyz_z;
                u *= inv_avg2f(r0, rn, y + 1 < P.NY);
                P.f[F_VY][i] = cen[4 * TT + tid] + u;
                u = dSxz_x;
                u += dSyz_y;
                u += dSzz_z;
                u *= inv_avg2f(r0, rz, C.z + 1 < P.NZ);
                P.f[F_VZ][i] = cen[5 * TT + tid] + u;
            };
            if (C.wint && Y.yi) body(std::true_type{});
            else body(std::false_type{});
        }
        // carry rho of plane y+1 into the next iteration
        r0 = rn;
        rx = rb[warp * PW + lane + 1];
        rz = rb[(warp + 1) * PW + lane];
        release_and_refill<NST>(it, total, cur, G, rel, &issued, &failed, issue);
        if (__any_sync(0xffffffffu, failed != 0)) break;
        cur.advance(G);
    }
    finish_ring<NST>(full, &issued, &failed);
}

// ------------------------------------------------------------------------
// stress pass (ForwardSolver3Delastic.cpp:283-409, FreeSurface3Delastic.cpp:15-47)
// ------------------------------------------------------------------------
template <int H>
__global__ void __launch_bounds__(NTHR, 2) el3d_str(const __grid_constant__ El3dMaps T, const StepParams P, const El3dSched S)
{
    using L = StrStage<H>;
    constexpr int NST = L::NST, HX = hx_of(H), BW = bw_of(H), TT = TX * TZ;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * L::BYTES);
    unsigned* rel = reinterpret_cast<unsigned*>(full + NST);   // per-stage release counters
    __shared__ Segs G;
    __shared__ int abortRun;
    __shared__ volatile int failed;
    __shared__ int issued;
    const int total = prologue<NST>(G, full, rel, &abortRun, &failed, P, S, H, T);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    auto issue = [&](int s, const Cursor& cur) {
        unsigned char* st = smem + s * L::BYTES;
        uint64_t* bar = full + s;
        const int tile = G.tile[cur.seg], ya = G.ya[cur.seg];
        const int q = ya - H + cur.k, c = ya - 2 * H + cur.k;
        const bool compute = c >= ya;
        const int x0 = (tile % S.ntx) * TX, z0 = (tile / S.ntx) * TZ;
        const PsiBoxes B = compute ? psi_boxes(P, x0, z0, c) : PsiBoxes{kNoBox, kNoBox, -1};
        uint32_t bytes = 3 * CB + PBYTES + B.bytes();
        if (compute) bytes += 3 * hbytes_of(H) + 7 * CB;
        mbar_expect_tx(bar, bytes);
        issue_psi(B, T.psS, st + L::PSI, bar, x0, z0, c);
        unsigned char* cen = st + L::CEN;
        tma_load(cen + 0 * CB, &T.cVx, bar, x0, z0, q);
        tma_load(cen + 1 * CB, &T.cVy, bar, x0, z0, q);
        tma_load(cen + 2 * CB, &T.cVz, bar, x0, z0, q);
        tma_load(st + L::PLUS, &T.pMu, bar, x0, z0, c + 1);
        if (compute) {
            tma_load(st + 0 * L::HB, &T.hVx, bar, x0 - HX, z0 - H, c);
            tma_load(st + 1 * L::HB, &T.hVy, bar, x0 - HX, z0 - H, c);
            tma_load(st + 2 * L::HB, &T.hVz, bar, x0 - HX, z0 - H, c);
            tma_load(cen + 3 * CB, &T.cSxx, bar, x0, z0, c);
            tma_load(cen + 4 * CB, &T.cSyy, bar, x0, z0, c);
            tma_load(cen + 5 * CB, &T.cSzz, bar, x0, z0, c);
            tma_load(cen + 6 * CB, &T.cSxy, bar, x0, z0, c);
            tma_load(cen + 7 * CB, &T.cSxz, bar, x0, z0, c);
            tma_load(cen + 8 * CB, &T.cSyz, bar, x0, z0, c);
            tma_load(cen + 9 * CB, &T.cM, bar, x0, z0, c);
        }
    };
    if (threadIdx.x == 0) start_feed<NST>(G, total, &issued, issue);

    const int tid = threadIdx.x;
    float qx[2 * H + 1], qy[2 * H + 1], qz[2 * H + 1];
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) qx[k] = qy[k] = qz[k] = 0.0f;
    // inverse clamped mu at the compute plane: (x,z), (x+1,z), (x,z+1), (x+1,z+1), and mu itself
    float i00 = 1.0f, i10 = 1.0f, i01 = 1.0f, i11 = 1.0f, m00 = 1.0f;
    const float scale = P.scale;
    const int ci = (warp + H) * BW + (lane + HX);
    Cursor cur{0, 0};
    Column C;

    for (int it = 0; it < total; ++it) {
        const int s = it % NST;
        const int tile = G.tile[cur.seg], ya = G.ya[cur.seg];
        if (cur.k == 0) column_setup(C, P, (tile % S.ntx) * TX, (tile / S.ntx) * TZ);
        const int y = ya - 2 * H + cur.k;
        const bool compute = y >= ya;
        if (!__all_sync(0xffffffffu, mbar_wait(full + s, (it / NST) & 1))) {
            failed = 1;
            report(S.err, WAVE_ERR_TIMEOUT);
            break;
        }
        const unsigned char* st = smem + s * L::BYTES;
        const float* cen = reinterpret_cast<const float*>(st + L::CEN);
#pragma unroll
        for (int k = 0; k < 2 * H; ++k) { qx[k] = qx[k + 1]; qy[k] = qy[k + 1]; qz[k] = qz[k + 1]; }
        qx[2 * H] = cen[0 * TT + tid];
        qy[2 * H] = cen[1 * TT + tid];
        qz[2 * H] = cen[2 * TT + tid];
        const float* mb = reinterpret_cast<const float*>(st + L::PLUS);
        const float n00 = mb[warp * PW + lane];
        const float j00 = inv_clampedf(n00), j10 = inv_clampedf(mb[warp * PW + lane + 1]);
        const float j01 = inv_clampedf(mb[(warp + 1) * PW + lane]), j11 = inv_clampedf(mb[(warp + 1) * PW + lane + 1]);
        if (compute && C.ok) {
            Plane Y;
            plane_setup(Y, P, y);
            const float* hVx = reinterpret_cast<const float*>(st + 0 * L::HB);
            const float* hVy = reinterpret_cast<const float*>(st + 1 * L::HB);
            const float* hVz = reinterpret_cast<const float*>(st + 2 * L::HB);
            const float* ps = reinterpret_cast<const float*>(st + L::PSI) + tid;
            const float* ryf = Y.yi ? nullptr : row_of(P.Dyf, y);
            const float* ryb = Y.yi ? nullptr : row_of(P.Dyb, y);
            const long long i = C.x + (long long)P.NX * (C.z + (long long)P.NZ * y);
            const bool inX = C.x + 1 < P.NX, inY = y + 1 < P.NY, inZ = C.z + 1 < P.NZ;
            const float M = cen[9 * TT + tid];
            const float mu = m00 < 1.0f ? 1.0f : m00;
            // XY: (x,y) (x+1,y) (x,y+1) (x+1,y+1); XZ: (x,z) (x+1,z) (x,z+1) (x+1,z+1);
            // YZ: (y,z) (y+1,z) (y,z+1) (y+1,z+1)  (calcAverageMatrixXY/XZ/YZ, Modelparameter.cpp:533-624)
            const float muXY = harm4f(i00, i10, j00, j10, inX, inY);
            const float muXZ = harm4f(i00, i10, i01, i11, inX, inZ);
            const float muYZ = harm4f(i00, j00, i01, j01, inY, inZ);

            auto finish = [&](float sxx, float syy, float szz, float sxy, float sxz, float syz, float vxx, float vyy, float vzz) {
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
                float d = 1.0f;
                if (P.abs) d = abs_damp(P, C.x, y, C.z);
                P.f[F_SXX][i] = sxx * d;
                P.f[F_SYY][i] = syy * d;
                P.f[F_SZZ][i] = szz * d;
                P.f[F_SXY][i] = sxy * d;
                P.f[F_SXZ][i] = sxz * d;
                P.f[F_SYZ][i] = syz * d;
            };
            auto body = [&](auto interior) {
                constexpr bool INT = decltype(interior)::value;
                // the nine velocity derivatives first (independent FMA chains), then CPML
                float vxx = dline<H, false, INT>(hVx, ci, 1, C.xi, C.rxb, scale);
                float vyx = dline<H, true, INT>(hVy, ci, 1, C.xi, C.rxf, scale);
                float vzx = dline<H, true, INT>(hVz, ci, 1, C.xi, C.rxf, scale);
                float vyy = dqueue<H, false, INT>(qy, Y.yi, ryb, scale);
                float vxy = dqueue<H, true, INT>(qx, Y.yi, ryf, scale);
                float vzy = dqueue<H, true, INT>(qz, Y.yi, ryf, scale);
                float vzz = dline<H, false, INT>(hVz, ci, BW, C.zi, C.rzb, scale);
                float vxz = dline<H, true, INT>(hVx, ci, BW, C.zi, C.rzf, scale);
                float vyz = dline<H, true, INT>(hVy, ci, BW, C.zi, C.rzf, scale);
                if (C.sx >= 0) {
                    cpml_s(vxx, ps[0 * TT], psi_x(P, PS_VXX, C, y), C.axf, C.bxf);
                    cpml_s(vyx, ps[1 * TT], psi_x(P, PS_VYX, C, y), C.axh, C.bxh);
                    cpml_s(vzx, ps[2 * TT], psi_x(P, PS_VZX, C, y), C.axh, C.bxh);
                }
                if (Y.sy >= 0) {
                    cpml_s(vyy, ps[3 * TT], psi_y(P, PS_VYY, C, Y), Y.ayf, Y.byf);
                    cpml_s(vxy, ps[4 * TT], psi_y(P, PS_VXY, C, Y), Y.ayh, Y.byh);
                    cpml_s(vzy, ps[5 * TT], psi_y(P, PS_VZY, C, Y), Y.ayh, Y.byh);
                }
                if (C.sz >= 0) {
                    cpml_s(vzz, ps[6 * TT], psi_z(P, PS_VZZ, C, y), C.azf, C.bzf);
                    cpml_s(vxz, ps[7 * TT], psi_z(P, PS_VXZ, C, y), C.azh, C.bzh);
                    cpml_s(vyz, ps[8 * TT], psi_z(P, PS_VYZ, C, y), C.azh, C.bzh);
                }
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
                u = vxy;
                u += vyx;
                u *= muXY;
                const float sxy = cen[6 * TT + tid] + u;
                u = vxz;
                u += vzx;
                u *= muXZ;
                const float sxz = cen[7 * TT + tid] + u;
                u = vyz;
                u += vzy;
                u *= muYZ;
                const float syz = cen[8 * TT + tid] + u;
                finish(sxx, syy, szz, sxy, sxz, syz, vxx, vyy, vzz);
            };
            if (C.wint && Y.yi) body(std::true_type{});
            else body(std::false_type{});
        }
        // carry mu of plane y+1 into the next iteration
        m00 = n00;
        i00 = j00; i10 = j10; i01 = j01; i11 = j11;
        release_and_refill<NST>(it, total, cur, G, rel, &issued, &failed, issue);
        if (__any_sync(0xffffffffu, failed != 0)) break;
        cur.advance(G);
    }
    finish_ring<NST>(full, &issued, &failed);
}

// ------------------------------------------------------------------------
// self-test of the bounded wait: an mbarrier that nothing completes
// ------------------------------------------------------------------------
__global__ void wait_selftest_kernel(int* err, uint32_t limit)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait(&bar, 0, limit)) report(err, WAVE_ERR_TIMEOUT);
}

// ------------------------------------------------------------------------
// host side: tensor maps and launches
// ------------------------------------------------------------------------
namespace {

using namespace el3d_host;

template <int H>
size_t vel_smem() { return VelStage<H>::NST * (VelStage<H>::BYTES + 2 * sizeof(uint64_t)); }
template <int H>
size_t str_smem() { return StrStage<H>::NST * (StrStage<H>::BYTES + 2 * sizeof(uint64_t)); }

template <int H>
cudaError_t configure_h()
{
    cudaError_t e = cudaFuncSetAttribute(el3d_vel<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vel_smem<H>());
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(el3d_str<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)str_smem<H>());
    if (e != cudaSuccess) return e;
    // a CTA (NTHR threads, the stage ring) must fit an SM; two are resident per SM
    int nv = 0, ns = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nv, el3d_vel<H>, NTHR, vel_smem<H>());
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ns, el3d_str<H>, NTHR, str_smem<H>());
    if (e != cudaSuccess) return e;
    return nv >= 1 && ns >= 1 ? cudaSuccess : cudaErrorInvalidConfiguration;
}

template <int H>
cudaError_t launch_h(const El3dPlan& plan, const StepParams& P, int pass, cudaStream_t s)
{
    const dim3 block(NTHR, 1, 1);
    if (pass == 0) el3d_vel<H><<<plan.grid, block, vel_smem<H>(), s>>>(plan.maps, P, plan.sched);
    else el3d_str<H><<<plan.grid, block, str_smem<H>(), s>>>(plan.maps, P, plan.sched);
    return cudaGetLastError();
}

cudaError_t configure(int H)
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

} // namespace

// A tile's x (or z) range may meet at most one CPML slab of that axis, and
// the compact slab layout must keep TMA's 16-byte rules (slab length and
// slab offset multiples of 4 floats along x).
static bool slab_tiles_ok(const Cpml1D& p, int T, bool xAxis)
{
    if (!p.on || p.n <= 2 * p.w) return true;
    if (xAxis && ((p.ns % 4) != 0 || ((p.n - p.ns) % 4) != 0)) return false;
    for (int c0 = 0; c0 < p.n; c0 += T)
        if (p.lo && c0 < p.w && c0 + T > p.n - p.w) return false;
    return true;
}

static bool make_psi_map(CUtensorMap* m, const float* base, int axis, const StepParams& P)
{
    if (!base) return false;
    switch (axis) {
    case 0: return make_map_dims(m, base, P.cx.ns, P.NZ, P.NY, TX, TZ);
    case 1: return make_map_dims(m, base, P.NX, P.NZ, P.cy.ns, TX, TZ);
    default: return make_map_dims(m, base, P.NX, P.cz.ns, P.NY, TX, TZ);
    }
}

// Builds the tensor maps for the current field/material pointers. Returns
// false when the streaming path does not apply (then the generic kernels run).
bool el3d_prepare(El3dPlan& plan, const StepParams& P, const float* rho, const float* M, const float* mu, int H, int* errWord)
{
    plan.ready = false;
    if (!P.is3d || H < 1 || H > 6 || (P.NX % 4) != 0 || P.NX < 8 || P.NZ < 2) return false;
    if (!rho || !M || !mu) return false;
    if (P.useCpml && (!slab_tiles_ok(P.cx, TX, true) || !slab_tiles_ok(P.cz, TZ, false))) return false;
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
    if (P.useCpml) {
        // order of the boxes in a stage: x-type, y-type, z-type (three each)
        const int vel[9] = {PS_SXX_X, PS_SXY_X, PS_SXZ_X, PS_SXY_Y, PS_SYY_Y, PS_SYZ_Y, PS_SXZ_Z, PS_SYZ_Z, PS_SZZ_Z};
        const int str[9] = {PS_VXX, PS_VYX, PS_VZX, PS_VYY, PS_VXY, PS_VZY, PS_VZZ, PS_VXZ, PS_VYZ};
        for (int j = 0; j < 9; ++j) {
            const int axis = j / 3 == 0 ? 0 : (j / 3 == 1 ? 1 : 2);
            const Cpml1D& ax = axis == 0 ? P.cx : (axis == 1 ? P.cy : P.cz);
            if (!ax.on) continue;
            ok &= make_psi_map(&T.psV[j], P.psi[vel[j]], axis, P);
            ok &= make_psi_map(&T.psS[j], P.psi[str[j]], axis, P);
        }
    }
    if (!ok) return false;
    plan.sched.ntx = (P.NX + TX - 1) / TX;
    plan.sched.ntz = (P.NZ + TZ - 1) / TZ;
    plan.sched.err = errWord;
    plan.H = H;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (long long)plan.sched.ntx * plan.sched.ntz;
    const long long work = tiles * P.NY;
    long long grid = 2LL * sms;           // two persistent CTAs per SM
    if (grid > work) grid = work;
    // each CTA's plane range must fit the segment table
    if (tiles / grid + 2 > MAXSEG) return false;
    plan.grid = static_cast<int>(grid);
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

// Runs the streaming kernels' bounded mbarrier wait on a barrier that no
// thread and no copy ever completes: the wait gives up after 2^14 polls and
// reports WAVE_ERR_TIMEOUT in *status, the kernel returns normally and the
// context stays usable. Diagnostic of the device-side failure path.
extern "C" int wave_selftest_bounded_wait(int* status)
{
    if (!status) return WAVE_ERR_ARG;
    int* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(int));
    if (e == cudaSuccess) {
        wave::wait_selftest_kernel<<<1, 32>>>(d, 1u << 14);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(status, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? WAVE_OK : WAVE_ERR_CUDA;
}
