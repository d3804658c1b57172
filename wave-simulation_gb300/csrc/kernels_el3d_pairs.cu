// kernels_el3d_pairs.cu — streaming sm_103a kernels for the 3-D elastic time
// step (FD3Delastic::run, ForwardSolver3Delastic.cpp:120-414) with two
// x-adjacent grid points per thread.
//
// The pipeline is the one of kernels_el3d.cu: persistent CTAs (two per SM)
// march column tiles down the depth axis y, TMA bulk-tensor copies fill a
// shared-memory stage ring whose "full" mbarriers carry the transaction bytes,
// the warp that releases a stage last refills it, and depth derivatives come
// from per-thread register queues. Here the tiles are 64 (x) x 8 (z): lane l
// of warp w owns the points x0 + 2l and x0 + 2l + 1 of row z0 + w, and both
// points travel as one 64-bit register pair. Shared-memory loads of the pair
// are 8-byte, the interior FD taps run as packed FP32 pairs (sub/fma .f32x2),
// the field and CPML psi stores are 8-byte, and the material averages share
// their neighbour reciprocals between the two points. Per grid point this
// roughly halves the load and FMA instructions of the one-point kernels and
// doubles the independent work each warp has in flight.
//
// Applies when NX % 4 == 0, every 64-wide tile meets at most one x CPML slab
// and the x slab width is even (a pair never straddles a slab edge). Interior
// rows use the compile-time FD coefficients times DT/DH; edge rows (order
// reduction, zero padding, free-surface image rows) use the operator's edge
// table, per point along x and per row along y and z.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "el3d.h"
#include "el3d_common.cuh"

namespace wave {
namespace el3dp {

using namespace el3d;

constexpr int TX = 64, TZ = 8, NTHR = 256;
static_assert(NTHR / 32 == NCWARP, "one warp per z row of the tile");
constexpr int CB = TX * TZ * 4;                  // centre box bytes
constexpr int PW = TX + 4, PH = TZ + 1;          // "+1" box (x0..x0+67, z0..z0+8)
constexpr int PBYTES = PW * PH * 4;
constexpr int PB = ((PBYTES + 127) / 128) * 128;

__host__ __device__ constexpr int hx_of(int H) { return H <= 4 ? 4 : 8; }
__host__ __device__ constexpr int bw_of(int H) { return TX + 2 * hx_of(H); }
__host__ __device__ constexpr int bh_of(int H) { return TZ + 2 * H; }
__host__ __device__ constexpr int hbytes_of(int H) { return bw_of(H) * bh_of(H) * 4; }
__host__ __device__ constexpr int hb_of(int H) { return ((hbytes_of(H) + 127) / 128) * 128; }

// ------------------------------------------------------------ packed pairs
__device__ __forceinline__ uint64_t pk(float2 v)
{
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y));
    return r;
}
__device__ __forceinline__ float2 upk(uint64_t r)
{
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}
__device__ __forceinline__ float2 add2(float2 a, float2 b)
{
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
    return upk(d);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
    return upk(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b)
{
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
    return upk(d);
}
// a * b + c per lane (fused, round to nearest: identical to fmaf per lane)
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)), "l"(pk(c)));
    return upk(d);
}
__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }
__device__ __forceinline__ float2 dup(float a) { return make_float2(a, a); }
// keeps the compiler from hoisting the shared-memory loads of later
// derivatives above this point (bounds the registers live at once)
__device__ __forceinline__ void sched_fence() { asm volatile("" ::: "memory"); }

// Interior coefficient pairs: c[j] = (fdc_j * DT/DH) for j < H; a derivative
// is sum_j c[j] * (u[lo_j] - u[hi_j]): tap j of the staggered operator and its
// mirror 2H-1-j carry coefficients c[j] and -c[j] (Derivatives.cpp:2000-2042)
// at offsets lo_j and hi_j (FWD: lo_j = j - H + 1, hi_j = H - j; BWD:
// lo_j = j - H, hi_j = H - 1 - j).
template <int H>
struct Coef {
    float2 c[H];
};
template <int H>
__device__ __forceinline__ Coef<H> make_coef(float scale)
{
    Coef<H> k;
#pragma unroll
    for (int j = 0; j < H; ++j) k.c[j] = dup(fdc(2 * H, j) * scale);
    return k;
}
template <int H, bool FWD>
__host__ __device__ constexpr int lo_tap(int j) { return FWD ? j - H + 1 : j - H; }
template <int H, bool FWD>
__host__ __device__ constexpr int hi_tap(int j) { return FWD ? H - j : H - 1 - j; }

// ------------------------------------------------------------ derivatives
// The step bodies first form all nine derivatives with the interior formulas
// (straight-line code, so the loads and FMAs of different derivatives
// interleave), then a rarely taken block replaces the ones that fall on edge
// rows: the outer pairs of the first and last x tile (per point), the outer
// z rows (per warp) and the outer y planes (per CTA).
//
// Along x, r points at the pair's first point in a shared-memory row (an even
// column, so pairs at even offsets are 8-byte aligned); the 2H + 2 values
// around the pair come from H + 1 aligned loads.
template <int H, bool FWD>
__device__ __forceinline__ float2 dx_int(const float* r, const Coef<H>& k)
{
    constexpr int A0 = -H - ((H & 1) ? 1 : 0);        // first aligned offset at or below -H
    constexpr int NA = (H + 1 - A0) / 2 + 1;           // pairs covering [A0, H + 1]
    float v[2 * NA];
#pragma unroll
    for (int m = 0; m < NA; ++m) {
        const float2 t = ld2(r + A0 + 2 * m);
        v[2 * m] = t.x;
        v[2 * m + 1] = t.y;
    }
    float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const int lo = lo_tap<H, FWD>(j) - A0, hi = hi_tap<H, FWD>(j) - A0;
        const float2 d = make_float2(v[lo] - v[hi], v[lo + 1] - v[hi + 1]);
        acc = j == 0 ? mul2(k.c[0], d) : fma2(k.c[j], d, acc);
    }
    return acc;
}

// Weighted x derivative used by the warps of the first and last x tile, whose
// outer pairs hold edge rows: d = sum_t W[t] * (u[t], u[t+1]) over the
// offsets t = -H..H of the pair's first point, with W the pair's row of the
// x-weight table in shared memory (each point's edge-table row, or the
// interior weights for an interior point). Uniform over the warp: no lane
// diverges.
template <int H>
__device__ __forceinline__ float2 dx_w(const float* r, const float2* W)
{
    constexpr int A0 = -H - ((H & 1) ? 1 : 0);
    constexpr int NA = (H + 1 - A0) / 2 + 1;
    float v[2 * NA];
#pragma unroll
    for (int m = 0; m < NA; ++m) {
        const float2 t = ld2(r + A0 + 2 * m);
        v[2 * m] = t.x;
        v[2 * m + 1] = t.y;
    }
    float2 a0 = make_float2(0.0f, 0.0f), a1 = a0;
#pragma unroll
    for (int t = -H; t <= H; ++t) {
        const float2 u = make_float2(v[t - A0], v[t + 1 - A0]);
        if ((t + H) & 1) a1 = fma2(W[t + H], u, a1);
        else a0 = fma2(W[t + H], u, a0);
    }
    return add2(a0, a1);
}

// rows of the x-weight table: 0 = interior pair, 1..NL = pairs starting at
// x = 0, 2, .., 2NL-2, NL+1..2NL = pairs starting at NX-2NL, .., NX-2, where
// NL pairs cover the edge band of H+1 columns on each side
template <int H>
struct XRows {
    static constexpr int NL = (H + 2) / 2;
    static constexpr int N = 1 + 2 * NL;
};
__device__ __forceinline__ int xrow_of(int xs, int NX, int NL)
{
    if (xs < 2 * NL) return 1 + xs / 2;
    if (xs >= NX - 2 * NL) return 1 + NL + (xs - (NX - 2 * NL)) / 2;
    return 0;
}
// weight of the point at column c for offset t (edge-table row or interior weights)
__device__ __forceinline__ float xweight(const Op1D& op, int c, int t)
{
    return interior_of(op, c) ? op.w[kMaxHalf + t] : __ldg(row_of(op, c) + t);
}
// fills the table for two x operators (called by all threads before the first barrier)
template <int H>
__device__ __forceinline__ void fill_xw(float2 (*xw)[XRows<H>::N][2 * H + 1], const Op1D& op0, const Op1D& op1, int NX)
{
    constexpr int NL = XRows<H>::NL, NR = XRows<H>::N, NT = 2 * H + 1;
    for (int e = threadIdx.x; e < 2 * NR * NT; e += blockDim.x) {
        const int o = e / (NR * NT), r = (e / NT) % NR, t = e % NT - H;
        const Op1D& op = o ? op1 : op0;
        const int xs = r == 0 ? NX / 2 - (NX / 2) % 2 : (r <= NL ? 2 * (r - 1) : NX - 2 * NL + 2 * (r - NL - 1));
        xw[o][r][t + H] = make_float2(xweight(op, xs, t), xweight(op, xs + 1, t));
    }
}

// along z (row stride BW): every row of the pair is aligned
template <int H, bool FWD>
__device__ __forceinline__ float2 dz_int(const float* p, int BW, const Coef<H>& k)
{
    float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const float2 d = sub2(ld2(p + lo_tap<H, FWD>(j) * BW), ld2(p + hi_tap<H, FWD>(j) * BW));
        acc = j == 0 ? mul2(k.c[0], d) : fma2(k.c[j], d, acc);
    }
    return acc;
}
template <int H>
__device__ __forceinline__ float2 dz_tab(const float* p, int BW, const float* row)
{
    float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int t = -H; t <= H; ++t) acc = fma2(dup(__ldg(row + t)), ld2(p + t * BW), acc);
    return acc;
}

// along y from the register queue (q[H] is the compute plane)
template <int H, bool FWD>
__device__ __forceinline__ float2 dy_int(const float2 (&q)[2 * H + 1], const Coef<H>& k)
{
    float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const float2 d = sub2(q[H + lo_tap<H, FWD>(j)], q[H + hi_tap<H, FWD>(j)]);
        acc = j == 0 ? mul2(k.c[0], d) : fma2(k.c[j], d, acc);
    }
    return acc;
}
template <int H>
__device__ __forceinline__ float2 dy_tab(const float2 (&q)[2 * H + 1], const float* row)
{
    float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int t = -H; t <= H; ++t) acc = fma2(dup(__ldg(row + t)), q[H + t], acc);
    return acc;
}

// ------------------------------------------------------------ per-column state
struct ColumnP {
    int x, z;                 // x: first point of the pair (even)
    bool ok;                  // the pair lies inside the grid (NX is even)
    bool zi;                  // interior row along z
    int xr;                   // row of the x-weight table (0: interior pair)
    bool xedge;               // some pair of the warp uses an edge row of the x-weight table
    int sx, sz;               // CPML slab indices (-1 outside); x + 1 is slab index sx + 1
    float2 axf, bxf, axh, bxh;
    float azf, bzf, azh, bzh;
    long long px, pz;         // psi offsets without the y term
};

__device__ __forceinline__ void column_setup(ColumnP& C, const StepParams& P, int x0, int z0, int NL)
{
    C.x = x0 + 2 * (threadIdx.x & 31);
    C.z = z0 + (threadIdx.x >> 5);
    C.ok = C.x < P.NX && C.z < P.NZ;
    C.xr = C.ok ? xrow_of(C.x, P.NX, NL) : 0;
    C.xedge = __any_sync(0xffffffffu, C.xr != 0);
    C.zi = interior_of(P.Dzf, C.z);
    C.sx = P.useCpml && C.ok ? slab_of(C.x, P.cx) : -1;
    C.sz = P.useCpml && C.ok ? slab_of(C.z, P.cz) : -1;
    C.axf = C.bxf = C.axh = C.bxh = make_float2(0.0f, 0.0f);
    C.azf = C.bzf = C.azh = C.bzh = 0.0f;
    if (C.sx >= 0) {
        C.axf = make_float2(P.cx.a_full[C.x], P.cx.a_full[C.x + 1]);
        C.bxf = make_float2(P.cx.b_full[C.x], P.cx.b_full[C.x + 1]);
        C.axh = make_float2(P.cx.a_half[C.x], P.cx.a_half[C.x + 1]);
        C.bxh = make_float2(P.cx.b_half[C.x], P.cx.b_half[C.x + 1]);
    }
    if (C.sz >= 0) { C.azf = P.cz.a_full[C.z]; C.bzf = P.cz.b_full[C.z]; C.azh = P.cz.a_half[C.z]; C.bzh = P.cz.b_half[C.z]; }
    C.px = C.sx + (long long)P.cx.ns * C.z;
    C.pz = C.x + (long long)P.NX * C.sz;
}

__device__ __forceinline__ float* psi_x(const StepParams& P, int slot, const ColumnP& C, int y)
{
    return P.psi[slot] + C.px + (long long)P.cx.ns * P.NZ * y;
}
__device__ __forceinline__ float* psi_z(const StepParams& P, int slot, const ColumnP& C, int y)
{
    return P.psi[slot] + C.pz + (long long)P.NX * P.cz.ns * y;
}
__device__ __forceinline__ float* psi_y(const StepParams& P, int slot, const ColumnP& C, const Plane& L)
{
    return P.psi[slot] + C.x + (long long)P.NX * (C.z + (long long)P.NZ * L.sy);
}

// CPML::applyCPML (CPML.cpp:84-95) on a pair: psi = b*psi + a*d; d += psi,
// old psi from the stage, new psi written to HBM
__device__ __forceinline__ void cpml2(float2& d, float2 ps, float* gpsi, float2 a, float2 b)
{
    ps = mul2(ps, b);
    ps = fma2(a, d, ps);
    st2(gpsi, ps);
    d = add2(d, ps);
}

// ------------------------------------------------------------ stage layout
template <int H, int NHALO, int NCEN>
struct Stage {
    static constexpr int HB = hb_of(H);
    static constexpr int CEN = NHALO * HB;
    static constexpr int PLUS = CEN + NCEN * CB;
    static constexpr int PSI = PLUS + PB;
    static constexpr int BYTES = PSI + 9 * CB;
    static constexpr int NST = 2;
};
// The velocity stage carries each stress field only with the halo its
// derivatives need: Sxx and Sxy along x (x-halo box), Syz and Szz along z
// (z-halo box), Sxz along both.
template <int H>
struct VelStage {
    static constexpr int XB = ((bw_of(H) * TZ * 4 + 127) / 128) * 128;   // x-halo box: BW x TZ
    static constexpr int HB = hb_of(H);                                  // x- and z-halo box: BW x BH
    static constexpr int ZB = ((TX * bh_of(H) * 4 + 127) / 128) * 128;   // z-halo box: TX x BH
    static constexpr int OXX = 0, OXY = XB, OXZ = 2 * XB, OYZ = 2 * XB + HB, OZZ = OYZ + ZB;
    static constexpr int CEN = OZZ + ZB;
    static constexpr int PLUS = CEN + 6 * CB;
    static constexpr int PSI = PLUS + PB;
    static constexpr int BYTES = PSI + 9 * CB;
    static constexpr int NST = 2;
    static constexpr uint32_t HALO_TX = 2 * bw_of(H) * TZ * 4 + hbytes_of(H) + 2 * TX * bh_of(H) * 4;   // delivered halo bytes
};
template <int H> using StrStage = Stage<H, 3, 10>;

struct PsiBoxes {
    int bx, bz, sy;
    __device__ __forceinline__ uint32_t bytes() const { return ((bx != kNoBox) + (sy >= 0) + (bz != kNoBox)) * 3u * CB; }
};
__device__ __forceinline__ PsiBoxes psi_boxes(const StepParams& P, int x0, int z0, int c)
{
    if (!P.useCpml) return {kNoBox, kNoBox, -1};
    return {slab_box(P.cx, x0, TX), slab_box(P.cz, z0, TZ), slab_of(c, P.cy)};
}
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

} // namespace el3dp

using namespace el3dp;

// ------------------------------------------------------------------------
// velocity pass (ForwardSolver3Delastic.cpp:174-277)
// ------------------------------------------------------------------------
template <int H>
__global__ void __launch_bounds__(NTHR, H <= 4 ? 2 : 1) el3dp_vel(const __grid_constant__ El3dMaps T, const StepParams P, const El3dSched S)
{
    using L = VelStage<H>;
    constexpr int NST = L::NST, HX = hx_of(H), BW = bw_of(H), TT = TX * TZ;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * L::BYTES);
    unsigned* rel = reinterpret_cast<unsigned*>(full + NST);
    __shared__ Segs G;
    __shared__ int abortRun;
    __shared__ volatile int failed;
    __shared__ int issued;
    __shared__ float2 xw[2][XRows<H>::N][2 * H + 1];   // x weights: Dxf, Dxb
    fill_xw<H>(xw, P.Dxf, P.Dxb, P.NX);
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
        if (compute) bytes += L::HALO_TX + 3 * CB;
        mbar_expect_tx(bar, bytes);
        issue_psi(B, T.psV, st + L::PSI, bar, x0, z0, c);
        unsigned char* cen = st + L::CEN;
        tma_load(cen + 0 * CB, &T.cSxy, bar, x0, z0, q);
        tma_load(cen + 1 * CB, &T.cSyy, bar, x0, z0, q);
        tma_load(cen + 2 * CB, &T.cSyz, bar, x0, z0, q);
        tma_load(st + L::PLUS, &T.pRho, bar, x0, z0, c + 1);
        if (compute) {
            tma_load(st + L::OXX, &T.hSxx, bar, x0 - HX, z0, c);
            tma_load(st + L::OXY, &T.hSxy, bar, x0 - HX, z0, c);
            tma_load(st + L::OXZ, &T.hSxz, bar, x0 - HX, z0 - H, c);
            tma_load(st + L::OYZ, &T.hSyz, bar, x0, z0 - H, c);
            tma_load(st + L::OZZ, &T.hSzz, bar, x0, z0 - H, c);
            tma_load(cen + 3 * CB, &T.cVx, bar, x0, z0, c);
            tma_load(cen + 4 * CB, &T.cVy, bar, x0, z0, c);
            tma_load(cen + 5 * CB, &T.cVz, bar, x0, z0, c);
        }
    };
    if (threadIdx.x == 0) start_feed<NST>(G, total, &issued, issue);

    const int pi = warp * TX + 2 * lane;            // the pair in a centre / psi box
    const int ci = (warp + H) * BW + (HX + 2 * lane);   // the pair in the x- and z-halo box
    const int xi = warp * BW + (HX + 2 * lane);         // the pair in an x-halo box
    const int zi = (warp + H) * TX + 2 * lane;          // the pair in a z-halo box
    const int ri = warp * PW + 2 * lane;            // the pair in the "+1" box
    float2 qxy[2 * H + 1], qyy[2 * H + 1], qyz[2 * H + 1];
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) qxy[k] = qyy[k] = qyz[k] = make_float2(0.0f, 0.0f);
    // rho at the compute plane: (x,z), (x+1,z), (x,z+1) for both points
    float2 r0 = make_float2(0.0f, 0.0f), rx = r0, rz = r0;
    const Op1D& DybS = P.fs ? P.DybS : P.Dyb;
    const Op1D& DyfS = P.fs ? P.DyfS : P.Dyf;
    const Coef<H> K = make_coef<H>(P.scale);
    Cursor cur{0, 0};
    ColumnP C;

    int it = 0;
    for (; it < total; ++it) {
        const int s = it % NST;
        const int tile = G.tile[cur.seg], ya = G.ya[cur.seg];
        if (cur.k == 0) column_setup(C, P, (tile % S.ntx) * TX, (tile / S.ntx) * TZ, XRows<H>::NL);
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
        qxy[2 * H] = ld2(cen + 0 * TT + pi);
        qyy[2 * H] = ld2(cen + 1 * TT + pi);
        qyz[2 * H] = ld2(cen + 2 * TT + pi);
        const float* rb = reinterpret_cast<const float*>(st + L::PLUS);
        const float2 rn = ld2(rb + ri);             // rho at (x, z, y+1), (x+1, z, y+1)
        if (compute && C.ok) {
            Plane Y;
            plane_setup(Y, P, y);
            const float* hSxx = reinterpret_cast<const float*>(st + L::OXX) + xi;
            const float* hSxy = reinterpret_cast<const float*>(st + L::OXY) + xi;
            const float* hSxz = reinterpret_cast<const float*>(st + L::OXZ) + ci;
            const float* hSyz = reinterpret_cast<const float*>(st + L::OYZ) + zi;
            const float* hSzz = reinterpret_cast<const float*>(st + L::OZZ) + zi;
            const float* ps = reinterpret_cast<const float*>(st + L::PSI) + pi;
            const float* ryb = Y.yi ? nullptr : row_of(DybS, y);
            const float* ryf = Y.yi ? nullptr : row_of(DyfS, y);
            const long long i = C.x + (long long)P.NX * (C.z + (long long)P.NZ * y);
            {
                float2 dSxx_x, dSxy_x, dSxz_x;
                if (C.xedge) {
                    dSxx_x = dx_w<H>(hSxx, xw[0][C.xr]);
                    dSxy_x = dx_w<H>(hSxy, xw[1][C.xr]);
                    dSxz_x = dx_w<H>(hSxz, xw[1][C.xr]);
                } else {
                    dSxx_x = dx_int<H, true>(hSxx, K);
                    dSxy_x = dx_int<H, false>(hSxy, K);
                    dSxz_x = dx_int<H, false>(hSxz, K);
                }
                float2 dSxy_y, dSyy_y, dSyz_y;
                if (Y.yi) {
                    dSxy_y = dy_int<H, false>(qxy, K);
                    dSyy_y = dy_int<H, true>(qyy, K);
                    dSyz_y = dy_int<H, false>(qyz, K);
                } else {
                    dSxy_y = dy_tab<H>(qxy, ryb);
                    dSyy_y = dy_tab<H>(qyy, ryf);
                    dSyz_y = dy_tab<H>(qyz, ryb);
                }
                float2 dSxz_z, dSyz_z, dSzz_z;
                if (C.zi) {
                    dSxz_z = dz_int<H, false>(hSxz, BW, K);
                    dSyz_z = dz_int<H, false>(hSyz, TX, K);
                    dSzz_z = dz_int<H, true>(hSzz, TX, K);
                } else {
                    dSxz_z = dz_tab<H>(hSxz, BW, row_of(P.Dzb, C.z));
                    dSyz_z = dz_tab<H>(hSyz, TX, row_of(P.Dzb, C.z));
                    dSzz_z = dz_tab<H>(hSzz, TX, row_of(P.Dzf, C.z));
                }
                if (C.sx >= 0) {
                    cpml2(dSxx_x, ld2(ps + 0 * TT), psi_x(P, PS_SXX_X, C, y), C.axh, C.bxh);
                    cpml2(dSxy_x, ld2(ps + 1 * TT), psi_x(P, PS_SXY_X, C, y), C.axf, C.bxf);
                    cpml2(dSxz_x, ld2(ps + 2 * TT), psi_x(P, PS_SXZ_X, C, y), C.axf, C.bxf);
                }
                if (Y.sy >= 0) {
                    cpml2(dSxy_y, ld2(ps + 3 * TT), psi_y(P, PS_SXY_Y, C, Y), dup(Y.ayf), dup(Y.byf));
                    cpml2(dSyy_y, ld2(ps + 4 * TT), psi_y(P, PS_SYY_Y, C, Y), dup(Y.ayh), dup(Y.byh));
                    cpml2(dSyz_y, ld2(ps + 5 * TT), psi_y(P, PS_SYZ_Y, C, Y), dup(Y.ayf), dup(Y.byf));
                }
                if (C.sz >= 0) {
                    cpml2(dSxz_z, ld2(ps + 6 * TT), psi_z(P, PS_SXZ_Z, C, y), dup(C.azf), dup(C.bzf));
                    cpml2(dSyz_z, ld2(ps + 7 * TT), psi_z(P, PS_SYZ_Z, C, y), dup(C.azf), dup(C.bzf));
                    cpml2(dSzz_z, ld2(ps + 8 * TT), psi_z(P, PS_SZZ_Z, C, y), dup(C.azh), dup(C.bzh));
                }
                const bool x2in = C.x + 2 < P.NX, yin = y + 1 < P.NY, zin = C.z + 1 < P.NZ;
                float2 u = add2(add2(dSxx_x, dSxy_y), dSxz_z);
                u = mul2(u, make_float2(inv_avg2f(r0.x, rx.x, true), inv_avg2f(r0.y, rx.y, x2in)));
                st2(P.f[F_VX] + i, add2(ld2(cen + 3 * TT + pi), u));
                u = add2(add2(dSxy_x, dSyy_y), dSyz_z);
                u = mul2(u, make_float2(inv_avg2f(r0.x, rn.x, yin), inv_avg2f(r0.y, rn.y, yin)));
                st2(P.f[F_VY] + i, add2(ld2(cen + 4 * TT + pi), u));
                u = add2(add2(dSxz_x, dSyz_y), dSzz_z);
                u = mul2(u, make_float2(inv_avg2f(r0.x, rz.x, zin), inv_avg2f(r0.y, rz.y, zin)));
                st2(P.f[F_VZ] + i, add2(ld2(cen + 5 * TT + pi), u));
            }
        }
        // carry rho of plane y+1 into the next iteration
        r0 = rn;
        rx = make_float2(rn.y, rb[ri + 2]);
        rz = ld2(rb + ri + PW);
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
__global__ void __launch_bounds__(NTHR, H <= 4 ? 2 : 1) el3dp_str(const __grid_constant__ El3dMaps T, const StepParams P, const El3dSched S)
{
    using L = StrStage<H>;
    constexpr int NST = L::NST, HX = hx_of(H), BW = bw_of(H), TT = TX * TZ;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * L::BYTES);
    unsigned* rel = reinterpret_cast<unsigned*>(full + NST);
    __shared__ Segs G;
    __shared__ int abortRun;
    __shared__ volatile int failed;
    __shared__ int issued;
    __shared__ float2 xw[2][XRows<H>::N][2 * H + 1];   // x weights: Dxb, Dxf
    fill_xw<H>(xw, P.Dxb, P.Dxf, P.NX);
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

    const int pi = warp * TX + 2 * lane;
    const int ci = (warp + H) * BW + (HX + 2 * lane);
    const int ri = warp * PW + 2 * lane;
    float2 qx[2 * H + 1], qy[2 * H + 1], qz[2 * H + 1];
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) qx[k] = qy[k] = qz[k] = make_float2(0.0f, 0.0f);
    // inverse clamped mu at the compute plane, row z: (x, x+1) and x+2; row z+1 likewise; and mu itself at (x, x+1)
    float2 i0 = make_float2(1.0f, 1.0f), i1 = i0, m00 = i0;
    float i0r = 1.0f, i1r = 1.0f;
    const Coef<H> K = make_coef<H>(P.scale);
    Cursor cur{0, 0};
    ColumnP C;

    int it = 0;
    for (; it < total; ++it) {
        const int s = it % NST;
        const int tile = G.tile[cur.seg], ya = G.ya[cur.seg];
        if (cur.k == 0) column_setup(C, P, (tile % S.ntx) * TX, (tile / S.ntx) * TZ, XRows<H>::NL);
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
        qx[2 * H] = ld2(cen + 0 * TT + pi);
        qy[2 * H] = ld2(cen + 1 * TT + pi);
        qz[2 * H] = ld2(cen + 2 * TT + pi);
        const float* mb = reinterpret_cast<const float*>(st + L::PLUS);
        if (compute && C.ok) {
            Plane Y;
            plane_setup(Y, P, y);
            const float* hVx = reinterpret_cast<const float*>(st + 0 * L::HB) + ci;
            const float* hVy = reinterpret_cast<const float*>(st + 1 * L::HB) + ci;
            const float* hVz = reinterpret_cast<const float*>(st + 2 * L::HB) + ci;
            const float* ps = reinterpret_cast<const float*>(st + L::PSI) + pi;
            const float* ryf = Y.yi ? nullptr : row_of(P.Dyf, y);
            const float* ryb = Y.yi ? nullptr : row_of(P.Dyb, y);
            const long long i = C.x + (long long)P.NX * (C.z + (long long)P.NZ * y);
            const bool x2in = C.x + 2 < P.NX, inY = y + 1 < P.NY, inZ = C.z + 1 < P.NZ;
            {
                float2 vxx, vyx, vzx;
                if (C.xedge) {
                    vxx = dx_w<H>(hVx, xw[0][C.xr]);
                    vyx = dx_w<H>(hVy, xw[1][C.xr]);
                    vzx = dx_w<H>(hVz, xw[1][C.xr]);
                } else {
                    vxx = dx_int<H, false>(hVx, K);
                    vyx = dx_int<H, true>(hVy, K);
                    vzx = dx_int<H, true>(hVz, K);
                }
                float2 vyy, vxy, vzy;
                if (Y.yi) {
                    vyy = dy_int<H, false>(qy, K);
                    vxy = dy_int<H, true>(qx, K);
                    vzy = dy_int<H, true>(qz, K);
                } else {
                    vyy = dy_tab<H>(qy, ryb);
                    vxy = dy_tab<H>(qx, ryf);
                    vzy = dy_tab<H>(qz, ryf);
                }
                float2 vzz, vxz, vyz;
                if (C.zi) {
                    vzz = dz_int<H, false>(hVz, BW, K);
                    vxz = dz_int<H, true>(hVx, BW, K);
                    vyz = dz_int<H, true>(hVy, BW, K);
                } else {
                    vzz = dz_tab<H>(hVz, BW, row_of(P.Dzb, C.z));
                    vxz = dz_tab<H>(hVx, BW, row_of(P.Dzf, C.z));
                    vyz = dz_tab<H>(hVy, BW, row_of(P.Dzf, C.z));
                }
                if (C.sx >= 0) {
                    cpml2(vxx, ld2(ps + 0 * TT), psi_x(P, PS_VXX, C, y), C.axf, C.bxf);
                    cpml2(vyx, ld2(ps + 1 * TT), psi_x(P, PS_VYX, C, y), C.axh, C.bxh);
                    cpml2(vzx, ld2(ps + 2 * TT), psi_x(P, PS_VZX, C, y), C.axh, C.bxh);
                }
                if (Y.sy >= 0) {
                    cpml2(vyy, ld2(ps + 3 * TT), psi_y(P, PS_VYY, C, Y), dup(Y.ayf), dup(Y.byf));
                    cpml2(vxy, ld2(ps + 4 * TT), psi_y(P, PS_VXY, C, Y), dup(Y.ayh), dup(Y.byh));
                    cpml2(vzy, ld2(ps + 5 * TT), psi_y(P, PS_VZY, C, Y), dup(Y.ayh), dup(Y.byh));
                }
                if (C.sz >= 0) {
                    cpml2(vzz, ld2(ps + 6 * TT), psi_z(P, PS_VZZ, C, y), dup(C.azf), dup(C.bzf));
                    cpml2(vxz, ld2(ps + 7 * TT), psi_z(P, PS_VXZ, C, y), dup(C.azh), dup(C.bzh));
                    cpml2(vyz, ld2(ps + 8 * TT), psi_z(P, PS_VYZ, C, y), dup(C.azh), dup(C.bzh));
                }
                // mu of plane y+1 at columns x, x+1, x+2 of rows z and z+1, its clamped inverses,
                // and the harmonic averages XY: (x,y) (x+1,y) (x,y+1) (x+1,y+1); XZ: (x,z) (x+1,z)
                // (x,z+1) (x+1,z+1); YZ: (y,z) (y+1,z) (y,z+1) (y+1,z+1)
                // (calcAverageMatrixXY/XZ/YZ, Modelparameter.cpp:533-624)
                const float2 n0 = ld2(mb + ri), n1 = ld2(mb + ri + PW);
                const float j0x = inv_clampedf(n0.x), j0y = inv_clampedf(n0.y), j0r = inv_clampedf(mb[ri + 2]);
                const float j1x = inv_clampedf(n1.x), j1y = inv_clampedf(n1.y);
                const float2 muXY = make_float2(harm4f(i0.x, i0.y, j0x, j0y, true, inY), harm4f(i0.y, i0r, j0y, j0r, x2in, inY));
                const float2 muXZ = make_float2(harm4f(i0.x, i0.y, i1.x, i1.y, true, inZ), harm4f(i0.y, i0r, i1.y, i1r, x2in, inZ));
                const float2 muYZ = make_float2(harm4f(i0.x, j0x, i1.x, j1x, inY, inZ), harm4f(i0.y, j0y, i1.y, j1y, inY, inZ));
                const float2 M = ld2(cen + 9 * TT + pi);
                const float2 mu = make_float2(m00.x < 1.0f ? 1.0f : m00.x, m00.y < 1.0f ? 1.0f : m00.y);
                float2 sxx = ld2(cen + 3 * TT + pi), syy = ld2(cen + 4 * TT + pi), szz = ld2(cen + 5 * TT + pi);
                float2 u = add2(add2(vxx, vyy), vzz);
                u = mul2(u, M);
                sxx = add2(sxx, u);
                syy = add2(syy, u);
                szz = add2(szz, u);
                const float2 two = dup(2.0f);
                u = mul2(add2(vyy, vzz), mu);
                sxx = sub2(sxx, mul2(two, u));
                u = mul2(add2(vxx, vzz), mu);
                syy = sub2(syy, mul2(two, u));
                u = mul2(add2(vxx, vyy), mu);
                szz = sub2(szz, mul2(two, u));
                const float2 sxy = add2(ld2(cen + 6 * TT + pi), mul2(add2(vxy, vyx), muXY));
                const float2 sxz = add2(ld2(cen + 7 * TT + pi), mul2(add2(vxz, vzx), muXZ));
                const float2 syz = add2(ld2(cen + 8 * TT + pi), mul2(add2(vyz, vzy), muYZ));
                if (P.fs && y == 0) {
                    // FreeSurface3Delastic.cpp:15-47 per point
                    float sv = M.x - 2.0f * mu.x, sh = sv * sv;
                    sh /= M.x;
                    sh *= -1.0f;
                    syy.x = 0.0f;
                    float t = sh * (vxx.x + vzz.x);
                    sxx.x += t; szz.x += t;
                    t = sv * vyy.x;
                    sxx.x -= t; szz.x -= t;
                    sv = M.y - 2.0f * mu.y;
                    sh = sv * sv;
                    sh /= M.y;
                    sh *= -1.0f;
                    syy.y = 0.0f;
                    t = sh * (vxx.y + vzz.y);
                    sxx.y += t; szz.y += t;
                    t = sv * vyy.y;
                    sxx.y -= t; szz.y -= t;
                }
                float2 d = make_float2(1.0f, 1.0f);
                if (P.abs) d = make_float2(abs_damp(P, C.x, y, C.z), abs_damp(P, C.x + 1, y, C.z));
                st2(P.f[F_SXX] + i, mul2(sxx, d));
                st2(P.f[F_SYY] + i, mul2(syy, d));
                st2(P.f[F_SZZ] + i, mul2(szz, d));
                st2(P.f[F_SXY] + i, mul2(sxy, d));
                st2(P.f[F_SXZ] + i, mul2(sxz, d));
                st2(P.f[F_SYZ] + i, mul2(syz, d));
            }
        }
        // carry mu of plane y+1 into the next iteration
        {
            const float2 n0 = ld2(mb + ri), n1 = ld2(mb + ri + PW);
            m00 = n0;
            i0 = make_float2(inv_clampedf(n0.x), inv_clampedf(n0.y));
            i0r = inv_clampedf(mb[ri + 2]);
            i1 = make_float2(inv_clampedf(n1.x), inv_clampedf(n1.y));
            i1r = inv_clampedf(mb[ri + PW + 2]);
        }
        release_and_refill<NST>(it, total, cur, G, rel, &issued, &failed, issue);
        if (__any_sync(0xffffffffu, failed != 0)) break;
        cur.advance(G);
    }
    finish_ring<NST>(full, &issued, &failed);
}

// ------------------------------------------------------------------------
// visco-elastic stress pass (ForwardSolver3Dviscoelastic.cpp:270-446, free
// surface FreeSurface3Dviscoelastic.cpp:17-75): the stress kernel's pipeline
// and derivatives; the stage also carries a tau_S "+1" box, from which the
// shear tau averages (4-point arithmetic, calc4PointAverageMatrixRow edge
// rules) and 1 + L tau_S are formed in-kernel. tau_P and the memory
// variables are read and written at the pair itself with 8-byte accesses
// (no halo). The update of each point follows visco_s_body (kernels.cu) op
// for op.
// ------------------------------------------------------------------------
template <int H>
struct VStrStage {
    static constexpr int HB = hb_of(H);
    static constexpr int CEN = 3 * HB;
    static constexpr int PLUS = CEN + 10 * CB;   // mu "+1" box
    static constexpr int PLUS2 = PLUS + PB;      // tau_S "+1" box
    static constexpr int PSI = PLUS2 + PB;
    static constexpr int BYTES = PSI + 9 * CB;
    static constexpr int NST = 2;
};

// 4-point arithmetic average with the edge fallbacks (the avg4 of the model
// preparation, kernels.cu), same operation order
__device__ __forceinline__ float avg4f(float a1, float a2, float a3, float a4, bool inA, bool inB)
{
    float s;
    if (inA && inB) {
        s = 0.25f * a1; s += 0.25f * a2; s += 0.25f * a3; s += 0.25f * a4;
    } else if (inA) {
        s = 0.5f * a2; s += 0.5f * a1;
    } else if (inB) {
        s = 0.5f * a3; s += 0.5f * a1;
    } else {
        s = 1.0f * a1;
    }
    return s;
}

// one point's visco-elastic stress update; d*: CPML-corrected derivatives
// (vxx = dx vx, vxy = dy vx, ...); S: sxx syy szz, Sh: sxy sxz syz, R[k][l]:
// the memory variables of rxx ryy rzz rxy rxz ryz (in/out)
template <int LL>
__device__ __forceinline__ void visco_point(const StepParams& P, float vxx, float vyy, float vzz, float vxy, float vyx, float vxz,
                                            float vzx, float vyz, float vzy, float M, float mu, float tauP, float tauS,
                                            float opP, float opS, const float muAv[3], const float tauAv[3], float S[3],
                                            float Sh[3], float (&R)[6][LL], bool fsRow)
{
    const float DTh = P.DThalf;
    float u = vxx;
    u += vyy;
    u += vzz;
    u *= M;
#pragma unroll
    for (int l = 0; l < LL; ++l) {
        float u2 = P.invRelax[l] * u;
        u2 *= tauP;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            S[k] += DTh * R[k][l];
            R[k][l] *= P.c1[l];
            R[k][l] -= u2;
        }
    }
    u *= opP;
#pragma unroll
    for (int k = 0; k < 3; ++k) S[k] += u;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float sum = k == 0 ? vyy + vzz : (k == 1 ? vxx + vzz : vxx + vyy);
        u = sum;
        u *= mu;
        u *= 2.0f;
#pragma unroll
        for (int l = 0; l < LL; ++l) {
            float u2 = P.invRelax[l] * u;
            u2 *= tauS;
            R[k][l] += u2;
            R[k][l] *= P.c2[l];
            S[k] += DTh * R[k][l];
        }
        u *= opS;
        S[k] -= u;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        u = k == 0 ? vxy : (k == 1 ? vxz : vyz);
        const float ut = k == 0 ? vyx : (k == 1 ? vzx : vzy);
        u += ut;
        u *= muAv[k];
        float sh = Sh[k];
#pragma unroll
        for (int l = 0; l < LL; ++l) {
            float r = R[3 + k][l];
            sh += DTh * r;
            r *= P.c1[l];
            float u2 = P.invRelax[l] * u;
            u2 *= tauAv[k];
            r -= u2;
            r *= P.c2[l];
            sh += DTh * r;
            R[3 + k][l] = r;
        }
        u *= opS;
        Sh[k] = sh + u;
    }
    if (fsRow) {
        // FreeSurfaceViscoelastic::setModelparameter (FreeSurfaceViscoelastic.cpp:12-97), as in visco_s_body
        float temp = -2.0f * mu * opS;
        float temp2 = M * opP;
        temp += temp2;
        const float itemp2 = 1.0f / temp2;
        const float sV = temp;
        float sH = -1.0f * temp;
        sH *= temp;
        sH *= itemp2;
        const float hsum = vxx + vzz;
        const int kk[2] = {0, 2};
#pragma unroll
        for (int l = 0; l < LL; ++l)
#pragma unroll
            for (int q = 0; q < 2; ++q) S[kk[q]] -= DTh * R[kk[q]][l];
#pragma unroll
        for (int q = 0; q < 2; ++q) S[kk[q]] += sH * hsum;
#pragma unroll
        for (int q = 0; q < 2; ++q) S[kk[q]] -= sV * vyy;
        float t3 = 2.0f * mu * tauS;
        t3 -= M * tauP;
        float ratio = 2.0f * mu * opS;
        ratio /= M * opP;
        ratio -= 1.0f;
#pragma unroll
        for (int l = 0; l < LL; ++l) {
            float rv = t3; rv *= P.c2[l]; rv /= P.relaxTime[l];
            float rh = t3; rh *= ratio; rh *= P.c2[l]; rh /= P.relaxTime[l];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                R[kk[q]][l] += rh * hsum;
                R[kk[q]][l] -= rv * vyy;
                S[kk[q]] += DTh * R[kk[q]][l];
            }
        }
        S[1] = 0.0f;
#pragma unroll
        for (int l = 0; l < LL; ++l) R[1][l] = 0.0f;
    }
}

template <int H, int LL>
__global__ void __launch_bounds__(NTHR, 2) el3dp_vstr(const __grid_constant__ El3dMaps T, const StepParams P, const El3dSched S)
{
    using L = VStrStage<H>;
    constexpr int NST = L::NST, HX = hx_of(H), BW = bw_of(H), TT = TX * TZ;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + NST * L::BYTES);
    unsigned* rel = reinterpret_cast<unsigned*>(full + NST);
    __shared__ Segs G;
    __shared__ int abortRun;
    __shared__ volatile int failed;
    __shared__ int issued;
    __shared__ float2 xw[2][XRows<H>::N][2 * H + 1];   // x weights: Dxb, Dxf
    fill_xw<H>(xw, P.Dxb, P.Dxf, P.NX);
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
        uint32_t bytes = 3 * CB + 2 * PBYTES + B.bytes();
        if (compute) bytes += 3 * hbytes_of(H) + 7 * CB;
        mbar_expect_tx(bar, bytes);
        issue_psi(B, T.psS, st + L::PSI, bar, x0, z0, c);
        unsigned char* cen = st + L::CEN;
        tma_load(cen + 0 * CB, &T.cVx, bar, x0, z0, q);
        tma_load(cen + 1 * CB, &T.cVy, bar, x0, z0, q);
        tma_load(cen + 2 * CB, &T.cVz, bar, x0, z0, q);
        tma_load(st + L::PLUS, &T.pMu, bar, x0, z0, c + 1);
        tma_load(st + L::PLUS2, &T.pTauS, bar, x0, z0, c + 1);
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

    const int pi = warp * TX + 2 * lane;
    const int ci = (warp + H) * BW + (HX + 2 * lane);
    const int ri = warp * PW + 2 * lane;
    float2 qx[2 * H + 1], qy[2 * H + 1], qz[2 * H + 1];
#pragma unroll
    for (int k = 0; k <= 2 * H; ++k) qx[k] = qy[k] = qz[k] = make_float2(0.0f, 0.0f);
    // plane-y values carried from the previous iteration's "+1" boxes:
    // inverse clamped mu and mu at (x, x+1), x+2 of rows z and z+1; tau_S likewise
    float2 i0 = make_float2(1.0f, 1.0f), i1 = i0, m00 = i0;
    float i0r = 1.0f, i1r = 1.0f;
    float2 t0 = make_float2(0.0f, 0.0f), t1 = t0;
    float t0r = 0.0f, t1r = 0.0f;
    const float Lf = static_cast<float>(LL);
    const Coef<H> K = make_coef<H>(P.scale);
    Cursor cur{0, 0};
    ColumnP C;

    int it = 0;
    for (; it < total; ++it) {
        const int s = it % NST;
        const int tile = G.tile[cur.seg], ya = G.ya[cur.seg];
        if (cur.k == 0) column_setup(C, P, (tile % S.ntx) * TX, (tile / S.ntx) * TZ, XRows<H>::NL);
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
        qx[2 * H] = ld2(cen + 0 * TT + pi);
        qy[2 * H] = ld2(cen + 1 * TT + pi);
        qz[2 * H] = ld2(cen + 2 * TT + pi);
        const float* mb = reinterpret_cast<const float*>(st + L::PLUS);
        const float* tb = reinterpret_cast<const float*>(st + L::PLUS2);
        if (compute && C.ok) {
            Plane Y;
            plane_setup(Y, P, y);
            const float* hVx = reinterpret_cast<const float*>(st + 0 * L::HB) + ci;
            const float* hVy = reinterpret_cast<const float*>(st + 1 * L::HB) + ci;
            const float* hVz = reinterpret_cast<const float*>(st + 2 * L::HB) + ci;
            const float* ps = reinterpret_cast<const float*>(st + L::PSI) + pi;
            const float* ryf = Y.yi ? nullptr : row_of(P.Dyf, y);
            const float* ryb = Y.yi ? nullptr : row_of(P.Dyb, y);
            const long long i = C.x + (long long)P.NX * (C.z + (long long)P.NZ * y);
            const bool x2in = C.x + 2 < P.NX, inY = y + 1 < P.NY, inZ = C.z + 1 < P.NZ;
            float2 vxx, vyx, vzx;
            if (C.xedge) {
                vxx = dx_w<H>(hVx, xw[0][C.xr]);
                vyx = dx_w<H>(hVy, xw[1][C.xr]);
                vzx = dx_w<H>(hVz, xw[1][C.xr]);
            } else {
                vxx = dx_int<H, false>(hVx, K);
                vyx = dx_int<H, true>(hVy, K);
                vzx = dx_int<H, true>(hVz, K);
            }
            float2 vyy, vxy, vzy;
            if (Y.yi) {
                vyy = dy_int<H, false>(qy, K);
                vxy = dy_int<H, true>(qx, K);
                vzy = dy_int<H, true>(qz, K);
            } else {
                vyy = dy_tab<H>(qy, ryb);
                vxy = dy_tab<H>(qx, ryf);
                vzy = dy_tab<H>(qz, ryf);
            }
            float2 vzz, vxz, vyz;
            if (C.zi) {
                vzz = dz_int<H, false>(hVz, BW, K);
                vxz = dz_int<H, true>(hVx, BW, K);
                vyz = dz_int<H, true>(hVy, BW, K);
            } else {
                vzz = dz_tab<H>(hVz, BW, row_of(P.Dzb, C.z));
                vxz = dz_tab<H>(hVx, BW, row_of(P.Dzf, C.z));
                vyz = dz_tab<H>(hVy, BW, row_of(P.Dzf, C.z));
            }
            if (C.sx >= 0) {
                cpml2(vxx, ld2(ps + 0 * TT), psi_x(P, PS_VXX, C, y), C.axf, C.bxf);
                cpml2(vyx, ld2(ps + 1 * TT), psi_x(P, PS_VYX, C, y), C.axh, C.bxh);
                cpml2(vzx, ld2(ps + 2 * TT), psi_x(P, PS_VZX, C, y), C.axh, C.bxh);
            }
            if (Y.sy >= 0) {
                cpml2(vyy, ld2(ps + 3 * TT), psi_y(P, PS_VYY, C, Y), dup(Y.ayf), dup(Y.byf));
                cpml2(vxy, ld2(ps + 4 * TT), psi_y(P, PS_VXY, C, Y), dup(Y.ayh), dup(Y.byh));
                cpml2(vzy, ld2(ps + 5 * TT), psi_y(P, PS_VZY, C, Y), dup(Y.ayh), dup(Y.byh));
            }
            if (C.sz >= 0) {
                cpml2(vzz, ld2(ps + 6 * TT), psi_z(P, PS_VZZ, C, y), dup(C.azf), dup(C.bzf));
                cpml2(vxz, ld2(ps + 7 * TT), psi_z(P, PS_VXZ, C, y), dup(C.azh), dup(C.bzh));
                cpml2(vyz, ld2(ps + 8 * TT), psi_z(P, PS_VYZ, C, y), dup(C.azh), dup(C.bzh));
            }
            // mu and tau_S of plane y+1 (the "+1" boxes) and the averages
            const float2 n0 = ld2(mb + ri), n1 = ld2(mb + ri + PW);
            const float j0x = inv_clampedf(n0.x), j0y = inv_clampedf(n0.y), j0r = inv_clampedf(mb[ri + 2]);
            const float j1x = inv_clampedf(n1.x), j1y = inv_clampedf(n1.y);
            const float muXY[2] = {harm4f(i0.x, i0.y, j0x, j0y, true, inY), harm4f(i0.y, i0r, j0y, j0r, x2in, inY)};
            const float muXZ[2] = {harm4f(i0.x, i0.y, i1.x, i1.y, true, inZ), harm4f(i0.y, i0r, i1.y, i1r, x2in, inZ)};
            const float muYZ[2] = {harm4f(i0.x, j0x, i1.x, j1x, inY, inZ), harm4f(i0.y, j0y, i1.y, j1y, inY, inZ)};
            const float2 u0 = ld2(tb + ri), u1 = ld2(tb + ri + PW);
            const float u0r = tb[ri + 2];
            const float tXY[2] = {avg4f(t0.x, t0.y, u0.x, u0.y, true, inY), avg4f(t0.y, t0r, u0.y, u0r, x2in, inY)};
            const float tXZ[2] = {avg4f(t0.x, t0.y, t1.x, t1.y, true, inZ), avg4f(t0.y, t0r, t1.y, t1r, x2in, inZ)};
            const float tYZ[2] = {avg4f(t0.x, u0.x, t1.x, u1.x, inY, inZ), avg4f(t0.y, u0.y, t1.y, u1.y, inY, inZ)};
            const float2 M = ld2(cen + 9 * TT + pi);
            const float2 tauP = ld2(P.m[M_TAUP] + i);
            float2 sxx = ld2(cen + 3 * TT + pi), syy = ld2(cen + 4 * TT + pi), szz = ld2(cen + 5 * TT + pi);
            float2 sxy = ld2(cen + 6 * TT + pi), sxz = ld2(cen + 7 * TT + pi), syz = ld2(cen + 8 * TT + pi);
            const int slotR[6] = {R_XX, R_YY, R_ZZ, R_XY, R_XZ, R_YZ};
            float Ra[6][LL], Rb[6][LL];
#pragma unroll
            for (int k = 0; k < 6; ++k)
#pragma unroll
                for (int l = 0; l < LL; ++l) {
                    const float2 r = ld2(P.r[slotR[k]][l] + i);
                    Ra[k][l] = r.x;
                    Rb[k][l] = r.y;
                }
            const bool fsRow = P.fs && y == 0;
            {
                float Sn[3] = {sxx.x, syy.x, szz.x}, Sh[3] = {sxy.x, sxz.x, syz.x};
                const float mav[3] = {muXY[0], muXZ[0], muYZ[0]}, tav[3] = {tXY[0], tXZ[0], tYZ[0]};
                const float mu = m00.x;   // the prepared modulus (already clamped)
                const float opP = 1.0f + Lf * tauP.x, opS = 1.0f + Lf * t0.x;
                visco_point<LL>(P, vxx.x, vyy.x, vzz.x, vxy.x, vyx.x, vxz.x, vzx.x, vyz.x, vzy.x, M.x, mu, tauP.x, t0.x, opP, opS,
                            mav, tav, Sn, Sh, Ra, fsRow);
                sxx.x = Sn[0]; syy.x = Sn[1]; szz.x = Sn[2]; sxy.x = Sh[0]; sxz.x = Sh[1]; syz.x = Sh[2];
            }
            {
                float Sn[3] = {sxx.y, syy.y, szz.y}, Sh[3] = {sxy.y, sxz.y, syz.y};
                const float mav[3] = {muXY[1], muXZ[1], muYZ[1]}, tav[3] = {tXY[1], tXZ[1], tYZ[1]};
                const float mu = m00.y;
                const float opP = 1.0f + Lf * tauP.y, opS = 1.0f + Lf * t0.y;
                visco_point<LL>(P, vxx.y, vyy.y, vzz.y, vxy.y, vyx.y, vxz.y, vzx.y, vyz.y, vzy.y, M.y, mu, tauP.y, t0.y, opP, opS,
                            mav, tav, Sn, Sh, Rb, fsRow);
                sxx.y = Sn[0]; syy.y = Sn[1]; szz.y = Sn[2]; sxy.y = Sh[0]; sxz.y = Sh[1]; syz.y = Sh[2];
            }
#pragma unroll
            for (int k = 0; k < 6; ++k)
#pragma unroll
                for (int l = 0; l < LL; ++l) st2(P.r[slotR[k]][l] + i, make_float2(Ra[k][l], Rb[k][l]));
            float2 d = make_float2(1.0f, 1.0f);
            if (P.abs) d = make_float2(abs_damp(P, C.x, y, C.z), abs_damp(P, C.x + 1, y, C.z));
            st2(P.f[F_SXX] + i, mul2(sxx, d));
            st2(P.f[F_SYY] + i, mul2(syy, d));
            st2(P.f[F_SZZ] + i, mul2(szz, d));
            st2(P.f[F_SXY] + i, mul2(sxy, d));
            st2(P.f[F_SXZ] + i, mul2(sxz, d));
            st2(P.f[F_SYZ] + i, mul2(syz, d));
        }
        // carry mu and tau_S of plane y+1 into the next iteration
        {
            const float2 n0 = ld2(mb + ri), n1 = ld2(mb + ri + PW);
            m00 = n0;
            i0 = make_float2(inv_clampedf(n0.x), inv_clampedf(n0.y));
            i0r = inv_clampedf(mb[ri + 2]);
            i1 = make_float2(inv_clampedf(n1.x), inv_clampedf(n1.y));
            i1r = inv_clampedf(mb[ri + PW + 2]);
            t0 = ld2(tb + ri);
            t0r = tb[ri + 2];
            t1 = ld2(tb + ri + PW);
            t1r = tb[ri + PW + 2];
        }
        release_and_refill<NST>(it, total, cur, G, rel, &issued, &failed, issue);
        if (__any_sync(0xffffffffu, failed != 0)) break;
        cur.advance(G);
    }
    finish_ring<NST>(full, &issued, &failed);
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
size_t vstr_smem() { return VStrStage<H>::NST * (VStrStage<H>::BYTES + 2 * sizeof(uint64_t)); }

// The visco-elastic stress kernel is built for orders 2-8 and one or two
// relaxation mechanisms (other set-ups run the generic kernel).
constexpr int kViscoMaxH = 4, kViscoMaxL = 2;

// resident CTAs per SM of the visco-elastic stress kernel (0: does not fit)
template <int H, int LL>
int configure_visco_hl()
{
    if (cudaFuncSetAttribute(el3dp_vstr<H, LL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vstr_smem<H>()) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, el3dp_vstr<H, LL>, NTHR, vstr_smem<H>()) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

template <int H>
int configure_visco_h(int L) { return L == 1 ? configure_visco_hl<H, 1>() : configure_visco_hl<H, 2>(); }

int configure_visco(int H, int L)
{
    if (L < 1 || L > kViscoMaxL) return 0;
    switch (H) {
    case 1: return configure_visco_h<1>(L);
    case 2: return configure_visco_h<2>(L);
    case 3: return configure_visco_h<3>(L);
    case 4: return configure_visco_h<4>(L);
    default: return 0;
    }
}

template <int H>
void launch_visco(const El3dPlan& plan, const StepParams& P, cudaStream_t s)
{
    const dim3 block(NTHR, 1, 1);
    if (P.L == 1) el3dp_vstr<H, 1><<<plan.gridVisco, block, vstr_smem<H>(), s>>>(plan.maps, P, plan.sched);
    else el3dp_vstr<H, 2><<<plan.gridVisco, block, vstr_smem<H>(), s>>>(plan.maps, P, plan.sched);
}

// CTAs of each kernel resident per SM (0: does not fit)
template <int H>
int configure_h()
{
    if (cudaFuncSetAttribute(el3dp_vel<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vel_smem<H>()) != cudaSuccess) return 0;
    if (cudaFuncSetAttribute(el3dp_str<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)str_smem<H>()) != cudaSuccess) return 0;
    int nv = 0, ns = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nv, el3dp_vel<H>, NTHR, vel_smem<H>()) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ns, el3dp_str<H>, NTHR, str_smem<H>()) != cudaSuccess) return 0;
    return nv < ns ? nv : ns;
}

int configure(int H)
{
    switch (H) {
    case 1: return configure_h<1>();
    case 2: return configure_h<2>();
    case 3: return configure_h<3>();
    case 4: return configure_h<4>();
    case 5: return configure_h<5>();
    case 6: return configure_h<6>();
    default: return 0;
    }
}

template <int H>
cudaError_t launch_h(const El3dPlan& plan, const StepParams& P, int pass, cudaStream_t s)
{
    const dim3 block(NTHR, 1, 1);
    if (pass == 0) el3dp_vel<H><<<plan.grid, block, vel_smem<H>(), s>>>(plan.maps, P, plan.sched);
    else if (P.L > 0) {
        if (plan.gridVisco < 1 || H > kViscoMaxH) return cudaErrorInvalidValue;
        launch_visco<(H <= kViscoMaxH ? H : 1)>(plan, P, s);
    } else el3dp_str<H><<<plan.grid, block, str_smem<H>(), s>>>(plan.maps, P, plan.sched);
    return cudaGetLastError();
}

// A tile's x (or z) range meets at most one CPML slab of that axis; the
// compact slab layout keeps TMA's 16-byte rules along x; along x the slab
// width is even so that a pair never straddles a slab edge.
bool slab_tiles_ok(const Cpml1D& p, int T, bool xAxis)
{
    if (!p.on || p.n <= 2 * p.w) return !xAxis || !p.on || (p.n % 2) == 0;
    if (xAxis && ((p.ns % 4) != 0 || ((p.n - p.ns) % 4) != 0 || (p.w % 2) != 0)) return false;
    for (int c0 = 0; c0 < p.n; c0 += T)
        if (p.lo && c0 < p.w && c0 + T > p.n - p.w) return false;
    return true;
}

bool make_psi_map(CUtensorMap* m, const float* base, int axis, const StepParams& P)
{
    if (!base) return false;
    switch (axis) {
    case 0: return make_map_dims(m, base, P.cx.ns, P.NZ, P.NY, TX, TZ);
    case 1: return make_map_dims(m, base, P.NX, P.NZ, P.cy.ns, TX, TZ);
    default: return make_map_dims(m, base, P.NX, P.cz.ns, P.NY, TX, TZ);
    }
}

} // namespace

// Builds the tensor maps of the pair kernels for the current field/material
// pointers. Returns false when they do not apply.
bool el3d_prepare_pairs(El3dPlan& plan, const StepParams& P, const float* rho, const float* M, const float* mu, int H, int* errWord,
                        const float* tauS)
{
    plan.ready = false;
    plan.gridVisco = 0;
    if (!P.is3d || H < 1 || H > 6 || (P.NX % 4) != 0 || P.NX < 8 || P.NZ < 2) return false;
    if (!rho || !M || !mu) return false;
    if (P.useCpml && (!slab_tiles_ok(P.cx, TX, true) || !slab_tiles_ok(P.cz, TZ, false))) return false;
    // the x-weight table holds the edge bands of both sides and one interior pair
    if (P.Dxf.full || P.Dxb.full || P.Dxf.E > H + 1 || P.Dxb.E > H + 1 || P.NX < 4 * ((H + 2) / 2) + 4) return false;
    const int bx = bw_of(H), bz = bh_of(H);
    El3dMaps& T = plan.maps;
    bool ok = true;
    ok &= make_map(&T.hSxx, P.f[F_SXX], P.NX, P.NZ, P.NY, bx, TZ);   // x halo only
    ok &= make_map(&T.hSxy, P.f[F_SXY], P.NX, P.NZ, P.NY, bx, TZ);
    ok &= make_map(&T.hSxz, P.f[F_SXZ], P.NX, P.NZ, P.NY, bx, bz);   // x and z halo
    ok &= make_map(&T.hSyz, P.f[F_SYZ], P.NX, P.NZ, P.NY, TX, bz);   // z halo only
    ok &= make_map(&T.hSzz, P.f[F_SZZ], P.NX, P.NZ, P.NY, TX, bz);
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
    if (tauS) ok &= make_map(&T.pTauS, tauS, P.NX, P.NZ, P.NY, PW, PH);
    if (P.useCpml) {
        const int vel[9] = {PS_SXX_X, PS_SXY_X, PS_SXZ_X, PS_SXY_Y, PS_SYY_Y, PS_SYZ_Y, PS_SXZ_Z, PS_SYZ_Z, PS_SZZ_Z};
        const int str[9] = {PS_VXX, PS_VYX, PS_VZX, PS_VYY, PS_VXY, PS_VZY, PS_VZZ, PS_VXZ, PS_VYZ};
        for (int j = 0; j < 9; ++j) {
            const int axis = j / 3;
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
    const int perSM = configure(H);
    if (perSM < 1) return false;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (long long)plan.sched.ntx * plan.sched.ntz;
    long long grid = (long long)perSM * sms;   // persistent: one wave of resident CTAs
    if (grid > tiles * P.NY) grid = tiles * P.NY;
    if (tiles / grid + 2 > MAXSEG) return false;
    plan.grid = static_cast<int>(grid);
    plan.ready = plan.grid > 0;
    if (plan.ready && tauS && P.L > 0 && P.L <= kViscoMaxL && H <= kViscoMaxH) {
        // the visco-elastic stress kernel: its larger stage may fit fewer CTAs per SM
        const int perV = configure_visco(H, P.L);
        long long gv = (long long)perV * sms;
        if (gv > tiles * P.NY) gv = tiles * P.NY;
        if (perV > 0 && tiles / gv + 2 <= MAXSEG) plan.gridVisco = static_cast<int>(gv);
    }
    return plan.ready;
}

cudaError_t el3d_launch_pairs(const El3dPlan& plan, const StepParams& P, int pass, cudaStream_t s)
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
