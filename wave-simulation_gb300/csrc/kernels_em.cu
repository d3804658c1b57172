// kernels_em.cu — sm_103a kernels of the EM time steps (TMz, TEz, 3-D EM and
// their visco variants; one thread per grid point, FP32), single-handle and
// batched, and their launch tables. The same two-pass structure as the
// seismic kernels in kernels.cu (H field, then E field with the memory
// variables and the ABS damping of E); a translation unit of its own so that
// the build compiles the two families in parallel.
#include <cuda_runtime.h>

#include "stencil.cuh"

namespace wave {

#define LD(ptr) __ldg((ptr) + p.i)

// --------------------------------------------------------------------------
// EM TMz: FD2Dtmem::run (ForwardSolverEM/ForwardSolver2Dtmem.cpp:128-170),
// FD2Dviscotmem::run (ForwardSolverEM/ForwardSolver2Dviscotmem.cpp:150-205)
// --------------------------------------------------------------------------
template <int H>
__device__ __forceinline__ void tm_h_body(const StepParams& P, const Pt& p)
{
    const float* ez = P.f[F_EZ];
    float u = dY<H, true>(P, p, ez, P.Dyf, PS_EZY);
    u *= LD(P.m[M_IMUYZ]);
    P.f[F_HX][p.i] -= u;
    float ut = dX<H, true>(P, p, ez, P.Dxf, PS_EZX);
    u = -ut;
    u *= LD(P.m[M_IMUXZ]);
    P.f[F_HY][p.i] -= u;
}

template <int H>
__global__ void __launch_bounds__(256) tm_h(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    tm_h_body<H>(P, p);
}


// memory variables of one E component (ForwardSolver2Dviscotmem.cpp:175-182,
// ForwardSolverEM/ForwardSolver2Dviscoemem.cpp:176-184): r_l = Cd_l e + Cc_l r_l,
// then the E update subtracts DT r_l for every mechanism
__device__ __forceinline__ void em_memory(const StepParams& P, const Pt& p, int rslot, int cd0, float e, float& u)
{
    for (int l = 0; l < P.L; ++l) {
        float* r = P.r[rslot][l] + p.i;
        const float ru = P.Cc[l] * *r;
        const float rt = __ldg(P.m[cd0 + l] + p.i) * e;
        const float rn = rt + ru;
        *r = rn;
        u -= P.DT * rn;
    }
}

template <int H>
__device__ __forceinline__ void tm_e_body(const StepParams& P, const Pt& p)
{
    const float e0 = P.f[F_EZ][p.i];
    float u = dX<H, false>(P, p, P.f[F_HY], P.Dxb, PS_HYX);
    float ut = dY<H, false>(P, p, P.f[F_HX], P.Dyb, PS_HXY);
    u -= ut;
    em_memory(P, p, R_EZ, M_CDZ0, e0, u);
    u *= LD(P.m[M_CBZ]);
    float e = LD(P.m[M_CAZ]) * e0;
    e = e + u;
    if (P.abs) e *= absDamp(P, p);
    P.f[F_EZ][p.i] = e;
}

template <int H>
__global__ void __launch_bounds__(256) tm_e(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    tm_e_body<H>(P, p);
}


// Batched TMz passes. A tile flagged kTileInterior (lossless 2-D shots only:
// wholly inside the grid, away from the operators' edge bands, the CPML slabs
// and the ABS frame) is staged in shared memory with 4-byte cp.async copies,
// every field of the tile and the halo its derivatives read, and then updated
// from there: each block keeps its whole tile in flight without holding it in
// registers (these passes are bound by load latency). Measured on the
// 128-shot TMz batch, this beat register-held prefetching (which cost more
// occupancy than it gained), 16-byte cp.async chunks of phase-matched rows
// and per-row bulk copies on an mbarrier. The point update runs the
// operations of tm_h_body / tm_e_body in their order (deriv's interior
// branch, no CPML, an ABS factor of 1), so both paths give the same bits.
// Other tiles run the generic bodies.
__device__ __forceinline__ void cp_async4(float* s, const float* g)
{
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(s));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}
// a W x R rectangle at g (row pitch NX) into s (row pitch W), by the 32 x 8 block
__device__ __forceinline__ void stage_rect(float* s, const float* g, int W, int R, int NX)
{
    for (int r = threadIdx.y; r < R; r += 8)
        for (int c = threadIdx.x; c < W; c += 32) cp_async4(s + r * W + c, g + (long long)r * NX + c);
}

template <int H>
__global__ void __launch_bounds__(256) tm_h_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    extern __shared__ float tile_smem[];
    int shot = -1;
    for (int t = blockIdx.x; t < S.ntiles; t += gridDim.x) {
        const BatchTile w = W[t];
        if (w.shot != shot) {
            __syncthreads();
            load_params(sP, Ps + w.shot);
            shot = w.shot;
        }
        if (!(w.flags & kTileInterior)) {
            tile_points(sP, w, S, [](const StepParams& P, const Pt& p) { tm_h_body<H>(P, p); });
            continue;
        }
        // Ez with the forward taps' halo (-H+1..H along x and y), 1/mu averages, Hx, Hy
        const int C = S.cols, R = S.rows, NX = sP.NX, PW = C + 2 * H - 1, PH = R + 2 * H - 1;
        float* sEz = tile_smem;
        float* sMy = sEz + PW * PH;
        float* sMx = sMy + C * R;
        float* sHx = sMx + C * R;
        float* sHy = sHx + C * R;
        const long long g0 = w.x0 + (long long)NX * w.r0;
        float* hx = sP.f[F_HX];
        float* hy = sP.f[F_HY];
        stage_rect(sEz, sP.f[F_EZ] + g0 - (H - 1) - (long long)(H - 1) * NX, PW, PH, NX);
        stage_rect(sMy, sP.m[M_IMUYZ] + g0, C, R, NX);
        stage_rect(sMx, sP.m[M_IMUXZ] + g0, C, R, NX);
        stage_rect(sHx, hx + g0, C, R, NX);
        stage_rect(sHy, hy + g0, C, R, NX);
        float wy[2 * H], wx[2 * H];
#pragma unroll
        for (int k = 0; k < 2 * H; ++k) {
            wy[k] = sP.Dyf.w[kMaxHalf - H + 1 + k];
            wx[k] = sP.Dxf.w[kMaxHalf - H + 1 + k];
        }
        cp_async_wait_all();
        __syncthreads();
        for (int ly = threadIdx.y; ly < R; ly += 8)
            for (int lx = threadIdx.x; lx < C; lx += 32) {
                const float* e = sEz + (ly + H - 1) * PW + (lx + H - 1);   // Ez at the point
                const int l = ly * C + lx;
                const long long i = g0 + lx + (long long)NX * ly;
                float u = 0.0f;
#pragma unroll
                for (int k = 0; k < 2 * H; ++k) u += wy[k] * e[(k - H + 1) * PW];
                u *= sMy[l];
                hx[i] = sHx[l] - u;
                float ut = 0.0f;
#pragma unroll
                for (int k = 0; k < 2 * H; ++k) ut += wx[k] * e[k - H + 1];
                u = -ut;
                u *= sMx[l];
                hy[i] = sHy[l] - u;
            }
        __syncthreads();   // the next tile reuses the staging area
    }
}

template <int H>
__global__ void __launch_bounds__(256) tm_e_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    extern __shared__ float tile_smem[];
    int shot = -1;
    for (int t = blockIdx.x; t < S.ntiles; t += gridDim.x) {
        const BatchTile w = W[t];
        if (w.shot != shot) {
            __syncthreads();
            load_params(sP, Ps + w.shot);
            shot = w.shot;
        }
        if (!(w.flags & kTileInterior)) {
            tile_points(sP, w, S, [](const StepParams& P, const Pt& p) { tm_e_body<H>(P, p); });
            continue;
        }
        // Hy with the backward taps' halo along x (-H..H-1), Hx with it along y, Ez, Ca, Cb
        const int C = S.cols, R = S.rows, NX = sP.NX, PW = C + 2 * H - 1, PH = R + 2 * H - 1;
        float* sHy = tile_smem;
        float* sHx = sHy + PW * R;
        float* sEz = sHx + C * PH;
        float* sCa = sEz + C * R;
        float* sCb = sCa + C * R;
        const long long g0 = w.x0 + (long long)NX * w.r0;
        float* ez = sP.f[F_EZ];
        stage_rect(sHy, sP.f[F_HY] + g0 - H, PW, R, NX);
        stage_rect(sHx, sP.f[F_HX] + g0 - (long long)H * NX, C, PH, NX);
        stage_rect(sEz, ez + g0, C, R, NX);
        stage_rect(sCa, sP.m[M_CAZ] + g0, C, R, NX);
        stage_rect(sCb, sP.m[M_CBZ] + g0, C, R, NX);
        float wx[2 * H], wy[2 * H];
#pragma unroll
        for (int k = 0; k < 2 * H; ++k) {
            wx[k] = sP.Dxb.w[kMaxHalf - H + k];
            wy[k] = sP.Dyb.w[kMaxHalf - H + k];
        }
        cp_async_wait_all();
        __syncthreads();
        for (int ly = threadIdx.y; ly < R; ly += 8)
            for (int lx = threadIdx.x; lx < C; lx += 32) {
                const float* a = sHy + ly * PW + (lx + H);   // Hy at the point
                const float* b = sHx + (ly + H) * C + lx;    // Hx at the point
                const int l = ly * C + lx;
                float u = 0.0f;
#pragma unroll
                for (int k = 0; k < 2 * H; ++k) u += wx[k] * a[k - H];
                float ut = 0.0f;
#pragma unroll
                for (int k = 0; k < 2 * H; ++k) ut += wy[k] * b[(k - H) * C];
                u -= ut;
                u *= sCb[l];
                float e = sCa[l] * sEz[l];
                e = e + u;
                ez[g0 + lx + (long long)NX * ly] = e;
            }
        __syncthreads();   // the next tile reuses the staging area
    }
}

// EM TEz: FD2Demem::run (ForwardSolverEM/ForwardSolver2Demem.cpp:132-180),
// FD2Dviscoemem::run (ForwardSolverEM/ForwardSolver2Dviscoemem.cpp:154-228)
template <int H>
__device__ __forceinline__ void te_h_body(const StepParams& P, const Pt& p)
{
    float u = dX<H, true>(P, p, P.f[F_EY], P.Dxf, PS_EYX);
    float ut = dY<H, true>(P, p, P.f[F_EX], P.Dyf, PS_EXY);
    u -= ut;
    u *= LD(P.m[M_IMUXY]);
    P.f[F_HZ][p.i] -= u;
}

template <int H>
__global__ void __launch_bounds__(256) te_h(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    te_h_body<H>(P, p);
}

template <int H>
__global__ void __launch_bounds__(256) te_h_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { te_h_body<H>(P, p); });
}

template <int H>
__device__ __forceinline__ void te_e_body(const StepParams& P, const Pt& p)
{
    const float* hz = P.f[F_HZ];
    const float d = P.abs ? absDamp(P, p) : 1.0f;
    const float ex0 = P.f[F_EX][p.i], ey0 = P.f[F_EY][p.i];
    float u = dY<H, false>(P, p, hz, P.Dyb, PS_HZY);
    em_memory(P, p, R_EX, M_CDX0, ex0, u);
    u *= LD(P.m[M_CBX]);
    float e = LD(P.m[M_CAX]) * ex0;
    P.f[F_EX][p.i] = (e + u) * d;
    const float ut = dX<H, false>(P, p, hz, P.Dxb, PS_HZX);
    u = -ut;
    em_memory(P, p, R_EY, M_CDY0, ey0, u);
    u *= LD(P.m[M_CBY]);
    e = LD(P.m[M_CAY]) * ey0;
    P.f[F_EY][p.i] = (e + u) * d;
}

template <int H>
__global__ void __launch_bounds__(256) te_e(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    te_e_body<H>(P, p);
}

template <int H>
__global__ void __launch_bounds__(256) te_e_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { te_e_body<H>(P, p); });
}

// --------------------------------------------------------------------------
// 3-D EM: FD3Demem::run (ForwardSolverEM/ForwardSolver3Demem.cpp:140-237),
// FD3Dviscoemem::run (ForwardSolverEM/ForwardSolver3Dviscoemem.cpp:186-309).
// CPML as CPMLEM3D.cpp:25-108: E derivatives on the half profile, H
// derivatives on the full one except hyx, which uses the half profile there.
// --------------------------------------------------------------------------
template <int H>
__device__ __forceinline__ void em3_h_body(const StepParams& P, const Pt& p)
{
    const float *ex = P.f[F_EX], *ey = P.f[F_EY], *ez = P.f[F_EZ];
    float u = dY<H, true>(P, p, ez, P.Dyf, PS_EZY);
    float ut = dZ<H, true>(P, p, ey, P.Dzf, PS_EYZ);
    u -= ut;
    u *= LD(P.m[M_IMUYZ]);
    P.f[F_HX][p.i] -= u;
    u = dZ<H, true>(P, p, ex, P.Dzf, PS_EXZ);
    ut = dX<H, true>(P, p, ez, P.Dxf, PS_EZX);
    u -= ut;
    u *= LD(P.m[M_IMUXZ]);
    P.f[F_HY][p.i] -= u;
    u = dX<H, true>(P, p, ey, P.Dxf, PS_EYX);
    ut = dY<H, true>(P, p, ex, P.Dyf, PS_EXY);
    u -= ut;
    u *= LD(P.m[M_IMUXY]);
    P.f[F_HZ][p.i] -= u;
}

template <int H>
__global__ void __launch_bounds__(256) em3_h(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    em3_h_body<H>(P, p);
}

template <int H>
__global__ void __launch_bounds__(256) em3_h_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { em3_h_body<H>(P, p); });
}

template <int H>
__device__ __forceinline__ void em3_e_body(const StepParams& P, const Pt& p)
{
    const float *hx = P.f[F_HX], *hy = P.f[F_HY], *hz = P.f[F_HZ];
    const float d = P.abs ? absDamp(P, p) : 1.0f;
    const float ex0 = P.f[F_EX][p.i], ey0 = P.f[F_EY][p.i], ez0 = P.f[F_EZ][p.i];
    // ex
    float u = dY<H, false>(P, p, hz, P.Dyb, PS_HZY);
    float ut = dZ<H, false>(P, p, hy, P.Dzb, PS_HYZ);
    u -= ut;
    em_memory(P, p, R_EX, M_CDX0, ex0, u);
    u *= LD(P.m[M_CBX]);
    float e = LD(P.m[M_CAX]) * ex0;
    P.f[F_EX][p.i] = (e + u) * d;
    // ey
    u = dZ<H, false>(P, p, hx, P.Dzb, PS_HXZ);
    ut = dX<H, false>(P, p, hz, P.Dxb, PS_HZX);
    u -= ut;
    em_memory(P, p, R_EY, M_CDY0, ey0, u);
    u *= LD(P.m[M_CBY]);
    e = LD(P.m[M_CAY]) * ey0;
    P.f[F_EY][p.i] = (e + u) * d;
    // ez
    u = dX<H, false, true>(P, p, hy, P.Dxb, PS_HYX);
    ut = dY<H, false>(P, p, hx, P.Dyb, PS_HXY);
    u -= ut;
    em_memory(P, p, R_EZ, M_CDZ0, ez0, u);
    u *= LD(P.m[M_CBZ]);
    e = LD(P.m[M_CAZ]) * ez0;
    P.f[F_EZ][p.i] = (e + u) * d;
}

template <int H>
__global__ void __launch_bounds__(256) em3_e(StepParams P)
{
    dependent_launch_prologue();
    Pt p;
    if (!point(P, p)) return;
    em3_e_body<H>(P, p);
}

template <int H>
__global__ void __launch_bounds__(256) em3_e_batch(const StepParams* __restrict__ Ps, const BatchTile* __restrict__ W, BatchSched S)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [](const StepParams& P, const Pt& p, int) { em3_e_body<H>(P, p); });
}

// --------------------------------------------------------------------------
// launch tables of the EM equations (kernel_eq numbering)
// --------------------------------------------------------------------------
#define WAVE_KTAB(name) { name<1>, name<2>, name<3>, name<4>, name<5>, name<6> }

StepKernel em_kernel_for(int eq, int pass, int H)
{
    static const StepKernel tmh[6] = WAVE_KTAB(tm_h), tme[6] = WAVE_KTAB(tm_e), teh[6] = WAVE_KTAB(te_h), tee[6] = WAVE_KTAB(te_e);
    static const StepKernel e3h[6] = WAVE_KTAB(em3_h), e3e[6] = WAVE_KTAB(em3_e);
    if (H < 1 || H > 6) return nullptr;
    const int k = H - 1;
    switch (eq) {
    case WAVE_EQ_EMEM + kEm3d:
    case WAVE_EQ_VISCOEMEM + kEm3d: return pass == 0 ? e3h[k] : e3e[k];
    case WAVE_EQ_TMEM:
    case WAVE_EQ_VISCOTMEM: return pass == 0 ? tmh[k] : tme[k];
    case WAVE_EQ_EMEM:
    case WAVE_EQ_VISCOEMEM: return pass == 0 ? teh[k] : tee[k];
    default: return nullptr;
    }
}

BatchKernel em_batch_kernel_for(int eq, int pass, int H)
{
    static const BatchKernel tmh[6] = WAVE_KTAB(tm_h_batch), tme[6] = WAVE_KTAB(tm_e_batch), teh[6] = WAVE_KTAB(te_h_batch),
                             tee[6] = WAVE_KTAB(te_e_batch);
    static const BatchKernel e3h[6] = WAVE_KTAB(em3_h_batch), e3e[6] = WAVE_KTAB(em3_e_batch);
    if (H < 1 || H > 6) return nullptr;
    const int k = H - 1;
    switch (eq) {
    case WAVE_EQ_EMEM + kEm3d:
    case WAVE_EQ_VISCOEMEM + kEm3d: return pass == 0 ? e3h[k] : e3e[k];
    case WAVE_EQ_TMEM:
    case WAVE_EQ_VISCOTMEM: return pass == 0 ? tmh[k] : tme[k];
    case WAVE_EQ_EMEM:
    case WAVE_EQ_VISCOEMEM: return pass == 0 ? teh[k] : tee[k];
    default: return nullptr;
    }
}

} // namespace wave
