// vargrid.cu — the acoustic time step on the variable (discontinuous) grid:
// FD2Dacoustic / FD3Dacoustic::run (ForwardSolver2Dacoustic.cpp:91-190,
// ForwardSolver3Dacoustic.cpp:91-230) with the grid's sparse operators.
//
// Layout in HBM: every field, psi and material array is one vector over the
// variable-grid index space (layer after layer). Each operator is an ELL
// block (W entries per row, entry-major: entry k of row i at k*N + i), so a
// warp's 32 rows read 32 consecutive column indices and weights per entry.
// The default kernels read instead one 32-bit stencil class per row and pass
// and take the (offset, weight) entries from the class table: the rows of a
// layer's interior share a handful of classes, so the operators cost 4 B per
// point and pass instead of 8 B per entry.
// One step is four launches plus the source/receiver kernel (and vg_abs
// with ABS):
//   vg_vel    Dxf p, Dyf p (or DyfFreeSurface p), Dzf p, CPML, velocity update
//   vg_interp velocity rows on the interfaces (InterpolationStaggeredX/Full/StaggeredZ)
//   vg_pres   Dxb vx + Dyb vy + Dzb vz, CPML, pressure update, surface zero
//   vg_interp pressure rows on the interfaces (InterpolationFull)
// The interpolations run in place where the rows they rewrite read only the
// coarse-aligned rows of the same interface (which they leave unchanged);
// otherwise (a 3:9 step) the new values go through a scratch array first.
//
// The elastic step (FD2Delastic::run, ForwardSolver2Delastic.cpp:117-297;
// FD3Delastic::run, ForwardSolver3Delastic.cpp:120-414) has the same shape
// with the ELL operators:
//   vge_vel   vx += (Dxf sxx + DybStaggeredX sxy [+ Dzb sxz]) / rho_x,
//             vy += (Dxb sxy + Dyf syy [+ Dzb syz]) / rho_y,
//             [vz += (Dxb sxz + DybStaggeredZ syz + Dzf szz) / rho_z]
//   vg_interp vx (StaggeredX), vy (Full) [, vz (StaggeredZ)]
//   vge_str   normal stresses from Dxb vx, Dyb vy [, Dzb vz]; sxy from
//             DyfStaggeredX vx + Dxf vy [; sxz from Dzf vx + Dxf vz; syz from
//             Dzf vy + DyfStaggeredZ vz]
//   vg_interp sxx, syy [, szz] (Full), sxy (StaggeredX) [, sxz (StaggeredXZ),
//             syz (StaggeredZ)]
//
// The end of the file holds the discrete adjoints of both steps (the
// gradient of the seismogram misfit): the transposes of the ELL blocks,
// interpolations and per-point factors applied in reverse order over a
// checkpointed sweep.
#include <algorithm>
#include <functional>
#include <stdexcept>
#include <vector>

#include <cuda_runtime.h>

#include "handle.h"
#include "stencil.cuh"
#include "vargrid.h"

namespace wave {

namespace {

struct VgParams {
    long long N, nSurface;
    int fs, cpml;
    float* vx;
    float* vy;
    float* vz;
    float* p;
    float* psi[6];              // p_x, p_y, p_z, vxx, vyy, vzz
    const float* M;
    const float* ir[3];
    const int* col[6];          // Dxf, Dyf, Dzf, Dxb, Dyb, Dzb
    const float* val[6];
    int W[6];
    const unsigned short* cpc[3];   // per axis: coefficient code of each point (0: none)
    const float* cpt[3];            // per axis: (a_full, b_full, a_half, b_half) per code
    // stencil classes of the launched pass (CLS kernels)
    const unsigned* cid;
    const int* coff;
    const float* cw;
    int KW;
    int base[3];
};

// phase 0: in place; 1: new values into tmp; 2: tmp into the field.
// srSlot >= 0: the blocks with blockIdx.y == srSlot run the step's sources
// and receivers instead (block 0 only), when none of them is on an interface
// row, so they touch no row the interpolation reads or writes.
constexpr int kMaxInterpLists = 6;
struct VgInterp {
    int n[kMaxInterpLists];
    int phase[kMaxInterpLists];
    float* f[kMaxInterpLists];
    float* tmp[kMaxInterpLists];
    const int* row[kMaxInterpLists];
    const int* col[kMaxInterpLists];
    const float* w[kMaxInterpLists];
    int srSlot;
    SrcRecParams Q;
    int* tcounter;
};

__device__ __forceinline__ float ell_row(const VgParams& P, int op, long long i, const float* __restrict__ u)
{
    const int* __restrict__ c = P.col[op] + i;
    const float* __restrict__ v = P.val[op] + i;
    float s = 0.0f;
    for (int k = 0; k < P.W[op]; ++k) s = __fmaf_rn(v[k * P.N], u[c[k * P.N]], s);
    return s;
}

// the same row through the row's stencil class: identical entries in the
// same order and explicit fused multiply-adds, so identical results; rows of
// one class in a warp share the table reads. (All arithmetic in these kernels
// is written with rounding intrinsics so that no kernel variant depends on
// the compiler's contraction choices.)
// WU: compile-time bound of the entry loop (every W <= WU), so the table
// reads and the gathers of a row are all issued before the sums
template <bool CLS, int WU>
__device__ __forceinline__ float op_row(const VgParams& P, int op, int q, long long i, unsigned cls, const float* __restrict__ u)
{
    if (!CLS) return ell_row(P, op, i, u);
    const size_t b = static_cast<size_t>(cls) * P.KW + P.base[q];
    const int* __restrict__ o = P.coff + b;
    const float* __restrict__ w = P.cw + b;
    const int W = P.W[op];
    float wk[WU], uk[WU];
#pragma unroll
    for (int k = 0; k < WU; ++k) {
        wk[k] = 0.0f;
        uk[k] = 0.0f;
        if (k < W) {
            wk[k] = __ldg(w + k);
            uk[k] = u[i + __ldg(o + k)];
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < WU; ++k)
        if (k < W) s = __fmaf_rn(wk[k], uk[k], s);
    return s;
}

// CPML::applyCPML (CPML.cpp:84-95); zero coefficients outside the frame
__device__ __forceinline__ void vg_cpml(const VgParams& P, float& d, int slot, int axis, bool half, long long i)
{
    const unsigned code = P.cpc[axis][i];
    if (code == 0) return;
    const float a = __ldg(P.cpt[axis] + 4 * code + (half ? 2 : 0));
    const float b = __ldg(P.cpt[axis] + 4 * code + (half ? 3 : 1));
    if (a == 0.0f && b == 0.0f) return;
    // the reference's three vector operations, each rounded (Psi *= b;
    // temp = a * Vec; Psi += temp; Vec += Psi), not contracted: the result
    // does not depend on which kernel variant the compiler fused
    const float ps = __fadd_rn(__fmul_rn(P.psi[slot][i], b), __fmul_rn(a, d));
    P.psi[slot][i] = ps;
    d = __fadd_rn(d, ps);
}

template <bool IS3D, bool CPML, bool CLS, int WU = 12>
__global__ void __launch_bounds__(256) vg_vel(VgParams P)
{
    dependent_launch_prologue();
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const float* p = P.p;
    const unsigned cls = CLS ? P.cid[i] : 0u;
    float d = op_row<CLS, WU>(P, 0, 0, i, cls, p);
    if (CPML) vg_cpml(P, d, 0, 0, true, i);
    P.vx[i] = __fadd_rn(P.vx[i], __fmul_rn(d, P.ir[0][i]));
    d = op_row<CLS, WU>(P, 1, 1, i, cls, p);
    if (CPML) vg_cpml(P, d, 1, 1, true, i);
    P.vy[i] = __fadd_rn(P.vy[i], __fmul_rn(d, P.ir[1][i]));
    if (IS3D) {
        d = op_row<CLS, WU>(P, 2, 2, i, cls, p);
        if (CPML) vg_cpml(P, d, 2, 2, true, i);
        P.vz[i] = __fadd_rn(P.vz[i], __fmul_rn(d, P.ir[2][i]));
    }
}

template <bool IS3D, bool CPML, bool CLS, int WU = 12>
__global__ void __launch_bounds__(256) vg_pres(VgParams P)
{
    dependent_launch_prologue();
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    const unsigned cls = CLS ? P.cid[i] : 0u;
    float d = op_row<CLS, WU>(P, 3, 0, i, cls, P.vx);
    if (CPML) vg_cpml(P, d, 3, 0, false, i);
    float d2 = op_row<CLS, WU>(P, 4, 1, i, cls, P.vy);
    if (CPML) vg_cpml(P, d2, 4, 1, false, i);
    d = __fadd_rn(d, d2);
    if (IS3D) {
        d2 = op_row<CLS, WU>(P, 5, 2, i, cls, P.vz);
        if (CPML) vg_cpml(P, d2, 5, 2, false, i);
        d = __fadd_rn(d, d2);
    }
    d = __fmul_rn(d, P.M[i]);
    float pv = __fadd_rn(P.p[i], d);
    // FreeSurface::setSurfaceZero (FreeSurface.cpp:14-19): the rows at y = 0
    // come first in the index order and never lie on an interface
    if (P.fs && i < P.nSurface) pv = 0.0f;
    P.p[i] = pv;
}

// blockIdx.y selects one of up to six (field, row list) pairs
__global__ void __launch_bounds__(256) vg_interp(VgInterp I)
{
    dependent_launch_prologue();
    const int s = blockIdx.y;
    if (s == I.srSlot) {
        if (blockIdx.x == 0) srcrec_body(I.Q, I.tcounter);
        return;
    }
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= I.n[s]) return;
    float* f = I.f[s];
    if (I.phase[s] == 2) {
        f[I.row[s][k]] = I.tmp[s][k];
        return;
    }
    const int* c = I.col[s] + 4 * k;
    const float* w = I.w[s] + 4 * k;
    float v = __fmul_rn(w[0], f[c[0]]);
    v = __fmaf_rn(w[1], f[c[1]], v);
    v = __fmaf_rn(w[2], f[c[2]], v);
    v = __fmaf_rn(w[3], f[c[3]], v);
    if (I.phase[s] == 1) I.tmp[s][k] = v;
    else f[I.row[s][k]] = v;
}

// DampingBoundary.apply (ABS2D.cpp:14-50, ABS3D.cpp:15-100): every listed
// field times the point's taper factor
struct VgAbs {
    long long N;
    const float* damp;
    float* f[9];
    int n;
};
__global__ void __launch_bounds__(256) vg_abs(VgAbs A)
{
    dependent_launch_prologue();
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    const float d = A.damp[i];
    if (d == 1.0f) return;
    for (int k = 0; k < A.n; ++k) A.f[k][i] = __fmul_rn(A.f[k][i], d);
}

// Acoustic::prepareForModelling on the variable grid: pWaveModulus = rho vp^2,
// inverse densities averaged with the grid's partners (Modelparameter.cpp:
// 336-446, 633-640; invalid values become 0)
__global__ void __launch_bounds__(256) vg_model(long long N, int naxes, const float* __restrict__ rho, const float* __restrict__ vp,
                                                const int* __restrict__ px, const int* __restrict__ py, const int* __restrict__ pz,
                                                float* M, float* irx, float* iry, float* irz)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float r = rho[i];
    float m = r;
    m *= vp[i];
    m *= vp[i];
    M[i] = m;
    const int* part[3] = {px, py, pz};
    float* out[3] = {irx, iry, irz};
    for (int a = 0; a < naxes; ++a) {
        const int j = part[a][i];
        const float avg = j >= 0 ? 0.5f * r + 0.5f * rho[j] : r;
        const float inv = 1.0f / avg;
        out[a][i] = isfinite(inv) ? inv : 0.0f;
    }
}

// ---------------------------------------------------------------- elastic
// CPML memory variables of the elastic step, in VgeParams::psi order
enum ElasticPsi {
    Q_SXX_X, Q_SXY_Y, Q_SXZ_Z, Q_SXY_X, Q_SYY_Y, Q_SYZ_Z, Q_SXZ_X, Q_SYZ_Y, Q_SZZ_Z,
    Q_VXX, Q_VYY, Q_VZZ, Q_VXY, Q_VYX, Q_VXZ, Q_VZX, Q_VYZ, Q_VZY, Q_COUNT
};
// operator slots of VarGridDev
enum ElasticOp { O_DXF, O_DYF, O_DZF, O_DXB, O_DYB, O_DZB, O_DYF_SX, O_DYB_SX, O_DYF_SZ, O_DYB_SZ };

struct VgeParams {
    long long N;
    long long nSurface;         // the y = 0 rows (first in the index order); free surface when fs
    int fs;
    float* v[3];                // vx vy vz
    float* s[6];                // sxx syy szz sxy sxz syz
    float* psi[Q_COUNT];
    const float* M;
    const float* mu;
    const float* muS[3];        // shear averages xy, xz, yz
    const float* ir[3];         // inverse density averages x, y, z
    const int* col[10];
    const float* val[10];
    int W[10];
    const unsigned short* cpc[3];
    const float* cpt[3];
};

__device__ __forceinline__ float vge_row(const VgeParams& P, int op, long long i, const float* __restrict__ u)
{
    const int* __restrict__ c = P.col[op] + i;
    const float* __restrict__ v = P.val[op] + i;
    float s = 0.0f;
    for (int k = 0; k < P.W[op]; ++k) s = __fmaf_rn(v[k * P.N], u[c[k * P.N]], s);
    return s;
}

// CPML::applyCPML (CPML.cpp:84-95), as vg_cpml
__device__ __forceinline__ void vge_cpml(const VgeParams& P, float& d, int slot, int axis, bool half, long long i)
{
    const unsigned code = P.cpc[axis][i];
    if (code == 0) return;
    const float a = __ldg(P.cpt[axis] + 4 * code + (half ? 2 : 0));
    const float b = __ldg(P.cpt[axis] + 4 * code + (half ? 3 : 1));
    if (a == 0.0f && b == 0.0f) return;
    const float ps = __fadd_rn(__fmul_rn(P.psi[slot][i], b), __fmul_rn(a, d));
    P.psi[slot][i] = ps;
    d = __fadd_rn(d, ps);
}

// one derivative term of an update: operator row, then its CPML correction
template <bool CPML>
__device__ __forceinline__ float vge_term(const VgeParams& P, int op, const float* u, int slot, int axis, bool half, long long i)
{
    float d = vge_row(P, op, i, u);
    if (CPML) vge_cpml(P, d, slot, axis, half, i);
    return d;
}

// velocities (ForwardSolver2Delastic.cpp:150-197, ForwardSolver3Delastic.cpp:
// 176-275); the CPML profiles of CPML2D / CPML3D: the forward derivatives
// (sxx_x, syy_y, szz_z) take the half-grid profiles, the others the full ones
template <bool IS3D, bool CPML>
__global__ void __launch_bounds__(256) vge_vel(VgeParams P)
{
    dependent_launch_prologue();
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    float* const* S = P.s;
    float d = vge_term<CPML>(P, O_DXF, S[0], Q_SXX_X, 0, true, i);
    d = __fadd_rn(d, vge_term<CPML>(P, O_DYB_SX, S[3], Q_SXY_Y, 1, false, i));
    if (IS3D) d = __fadd_rn(d, vge_term<CPML>(P, O_DZB, S[4], Q_SXZ_Z, 2, false, i));
    P.v[0][i] = __fadd_rn(P.v[0][i], __fmul_rn(d, P.ir[0][i]));
    d = vge_term<CPML>(P, O_DXB, S[3], Q_SXY_X, 0, false, i);
    d = __fadd_rn(d, vge_term<CPML>(P, O_DYF, S[1], Q_SYY_Y, 1, true, i));
    if (IS3D) d = __fadd_rn(d, vge_term<CPML>(P, O_DZB, S[5], Q_SYZ_Z, 2, false, i));
    P.v[1][i] = __fadd_rn(P.v[1][i], __fmul_rn(d, P.ir[1][i]));
    if (IS3D) {
        d = vge_term<CPML>(P, O_DXB, S[4], Q_SXZ_X, 0, false, i);
        d = __fadd_rn(d, vge_term<CPML>(P, O_DYB_SZ, S[5], Q_SYZ_Y, 1, false, i));
        d = __fadd_rn(d, vge_term<CPML>(P, O_DZF, S[2], Q_SZZ_Z, 2, true, i));
        P.v[2][i] = __fadd_rn(P.v[2][i], __fmul_rn(d, P.ir[2][i]));
    }
}

// stresses (ForwardSolver2Delastic.cpp:200-260, ForwardSolver3Delastic.cpp:
// 280-384): vxx, vyy, vzz with the full profiles, the shear derivatives
// (vxy, vyx, vxz, vzx, vyz, vzy) with the half ones
template <bool IS3D, bool CPML>
__global__ void __launch_bounds__(256) vge_str(VgeParams P)
{
    dependent_launch_prologue();
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= P.N) return;
    float* const* V = P.v;
    const float vxx = vge_term<CPML>(P, O_DXB, V[0], Q_VXX, 0, false, i);
    const float vyy = vge_term<CPML>(P, O_DYB, V[1], Q_VYY, 1, false, i);
    const float vzz = IS3D ? vge_term<CPML>(P, O_DZB, V[2], Q_VZZ, 2, false, i) : 0.0f;
    float sum = __fadd_rn(vxx, vyy);
    if (IS3D) sum = __fadd_rn(sum, vzz);
    const float M = P.M[i];
    const float u = __fmul_rn(sum, M);
    const float mu = P.mu[i];
    float sxx, syy, szz = 0.0f;
    if (IS3D) {
        sxx = __fsub_rn(__fadd_rn(P.s[0][i], u), __fmul_rn(2.0f, __fmul_rn(__fadd_rn(vyy, vzz), mu)));
        syy = __fsub_rn(__fadd_rn(P.s[1][i], u), __fmul_rn(2.0f, __fmul_rn(__fadd_rn(vxx, vzz), mu)));
        szz = __fsub_rn(__fadd_rn(P.s[2][i], u), __fmul_rn(2.0f, __fmul_rn(__fadd_rn(vxx, vyy), mu)));
    } else {
        sxx = __fsub_rn(__fadd_rn(P.s[0][i], u), __fmul_rn(2.0f, __fmul_rn(vyy, mu)));
        syy = __fsub_rn(__fadd_rn(P.s[1][i], u), __fmul_rn(2.0f, __fmul_rn(vxx, mu)));
    }
    if (P.fs && i < P.nSurface) {
        // FreeSurfaceElastic::setModelparameter (FreeSurfaceElastic.cpp:11-47):
        // scaleV = M - 2 mu, scaleH = -(M - 2 mu)^2 / M; exchangeHorizontalUpdate
        // and setSurfaceZero (FreeSurface2Delastic.cpp:14-40,
        // FreeSurface3Delastic.cpp:15-47). The surface rows are never
        // interface rows, so doing it before the interpolations changes nothing.
        const float t = __fsub_rn(M, __fmul_rn(2.0f, mu));
        const float scaleH = -__fdiv_rn(__fmul_rn(t, t), M);
        if (IS3D) {
            const float h = __fmul_rn(scaleH, __fadd_rn(vxx, vzz)), v = __fmul_rn(t, vyy);
            sxx = __fsub_rn(__fadd_rn(sxx, h), v);
            szz = __fsub_rn(__fadd_rn(szz, h), v);
        } else {
            sxx = __fsub_rn(__fadd_rn(sxx, __fmul_rn(scaleH, vxx)), __fmul_rn(t, vyy));
        }
        syy = 0.0f;
    }
    P.s[0][i] = sxx;
    P.s[1][i] = syy;
    if (IS3D) P.s[2][i] = szz;
    float a = vge_term<CPML>(P, O_DYF_SX, V[0], Q_VXY, 1, true, i);
    float b = vge_term<CPML>(P, O_DXF, V[1], Q_VYX, 0, true, i);
    P.s[3][i] = __fadd_rn(P.s[3][i], __fmul_rn(__fadd_rn(a, b), P.muS[0][i]));
    if (IS3D) {
        a = vge_term<CPML>(P, O_DZF, V[0], Q_VXZ, 2, true, i);
        b = vge_term<CPML>(P, O_DXF, V[2], Q_VZX, 0, true, i);
        P.s[4][i] = __fadd_rn(P.s[4][i], __fmul_rn(__fadd_rn(a, b), P.muS[1][i]));
        a = vge_term<CPML>(P, O_DZF, V[1], Q_VYZ, 2, true, i);
        b = vge_term<CPML>(P, O_DYF_SZ, V[2], Q_VZY, 1, true, i);
        P.s[5][i] = __fadd_rn(P.s[5][i], __fmul_rn(__fadd_rn(a, b), P.muS[2][i]));
    }
}

// Elastic::prepareForModelling on the variable grid: M = rho vp^2,
// mu = rho vs^2; inverse densities averaged with the grid's partners
// (Modelparameter.cpp:336-446, 633-640)
__global__ void __launch_bounds__(256) vge_model(long long N, int naxes, const float* __restrict__ rho,
                                                 const float* __restrict__ vp, const float* __restrict__ vs,
                                                 const int* __restrict__ px, const int* __restrict__ py,
                                                 const int* __restrict__ pz, float* M, float* mu, float* irx, float* iry,
                                                 float* irz)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float r = rho[i];
    M[i] = __fmul_rn(__fmul_rn(r, vp[i]), vp[i]);
    mu[i] = __fmul_rn(__fmul_rn(r, vs[i]), vs[i]);
    const int* part[3] = {px, py, pz};
    float* out[3] = {irx, iry, irz};
    for (int a = 0; a < naxes; ++a) {
        const int j = part[a][i];
        const float avg = j >= 0 ? __fadd_rn(__fmul_rn(0.5f, r), __fmul_rn(0.5f, rho[j])) : r;
        const float inv = __fdiv_rn(1.0f, avg);
        out[a][i] = isfinite(inv) ? inv : 0.0f;
    }
}

// the shear modulus at a staggered point of one axis pair: calc4PointAverage
// MatrixRow's average of 1/max(mu, 1) over the point and its neighbours along
// the pair's first axis (s1), second axis (s2) and both (s3); with one axis
// past the grid the point and its neighbour along the other, with both the
// point alone; inverted, results below 4 set to 0 (Modelparameter.cpp:
// 449-624, ModelparameterSeismic.cpp:421-432). A partner the index map does
// not find counts as the point itself. Runs after vge_model (reads mu).
__device__ __forceinline__ float inv_mu(const float* mu, int j) { return __fdiv_rn(1.0f, fmaxf(mu[j], 1.0f)); }

__global__ void __launch_bounds__(256) vge_shear(long long N, const float* __restrict__ mu, const int* __restrict__ s1,
                                                 const int* __restrict__ s2, const int* __restrict__ s3, float* muS)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const int a = s1[i], b = s2[i], c = s3[i];
    const float ii = inv_mu(mu, static_cast<int>(i));
    float s;
    if (a >= 0 && b >= 0) {
        s = __fmul_rn(0.25f, ii);
        s = __fadd_rn(s, __fmul_rn(0.25f, inv_mu(mu, a)));
        s = __fadd_rn(s, __fmul_rn(0.25f, inv_mu(mu, b)));
        s = __fadd_rn(s, __fmul_rn(0.25f, c >= 0 ? inv_mu(mu, c) : ii));
    } else if (a >= 0) {
        s = __fadd_rn(__fmul_rn(0.5f, inv_mu(mu, a)), __fmul_rn(0.5f, ii));
    } else if (b >= 0) {
        s = __fadd_rn(__fmul_rn(0.5f, inv_mu(mu, b)), __fmul_rn(0.5f, ii));
    } else {
        s = ii;
    }
    const float av = __fdiv_rn(1.0f, s);
    muS[i] = av < 4.0f ? 0.0f : av;
}

template <class K, class Prm>
void launch(K kernel, dim3 grid, dim3 block, bool dep, cudaStream_t s, const Prm& P)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = dep ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, P);
}

// the elastic step's CPML memory variables, in VgeParams::psi order
constexpr int kElasticPsi[Q_COUNT] = {PS_SXX_X, PS_SXY_Y, PS_SXZ_Z, PS_SXY_X, PS_SYY_Y, PS_SYZ_Z, PS_SXZ_X, PS_SYZ_Y, PS_SZZ_Z,
                                      PS_VXX, PS_VYY, PS_VZZ, PS_VXY, PS_VYX, PS_VXZ, PS_VZX, PS_VYZ, PS_VZY};
// the ones the 2-D step uses
constexpr int kElasticPsi2D[8] = {Q_SXX_X, Q_SXY_Y, Q_SXY_X, Q_SYY_Y, Q_VXX, Q_VYY, Q_VXY, Q_VYX};

VgeParams elastic_params_of(wave_handle* h)
{
    const VarGridDev& G = *h->vg;
    VgeParams P{};
    P.N = G.N;
    P.nSurface = G.nSurface;
    P.fs = G.fs;
    const int vf[3] = {F_VX, F_VY, F_VZ}, sf[6] = {F_SXX, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ};
    for (int k = 0; k < 3; ++k) P.v[k] = h->f[vf[k]];
    for (int k = 0; k < 6; ++k) P.s[k] = h->f[sf[k]];
    for (int k = 0; k < Q_COUNT; ++k) P.psi[k] = h->psi[kElasticPsi[k]];
    P.M = h->m[M_M];
    P.mu = h->m[M_MU];
    P.muS[0] = h->m[M_MUXY];
    P.muS[1] = h->m[M_MUXZ];
    P.muS[2] = h->m[M_MUYZ];
    P.ir[0] = h->m[M_IRX];
    P.ir[1] = h->m[M_IRY];
    P.ir[2] = h->m[M_IRZ];
    for (int k = 0; k < 10; ++k) {
        P.col[k] = G.col[k];
        P.val[k] = G.val[k];
        P.W[k] = G.W[k];
    }
    for (int a = 0; a < 3; ++a) {
        P.cpc[a] = G.cpCode[a];
        P.cpt[a] = G.cpTab[a];
    }
    return P;
}

VgParams params_of(wave_handle* h)
{
    const VarGridDev& G = *h->vg;
    VgParams P{};
    P.N = G.N;
    P.nSurface = G.nSurface;
    P.fs = G.fs;
    P.cpml = G.cpCode[0] != nullptr;
    P.vx = h->f[F_VX];
    P.vy = h->f[F_VY];
    P.vz = G.is3d ? h->f[F_VZ] : nullptr;
    P.p = h->f[F_P];
    const int slots[6] = {PS_P_X, PS_P_Y, PS_P_Z, PS_VXX, PS_VYY, PS_VZZ};
    for (int k = 0; k < 6; ++k) P.psi[k] = h->psi[slots[k]];
    P.M = h->m[M_M];
    P.ir[0] = h->m[M_IRX];
    P.ir[1] = h->m[M_IRY];
    P.ir[2] = G.is3d ? h->m[M_IRZ] : nullptr;
    for (int k = 0; k < 6; ++k) {
        P.col[k] = G.col[k];
        P.val[k] = G.val[k];
        P.W[k] = G.W[k];
    }
    for (int a = 0; a < 3; ++a) {
        P.cpc[a] = G.cpCode[a];
        P.cpt[a] = G.cpTab[a];
    }
    return P;
}

template <class T>
const T* upload(wave_handle* h, const std::vector<T>& v)
{
    T* d = h->alloc<T>(v.size());
    if (!v.empty()) h->check(cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "variable grid upload");
    return d;
}

} // namespace

void vargrid_setup(wave_handle* h, const VarGridHost& G)
{
    auto D = std::make_shared<VarGridDev>();
    D->L = G.L;
    const bool is3d = h->is3d();
    D->N = G.L.N;
    D->is3d = is3d;
    const bool elastic = h->cfg.equation == WAVE_EQ_ELASTIC;
    D->elastic = elastic ? 1 : 0;
    const EllHost* ops[10] = {&G.Dxf, &G.Dyf, &G.Dzf, &G.Dxb, &G.Dyb, &G.Dzb, &G.DyfSX, &G.DybSX, &G.DyfSZ, &G.DybSZ};
    for (int k = 0; k < (elastic ? (is3d ? 10 : 8) : 6); ++k) {
        if (!is3d && (k == 2 || k == 5)) continue;
        D->W[k] = ops[k]->W;
        D->col[k] = upload(h, ops[k]->col);
        D->val[k] = upload(h, ops[k]->val);
    }
    const InterpHost* in[4] = {&G.full, &G.stagX, &G.stagZ, &G.stagXZ};
    long long total = 0;
    for (int k = 0; k < 4; ++k) {
        D->nInterp[k] = static_cast<int>(in[k]->row.size());
        D->inplace[k] = in[k]->inplace ? 1 : 0;
        total += D->nInterp[k];
        if (D->nInterp[k] == 0) continue;
        D->irow[k] = upload(h, in[k]->row);
        D->icol[k] = upload(h, in[k]->col);
        D->iw[k] = upload(h, in[k]->w);
    }
    // scratch of the two-phase interpolation: the elastic stress launch
    // rewrites up to three fields with the Full rows
    if (total > 0) D->itmp = h->alloc<float>(elastic ? 3 * total : total);
    if (h->cfg.DampingBoundary == 2) {
        for (int a = 0; a < (is3d ? 3 : 2); ++a) {
            D->cpCode[a] = upload(h, G.cpCode[a]);
            D->cpTab[a] = upload(h, G.cpTab[a]);
        }
        if (elastic) {
            for (int q = 0; q < (is3d ? static_cast<int>(Q_COUNT) : 8); ++q) {
                const int slot = kElasticPsi[is3d ? q : kElasticPsi2D[q]];
                h->psi[slot] = h->alloc<float>(D->N);
                h->psiLen[slot] = D->N;
            }
        } else {
            const int slots[6] = {PS_P_X, PS_P_Y, PS_P_Z, PS_VXX, PS_VYY, PS_VZZ};
            for (int k = 0; k < 6; ++k) {
                if (!is3d && (k == 2 || k == 5)) continue;
                h->psi[slots[k]] = h->alloc<float>(D->N);
                h->psiLen[slots[k]] = D->N;
            }
        }
    }
    for (int a = 0; a < (is3d ? 3 : 2); ++a) D->partner[a] = upload(h, G.avgPartner[a]);
    if (elastic)
        for (int q = 0; q < (is3d ? 3 : 1); ++q)
            for (int a = 0; a < 3; ++a) D->shear[q][a] = upload(h, G.shearPartner[q][a]);
    for (int pass = 0; pass < 2; ++pass) {
        const ClassHost& C = G.cls[pass];
        if (!C.ok) continue;
        D->clsId[pass] = upload(h, C.id);
        D->clsOff[pass] = upload(h, C.off);
        D->clsW[pass] = upload(h, C.w);
        D->clsKW[pass] = C.KW;
        for (int q = 0; q < 3; ++q) D->clsBase[pass][q] = C.opBase[q];
    }
    D->nSurface = G.nSurface;
    D->fs = h->cfg.FreeSurface == 1 ? 1 : 0;
    if (!G.absDamp.empty()) D->absDamp = upload(h, G.absDamp);
    h->vg = D;
}

void vargrid_set_model(wave_handle* h, const float* rho, const float* vp, const float* vs)
{
    const VarGridDev& G = *h->vg;
    auto mat = [&](int slot) {
        if (!h->m[slot]) h->m[slot] = h->alloc<float>(h->N);
        h->sp.m[slot] = h->m[slot];
        return h->m[slot];
    };
    if (G.elastic) {
        const unsigned blocks = static_cast<unsigned>((G.N + 255) / 256);
        float* mu = mat(M_MU);
        vge_model<<<blocks, 256, 0, h->stream>>>(G.N, G.is3d ? 3 : 2, rho, vp, vs, G.partner[0], G.partner[1], G.partner[2],
                                                 mat(M_M), mu, mat(M_IRX), mat(M_IRY), G.is3d ? mat(M_IRZ) : nullptr);
        const int slots[3] = {M_MUXY, M_MUXZ, M_MUYZ};
        for (int q = 0; q < (G.is3d ? 3 : 1); ++q)
            vge_shear<<<blocks, 256, 0, h->stream>>>(G.N, mu, G.shear[q][0], G.shear[q][1], G.shear[q][2], mat(slots[q]));
        h->check(cudaGetLastError(), "variable grid model preparation");
        return;
    }
    float* M = mat(M_M);
    float* irx = mat(M_IRX);
    float* iry = mat(M_IRY);
    float* irz = G.is3d ? mat(M_IRZ) : nullptr;
    const unsigned blocks = static_cast<unsigned>((G.N + 255) / 256);
    vg_model<<<blocks, 256, 0, h->stream>>>(G.N, G.is3d ? 3 : 2, rho, vp, G.partner[0], G.partner[1], G.partner[2], M, irx, iry, irz);
    h->check(cudaGetLastError(), "variable grid model preparation");
}

int vargrid_launch_step(wave_handle* h, bool dep, cudaEvent_t* mid, bool* srcrecDone)
{
    *srcrecDone = false;
    const VarGridDev& G = *h->vg;
    const VgParams P = params_of(h);
    const dim3 block(256);
    const dim3 grid(static_cast<unsigned>((G.N + 255) / 256));
    const bool cp = G.cpCode[0] != nullptr;
    // kernel path 1 (generic only) keeps the ELL blocks; otherwise the
    // stencil classes wherever they were built
    const bool cls[2] = {h->kernelPath != 1 && G.clsId[0] != nullptr, h->kernelPath != 1 && G.clsId[1] != nullptr};
    using K = void (*)(VgParams);
    // class kernels with an entry loop of 6 (orders up to 6) or 12
    int wmax = 0;
    for (int k = 0; k < 6; ++k) wmax = G.W[k] > wmax ? G.W[k] : wmax;
    const bool w6 = wmax <= 6;
    const K velK[2][2][2] = {{{vg_vel<false, false, false>, w6 ? vg_vel<false, false, true, 6> : vg_vel<false, false, true>},
                              {vg_vel<false, true, false>, w6 ? vg_vel<false, true, true, 6> : vg_vel<false, true, true>}},
                             {{vg_vel<true, false, false>, w6 ? vg_vel<true, false, true, 6> : vg_vel<true, false, true>},
                              {vg_vel<true, true, false>, w6 ? vg_vel<true, true, true, 6> : vg_vel<true, true, true>}}};
    const K presK[2][2][2] = {{{vg_pres<false, false, false>, w6 ? vg_pres<false, false, true, 6> : vg_pres<false, false, true>},
                               {vg_pres<false, true, false>, w6 ? vg_pres<false, true, true, 6> : vg_pres<false, true, true>}},
                              {{vg_pres<true, false, false>, w6 ? vg_pres<true, false, true, 6> : vg_pres<true, false, true>},
                               {vg_pres<true, true, false>, w6 ? vg_pres<true, true, true, 6> : vg_pres<true, true, true>}}};
    auto with_classes = [&](int pass) {
        VgParams Q = P;
        if (cls[pass]) {
            Q.cid = G.clsId[pass];
            Q.coff = G.clsOff[pass];
            Q.cw = G.clsW[pass];
            Q.KW = G.clsKW[pass];
            for (int q = 0; q < 3; ++q) Q.base[q] = G.clsBase[pass][q];
        }
        return Q;
    };
    K vel = velK[G.is3d ? 1 : 0][cp ? 1 : 0][cls[0] ? 1 : 0];
    K pres = presK[G.is3d ? 1 : 0][cp ? 1 : 0][cls[1] ? 1 : 0];
    int launches = 0;
    const VgeParams E = G.elastic ? elastic_params_of(h) : VgeParams{};
    if (G.elastic) {
        launch(G.is3d ? (cp ? vge_vel<true, true> : vge_vel<true, false>) : (cp ? vge_vel<false, true> : vge_vel<false, false>), grid,
               block, dep, h->stream, E);
    } else {
        launch(vel, grid, block, dep, h->stream, with_classes(0));
    }
    ++launches;
    const bool interp = G.nInterp[0] + G.nInterp[1] + G.nInterp[2] + G.nInterp[3] > 0;
    auto run_interp = [&](VgInterp I, int lists) {
        int mx = 0;
        for (int s = 0; s < lists; ++s) mx = I.n[s] > mx ? I.n[s] : mx;
        if (mx == 0) return;
        const int slots = I.srSlot >= 0 ? lists + 1 : lists;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(static_cast<unsigned>((mx + 255) / 256), static_cast<unsigned>(slots));
        cfg.blockDim = dim3(256);
        cfg.stream = h->stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = dep ? 1 : 0;
        cudaLaunchKernelEx(&cfg, vg_interp, I);
        ++launches;
    };
    // the lists of one launch: in place where allowed, else gather into the
    // scratch in one launch and scatter back in a second
    auto interp_fields = [&](const int* kinds, float* const* fields, int m, bool withSrcrec) {
        VgInterp I{};
        I.srSlot = -1;
        int n = 0;
        bool twoPhase = false;
        long long off = 0;
        for (int q = 0; q < m; ++q) {
            const int kind = kinds[q];
            if (!fields[q] || G.nInterp[kind] == 0) continue;
            I.n[n] = G.nInterp[kind];
            I.f[n] = fields[q];
            I.row[n] = G.irow[kind];
            I.col[n] = G.icol[kind];
            I.w[n] = G.iw[kind];
            I.tmp[n] = G.itmp + off;
            off += G.nInterp[kind];
            I.phase[n] = G.inplace[kind] ? 0 : 1;
            twoPhase = twoPhase || !G.inplace[kind];
            ++n;
        }
        if (withSrcrec && !twoPhase && n > 0) {
            I.srSlot = n;
            I.Q = h->sq;
            I.tcounter = h->tcounter;
            *srcrecDone = true;
        }
        run_interp(I, n);
        if (twoPhase) {
            for (int q = 0; q < n; ++q) I.n[q] = I.phase[q] == 1 ? I.n[q] : 0;
            for (int q = 0; q < n; ++q) I.phase[q] = 2;
            if (withSrcrec && n > 0) {   // after the scatter
                I.srSlot = n;
                I.Q = h->sq;
                I.tcounter = h->tcounter;
                *srcrecDone = true;
            }
            run_interp(I, n);
        }
    };
    if (interp) {
        // vx: StaggeredX, vy: Full, vz: StaggeredZ (ForwardSolver3Dacoustic.cpp:139-197,
        // ForwardSolver2Delastic.cpp:190-197)
        const int kinds[3] = {1, 0, 2};
        float* const fields[3] = {P.vx, P.vy, G.is3d ? P.vz : nullptr};
        interp_fields(kinds, fields, 3, false);
    }
    if (mid) cudaEventRecord(*mid, h->stream);
    if (G.elastic) {
        launch(G.is3d ? (cp ? vge_str<true, true> : vge_str<true, false>) : (cp ? vge_str<false, true> : vge_str<false, false>), grid,
               block, dep, h->stream, E);
    } else {
        launch(pres, grid, block, dep, h->stream, with_classes(1));
    }
    ++launches;
    // ABS: every field of the step times the taper, after the pressure update
    // and before its interpolation (ForwardSolver2Dacoustic.cpp:176-184,
    // ForwardSolver3Dacoustic.cpp:212-221), after the stress interpolations
    // and the free surface (ForwardSolver2Delastic.cpp:283-285,
    // ForwardSolver3Delastic.cpp:407-409)
    auto run_abs = [&](std::initializer_list<float*> fields) {
        VgAbs A{};
        A.N = G.N;
        A.damp = G.absDamp;
        for (float* f : fields)
            if (f) A.f[A.n++] = f;
        launch(vg_abs, grid, block, dep, h->stream, A);
        ++launches;
    };
    if (G.absDamp && !G.elastic) run_abs({P.p, P.vx, P.vy, G.is3d ? P.vz : nullptr});
    if (interp && G.elastic) {
        // sxx, syy: Full, sxy: StaggeredX (ForwardSolver2Delastic.cpp:262-270); sources
        // and receivers in the same launch when none is on an interface row
        bool apart = true;
        auto off_interface = [&](const std::vector<long long>& idx) {
            for (long long i : idx) {
                int x, y, z;
                G.L.coord(i, x, y, z);
                if (G.L.onIfaceY[y]) apart = false;
            }
        };
        off_interface(h->hSrcIdx);
        off_interface(h->hRecIdx);
        // 3-D (ForwardSolver3Delastic.cpp:315-392): szz Full, sxz StaggeredXZ,
        // syz StaggeredZ, which the reference applies twice: the second pass
        // changes nothing where the interpolation runs in place (its rows
        // read only rows it leaves unchanged), so only a two-phase StaggeredZ
        // list is applied again
        const bool again = G.is3d && G.nInterp[2] > 0 && !G.inplace[2];
        const bool fuse = apart && h->kernelPath != 1 && !G.absDamp;   // the taper comes before the sources
        const int kinds[6] = {0, 0, 1, 0, 3, 2};
        float* const fields[6] = {E.s[0], E.s[1], E.s[3], G.is3d ? E.s[2] : nullptr, G.is3d ? E.s[4] : nullptr,
                                  G.is3d ? E.s[5] : nullptr};
        interp_fields(kinds, fields, 6, !again && fuse);
        if (again) {
            const int k2[1] = {2};
            float* const f2[1] = {E.s[5]};
            interp_fields(k2, f2, 1, fuse);
        }
    } else if (interp && G.nInterp[0] > 0) {
        // sources and receivers in the same launch when none is on an interface row
        bool apart = true;
        auto off_interface = [&](const std::vector<long long>& idx) {
            for (long long i : idx) {
                int x, y, z;
                G.L.coord(i, x, y, z);
                if (G.L.onIfaceY[y]) apart = false;
            }
        };
        off_interface(h->hSrcIdx);
        off_interface(h->hRecIdx);
        const int kinds[1] = {0};
        float* const fields[1] = {P.p};
        interp_fields(kinds, fields, 1, apart && h->kernelPath != 1);
    }
    if (G.absDamp && G.elastic)
        run_abs({E.s[0], E.s[1], G.is3d ? E.s[2] : nullptr, E.s[3], G.is3d ? E.s[4] : nullptr, G.is3d ? E.s[5] : nullptr,
                 E.v[0], E.v[1], G.is3d ? E.v[2] : nullptr});
    h->check(cudaGetLastError(), "variable grid step launch");
    return launches;
}

// ---------------------------------------------------------------- adjoint
// Discrete adjoint of the acoustic step above (vg_vel, the velocity
// interpolations, vg_pres with the surface zero, vg_abs, the pressure
// interpolation, sources and receivers), for J = 1/2 sum (d - d_obs)^2 over
// receivers and steps. Every operator of the step is an ELL block, an
// interpolation row list or a per-point factor, so the backward step applies
// their transposes in reverse order: the ELL blocks' transposes are built
// once on the host, an interpolation's transpose moves each rewritten row's
// adjoint onto its four source rows (atomics: a few rows per interface). The
// forward intermediates a step's gradient terms need (Df p + CPML, the
// interpolated velocities, Db v + CPML) are re-formed from the stored state.

namespace {

struct VgAdj {
    long long N, nSurface;
    int fs, cpml, naxes;
    // forward state n and the intermediates re-formed from it
    const float* p;
    const float* v[3];
    const float* psiP[3];       // p_x, p_y, p_z
    const float* psiV[3];       // vxx, vyy, vzz
    float* gx[3];               // Df p + CPML per axis
    float* v2[3];               // velocities after the update (then interpolated in place)
    float* d;                   // Dxb vx + Dyb vy [+ Dzb vz] with CPML
    // adjoint state: of the state after step n on entry, of state n on exit
    float* lp;
    float* lv[3];
    float* lpsiP[3];
    float* lpsiV[3];
    // adjoint temporaries and gradient sums
    float* lp3;
    float* lv2[3];
    float* ldx[3];
    float* lu[3];
    float* gM;
    float* gir[3];
    const float* M;
    const float* ir[3];
    const float* damp;
    const int* col[6];
    const float* val[6];
    int W[6];
    const int* colT[6];
    const float* valT[6];
    int WT[6];
    const unsigned short* cpc[3];
    const float* cpt[3];
};

__device__ __forceinline__ float ell_gather(const int* __restrict__ col, const float* __restrict__ val, int W, long long N, long long i,
                                            const float* __restrict__ u)
{
    float s = 0.0f;
    for (int k = 0; k < W; ++k) s = __fmaf_rn(val[k * N + i], u[col[k * N + i]], s);
    return s;
}

// CPML coefficients of point i on an axis (half: the velocity update's);
// false where the point has none
__device__ __forceinline__ bool adj_cpml(const VgAdj& A, int axis, bool half, long long i, float& a, float& b)
{
    if (!A.cpml) return false;
    const unsigned code = A.cpc[axis][i];
    if (code == 0) return false;
    a = A.cpt[axis][4 * code + (half ? 2 : 0)];
    b = A.cpt[axis][4 * code + (half ? 3 : 1)];
    return a != 0.0f || b != 0.0f;
}

// the velocity update of step n again: gx = Df p + CPML, v2 = v + gx / rho
__global__ void __launch_bounds__(256) vga_fwd_vel(VgAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    for (int ax = 0; ax < A.naxes; ++ax) {
        float u = ell_gather(A.col[ax], A.val[ax], A.W[ax], A.N, i, A.p);
        float a, b;
        if (adj_cpml(A, ax, true, i, a, b)) u = __fadd_rn(u, __fadd_rn(__fmul_rn(A.psiP[ax][i], b), __fmul_rn(a, u)));
        A.gx[ax][i] = u;
        A.v2[ax][i] = __fadd_rn(A.v[ax][i], __fmul_rn(u, A.ir[ax][i]));
    }
}

// the pressure update's derivative sum of step n from the interpolated velocities
__global__ void __launch_bounds__(256) vga_fwd_div(VgAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    float d = 0.0f;
    for (int ax = 0; ax < A.naxes; ++ax) {
        float u = ell_gather(A.col[3 + ax], A.val[3 + ax], A.W[3 + ax], A.N, i, A.v2[ax]);
        float a, b;
        if (adj_cpml(A, ax, false, i, a, b)) u = __fadd_rn(u, __fadd_rn(__fmul_rn(A.psiV[ax][i], b), __fmul_rn(a, u)));
        d = ax == 0 ? u : __fadd_rn(d, u);
    }
    A.d[i] = d;
}

// the residual of step n at the receivers into the adjoint of the field each reads
__global__ void vga_inject(VgAdj A, int nrec, int nt, int n, const long long* __restrict__ ridx, const int* __restrict__ rtype,
                           const float* __restrict__ res)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const int t = rtype[r];
    float* f = t == 1 ? A.lp : (t >= 2 && t - 2 < A.naxes) ? A.lv[t - 2] : nullptr;
    if (f) atomicAdd(f + ridx[r], res[static_cast<long long>(r) * nt + n]);
}

// transposed surface zero (FreeSurface.cpp:14-19): lp3 = lp outside the surface rows
__global__ void __launch_bounds__(256) vga_surface(VgAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    A.lp3[i] = (A.fs && i < A.nSurface) ? 0.0f : A.lp[i];
}

// transposed ABS taper and pressure update, the pressure update's CPML
__global__ void __launch_bounds__(256) vga_pres(VgAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    const float dm = A.damp ? A.damp[i] : 1.0f;
    const float l1 = A.lp3[i] * dm;
    for (int ax = 0; ax < A.naxes; ++ax) A.lv2[ax][i] = A.lv[ax][i] * dm;
    A.gM[i] += l1 * A.d[i];
    const float ld = A.M[i] * l1;
    A.lp[i] = l1;
    for (int ax = 0; ax < A.naxes; ++ax) {
        float a, b;
        if (adj_cpml(A, ax, false, i, a, b)) {
            const float tot = A.lpsiV[ax][i] + ld;
            A.ldx[ax][i] = ld + a * tot;
            A.lpsiV[ax][i] = b * tot;
        } else {
            A.ldx[ax][i] = ld;
        }
    }
}

// lv = lv2 + Db^T ldx per axis
__global__ void __launch_bounds__(256) vga_div_t(VgAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    for (int ax = 0; ax < A.naxes; ++ax)
        A.lv[ax][i] = A.lv2[ax][i] + ell_gather(A.colT[3 + ax], A.valT[3 + ax], A.WT[3 + ax], A.N, i, A.ldx[ax]);
}

// transposed velocity update and its CPML: the density-average gradient, lu = adjoint of Df p
__global__ void __launch_bounds__(256) vga_vel(VgAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    for (int ax = 0; ax < A.naxes; ++ax) {
        const float l1 = A.lv[ax][i];
        const float lg = A.ir[ax][i] * l1;
        A.gir[ax][i] += l1 * A.gx[ax][i];
        float a, b;
        if (adj_cpml(A, ax, true, i, a, b)) {
            const float tot = A.lpsiP[ax][i] + lg;
            A.lu[ax][i] = lg + a * tot;
            A.lpsiP[ax][i] = b * tot;
        } else {
            A.lu[ax][i] = lg;
        }
    }
}

// lp += sum over axes of Df^T lu
__global__ void __launch_bounds__(256) vga_grad_t(VgAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    float s = A.lp[i];
    for (int ax = 0; ax < A.naxes; ++ax) s += ell_gather(A.colT[ax], A.valT[ax], A.WT[ax], A.N, i, A.lu[ax]);
    A.lp[i] = s;
}

// transposed interpolation rows: every list's rewritten rows hand their
// adjoint to their four source rows. Phase 0 takes each row's adjoint into
// the scratch and clears the row, phase 1 adds it onto the source rows.
struct VgInterpT {
    int n[kMaxInterpLists];
    float* f[kMaxInterpLists];
    float* tmp[kMaxInterpLists];
    const int* row[kMaxInterpLists];
    const int* col[kMaxInterpLists];
    const float* w[kMaxInterpLists];
};
__global__ void __launch_bounds__(256) vga_interp_t(VgInterpT I, int phase)
{
    const int s = blockIdx.y;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= I.n[s]) return;
    float* f = I.f[s];
    if (phase == 0) {
        const int r = I.row[s][k];
        I.tmp[s][k] = f[r];
        f[r] = 0.0f;
        return;
    }
    const float t = I.tmp[s][k];
    for (int q = 0; q < 4; ++q) atomicAdd(f + I.col[s][4 * k + q], I.w[s][4 * k + q] * t);
}

// dJ/dvp, dJ/drho from the sums over the steps: M = rho vp^2
// (ModelparameterSeismic.cpp:131-136) and the inverse density averages
// 1 / (rho_i / 2 + rho_j / 2) with the axis partner j, or 1 / rho_i alone
// (Modelparameter.cpp:336-446, 633-640); grho starts at zero
__global__ void __launch_bounds__(256) vga_chain(VgAdj A, const float* __restrict__ rho, const float* __restrict__ vp,
                                                 const int* __restrict__ px, const int* __restrict__ py, const int* __restrict__ pz,
                                                 float* gvp, float* grho)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    const float g = A.gM[i];
    gvp[i] = g * 2.0f * rho[i] * vp[i];
    float own = g * vp[i] * vp[i];
    const int* part[3] = {px, py, pz};
    for (int ax = 0; ax < A.naxes; ++ax) {
        const float r = A.ir[ax][i];
        const float w = -A.gir[ax][i] * r * r;
        const int j = part[ax][i];
        if (j >= 0) {
            own += 0.5f * w;
            atomicAdd(grho + j, 0.5f * w);
        } else {
            own += w;
        }
    }
    atomicAdd(grho + i, own);
}

// residuals seis - dobs and the misfit 1/2 sum res^2 (double, one atomic per block)
__global__ void __launch_bounds__(256) vga_residual(const float* __restrict__ seis, const float* __restrict__ dobs, float* res, long long n,
                                                    double* misfit)
{
    __shared__ double part[256];
    double acc = 0.0;
    for (long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += static_cast<long long>(gridDim.x) * blockDim.x) {
        const float r = seis[k] - dobs[k];
        res[k] = r;
        acc += 0.5 * static_cast<double>(r) * r;
    }
    part[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(misfit, part[0]);
}

// the ELL blocks' transposes (entry-major like the forward blocks; padding
// entries point at the row itself with weight 0)
void build_transposes(wave_handle* h)
{
    VarGridDev& G = *h->vg;
    if (G.transposed) return;
    const long long N = G.N;
    for (int op = 0; op < 10; ++op) {
        if (!G.col[op] || G.W[op] == 0) continue;
        const int W = G.W[op];
        std::vector<int> col(static_cast<size_t>(W) * N);
        std::vector<float> val(col.size());
        h->check(cudaMemcpy(col.data(), G.col[op], col.size() * sizeof(int), cudaMemcpyDeviceToHost), "operator download");
        h->check(cudaMemcpy(val.data(), G.val[op], val.size() * sizeof(float), cudaMemcpyDeviceToHost), "operator download");
        std::vector<int> count(N, 0);
        for (long long i = 0; i < N; ++i)
            for (int k = 0; k < W; ++k)
                if (val[k * N + i] != 0.0f) ++count[col[k * N + i]];
        int WT = 1;
        for (long long c = 0; c < N; ++c) WT = count[c] > WT ? count[c] : WT;
        std::vector<int> colT(static_cast<size_t>(WT) * N);
        std::vector<float> valT(colT.size(), 0.0f);
        for (long long c = 0; c < N; ++c)
            for (int k = 0; k < WT; ++k) colT[k * N + c] = static_cast<int>(c);
        std::fill(count.begin(), count.end(), 0);
        for (long long i = 0; i < N; ++i)
            for (int k = 0; k < W; ++k) {
                const float v = val[k * N + i];
                if (v == 0.0f) continue;
                const int c = col[k * N + i];
                const int slot = count[c]++;
                colT[slot * N + c] = static_cast<int>(i);
                valT[slot * N + c] = v;
            }
        G.WT[op] = WT;
        G.colT[op] = upload(h, colT);
        G.valT[op] = upload(h, valT);
    }
    G.transposed = true;
}

// the interpolation of the listed fields (kinds: 0 Full, 1 StaggeredX, 2
// StaggeredZ), as the forward step runs it, without sources and receivers
void interp_apply(wave_handle* h, const int* kinds, float* const* fields, int m)
{
    const VarGridDev& G = *h->vg;
    VgInterp I{};
    I.srSlot = -1;
    int n = 0, mx = 0;
    bool twoPhase = false;
    long long off = 0;
    if (m > kMaxInterpLists) throw std::runtime_error("interp_apply: too many lists");
    for (int q = 0; q < m; ++q) {
        const int kind = kinds[q];
        if (!fields[q] || G.nInterp[kind] == 0) continue;
        I.n[n] = G.nInterp[kind];
        I.f[n] = fields[q];
        I.row[n] = G.irow[kind];
        I.col[n] = G.icol[kind];
        I.w[n] = G.iw[kind];
        I.tmp[n] = G.itmp + off;
        off += G.nInterp[kind];
        I.phase[n] = G.inplace[kind] ? 0 : 1;
        twoPhase = twoPhase || !G.inplace[kind];
        mx = I.n[n] > mx ? I.n[n] : mx;
        ++n;
    }
    if (n == 0) return;
    const dim3 grid(static_cast<unsigned>((mx + 255) / 256), static_cast<unsigned>(n));
    vg_interp<<<grid, 256, 0, h->stream>>>(I);
    if (twoPhase) {
        for (int q = 0; q < n; ++q) I.n[q] = I.phase[q] == 1 ? I.n[q] : 0;
        for (int q = 0; q < n; ++q) I.phase[q] = 2;
        vg_interp<<<grid, 256, 0, h->stream>>>(I);
    }
}

// the transpose of interp_apply on adjoint fields (tmp: scratch of the
// summed row counts)
void interp_transpose(wave_handle* h, const int* kinds, float* const* fields, int m, float* tmp)
{
    const VarGridDev& G = *h->vg;
    VgInterpT I{};
    int n = 0, mx = 0;
    long long off = 0;
    if (m > kMaxInterpLists) throw std::runtime_error("interp_transpose: too many lists");
    for (int q = 0; q < m; ++q) {
        const int kind = kinds[q];
        if (!fields[q] || G.nInterp[kind] == 0) continue;
        I.n[n] = G.nInterp[kind];
        I.f[n] = fields[q];
        I.row[n] = G.irow[kind];
        I.col[n] = G.icol[kind];
        I.w[n] = G.iw[kind];
        I.tmp[n] = tmp + off;
        off += G.nInterp[kind];
        mx = I.n[n] > mx ? I.n[n] : mx;
        ++n;
    }
    if (n == 0) return;
    const dim3 grid(static_cast<unsigned>((mx + 255) / 256), static_cast<unsigned>(n));
    vga_interp_t<<<grid, 256, 0, h->stream>>>(I, 0);
    vga_interp_t<<<grid, 256, 0, h->stream>>>(I, 1);
}

// device buffers of one adjoint call, freed when it returns
struct AdjPool {
    wave_handle* h;
    std::vector<void*> bufs;
    ~AdjPool() { for (void* p : bufs) cudaFree(p); }
    template <class T = float>
    T* get(size_t count)
    {
        void* p = nullptr;
        h->check(cudaMalloc(&p, (count > 0 ? count : 1) * sizeof(T)), "cudaMalloc");
        bufs.push_back(p);
        return static_cast<T*>(p);
    }
    float* zeros(size_t count)
    {
        float* p = get(count);
        h->check(cudaMemsetAsync(p, 0, (count > 0 ? count : 1) * sizeof(float), h->stream), "memset");
        return p;
    }
};

// The sweep both variable-grid adjoints share: the forward from a zero state
// with a copy of the state parts every K steps, the residuals and misfit,
// then per checkpoint segment the recomputed states and back(n, state n) for
// n from the segment's last step down to its first.
void adjoint_sweep(wave_handle* h, AdjPool& pool, const std::vector<float*>& parts, const float* dobs, int K, double* misfit,
                   float* res, const std::function<void(int, const float*)>& back)
{
    cudaStream_t st = h->stream;
    const long long N = h->vg->N;
    const int NT = h->NT;
    const size_t S = parts.size();
    const int nck = (NT + K - 1) / K;
    float* ckpt = pool.get(static_cast<size_t>(nck) * S * N);
    float* view = pool.get(static_cast<size_t>(K) * S * N);
    auto save = [&](float* dst) {
        for (size_t k = 0; k < S; ++k)
            h->check(cudaMemcpyAsync(dst + k * N, parts[k], N * sizeof(float), cudaMemcpyDeviceToDevice, st), "state copy");
    };
    auto restore = [&](const float* src) {
        for (size_t k = 0; k < S; ++k)
            h->check(cudaMemcpyAsync(parts[k], src + k * N, N * sizeof(float), cudaMemcpyDeviceToDevice, st), "state copy");
    };
    for (float* f : parts) h->check(cudaMemsetAsync(f, 0, N * sizeof(float), st), "memset");
    launch_set_counter(h->tcounter, 0, st);
    for (int n = 0; n < NT; ++n) {
        if (n % K == 0) save(ckpt + static_cast<size_t>(n / K) * S * N);
        step_once(h);
    }
    const long long nd = static_cast<long long>(h->nrec) * NT;
    double* dMis = pool.get<double>(1);
    h->check(cudaMemsetAsync(dMis, 0, sizeof(double), st), "memset");
    vga_residual<<<256, 256, 0, st>>>(h->seis, dobs, res, nd, dMis);
    for (int seg = nck - 1; seg >= 0; --seg) {
        const int n0 = seg * K, n1 = n0 + K < NT ? n0 + K : NT;
        restore(ckpt + static_cast<size_t>(seg) * S * N);
        launch_set_counter(h->tcounter, n0, st);
        for (int n = n0; n < n1; ++n) {
            save(view + static_cast<size_t>(n - n0) * S * N);
            if (n + 1 < n1) step_once(h);
        }
        for (int n = n1 - 1; n >= n0; --n) back(n, view + static_cast<size_t>(n - n0) * S * N);
        h->check(cudaGetLastError(), "variable grid adjoint");
    }
    double J = 0.0;
    h->check(cudaMemcpyAsync(&J, dMis, sizeof(double), cudaMemcpyDeviceToHost, st), "misfit");
    h->check(cudaStreamSynchronize(st), "variable grid adjoint");
    *misfit = J;
    h->stepsSinceReset = NT;
}

void adjoint_acoustic(wave_handle* h, const float* dobs, int K, double* misfit, float* gvp, float* grho)
{
    const VarGridDev& G = *h->vg;
    cudaStream_t st = h->stream;
    const long long N = G.N;
    const int NT = h->NT;
    const int na = G.is3d ? 3 : 2;
    const VgParams P = params_of(h);
    const bool cp = P.cpml != 0;
    AdjPool pool{h};

    // state parts: p, vx, vy [, vz] and the CPML memory variables
    std::vector<float*> parts = {P.p, P.vx, P.vy};
    if (G.is3d) parts.push_back(P.vz);
    if (cp)
        for (int a = 0; a < na; ++a) {
            parts.push_back(P.psi[a]);        // p_x, p_y, p_z
            parts.push_back(P.psi[3 + a]);    // vxx, vyy, vzz
        }

    VgAdj A{};
    A.N = N;
    A.nSurface = G.nSurface;
    A.fs = G.fs;
    A.cpml = cp ? 1 : 0;
    A.naxes = na;
    A.M = P.M;
    A.damp = G.absDamp;
    for (int k = 0; k < 6; ++k) {
        A.col[k] = G.col[k];
        A.val[k] = G.val[k];
        A.W[k] = G.W[k];
        A.colT[k] = G.colT[k];
        A.valT[k] = G.valT[k];
        A.WT[k] = G.WT[k];
    }
    for (int a = 0; a < 3; ++a) {
        A.cpc[a] = G.cpCode[a];
        A.cpt[a] = G.cpTab[a];
        A.ir[a] = P.ir[a];
    }
    const size_t nAdj = 1 + na + (cp ? 2 * na : 0);
    float* adj = pool.zeros(nAdj * N);
    A.lp = adj;
    for (int a = 0; a < na; ++a) {
        A.lv[a] = adj + (1 + a) * N;
        if (cp) {
            A.lpsiP[a] = adj + (1 + na + 2 * a) * N;
            A.lpsiV[a] = adj + (2 + na + 2 * a) * N;
        }
    }
    float* tmp = pool.get((5 * na + 2) * static_cast<size_t>(N));
    for (int a = 0; a < na; ++a) {
        A.gx[a] = tmp + a * N;
        A.v2[a] = tmp + (na + a) * N;
        A.lv2[a] = tmp + (2 * na + a) * N;
        A.ldx[a] = tmp + (3 * na + a) * N;
        A.lu[a] = tmp + (4 * na + a) * N;
    }
    A.d = tmp + 5 * na * N;
    A.lp3 = tmp + (5 * na + 1) * N;
    A.gM = pool.zeros(N);
    float* gir = pool.zeros(static_cast<size_t>(na) * N);
    for (int a = 0; a < na; ++a) A.gir[a] = gir + a * N;
    float* itmp = pool.get(3 * static_cast<size_t>(G.nInterp[0] + G.nInterp[1] + G.nInterp[2] + 1));
    float* res = pool.get(static_cast<size_t>(h->nrec) * NT);

    const dim3 grid(static_cast<unsigned>((N + 255) / 256)), block(256);
    const int velKinds[3] = {1, 0, 2};   // vx StaggeredX, vy Full, vz StaggeredZ
    const int presKind[1] = {0};
    adjoint_sweep(h, pool, parts, dobs, K, misfit, res, [&](int n, const float* sv) {
        A.p = sv;
        for (int a = 0; a < na; ++a) {
            A.v[a] = sv + (1 + a) * N;
            A.psiP[a] = cp ? sv + (1 + na + 2 * a) * N : nullptr;
            A.psiV[a] = cp ? sv + (2 + na + 2 * a) * N : nullptr;
        }
        vga_inject<<<(h->nrec + 127) / 128, 128, 0, st>>>(A, h->nrec, NT, n, h->ridx, h->rtype, res);
        vga_fwd_vel<<<grid, block, 0, st>>>(A);
        float* v2f[3] = {A.v2[0], A.v2[1], na == 3 ? A.v2[2] : nullptr};
        interp_apply(h, velKinds, v2f, 3);
        vga_fwd_div<<<grid, block, 0, st>>>(A);
        vga_surface<<<grid, block, 0, st>>>(A);
        float* lp3f[1] = {A.lp3};
        interp_transpose(h, presKind, lp3f, 1, itmp);
        vga_pres<<<grid, block, 0, st>>>(A);
        vga_div_t<<<grid, block, 0, st>>>(A);
        float* lvf[3] = {A.lv[0], A.lv[1], na == 3 ? A.lv[2] : nullptr};
        interp_transpose(h, velKinds, lvf, 3, itmp);
        vga_vel<<<grid, block, 0, st>>>(A);
        vga_grad_t<<<grid, block, 0, st>>>(A);
    });
    h->check(cudaMemsetAsync(grho, 0, N * sizeof(float), st), "memset");
    vga_chain<<<grid, block, 0, st>>>(A, h->m[M_RHO], h->m[M_VP], G.partner[0], G.partner[1], G.is3d ? G.partner[2] : nullptr,
                                      gvp, grho);
    h->check(cudaGetLastError(), "variable grid adjoint");
    h->check(cudaStreamSynchronize(st), "variable grid adjoint");
}

// ---- 2-D elastic (vge_vel, the velocity interpolations, vge_str with the
// free-surface exchange, the stress interpolations, the ABS taper, sources
// and receivers: FD2Delastic::run, ForwardSolver2Delastic.cpp:117-297)

struct VgeAdj {
    long long N, nSurface;
    int fs, cpml;
    // state n: vx, vy; sxx, syy, sxy; its CPML memory variables
    const float* v[2];
    const float* s[3];
    const float* psi[Q_COUNT];
    // forward intermediates re-formed from state n
    float* gv[2];               // the velocity updates' derivative sums with CPML
    float* v2[2];               // updated velocities (interpolated in place)
    float* e[3];                // vxx, vyy with CPML; the shear sum vxy + vyx
    // adjoint state (vx, vy; sxx, syy, sxy; memory variables) and temporaries
    float* lv[2];
    float* ls[3];
    float* lpsi[Q_COUNT];
    float* lfs[2];              // the surface exchange's adjoint onto vxx, vyy
    float* ld[4];               // adjoints of the raw derivative terms of one pass
    float* gM;
    float* gmu;
    float* gmuXY;
    float* gir[2];
    float* gsH;
    float* gsV;
    const float* M;
    const float* mu;
    const float* muXY;
    const float* ir[2];
    const float* damp;
    const int* col[8];
    const float* val[8];
    int W[8];
    const int* colT[8];
    const float* valT[8];
    int WT[8];
    const unsigned short* cpc[2];
    const float* cpt[2];
};

template <class Adj>
__device__ __forceinline__ bool vge_adj_cpml(const Adj& A, int axis, bool half, long long i, float& a, float& b)
{
    if (!A.cpml) return false;
    const unsigned code = A.cpc[axis][i];
    if (code == 0) return false;
    a = A.cpt[axis][4 * code + (half ? 2 : 0)];
    b = A.cpt[axis][4 * code + (half ? 3 : 1)];
    return a != 0.0f || b != 0.0f;
}

// one derivative term of the forward step from state n: operator row and CPML
template <class Adj>
__device__ __forceinline__ float vge_fwd_term(const Adj& A, int op, const float* u, int slot, int axis, bool half, long long i)
{
    float d = ell_gather(A.col[op], A.val[op], A.W[op], A.N, i, u);
    float a, b;
    if (vge_adj_cpml(A, axis, half, i, a, b)) d = __fadd_rn(d, __fadd_rn(__fmul_rn(A.psi[slot][i], b), __fmul_rn(a, d)));
    return d;
}

// the transposed CPML of one term: the adjoint of the raw derivative, and
// the memory variable's adjoint carried to the step before
template <class Adj>
__device__ __forceinline__ float vge_term_t(const Adj& A, float l, int slot, int axis, bool half, long long i)
{
    float a, b;
    if (!vge_adj_cpml(A, axis, half, i, a, b)) return l;
    const float tot = A.lpsi[slot][i] + l;
    A.lpsi[slot][i] = b * tot;
    return l + a * tot;
}

__global__ void __launch_bounds__(256) vgea_fwd_vel(VgeAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    float d = vge_fwd_term(A, O_DXF, A.s[0], Q_SXX_X, 0, true, i);
    d = __fadd_rn(d, vge_fwd_term(A, O_DYB_SX, A.s[2], Q_SXY_Y, 1, false, i));
    A.gv[0][i] = d;
    A.v2[0][i] = __fadd_rn(A.v[0][i], __fmul_rn(d, A.ir[0][i]));
    d = vge_fwd_term(A, O_DXB, A.s[2], Q_SXY_X, 0, false, i);
    d = __fadd_rn(d, vge_fwd_term(A, O_DYF, A.s[1], Q_SYY_Y, 1, true, i));
    A.gv[1][i] = d;
    A.v2[1][i] = __fadd_rn(A.v[1][i], __fmul_rn(d, A.ir[1][i]));
}

__global__ void __launch_bounds__(256) vgea_fwd_str(VgeAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    A.e[0][i] = vge_fwd_term(A, O_DXB, A.v2[0], Q_VXX, 0, false, i);
    A.e[1][i] = vge_fwd_term(A, O_DYB, A.v2[1], Q_VYY, 1, false, i);
    A.e[2][i] = __fadd_rn(vge_fwd_term(A, O_DYF_SX, A.v2[0], Q_VXY, 1, true, i), vge_fwd_term(A, O_DXF, A.v2[1], Q_VYX, 0, true, i));
}

// receivers: pressure (type 1) reads (sxx + syy) / 2, types 2 and 3 vx, vy
__global__ void vgea_inject(VgeAdj A, int nrec, int nt, int n, const long long* __restrict__ ridx, const int* __restrict__ rtype,
                            const float* __restrict__ res)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const float v = res[static_cast<long long>(r) * nt + n];
    const long long i = ridx[r];
    const int t = rtype[r];
    if (t == 1) {
        atomicAdd(A.ls[0] + i, 0.5f * v);
        atomicAdd(A.ls[1] + i, 0.5f * v);
    } else if (t == 2 || t == 3) {
        atomicAdd(A.lv[t - 2] + i, v);
    }
}

// transposed ABS taper and free-surface exchange (FreeSurface2Delastic.cpp:14-40)
__global__ void __launch_bounds__(256) vgea_abs_fs(VgeAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    if (A.damp) {
        const float d = A.damp[i];
        A.lv[0][i] *= d;
        A.lv[1][i] *= d;
        for (int k = 0; k < 3; ++k) A.ls[k][i] *= d;
    }
    float fx = 0.0f, fy = 0.0f;
    if (A.fs && i < A.nSurface) {
        const float M = A.M[i], t = M - 2.0f * A.mu[i];
        const float sH = -(t * t) / M;
        const float l = A.ls[0][i];
        A.gsH[i] += l * A.e[0][i];
        A.gsV[i] -= l * A.e[1][i];
        fx = sH * l;
        fy = -t * l;
        A.ls[1][i] = 0.0f;
    }
    A.lfs[0][i] = fx;
    A.lfs[1][i] = fy;
}

// transposed stress updates and their CPML (after the stress interpolations' transposes)
__global__ void __launch_bounds__(256) vgea_str(VgeAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    const float l3 = A.ls[2][i];
    A.gmuXY[i] += l3 * A.e[2][i];
    const float lu = A.muXY[i] * l3;
    A.ld[0][i] = vge_term_t(A, lu, Q_VXY, 1, true, i);
    A.ld[1][i] = vge_term_t(A, lu, Q_VYX, 0, true, i);
    const float lx = A.ls[0][i], ly = A.ls[1][i], vxx = A.e[0][i], vyy = A.e[1][i];
    const float l2 = lx + ly, M = A.M[i], mu = A.mu[i];
    A.gM[i] += l2 * (vxx + vyy);
    A.gmu[i] -= 2.0f * (vyy * lx + vxx * ly);
    A.ld[2][i] = vge_term_t(A, M * l2 - 2.0f * mu * ly + A.lfs[0][i], Q_VXX, 0, false, i);
    A.ld[3][i] = vge_term_t(A, M * l2 - 2.0f * mu * lx + A.lfs[1][i], Q_VYY, 1, false, i);
}

// lvx += DyfSX^T ld0 + Dxb^T ld2, lvy += Dxf^T ld1 + Dyb^T ld3
__global__ void __launch_bounds__(256) vgea_str_t(VgeAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    A.lv[0][i] += ell_gather(A.colT[O_DYF_SX], A.valT[O_DYF_SX], A.WT[O_DYF_SX], A.N, i, A.ld[0]) +
                  ell_gather(A.colT[O_DXB], A.valT[O_DXB], A.WT[O_DXB], A.N, i, A.ld[2]);
    A.lv[1][i] += ell_gather(A.colT[O_DXF], A.valT[O_DXF], A.WT[O_DXF], A.N, i, A.ld[1]) +
                  ell_gather(A.colT[O_DYB], A.valT[O_DYB], A.WT[O_DYB], A.N, i, A.ld[3]);
}

// transposed velocity updates and their CPML (after the velocity interpolations' transposes)
__global__ void __launch_bounds__(256) vgea_vel(VgeAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    const float ly = A.lv[1][i];
    A.gir[1][i] += ly * A.gv[1][i];
    const float gy = A.ir[1][i] * ly;
    A.ld[2][i] = vge_term_t(A, gy, Q_SXY_X, 0, false, i);
    A.ld[3][i] = vge_term_t(A, gy, Q_SYY_Y, 1, true, i);
    const float lx = A.lv[0][i];
    A.gir[0][i] += lx * A.gv[0][i];
    const float gx = A.ir[0][i] * lx;
    A.ld[0][i] = vge_term_t(A, gx, Q_SXX_X, 0, true, i);
    A.ld[1][i] = vge_term_t(A, gx, Q_SXY_Y, 1, false, i);
}

// lsxx += Dxf^T ld0, lsyy += Dyf^T ld3, lsxy += Dxb^T ld2 + DybSX^T ld1
__global__ void __launch_bounds__(256) vgea_vel_t(VgeAdj A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    A.ls[0][i] += ell_gather(A.colT[O_DXF], A.valT[O_DXF], A.WT[O_DXF], A.N, i, A.ld[0]);
    A.ls[1][i] += ell_gather(A.colT[O_DYF], A.valT[O_DYF], A.WT[O_DYF], A.N, i, A.ld[3]);
    A.ls[2][i] += ell_gather(A.colT[O_DXB], A.valT[O_DXB], A.WT[O_DXB], A.N, i, A.ld[2]) +
                  ell_gather(A.colT[O_DYB_SX], A.valT[O_DYB_SX], A.WT[O_DYB_SX], A.N, i, A.ld[1]);
}

// chain rule, first half: the surface scales' sensitivities (scaleV = M - 2 mu,
// scaleH = -(M - 2 mu)^2 / M), the XY shear average's (vge_shear: 1 / the
// weighted mean of 1 / max(mu, 1), zero below 4) scattered onto its points,
// the inverse density averages' onto rho; gMt receives the point's dJ/dM,
// gmuT (zeroed) and grho (zeroed) the scattered sums
__global__ void __launch_bounds__(256) vgea_chain1(VgeAdj A, const float* __restrict__ rho, const int* __restrict__ px,
                                                   const int* __restrict__ py, const int* __restrict__ s1, const int* __restrict__ s2,
                                                   const int* __restrict__ s3, float* gMt, float* gmuT, float* grho)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    float g = A.gM[i], gm = A.gmu[i];
    if (A.fs && i < A.nSurface) {
        const float M = A.M[i], t = M - 2.0f * A.mu[i];
        const float sH = A.gsH[i], sV = A.gsV[i];
        g += sV + sH * (-2.0f * t / M + t * t / (M * M));
        gm += -2.0f * sV + sH * 4.0f * t / M;
    }
    gMt[i] = g;
    atomicAdd(gmuT + i, gm);
    const float mxy = A.muXY[i];
    if (mxy >= 4.0f) {
        const float coef = A.gmuXY[i] * mxy * mxy;
        const int a = s1[i], b = s2[i], c = s3[i];
        const int ii = static_cast<int>(i);
        int pts[4];
        float w[4];
        int np = 0;
        if (a >= 0 && b >= 0) {
            pts[0] = ii; pts[1] = a; pts[2] = b; pts[3] = c >= 0 ? c : ii;
            w[0] = w[1] = w[2] = w[3] = 0.25f;
            np = 4;
        } else if (a >= 0 || b >= 0) {
            pts[0] = a >= 0 ? a : b; pts[1] = ii;
            w[0] = w[1] = 0.5f;
            np = 2;
        } else {
            pts[0] = ii;
            w[0] = 1.0f;
            np = 1;
        }
        for (int k = 0; k < np; ++k) {
            const float m = A.mu[pts[k]];
            if (m > 1.0f) atomicAdd(gmuT + pts[k], coef * w[k] / (m * m));
        }
    }
    const int* part[2] = {px, py};
    float own = 0.0f;
    for (int ax = 0; ax < 2; ++ax) {
        const float r = A.ir[ax][i];
        const float wv = -A.gir[ax][i] * r * r;
        const int j = part[ax][i];
        if (j >= 0) {
            own += 0.5f * wv;
            atomicAdd(grho + j, 0.5f * wv);
        } else {
            own += wv;
        }
    }
    atomicAdd(grho + i, own);
}

// chain rule, second half: M = rho vp^2, mu = rho vs^2
__global__ void __launch_bounds__(256) vgea_chain2(long long N, const float* __restrict__ rho, const float* __restrict__ vp,
                                                   const float* __restrict__ vs, const float* __restrict__ gMt,
                                                   const float* __restrict__ gmuT, float* gvp, float* gvs, float* grho)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float g = gMt[i], gm = gmuT[i];
    gvp[i] = g * 2.0f * rho[i] * vp[i];
    gvs[i] = gm * 2.0f * rho[i] * vs[i];
    grho[i] += g * vp[i] * vp[i] + gm * vs[i] * vs[i];
}

void adjoint_elastic2d(wave_handle* h, const float* dobs, int K, double* misfit, float* gvp, float* gvs, float* grho)
{
    const VarGridDev& G = *h->vg;
    cudaStream_t st = h->stream;
    const long long N = G.N;
    const int NT = h->NT;
    const VgeParams E = elastic_params_of(h);
    const bool cp = G.cpCode[0] != nullptr;
    AdjPool pool{h};
    const int psiSlots[8] = {Q_SXX_X, Q_SXY_Y, Q_SXY_X, Q_SYY_Y, Q_VXX, Q_VYY, Q_VXY, Q_VYX};
    std::vector<float*> parts = {E.v[0], E.v[1], E.s[0], E.s[1], E.s[3]};
    if (cp)
        for (int q : psiSlots) parts.push_back(E.psi[q]);

    VgeAdj A{};
    A.N = N;
    A.nSurface = G.nSurface;
    A.fs = G.fs;
    A.cpml = cp ? 1 : 0;
    A.M = E.M;
    A.mu = E.mu;
    A.muXY = E.muS[0];
    A.ir[0] = E.ir[0];
    A.ir[1] = E.ir[1];
    A.damp = G.absDamp;
    for (int k = 0; k < 8; ++k) {
        A.col[k] = G.col[k];
        A.val[k] = G.val[k];
        A.W[k] = G.W[k];
        A.colT[k] = G.colT[k];
        A.valT[k] = G.valT[k];
        A.WT[k] = G.WT[k];
    }
    for (int a = 0; a < 2; ++a) {
        A.cpc[a] = G.cpCode[a];
        A.cpt[a] = G.cpTab[a];
    }
    float* adj = pool.zeros((5 + (cp ? 8 : 0)) * static_cast<size_t>(N));
    for (int k = 0; k < 2; ++k) A.lv[k] = adj + k * N;
    for (int k = 0; k < 3; ++k) A.ls[k] = adj + (2 + k) * N;
    if (cp)
        for (int k = 0; k < 8; ++k) A.lpsi[psiSlots[k]] = adj + (5 + k) * N;
    float* tmp = pool.get(13 * static_cast<size_t>(N));
    for (int k = 0; k < 2; ++k) {
        A.gv[k] = tmp + k * N;
        A.v2[k] = tmp + (2 + k) * N;
        A.lfs[k] = tmp + (4 + k) * N;
    }
    for (int k = 0; k < 3; ++k) A.e[k] = tmp + (6 + k) * N;
    for (int k = 0; k < 4; ++k) A.ld[k] = tmp + (9 + k) * N;
    float* sums = pool.zeros(7 * static_cast<size_t>(N));
    A.gM = sums;
    A.gmu = sums + N;
    A.gmuXY = sums + 2 * N;
    A.gir[0] = sums + 3 * N;
    A.gir[1] = sums + 4 * N;
    A.gsH = sums + 5 * N;
    A.gsV = sums + 6 * N;
    float* itmp = pool.get(3 * static_cast<size_t>(G.nInterp[0] + G.nInterp[1] + G.nInterp[2] + 1));
    float* res = pool.get(static_cast<size_t>(h->nrec) * NT);

    const dim3 grid(static_cast<unsigned>((N + 255) / 256)), block(256);
    const int velKinds[2] = {1, 0};      // vx StaggeredX, vy Full
    const int strKinds[3] = {0, 0, 1};   // sxx, syy Full, sxy StaggeredX
    adjoint_sweep(h, pool, parts, dobs, K, misfit, res, [&](int n, const float* sv) {
        A.v[0] = sv;
        A.v[1] = sv + N;
        for (int k = 0; k < 3; ++k) A.s[k] = sv + (2 + k) * N;
        for (int k = 0; k < 8; ++k) A.psi[psiSlots[k]] = cp ? sv + (5 + k) * N : nullptr;
        vgea_inject<<<(h->nrec + 127) / 128, 128, 0, st>>>(A, h->nrec, NT, n, h->ridx, h->rtype, res);
        vgea_fwd_vel<<<grid, block, 0, st>>>(A);
        float* v2f[2] = {A.v2[0], A.v2[1]};
        interp_apply(h, velKinds, v2f, 2);
        vgea_fwd_str<<<grid, block, 0, st>>>(A);
        vgea_abs_fs<<<grid, block, 0, st>>>(A);
        float* lsf[3] = {A.ls[0], A.ls[1], A.ls[2]};
        interp_transpose(h, strKinds, lsf, 3, itmp);
        vgea_str<<<grid, block, 0, st>>>(A);
        vgea_str_t<<<grid, block, 0, st>>>(A);
        float* lvf[2] = {A.lv[0], A.lv[1]};
        interp_transpose(h, velKinds, lvf, 2, itmp);
        vgea_vel<<<grid, block, 0, st>>>(A);
        vgea_vel_t<<<grid, block, 0, st>>>(A);
    });
    float* gMt = pool.get(N);
    float* gmuT = pool.zeros(N);
    h->check(cudaMemsetAsync(grho, 0, N * sizeof(float), st), "memset");
    vgea_chain1<<<grid, block, 0, st>>>(A, h->m[M_RHO], G.partner[0], G.partner[1], G.shear[0][0], G.shear[0][1], G.shear[0][2], gMt,
                                        gmuT, grho);
    vgea_chain2<<<grid, block, 0, st>>>(N, h->m[M_RHO], h->m[M_VP], h->m[M_VS], gMt, gmuT, gvp, gvs, grho);
    h->check(cudaGetLastError(), "variable grid adjoint");
    h->check(cudaStreamSynchronize(st), "variable grid adjoint");
}

// ---- 3-D elastic (FD3Delastic::run, ForwardSolver3Delastic.cpp:120-414):
// the same sweep with the z terms, the XZ and YZ shear averages, the
// StaggeredXZ interpolation of sxz, the StaggeredZ one of syz (applied again
// where it runs in two phases, as the forward step does) and the surface
// exchange of sxx and szz with vxx + vzz (FreeSurface3Delastic.cpp:15-47)

struct VgeAdj3 {
    long long N, nSurface;
    int fs, cpml;
    const float* v[3];
    const float* s[6];          // sxx syy szz sxy sxz syz
    const float* psi[Q_COUNT];
    float* gv[3];
    float* v2[3];
    float* e[6];                // vxx, vyy, vzz with CPML; the shear sums of sxy, sxz, syz
    float* lv[3];
    float* ls[6];
    float* lpsi[Q_COUNT];
    float* lfs[2];              // the surface exchange's adjoint onto vxx + vzz and onto vyy
    float* ld[9];
    float* gM;
    float* gmu;
    float* gmuS[3];
    float* gir[3];
    float* gsH;
    float* gsV;
    const float* M;
    const float* mu;
    const float* muS[3];
    const float* ir[3];
    const float* damp;
    const int* col[10];
    const float* val[10];
    int W[10];
    const int* colT[10];
    const float* valT[10];
    int WT[10];
    const unsigned short* cpc[3];
    const float* cpt[3];
};

__device__ __forceinline__ float gatherT(const VgeAdj3& A, int op, long long i, const float* u)
{
    return ell_gather(A.colT[op], A.valT[op], A.WT[op], A.N, i, u);
}

__global__ void __launch_bounds__(256) vgea3_fwd_vel(VgeAdj3 A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    float d = vge_fwd_term(A, O_DXF, A.s[0], Q_SXX_X, 0, true, i);
    d = __fadd_rn(d, vge_fwd_term(A, O_DYB_SX, A.s[3], Q_SXY_Y, 1, false, i));
    d = __fadd_rn(d, vge_fwd_term(A, O_DZB, A.s[4], Q_SXZ_Z, 2, false, i));
    A.gv[0][i] = d;
    A.v2[0][i] = __fadd_rn(A.v[0][i], __fmul_rn(d, A.ir[0][i]));
    d = vge_fwd_term(A, O_DXB, A.s[3], Q_SXY_X, 0, false, i);
    d = __fadd_rn(d, vge_fwd_term(A, O_DYF, A.s[1], Q_SYY_Y, 1, true, i));
    d = __fadd_rn(d, vge_fwd_term(A, O_DZB, A.s[5], Q_SYZ_Z, 2, false, i));
    A.gv[1][i] = d;
    A.v2[1][i] = __fadd_rn(A.v[1][i], __fmul_rn(d, A.ir[1][i]));
    d = vge_fwd_term(A, O_DXB, A.s[4], Q_SXZ_X, 0, false, i);
    d = __fadd_rn(d, vge_fwd_term(A, O_DYB_SZ, A.s[5], Q_SYZ_Y, 1, false, i));
    d = __fadd_rn(d, vge_fwd_term(A, O_DZF, A.s[2], Q_SZZ_Z, 2, true, i));
    A.gv[2][i] = d;
    A.v2[2][i] = __fadd_rn(A.v[2][i], __fmul_rn(d, A.ir[2][i]));
}

__global__ void __launch_bounds__(256) vgea3_fwd_str(VgeAdj3 A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    A.e[0][i] = vge_fwd_term(A, O_DXB, A.v2[0], Q_VXX, 0, false, i);
    A.e[1][i] = vge_fwd_term(A, O_DYB, A.v2[1], Q_VYY, 1, false, i);
    A.e[2][i] = vge_fwd_term(A, O_DZB, A.v2[2], Q_VZZ, 2, false, i);
    A.e[3][i] = __fadd_rn(vge_fwd_term(A, O_DYF_SX, A.v2[0], Q_VXY, 1, true, i), vge_fwd_term(A, O_DXF, A.v2[1], Q_VYX, 0, true, i));
    A.e[4][i] = __fadd_rn(vge_fwd_term(A, O_DZF, A.v2[0], Q_VXZ, 2, true, i), vge_fwd_term(A, O_DXF, A.v2[2], Q_VZX, 0, true, i));
    A.e[5][i] = __fadd_rn(vge_fwd_term(A, O_DZF, A.v2[1], Q_VYZ, 2, true, i), vge_fwd_term(A, O_DYF_SZ, A.v2[2], Q_VZY, 1, true, i));
}

// receivers: pressure (type 1) reads (sxx + syy + szz) / 3, types 2-4 vx, vy, vz
__global__ void vgea3_inject(VgeAdj3 A, int nrec, int nt, int n, const long long* __restrict__ ridx, const int* __restrict__ rtype,
                             const float* __restrict__ res)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const float v = res[static_cast<long long>(r) * nt + n];
    const long long i = ridx[r];
    const int t = rtype[r];
    if (t == 1) {
        for (int k = 0; k < 3; ++k) atomicAdd(A.ls[k] + i, v / 3.0f);
    } else if (t >= 2 && t <= 4) {
        atomicAdd(A.lv[t - 2] + i, v);
    }
}

__global__ void __launch_bounds__(256) vgea3_abs_fs(VgeAdj3 A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    if (A.damp) {
        const float d = A.damp[i];
        for (int k = 0; k < 3; ++k) A.lv[k][i] *= d;
        for (int k = 0; k < 6; ++k) A.ls[k][i] *= d;
    }
    float fh = 0.0f, fv = 0.0f;
    if (A.fs && i < A.nSurface) {
        const float M = A.M[i], t = M - 2.0f * A.mu[i];
        const float sH = -(t * t) / M;
        const float l = A.ls[0][i] + A.ls[2][i];
        A.gsH[i] += l * (A.e[0][i] + A.e[2][i]);
        A.gsV[i] -= l * A.e[1][i];
        fh = sH * l;
        fv = -t * l;
        A.ls[1][i] = 0.0f;
    }
    A.lfs[0][i] = fh;
    A.lfs[1][i] = fv;
}

__global__ void __launch_bounds__(256) vgea3_str(VgeAdj3 A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    // shear stresses: (first term's memory slot, axis), (second term's)
    const int slot[3][2] = {{Q_VXY, Q_VYX}, {Q_VXZ, Q_VZX}, {Q_VYZ, Q_VZY}};
    const int axis[3][2] = {{1, 0}, {2, 0}, {2, 1}};
    for (int c = 0; c < 3; ++c) {
        const float l = A.ls[3 + c][i];
        A.gmuS[c][i] += l * A.e[3 + c][i];
        const float lu = A.muS[c][i] * l;
        A.ld[2 * c][i] = vge_term_t(A, lu, slot[c][0], axis[c][0], true, i);
        A.ld[2 * c + 1][i] = vge_term_t(A, lu, slot[c][1], axis[c][1], true, i);
    }
    const float lx = A.ls[0][i], ly = A.ls[1][i], lz = A.ls[2][i];
    const float ex = A.e[0][i], ey = A.e[1][i], ez = A.e[2][i];
    const float l3 = lx + ly + lz, M = A.M[i], mu = A.mu[i];
    A.gM[i] += l3 * (ex + ey + ez);
    A.gmu[i] -= 2.0f * ((ey + ez) * lx + (ex + ez) * ly + (ex + ey) * lz);
    A.ld[6][i] = vge_term_t(A, M * l3 - 2.0f * mu * (ly + lz) + A.lfs[0][i], Q_VXX, 0, false, i);
    A.ld[7][i] = vge_term_t(A, M * l3 - 2.0f * mu * (lx + lz) + A.lfs[1][i], Q_VYY, 1, false, i);
    A.ld[8][i] = vge_term_t(A, M * l3 - 2.0f * mu * (lx + ly) + A.lfs[0][i], Q_VZZ, 2, false, i);
}

__global__ void __launch_bounds__(256) vgea3_str_t(VgeAdj3 A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    A.lv[0][i] += gatherT(A, O_DYF_SX, i, A.ld[0]) + gatherT(A, O_DZF, i, A.ld[2]) + gatherT(A, O_DXB, i, A.ld[6]);
    A.lv[1][i] += gatherT(A, O_DXF, i, A.ld[1]) + gatherT(A, O_DZF, i, A.ld[4]) + gatherT(A, O_DYB, i, A.ld[7]);
    A.lv[2][i] += gatherT(A, O_DXF, i, A.ld[3]) + gatherT(A, O_DYF_SZ, i, A.ld[5]) + gatherT(A, O_DZB, i, A.ld[8]);
}

__global__ void __launch_bounds__(256) vgea3_vel(VgeAdj3 A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    // per velocity: (memory slot, axis, half) of its three terms
    const int slot[3][3] = {{Q_SXX_X, Q_SXY_Y, Q_SXZ_Z}, {Q_SXY_X, Q_SYY_Y, Q_SYZ_Z}, {Q_SXZ_X, Q_SYZ_Y, Q_SZZ_Z}};
    for (int k = 0; k < 3; ++k) {
        const float l = A.lv[k][i];
        A.gir[k][i] += l * A.gv[k][i];
        const float g = A.ir[k][i] * l;
        for (int a = 0; a < 3; ++a) A.ld[3 * k + a][i] = vge_term_t(A, g, slot[k][a], a, a == k, i);
    }
}

__global__ void __launch_bounds__(256) vgea3_vel_t(VgeAdj3 A)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    A.ls[0][i] += gatherT(A, O_DXF, i, A.ld[0]);
    A.ls[1][i] += gatherT(A, O_DYF, i, A.ld[4]);
    A.ls[2][i] += gatherT(A, O_DZF, i, A.ld[8]);
    A.ls[3][i] += gatherT(A, O_DYB_SX, i, A.ld[1]) + gatherT(A, O_DXB, i, A.ld[3]);
    A.ls[4][i] += gatherT(A, O_DZB, i, A.ld[2]) + gatherT(A, O_DXB, i, A.ld[6]);
    A.ls[5][i] += gatherT(A, O_DZB, i, A.ld[5]) + gatherT(A, O_DYB_SZ, i, A.ld[7]);
}

// chain rule, first half (as vgea_chain1 with the three shear averages and axes)
__global__ void __launch_bounds__(256) vgea3_chain1(VgeAdj3 A, const int* __restrict__ px, const int* __restrict__ py,
                                                    const int* __restrict__ pz, const int* const* __restrict__ shear, float* gMt,
                                                    float* gmuT, float* grho)
{
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= A.N) return;
    float g = A.gM[i], gm = A.gmu[i];
    if (A.fs && i < A.nSurface) {
        const float M = A.M[i], t = M - 2.0f * A.mu[i];
        const float sH = A.gsH[i], sV = A.gsV[i];
        g += sV + sH * (-2.0f * t / M + t * t / (M * M));
        gm += -2.0f * sV + sH * 4.0f * t / M;
    }
    gMt[i] = g;
    atomicAdd(gmuT + i, gm);
    const int ii = static_cast<int>(i);
    for (int q = 0; q < 3; ++q) {
        const float m = A.muS[q][i];
        if (m < 4.0f) continue;
        const float coef = A.gmuS[q][i] * m * m;
        const int a = shear[3 * q][i], b = shear[3 * q + 1][i], c = shear[3 * q + 2][i];
        int pts[4];
        float w[4];
        int np;
        if (a >= 0 && b >= 0) {
            pts[0] = ii; pts[1] = a; pts[2] = b; pts[3] = c >= 0 ? c : ii;
            w[0] = w[1] = w[2] = w[3] = 0.25f;
            np = 4;
        } else if (a >= 0 || b >= 0) {
            pts[0] = a >= 0 ? a : b; pts[1] = ii;
            w[0] = w[1] = 0.5f;
            np = 2;
        } else {
            pts[0] = ii;
            w[0] = 1.0f;
            np = 1;
        }
        for (int k = 0; k < np; ++k) {
            const float mk = A.mu[pts[k]];
            if (mk > 1.0f) atomicAdd(gmuT + pts[k], coef * w[k] / (mk * mk));
        }
    }
    const int* part[3] = {px, py, pz};
    float own = 0.0f;
    for (int ax = 0; ax < 3; ++ax) {
        const float r = A.ir[ax][i];
        const float wv = -A.gir[ax][i] * r * r;
        const int j = part[ax][i];
        if (j >= 0) {
            own += 0.5f * wv;
            atomicAdd(grho + j, 0.5f * wv);
        } else {
            own += wv;
        }
    }
    atomicAdd(grho + i, own);
}

void adjoint_elastic3d(wave_handle* h, const float* dobs, int K, double* misfit, float* gvp, float* gvs, float* grho)
{
    const VarGridDev& G = *h->vg;
    cudaStream_t st = h->stream;
    const long long N = G.N;
    const int NT = h->NT;
    const VgeParams E = elastic_params_of(h);
    const bool cp = G.cpCode[0] != nullptr;
    AdjPool pool{h};
    std::vector<float*> parts = {E.v[0], E.v[1], E.v[2]};
    for (int k = 0; k < 6; ++k) parts.push_back(E.s[k]);
    if (cp)
        for (int q = 0; q < Q_COUNT; ++q) parts.push_back(E.psi[q]);

    VgeAdj3 A{};
    A.N = N;
    A.nSurface = G.nSurface;
    A.fs = G.fs;
    A.cpml = cp ? 1 : 0;
    A.M = E.M;
    A.mu = E.mu;
    for (int k = 0; k < 3; ++k) {
        A.muS[k] = E.muS[k];
        A.ir[k] = E.ir[k];
        A.cpc[k] = G.cpCode[k];
        A.cpt[k] = G.cpTab[k];
    }
    A.damp = G.absDamp;
    for (int k = 0; k < 10; ++k) {
        A.col[k] = G.col[k];
        A.val[k] = G.val[k];
        A.W[k] = G.W[k];
        A.colT[k] = G.colT[k];
        A.valT[k] = G.valT[k];
        A.WT[k] = G.WT[k];
    }
    float* adj = pool.zeros((9 + (cp ? Q_COUNT : 0)) * static_cast<size_t>(N));
    for (int k = 0; k < 3; ++k) A.lv[k] = adj + k * N;
    for (int k = 0; k < 6; ++k) A.ls[k] = adj + (3 + k) * N;
    if (cp)
        for (int q = 0; q < Q_COUNT; ++q) A.lpsi[q] = adj + (9 + q) * N;
    float* tmp = pool.get(26 * static_cast<size_t>(N));
    for (int k = 0; k < 3; ++k) {
        A.gv[k] = tmp + k * N;
        A.v2[k] = tmp + (3 + k) * N;
    }
    for (int k = 0; k < 6; ++k) A.e[k] = tmp + (6 + k) * N;
    for (int k = 0; k < 2; ++k) A.lfs[k] = tmp + (12 + k) * N;
    for (int k = 0; k < 9; ++k) A.ld[k] = tmp + (14 + k) * N;
    float* sums = pool.zeros(10 * static_cast<size_t>(N));
    A.gM = sums;
    A.gmu = sums + N;
    for (int k = 0; k < 3; ++k) {
        A.gmuS[k] = sums + (2 + k) * N;
        A.gir[k] = sums + (5 + k) * N;
    }
    A.gsH = sums + 8 * N;
    A.gsV = sums + 9 * N;
    float* itmp = pool.get(6 * static_cast<size_t>(G.nInterp[0] + G.nInterp[1] + G.nInterp[2] + G.nInterp[3] + 1));
    float* res = pool.get(static_cast<size_t>(h->nrec) * NT);

    const dim3 grid(static_cast<unsigned>((N + 255) / 256)), block(256);
    const int velKinds[3] = {1, 0, 2};            // vx StaggeredX, vy Full, vz StaggeredZ
    const int strKinds[6] = {0, 0, 0, 1, 3, 2};   // sxx syy szz Full, sxy StaggeredX, sxz StaggeredXZ, syz StaggeredZ
    const int zKind[1] = {2};
    const bool again = G.nInterp[2] > 0 && !G.inplace[2];
    adjoint_sweep(h, pool, parts, dobs, K, misfit, res, [&](int n, const float* sv) {
        for (int k = 0; k < 3; ++k) A.v[k] = sv + k * N;
        for (int k = 0; k < 6; ++k) A.s[k] = sv + (3 + k) * N;
        for (int q = 0; q < Q_COUNT; ++q) A.psi[q] = cp ? sv + (9 + q) * N : nullptr;
        vgea3_inject<<<(h->nrec + 127) / 128, 128, 0, st>>>(A, h->nrec, NT, n, h->ridx, h->rtype, res);
        vgea3_fwd_vel<<<grid, block, 0, st>>>(A);
        float* v2f[3] = {A.v2[0], A.v2[1], A.v2[2]};
        interp_apply(h, velKinds, v2f, 3);
        vgea3_fwd_str<<<grid, block, 0, st>>>(A);
        vgea3_abs_fs<<<grid, block, 0, st>>>(A);
        if (again) {   // the second StaggeredZ pass of syz, transposed first
            float* f5[1] = {A.ls[5]};
            interp_transpose(h, zKind, f5, 1, itmp);
        }
        float* lsf[6] = {A.ls[0], A.ls[1], A.ls[2], A.ls[3], A.ls[4], A.ls[5]};
        interp_transpose(h, strKinds, lsf, 6, itmp);
        vgea3_str<<<grid, block, 0, st>>>(A);
        vgea3_str_t<<<grid, block, 0, st>>>(A);
        float* lvf[3] = {A.lv[0], A.lv[1], A.lv[2]};
        interp_transpose(h, velKinds, lvf, 3, itmp);
        vgea3_vel<<<grid, block, 0, st>>>(A);
        vgea3_vel_t<<<grid, block, 0, st>>>(A);
    });
    float* gMt = pool.get(N);
    float* gmuT = pool.zeros(N);
    const int** shear = pool.get<const int*>(9);
    const int* hs[9];
    for (int q = 0; q < 3; ++q)
        for (int a = 0; a < 3; ++a) hs[3 * q + a] = G.shear[q][a];
    h->check(cudaMemcpyAsync(shear, hs, sizeof(hs), cudaMemcpyHostToDevice, st), "copy");
    h->check(cudaMemsetAsync(grho, 0, N * sizeof(float), st), "memset");
    vgea3_chain1<<<grid, block, 0, st>>>(A, G.partner[0], G.partner[1], G.partner[2], shear, gMt, gmuT, grho);
    vgea_chain2<<<grid, block, 0, st>>>(N, h->m[M_RHO], h->m[M_VP], h->m[M_VS], gMt, gmuT, gvp, gvs, grho);
    h->check(cudaGetLastError(), "variable grid adjoint");
    h->check(cudaStreamSynchronize(st), "variable grid adjoint");
}

} // namespace

void vargrid_adjoint(wave_handle* h, const float* dobs, int K, double* misfit, float* gvp, float* gvs, float* grho)
{
    build_transposes(h);
    if (h->vg->elastic) {
        if (h->vg->is3d) adjoint_elastic3d(h, dobs, K, misfit, gvp, gvs, grho);
        else adjoint_elastic2d(h, dobs, K, misfit, gvp, gvs, grho);
        return;
    }
    h->check(cudaMemsetAsync(gvs, 0, h->vg->N * sizeof(float), h->stream), "memset");
    adjoint_acoustic(h, dobs, K, misfit, gvp, grho);
}

} // namespace wave
