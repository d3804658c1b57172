// adjoint.cu — gradient of the seismogram misfit J = 1/2 sum (d - d_obs)^2 with
// respect to vp, vs and rho for the 2-D elastic time step, by the discrete
// adjoint of the forward step (FD2Delastic::run, ForwardSolver2Delastic.cpp:
// 117-297) with CPML (CPML.cpp:84-95), the free surface (image operators and
// FreeSurface2Delastic.cpp:14-45), the ABS taper (ABS2D.cpp:14-50) and
// checkpointing.
//
// The forward step is linear in the state X = (vx, vy, sxx, syy, sxy, psi):
//   velocity pass   a_k = D_k sigma,  P_k' = b P_k + a a_k,  a_k' = a_k + P_k',
//                   vx' = vx + irx (a1' + a2'),  vy' = vy + iry (a3' + a4')
//   stress pass     c_k = D_k v',     Q_k' = b Q_k + a c_k,  c_k' = c_k + Q_k',
//                   sxx' = sxx + M (c1' + c2') - 2 mu c2', syy' = syy + M (c1' + c2') - 2 mu c1',
//                   sxy' = sxy + mu_xy (c3' + c4')
// then at y = 0 with the free surface sxx' += sh c1' - sv c2', syy' = 0
// (sv = M - 2 mu, sh = -sv^2 / M), then the ABS taper d on all five fields,
// plus source terms, and receivers read X after each step. The stress pass
// reads the velocities before the taper and the sources, v' = (v_{n+1} - s) / d,
// re-formed from the saved state when ABS or velocity sources are on. The adjoint runs
// the transposed pieces backwards (three stages per step: stress transpose,
// velocity transpose, stress-derivative transpose; the third stage of a step
// runs inside the first kernel of the next one back, so two kernels per
// step) and accumulates
// dJ/dM, dJ/dmu, dJ/dmu_xy, dJ/dirx, dJ/diry, which a last kernel maps to
// vp, vs, rho through the model preparation (moduli, 2-point inverse density
// averages, harmonic 4-point shear average with its edge fallbacks and vacuum
// rules; Modelparameter.cpp:336-639, ModelparameterSeismic.cpp:131-136, 421-432).
//
// The lossless 2-D TMz step (FD2Dtmem::run, ForwardSolver2Dtmem.cpp:108-174)
// has its own stages on the same driver (again two kernels per step):
//   hx' = hx - iMyz (Dyf ez + P_ezy)'   hy' = hy + iMxz (Dxf ez + P_ezx)'
//   ez' = Ca ez + Cb ((Dxb hy' + P_hyx)' - (Dyb hx' + P_hxy)'), then the ABS taper,
// and a last kernel maps dJ/dCa, dJ/dCb, dJ/diMxz, dJ/diMyz to eps_r, sigma
// and mu_r (Ca, Cb of ForwardSolverEM.cpp:14-67 with eps = eps_r eps0; the
// inverse 2-point mu averages of TMEM.cpp:366-374).
//
// The 2-D SH step (FD2Dsh::run, ForwardSolver2Dsh.cpp:108-196) likewise:
//   vz' = vz + irho ((Dxb sxz + P_sxz_x)' + (DybS syz + P_syz_y)')
//   sxz' = sxz + muXZ (Dxf vz' + P_vzx)',  syz' = syz + muYZ (Dyf vz' + P_vzy)',
// then the ABS taper on all three, and a last kernel maps dJ/dmuXZ, dJ/dmuYZ,
// dJ/dirho to vs and rho (mu = max(rho vs^2, 1), its harmonic 2-point averages
// along x and y, SH.cpp:424-431; irho = 1 / rho).
//
// The lossless 2-D TEz step (FD2Demem::run, ForwardSolver2Demem.cpp:112-185):
//   hz' = hz - iMxy ((Dxf ey + P_eyx)' - (Dyf ex + P_exy)')
//   ex' = CaX ex + CbX (Dyb hz' + P_hzy)',  ey' = CaY ey - CbY (Dxb hz' + P_hzx)',
// then the ABS taper on all three, and a last kernel maps dJ/dCaX, dJ/dCbX,
// dJ/dCaY, dJ/dCbY, dJ/diMxy to eps_r, sigma and mu_r (Ca, Cb of the 2-point
// averages of eps and sigma along x and y, EMEM.cpp:378-392; iMxy the inverse
// 4-point average of mu).
//
// Checkpointing: the forward run saves the state every K steps; the backward
// sweep recomputes each K-step segment into a buffer of K+1 states and walks
// it backwards. The reference has no adjoint (its inversion lives in a
// separate project); this file has no counterpart there.
#include <cmath>
#include <functional>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "handle.h"
#include "stencil.cuh"

namespace wave {

// parts of one saved state, in view order
enum AdjPart { AV_VX, AV_VY, AV_SXX, AV_SYY, AV_SXY, AV_P1, AV_P2, AV_P3, AV_P4, AV_Q1, AV_Q2, AV_Q3, AV_Q4, AV_COUNT };

// psi slot of each psi part: velocity pass P1..P4, stress pass Q1..Q4
static const int kAdjPsiSlot[8] = {PS_SXX_X, PS_SXY_Y, PS_SXY_X, PS_SYY_Y, PS_VXX, PS_VYY, PS_VXY, PS_VYX};

struct AdjShot {
    float* view;                 // recompute buffer: K+1 states
    long long stride;            // floats per state
    long long off[AV_COUNT];     // part offsets within a state (0 = absent psi)
    float* lf[5];                // adjoint fields: vx, vy, sxx, syy, sxy
    float* lpsi[8];              // adjoint psi (slab layout of the forward psi)
    float* T[8];                 // adjoints of the raw derivatives c1..c4, a1..a4
    float* g[5];                 // dJ/dM, dJ/dmu, dJ/dmu_xy, dJ/dirx, dJ/diry
    const long long* ridx;
    const int* rtype;
    const float* res;            // residual d - d_obs, nrec x nt
    int nrec, nt;
    int tm;                      // 1: lossless 2-D TMz (parts: hx, hy, ez; psi ezy, ezx, hyx, hxy)
    int sh;                      // 1: 2-D SH (parts: vz, sxz, syz; psi sxz_x, syz_y, vzx, vzy)
    int te;                      // 1: lossless 2-D TEz (parts: hz, ex, ey; psi eyx, exy, hzy, hzx)
    float* vprime[2];            // vx', vy' (TMz: hx', hy') of the current step (null: the saved state's are they)
    const long long* sidx;       // sources (velocity sources are taken out of v')
    const int* stype;
    const float* signals;        // nsrc x nt
    int nsrc;
};

struct CopyPart {
    const float* src;
    float* dst;
    long long n;
    long long srcStride, dstStride;   // per state index
};

namespace {

// (D^T lam)[c] = sum_k w_{c-k}(k) lam[c-k] over the rows c-k inside the axis,
// with the row weights of deriv(): interior weights or the edge-table row
template <int H, bool FWD>
__device__ __forceinline__ float derivT(const float* __restrict__ lam, long long i, long long st, int c, const Op1D& op)
{
    float s = 0.0f;
    if (!op.full && c - H >= op.E && c + H < op.n - op.E) {
        // every row c-k is an interior row: its weight at offset k is the interior weight
#pragma unroll
        for (int k = (FWD ? -H + 1 : -H); k <= (FWD ? H : H - 1); ++k) s += op.w[kMaxHalf + k] * __ldg(lam + i - k * st);
        return s;
    }
#pragma unroll
    for (int k = -H; k <= H; ++k) {
        const int r = c - k;
        if (r < 0 || r >= op.n) continue;
        float w;
        if (!op.full && r >= op.E && r < op.n - op.E) {
            w = op.w[kMaxHalf + k];
        } else {
            const int slot = op.full ? r : (r < op.E ? r : op.E + r - (op.n - op.E));
            w = __ldg(op.tab + slot * kTabW + kMaxHalf + k);
        }
        if (w != 0.0f) s += w * __ldg(lam + i - k * st);
    }
    return s;
}

// adjoint of (c, Q) -> (c' = (1 + a) c + b Q, Q' = a c + b Q)
__device__ __forceinline__ void cpml_adj(float& l, float* lpsi, float a, float b)
{
    const float lq = *lpsi;
    const float lc = (1.0f + a) * l + a * lq;
    *lpsi = b * (l + lq);
    l = lc;
}

struct Slabs {
    int sx, sy;
    long long px, py;
};

__device__ __forceinline__ Slabs slabs_of(const StepParams& P, const Pt& p)
{
    Slabs S;
    S.sx = P.useCpml ? slab(p.x, P.cx) : -1;
    S.sy = P.useCpml ? slab(p.y, P.cy) : -1;
    S.px = S.sx >= 0 ? pix(P, p, S.sx) : 0;
    S.py = S.sy >= 0 ? piy(P, p, S.sy) : 0;
    return S;
}

// stress-pass transpose at step n (state n = view vn, state n+1 = view vn+1)
template <int H>
__device__ __forceinline__ void adj_stress_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn, bool pending)
{
    const float* X1 = A.view + (long long)(vn + 1) * A.stride;
    const long long i = p.i, sy = P.NX;
    const float* vx1 = A.vprime[0] ? A.vprime[0] : X1 + A.off[AV_VX];
    const float* vy1 = A.vprime[1] ? A.vprime[1] : X1 + A.off[AV_VY];
    const float M = __ldg(P.m[M_M] + i), mu = __ldg(P.m[M_MU] + i), mxy = __ldg(P.m[M_MUXY] + i);
    const Slabs S = slabs_of(P, p);
    // forward derivatives with their CPML correction, c' = c + Q_{n+1}
    float c1 = deriv<H, false>(vx1, i, 1, p.x, P.Dxb);
    float c2 = deriv<H, false>(vy1, i, sy, p.y, P.Dyb);
    float c3 = deriv<H, true>(vx1, i, sy, p.y, P.Dyf);
    float c4 = deriv<H, true>(vy1, i, 1, p.x, P.Dxf);
    if (S.sx >= 0) { c1 += X1[A.off[AV_Q1] + S.px]; c4 += X1[A.off[AV_Q4] + S.px]; }
    if (S.sy >= 0) { c2 += X1[A.off[AV_Q2] + S.py]; c3 += X1[A.off[AV_Q3] + S.py]; }
    float lxx = A.lf[2][i], lyy = A.lf[3][i], lxy = A.lf[4][i];
    if (pending) {
        // the transposed velocity-pass derivatives of sigma from the step after
        // this one (its third stage, folded in here to save a launch)
        const Op1D& DybS = P.fs ? P.DybS : P.Dyb;
        const Op1D& DyfS = P.fs ? P.DyfS : P.Dyf;
        lxx += derivT<H, true>(A.T[4], i, 1, p.x, P.Dxf);
        float u = derivT<H, false>(A.T[5], i, sy, p.y, DybS);
        u += derivT<H, false>(A.T[6], i, 1, p.x, P.Dxb);
        lxy += u;
        lyy += derivT<H, true>(A.T[7], i, sy, p.y, DyfS);
    }
    if (P.abs) {
        // the taper multiplied all five fields last: their adjoints first
        const float d = absDamp(P, p);
        lxx *= d; lyy *= d; lxy *= d;
        A.lf[0][i] *= d;
        A.lf[1][i] *= d;
    }
    const bool fsRow = P.fs && p.y == 0;
    if (fsRow) lyy = 0.0f;                 // syy' = 0 on the surface
    A.lf[2][i] = lxx;
    A.lf[3][i] = lyy;
    A.lf[4][i] = lxy;
    const float lam = M - 2.0f * mu;
    float l1 = M * lxx + lam * lyy;
    float l2 = lam * lxx + M * lyy;
    float l3 = mxy * lxy, l4 = l3;
    if (fsRow) {
        // sxx' += sh c1' - sv c2' with sv = M - 2 mu, sh = -sv^2 / M
        const float sv = lam, sh = -(sv * sv) / M;
        l1 += sh * lxx;
        l2 -= sv * lxx;
        // dJ/dsh = lxx c1', dJ/dsv = -lxx c2' (c1, c2 carry their CPML correction here);
        // d sv / dM = 1, d sv / dmu = -2; d sh / dM = -(2 sv / M - sv^2 / M^2), d sh / dmu = 4 sv / M
        const float gh = lxx * c1, gv = -lxx * c2;
        A.g[0][i] += gv - gh * (2.0f * sv / M - (sv * sv) / (M * M));
        A.g[1][i] += -2.0f * gv + gh * 4.0f * sv / M;
    }
    if (S.sx >= 0) {
        cpml_adj(l1, A.lpsi[4] + S.px, P.cx.a_full[p.x], P.cx.b_full[p.x]);   // Q1 (vxx): x, full profile
        cpml_adj(l4, A.lpsi[7] + S.px, P.cx.a_half[p.x], P.cx.b_half[p.x]);   // Q4 (vyx): x, half profile
    }
    if (S.sy >= 0) {
        cpml_adj(l2, A.lpsi[5] + S.py, P.cy.a_full[p.y], P.cy.b_full[p.y]);   // Q2 (vyy): y, full profile
        cpml_adj(l3, A.lpsi[6] + S.py, P.cy.a_half[p.y], P.cy.b_half[p.y]);   // Q3 (vxy): y, half profile
    }
    A.T[0][i] = l1;
    A.T[1][i] = l2;
    A.T[2][i] = l3;
    A.T[3][i] = l4;
    A.g[0][i] += (lxx + lyy) * (c1 + c2);
    A.g[1][i] += -2.0f * (lxx * c2 + lyy * c1);
    A.g[2][i] += lxy * (c3 + c4);
}

// velocity-pass transpose (and the transposed stress-pass derivatives of v)
template <int H>
__device__ __forceinline__ void adj_vel_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn)
{
    const float* X0 = A.view + (long long)vn * A.stride;
    const float* X1 = X0 + A.stride;
    const long long i = p.i, sy = P.NX;
    float lvx = A.lf[0][i];
    lvx += derivT<H, false>(A.T[0], i, 1, p.x, P.Dxb);
    lvx += derivT<H, true>(A.T[2], i, sy, p.y, P.Dyf);
    float lvy = A.lf[1][i];
    lvy += derivT<H, false>(A.T[1], i, sy, p.y, P.Dyb);
    lvy += derivT<H, true>(A.T[3], i, 1, p.x, P.Dxf);
    const Slabs S = slabs_of(P, p);
    const float *sxx = X0 + A.off[AV_SXX], *syy = X0 + A.off[AV_SYY], *sxy = X0 + A.off[AV_SXY];
    const Op1D& DybS = P.fs ? P.DybS : P.Dyb;
    const Op1D& DyfS = P.fs ? P.DyfS : P.Dyf;
    float a1 = deriv<H, true>(sxx, i, 1, p.x, P.Dxf);
    float a2 = deriv<H, false>(sxy, i, sy, p.y, DybS);
    float a3 = deriv<H, false>(sxy, i, 1, p.x, P.Dxb);
    float a4 = deriv<H, true>(syy, i, sy, p.y, DyfS);
    if (S.sx >= 0) { a1 += X1[A.off[AV_P1] + S.px]; a3 += X1[A.off[AV_P3] + S.px]; }
    if (S.sy >= 0) { a2 += X1[A.off[AV_P2] + S.py]; a4 += X1[A.off[AV_P4] + S.py]; }
    const float irx = __ldg(P.m[M_IRX] + i), iry = __ldg(P.m[M_IRY] + i);
    float l1 = irx * lvx, l2 = l1, l3 = iry * lvy, l4 = l3;
    if (S.sx >= 0) {
        cpml_adj(l1, A.lpsi[0] + S.px, P.cx.a_half[p.x], P.cx.b_half[p.x]);   // P1 (sxx_x): x, half profile
        cpml_adj(l3, A.lpsi[2] + S.px, P.cx.a_full[p.x], P.cx.b_full[p.x]);   // P3 (sxy_x): x, full profile
    }
    if (S.sy >= 0) {
        cpml_adj(l2, A.lpsi[1] + S.py, P.cy.a_full[p.y], P.cy.b_full[p.y]);   // P2 (sxy_y): y, full profile
        cpml_adj(l4, A.lpsi[3] + S.py, P.cy.a_half[p.y], P.cy.b_half[p.y]);   // P4 (syy_y): y, half profile
    }
    A.T[4][i] = l1;
    A.T[5][i] = l2;
    A.T[6][i] = l3;
    A.T[7][i] = l4;
    A.lf[0][i] = lvx;
    A.lf[1][i] = lvy;
    A.g[3][i] += lvx * (a1 + a2);
    A.g[4][i] += lvy * (a3 + a4);
}


// ---- lossless 2-D TMz --------------------------------------------------------
// parts of a TMz state in the view: AV_VX = hx, AV_VY = hy, AV_SXX = ez,
// AV_P1..AV_P4 = psi of ezy, ezx, hyx, hxy; lf[0..2] = adjoints of hx, hy, ez;
// T[0..3] = adjoints of c1, c2, a1, a2; g[0..3] = dJ/dCa, dJ/dCb, dJ/diMyz, dJ/diMxz

// E-update transpose at step n
template <int H>
__device__ __forceinline__ void adj_tm_e_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn, bool pending)
{
    const float* X0 = A.view + (long long)vn * A.stride;
    const float* X1 = X0 + A.stride;
    const long long i = p.i, sy = P.NX;
    const float* hx1 = A.vprime[0] ? A.vprime[0] : X1 + A.off[AV_VX];
    const float* hy1 = A.vprime[1] ? A.vprime[1] : X1 + A.off[AV_VY];
    const Slabs S = slabs_of(P, p);
    float c1 = deriv<H, false>(hy1, i, 1, p.x, P.Dxb);
    float c2 = deriv<H, false>(hx1, i, sy, p.y, P.Dyb);
    if (S.sx >= 0) c1 += X1[A.off[AV_P3] + S.px];
    if (S.sy >= 0) c2 += X1[A.off[AV_P4] + S.py];
    float lez = A.lf[2][i];
    if (pending) {
        // the transposed H-update derivatives of ez from the step after this one
        float u = derivT<H, true>(A.T[2], i, sy, p.y, P.Dyf);
        u += derivT<H, true>(A.T[3], i, 1, p.x, P.Dxf);
        lez += u;
    }
    if (P.abs) {
        // the taper multiplied ez, hx and hy last: their adjoints first
        const float d = absDamp(P, p);
        lez *= d;
        A.lf[0][i] *= d;
        A.lf[1][i] *= d;
    }
    const float ca = __ldg(P.m[M_CAZ] + i), cb = __ldg(P.m[M_CBZ] + i);
    float l1 = cb * lez, l2 = -l1;
    A.g[0][i] += lez * X0[A.off[AV_SXX] + i];
    A.g[1][i] += lez * (c1 - c2);
    A.lf[2][i] = ca * lez;
    if (S.sx >= 0) cpml_adj(l1, A.lpsi[2] + S.px, P.cx.a_full[p.x], P.cx.b_full[p.x]);   // hyx: x, full profile
    if (S.sy >= 0) cpml_adj(l2, A.lpsi[3] + S.py, P.cy.a_full[p.y], P.cy.b_full[p.y]);   // hxy: y, full profile
    A.T[0][i] = l1;
    A.T[1][i] = l2;
}

// H-update transpose at step n (after the E transpose of every point)
template <int H>
__device__ __forceinline__ void adj_tm_h_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn)
{
    const float* X0 = A.view + (long long)vn * A.stride;
    const float* X1 = X0 + A.stride;
    const long long i = p.i, sy = P.NX;
    const float lhy = A.lf[1][i] + derivT<H, false>(A.T[0], i, 1, p.x, P.Dxb);
    const float lhx = A.lf[0][i] + derivT<H, false>(A.T[1], i, sy, p.y, P.Dyb);
    const float* ez0 = X0 + A.off[AV_SXX];
    const Slabs S = slabs_of(P, p);
    float a1 = deriv<H, true>(ez0, i, sy, p.y, P.Dyf);
    float a2 = deriv<H, true>(ez0, i, 1, p.x, P.Dxf);
    if (S.sy >= 0) a1 += X1[A.off[AV_P1] + S.py];
    if (S.sx >= 0) a2 += X1[A.off[AV_P2] + S.px];
    const float imyz = __ldg(P.m[M_IMUYZ] + i), imxz = __ldg(P.m[M_IMUXZ] + i);
    float l1 = -imyz * lhx, l2 = imxz * lhy;
    A.g[2][i] += -lhx * a1;
    A.g[3][i] += lhy * a2;
    if (S.sy >= 0) cpml_adj(l1, A.lpsi[0] + S.py, P.cy.a_half[p.y], P.cy.b_half[p.y]);   // ezy: y, half profile
    if (S.sx >= 0) cpml_adj(l2, A.lpsi[1] + S.px, P.cx.a_half[p.x], P.cx.b_half[p.x]);   // ezx: x, half profile
    A.T[2][i] = l1;
    A.T[3][i] = l2;
    A.lf[0][i] = lhx;
    A.lf[1][i] = lhy;
}


// ---- 2-D SH ---------------------------------------------------------------
// parts of an SH state in the view: AV_VX = vz, AV_SXX = sxz, AV_SYY = syz,
// AV_P1, AV_P2 = psi of sxz_x, syz_y, AV_Q1, AV_Q2 = psi of vzx, vzy;
// lf[0], lf[2], lf[3] = adjoints of vz, sxz, syz; T[0..1] = adjoints of the
// stress-pass derivatives c1, c2, T[2..3] of the velocity-pass ones a1, a2;
// g[0..2] = dJ/dmuXZ, dJ/dmuYZ, dJ/dirho

// stress-update transpose at step n
template <int H>
__device__ __forceinline__ void adj_sh_s_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn, bool pending)
{
    const float* X1 = A.view + (long long)(vn + 1) * A.stride;
    const long long i = p.i, sy = P.NX;
    const float* vz1 = A.vprime[0] ? A.vprime[0] : X1 + A.off[AV_VX];
    const Slabs S = slabs_of(P, p);
    float c1 = deriv<H, true>(vz1, i, 1, p.x, P.Dxf);
    float c2 = deriv<H, true>(vz1, i, sy, p.y, P.Dyf);
    if (S.sx >= 0) c1 += X1[A.off[AV_Q1] + S.px];
    if (S.sy >= 0) c2 += X1[A.off[AV_Q2] + S.py];
    float lxz = A.lf[2][i], lyz = A.lf[3][i];
    if (pending) {
        // the transposed velocity-update derivatives of the stresses from the step after this one
        lxz += derivT<H, false>(A.T[2], i, 1, p.x, P.Dxb);
        lyz += derivT<H, false>(A.T[3], i, sy, p.y, P.fs ? P.DybS : P.Dyb);
    }
    if (P.abs) {
        // the taper multiplied sxz, syz and vz last: their adjoints first
        const float d = absDamp(P, p);
        lxz *= d;
        lyz *= d;
        A.lf[0][i] *= d;
    }
    A.lf[2][i] = lxz;
    A.lf[3][i] = lyz;
    float l1 = __ldg(P.m[M_MUXZ] + i) * lxz, l2 = __ldg(P.m[M_MUYZ] + i) * lyz;
    A.g[0][i] += lxz * c1;
    A.g[1][i] += lyz * c2;
    if (S.sx >= 0) cpml_adj(l1, A.lpsi[4] + S.px, P.cx.a_half[p.x], P.cx.b_half[p.x]);   // vzx: x, half profile
    if (S.sy >= 0) cpml_adj(l2, A.lpsi[5] + S.py, P.cy.a_half[p.y], P.cy.b_half[p.y]);   // vzy: y, half profile
    A.T[0][i] = l1;
    A.T[1][i] = l2;
}

// velocity-update transpose at step n (after the stress transpose of every point)
template <int H>
__device__ __forceinline__ void adj_sh_v_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn)
{
    const float* X0 = A.view + (long long)vn * A.stride;
    const float* X1 = X0 + A.stride;
    const long long i = p.i, sy = P.NX;
    float lvz = A.lf[0][i];
    lvz += derivT<H, true>(A.T[0], i, 1, p.x, P.Dxf);
    lvz += derivT<H, true>(A.T[1], i, sy, p.y, P.Dyf);
    const Slabs S = slabs_of(P, p);
    float a1 = deriv<H, false>(X0 + A.off[AV_SXX], i, 1, p.x, P.Dxb);
    float a2 = deriv<H, false>(X0 + A.off[AV_SYY], i, sy, p.y, P.fs ? P.DybS : P.Dyb);
    if (S.sx >= 0) a1 += X1[A.off[AV_P1] + S.px];
    if (S.sy >= 0) a2 += X1[A.off[AV_P2] + S.py];
    const float ir = __ldg(P.m[M_IR] + i);
    float l1 = ir * lvz, l2 = l1;
    A.g[2][i] += lvz * (a1 + a2);
    if (S.sx >= 0) cpml_adj(l1, A.lpsi[0] + S.px, P.cx.a_full[p.x], P.cx.b_full[p.x]);   // sxz_x: x, full profile
    if (S.sy >= 0) cpml_adj(l2, A.lpsi[1] + S.py, P.cy.a_full[p.y], P.cy.b_full[p.y]);   // syz_y: y, full profile
    A.T[2][i] = l1;
    A.T[3][i] = l2;
    A.lf[0][i] = lvz;
}


// ---- lossless 2-D TEz -------------------------------------------------------
// parts of a TEz state in the view: AV_VX = hz, AV_SXX = ex, AV_SYY = ey,
// AV_P1, AV_P2 = psi of eyx, exy, AV_Q1, AV_Q2 = psi of hzy, hzx; lf[0], lf[2],
// lf[3] = adjoints of hz, ex, ey; T[0..1] = adjoints of the E-update
// derivatives c1, c2, T[2..3] of the H-update ones a1, a2; g[0..4] = dJ/dCaX,
// dJ/dCbX, dJ/dCaY, dJ/dCbY, dJ/diMxy

// E-update transpose at step n
template <int H>
__device__ __forceinline__ void adj_te_e_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn, bool pending)
{
    const float* X0 = A.view + (long long)vn * A.stride;
    const float* X1 = X0 + A.stride;
    const long long i = p.i, sy = P.NX;
    const float* hz1 = A.vprime[0] ? A.vprime[0] : X1 + A.off[AV_VX];
    const Slabs S = slabs_of(P, p);
    float c1 = deriv<H, false>(hz1, i, sy, p.y, P.Dyb);
    float c2 = deriv<H, false>(hz1, i, 1, p.x, P.Dxb);
    if (S.sy >= 0) c1 += X1[A.off[AV_Q1] + S.py];
    if (S.sx >= 0) c2 += X1[A.off[AV_Q2] + S.px];
    float lex = A.lf[2][i], ley = A.lf[3][i];
    if (pending) {
        // the transposed H-update derivatives of ey and ex from the step after this one
        ley += derivT<H, true>(A.T[2], i, 1, p.x, P.Dxf);
        lex += derivT<H, true>(A.T[3], i, sy, p.y, P.Dyf);
    }
    if (P.abs) {
        // the taper multiplied ey, ex and hz last: their adjoints first
        const float d = absDamp(P, p);
        lex *= d;
        ley *= d;
        A.lf[0][i] *= d;
    }
    const float cax = __ldg(P.m[M_CAX] + i), cbx = __ldg(P.m[M_CBX] + i);
    const float cay = __ldg(P.m[M_CAY] + i), cby = __ldg(P.m[M_CBY] + i);
    A.g[0][i] += lex * X0[A.off[AV_SXX] + i];
    A.g[1][i] += lex * c1;
    A.g[2][i] += ley * X0[A.off[AV_SYY] + i];
    A.g[3][i] -= ley * c2;
    float l1 = cbx * lex, l2 = -cby * ley;
    A.lf[2][i] = cax * lex;
    A.lf[3][i] = cay * ley;
    if (S.sy >= 0) cpml_adj(l1, A.lpsi[4] + S.py, P.cy.a_full[p.y], P.cy.b_full[p.y]);   // hzy: y, full profile
    if (S.sx >= 0) cpml_adj(l2, A.lpsi[5] + S.px, P.cx.a_full[p.x], P.cx.b_full[p.x]);   // hzx: x, full profile
    A.T[0][i] = l1;
    A.T[1][i] = l2;
}

// H-update transpose at step n (after the E transpose of every point)
template <int H>
__device__ __forceinline__ void adj_te_h_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn)
{
    const float* X0 = A.view + (long long)vn * A.stride;
    const float* X1 = X0 + A.stride;
    const long long i = p.i, sy = P.NX;
    float lhz = A.lf[0][i];
    lhz += derivT<H, false>(A.T[0], i, sy, p.y, P.Dyb);
    lhz += derivT<H, false>(A.T[1], i, 1, p.x, P.Dxb);
    const Slabs S = slabs_of(P, p);
    float a1 = deriv<H, true>(X0 + A.off[AV_SYY], i, 1, p.x, P.Dxf);
    float a2 = deriv<H, true>(X0 + A.off[AV_SXX], i, sy, p.y, P.Dyf);
    if (S.sx >= 0) a1 += X1[A.off[AV_P1] + S.px];
    if (S.sy >= 0) a2 += X1[A.off[AV_P2] + S.py];
    const float im = __ldg(P.m[M_IMUXY] + i);
    float l1 = -im * lhz, l2 = im * lhz;
    A.g[4][i] -= lhz * (a1 - a2);
    if (S.sx >= 0) cpml_adj(l1, A.lpsi[0] + S.px, P.cx.a_half[p.x], P.cx.b_half[p.x]);   // eyx: x, half profile
    if (S.sy >= 0) cpml_adj(l2, A.lpsi[1] + S.py, P.cy.a_half[p.y], P.cy.b_half[p.y]);   // exy: y, half profile
    A.T[2][i] = l1;
    A.T[3][i] = l2;
    A.lf[0][i] = lhz;
}


template <int H, int PASS>
__global__ void __launch_bounds__(256) adj_pass(const StepParams* __restrict__ Ps, const AdjShot* __restrict__ As,
                                                const BatchTile* __restrict__ W, BatchSched S, int vn, int pending)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [&](const StepParams& P, const Pt& p, int shot) {
        const AdjShot& A = As[shot];
        if (PASS == 0) adj_stress_body<H>(P, A, p, vn, pending != 0);
        else if (PASS == 1) adj_vel_body<H>(P, A, p, vn);
        else if (PASS == 3) adj_tm_e_body<H>(P, A, p, vn, pending != 0);
        else if (PASS == 4) adj_tm_h_body<H>(P, A, p, vn);
        else if (PASS == 5) adj_sh_s_body<H>(P, A, p, vn, pending != 0);
        else if (PASS == 6) adj_sh_v_body<H>(P, A, p, vn);
        else if (PASS == 7) adj_te_e_body<H>(P, A, p, vn, pending != 0);
        else adj_te_h_body<H>(P, A, p, vn);
    });
}

// v' = (v_{n+1} - sources of step n) / d: the velocities the stress pass of
// step n read (before the ABS taper and the source injection)
__global__ void adj_vprime(const StepParams* __restrict__ Ps, const AdjShot* __restrict__ As, const BatchTile* __restrict__ W,
                           BatchSched S, int vn)
{
    BATCH_SHARED_PARAMS(sP);
    batch_loop(Ps, W, S, sP, [&](const StepParams& P, const Pt& p, int shot) {
        const AdjShot& A = As[shot];
        if (!A.vprime[0]) return;
        const float* X1 = A.view + (long long)(vn + 1) * A.stride;
        const float d = P.abs ? absDamp(P, p) : 1.0f;
        A.vprime[0][p.i] = X1[A.off[AV_VX] + p.i] / d;
        if (!A.sh && !A.te) A.vprime[1][p.i] = X1[A.off[AV_VY] + p.i] / d;
    });
}

__global__ void adj_vprime_sources(const StepParams* __restrict__ Ps, const AdjShot* __restrict__ As, int n)
{
    const StepParams& P = Ps[blockIdx.x];
    const AdjShot& A = As[blockIdx.x];
    if (!A.vprime[0]) return;
    for (int k = threadIdx.x; k < A.nsrc; k += blockDim.x) {
        const int t = A.stype[k];
        if (A.te ? t != WAVE_TYPE_HZ : A.sh ? t != WAVE_TYPE_VZ : (t != WAVE_TYPE_VX && t != WAVE_TYPE_VY)) continue;
        const long long i = A.sidx[k];
        Pt p;
        p.i = i;
        p.x = static_cast<int>(i % P.NX);
        p.y = static_cast<int>(i / P.NX);
        p.z = 0;
        const float d = P.abs ? absDamp(P, p) : 1.0f;
        atomicAdd(A.vprime[(A.sh || A.te || t == WAVE_TYPE_VX) ? 0 : 1] + i, -A.signals[(long long)k * A.nt + n] / d);
    }
}

// residual of step n at the receivers into the adjoint state (transposed gather;
// a pressure trace is (sxx + syy) / 2, FDTD2Delastic.cpp:12-49)
__global__ void adj_inject(const AdjShot* __restrict__ As, int n)
{
    const AdjShot& A = As[blockIdx.x];
    for (int r = threadIdx.x; r < A.nrec; r += blockDim.x) {
        const float v = A.res[(long long)r * A.nt + n];
        const long long i = A.ridx[r];
        if (A.tm) {   // Ez receivers
            atomicAdd(A.lf[2] + i, v);
            continue;
        }
        if (A.sh) {   // vz receivers
            atomicAdd(A.lf[0] + i, v);
            continue;
        }
        if (A.te) {   // Ex, Ey and Hz receivers
            const int t = A.rtype[r];
            atomicAdd(A.lf[t == WAVE_TYPE_EX ? 2 : t == WAVE_TYPE_EY ? 3 : 0] + i, v);
            continue;
        }
        switch (A.rtype[r]) {
        case WAVE_TYPE_P:
            atomicAdd(A.lf[2] + i, 0.5f * v);
            atomicAdd(A.lf[3] + i, 0.5f * v);
            break;
        case WAVE_TYPE_VX: atomicAdd(A.lf[0] + i, v); break;
        default: atomicAdd(A.lf[1] + i, v); break;
        }
    }
}

__global__ void copy_parts(const CopyPart* __restrict__ parts, long long srcIdx, long long dstIdx)
{
    const CopyPart c = parts[blockIdx.y];
    const float* s = c.src + srcIdx * c.srcStride;
    float* d = c.dst + dstIdx * c.dstStride;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < c.n; k += (long long)gridDim.x * blockDim.x) d[k] = s[k];
}

__global__ void residual_kernel(const float* __restrict__ seis, const float* __restrict__ dobs, float* res, long long n, double* misfit)
{
    double acc = 0.0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        const float r = seis[k] - dobs[k];
        res[k] = r;
        acc += 0.5 * static_cast<double>(r) * static_cast<double>(r);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(misfit, acc);
}

// weight of point (kx, ky) in the 4-point XY average row at (x, y), with the
// edge fallbacks of calc4PointAverageMatrixRow (Modelparameter.cpp:448-527)
__device__ __forceinline__ float w4(int x, int y, int kx, int ky, int NX, int NY)
{
    const bool inX = x + 1 < NX, inY = y + 1 < NY;
    const bool mx = kx == x || kx == x + 1, my = ky == y || ky == y + 1;
    if (inX && inY) return (mx && my) ? 0.25f : 0.0f;
    if (inX) return (ky == y && mx) ? 0.5f : 0.0f;
    if (inY) return (kx == x && my) ? 0.5f : 0.0f;
    return (kx == x && ky == y) ? 1.0f : 0.0f;
}

// chain rule from the prepared materials to vp, vs, rho (2-D elastic):
// M = rho vp^2; mu = max(rho vs^2, 1); mu_xy = 1 / sum_k w_k / mu_k (0 below 4);
// irx = 1 / (2-point average of rho along x), iry along y (0 where invalid)
__global__ void adj_grad_final(PrepParams G, const StepParams P, const AdjShot A, float* gvp, float* gvs, float* grho, int accumulate)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < G.N; k += (long long)gridDim.x * blockDim.x) {
        const int kx = static_cast<int>(k % G.NX), ky = static_cast<int>(k / G.NX);
        const float rho = P.m[M_RHO][k], vp = P.m[M_VP][k], vs = P.m[M_VS][k];
        const float muk = P.m[M_MU][k];
        float gmu = A.g[1][k];
        for (int dy = 0; dy <= 1; ++dy)
            for (int dx = 0; dx <= 1; ++dx) {
                const int x = kx - dx, y = ky - dy;
                if (x < 0 || y < 0) continue;
                const long long r = x + (long long)G.NX * y;
                const float mxy = P.m[M_MUXY][r];
                if (mxy == 0.0f) continue;
                const float w = w4(x, y, kx, ky, G.NX, G.NY);
                if (w != 0.0f) gmu += A.g[2][r] * w * (mxy / muk) * (mxy / muk);
            }
        const bool unclamped = rho * vs * vs >= 1.0f;
        float gr = A.g[0][k] * vp * vp;
        if (unclamped) gr += gmu * vs * vs;
        // inverse density averages: rows (kx, ky) and (kx-1, ky) along x, (kx, ky-1) along y
        for (int d = 0; d <= 1; ++d) {
            if (kx - d >= 0) {
                const long long r = k - d;
                const float ir = P.m[M_IRX][r];
                const float w = (kx - d + 1 < G.NX) ? 0.5f : 1.0f;
                if (ir != 0.0f && (d == 0 || w == 0.5f)) gr -= A.g[3][r] * ir * ir * w;
            }
            if (ky - d >= 0) {
                const long long r = k - d * (long long)G.NX;
                const float ir = P.m[M_IRY][r];
                const float w = (ky - d + 1 < G.NY) ? 0.5f : 1.0f;
                if (ir != 0.0f && (d == 0 || w == 0.5f)) gr -= A.g[4][r] * ir * ir * w;
            }
        }
        const float gp = A.g[0][k] * 2.0f * rho * vp;
        const float gs = unclamped ? gmu * 2.0f * rho * vs : 0.0f;
        if (accumulate) { gvp[k] += gp; gvs[k] += gs; grho[k] += gr; }
        else { gvp[k] = gp; gvs[k] = gs; grho[k] = gr; }
    }
}

// chain rule for TMz: Ca = (1 - k) / (1 + k), Cb = (1 / eps) / (1 + k) with
// k = sigma DT / (2 eps), eps = eps_r eps0; iMxz, iMyz = 1 / (2-point average of
// mu = mu_r mu0) along x, y (0 where invalid)
__global__ void adj_tm_final(PrepParams G, const StepParams P, const AdjShot A, float DT, float* geps, float* gsig, float* gmu,
                             int accumulate)
{
    const float eps0 = 8.8541878176e-12f, mu0 = 1.2566370614e-6f;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < G.N; k += (long long)gridDim.x * blockDim.x) {
        const int kx = static_cast<int>(k % G.NX), ky = static_cast<int>(k / G.NX);
        const float e = P.m[M_EPSR][k] * eps0, sg = P.m[M_SIG][k];
        const float kk = sg * DT / (2.0f * e), q = 1.0f + kk;
        const float gca = A.g[0][k], gcb = A.g[1][k];
        const float dca_de = 2.0f * kk / (e * q * q), dca_ds = -2.0f / (q * q) * (DT / (2.0f * e));
        const float dcb_de = (-1.0f / (e * q) + kk / (e * q * q)) / e, dcb_ds = -(1.0f / e) / (q * q) * (DT / (2.0f * e));
        const float ge = eps0 * (gca * dca_de + gcb * dcb_de);
        const float gs = gca * dca_ds + gcb * dcb_ds;
        // rows (kx, ky) and (kx-1, ky) of the x average, (kx, ky) and (kx, ky-1) of the y average
        float gm = 0.0f;
        for (int d = 0; d <= 1; ++d) {
            if (kx - d >= 0) {
                const long long r = k - d;
                const float im = P.m[M_IMUXZ][r];
                const float w = (kx - d + 1 < G.NX) ? 0.5f : 1.0f;
                if (im != 0.0f && (d == 0 || w == 0.5f)) gm -= A.g[3][r] * im * im * w;
            }
            if (ky - d >= 0) {
                const long long r = k - d * (long long)G.NX;
                const float im = P.m[M_IMUYZ][r];
                const float w = (ky - d + 1 < G.NY) ? 0.5f : 1.0f;
                if (im != 0.0f && (d == 0 || w == 0.5f)) gm -= A.g[2][r] * im * im * w;
            }
        }
        gm *= mu0;
        if (accumulate) { geps[k] += ge; gsig[k] += gs; gmu[k] += gm; }
        else { geps[k] = ge; gsig[k] = gs; gmu[k] = gm; }
    }
}

// chain rule for SH: mu = max(rho vs^2, 1); muXZ, muYZ = 1 / (2-point average
// of 1 / mu) along x, y (0 below 4); irho = 1 / rho. grad_vp is zero.
__global__ void adj_sh_final(PrepParams G, const StepParams P, const AdjShot A, float* gvp, float* gvs, float* grho, int accumulate)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < G.N; k += (long long)gridDim.x * blockDim.x) {
        const int kx = static_cast<int>(k % G.NX), ky = static_cast<int>(k / G.NX);
        const float rho = P.m[M_RHO][k], vs = P.m[M_VS][k], muk = P.m[M_MU][k];
        // rows (kx, ky) and (kx-1, ky) of the x average, (kx, ky) and (kx, ky-1) of the y average
        float gmu = 0.0f;
        for (int d = 0; d <= 1; ++d) {
            if (kx - d >= 0) {
                const long long r = k - d;
                const float m = P.m[M_MUXZ][r];
                const float w = (kx - d + 1 < G.NX) ? 0.5f : 1.0f;
                if (m != 0.0f && (d == 0 || w == 0.5f)) gmu += A.g[0][r] * w * (m / muk) * (m / muk);
            }
            if (ky - d >= 0) {
                const long long r = k - d * (long long)G.NX;
                const float m = P.m[M_MUYZ][r];
                const float w = (ky - d + 1 < G.NY) ? 0.5f : 1.0f;
                if (m != 0.0f && (d == 0 || w == 0.5f)) gmu += A.g[1][r] * w * (m / muk) * (m / muk);
            }
        }
        float raw = rho;
        raw *= vs;
        raw *= vs;
        const bool unclamped = raw >= 1.0f;
        const float ir = P.m[M_IR][k];
        const float gs = unclamped ? gmu * 2.0f * rho * vs : 0.0f;
        const float gr = (unclamped ? gmu * vs * vs : 0.0f) - A.g[2][k] * ir * ir;
        if (accumulate) { gvs[k] += gs; grho[k] += gr; }
        else { gvp[k] = 0.0f; gvs[k] = gs; grho[k] = gr; }
    }
}

// d Ca / d eps, d Ca / d sigma, d Cb / d eps, d Cb / d sigma of
// Ca = (1 - k) / (1 + k), Cb = (1 / eps) / (1 + k), k = sigma DT / (2 eps),
// applied to the adjoints of Ca and Cb
__device__ __forceinline__ void cacb_adj(float e, float sg, float DT, float gca, float gcb, float& ge, float& gs)
{
    const float kk = sg * DT / (2.0f * e), q = 1.0f + kk;
    const float dca_de = 2.0f * kk / (e * q * q), dca_ds = -2.0f / (q * q) * (DT / (2.0f * e));
    const float dcb_de = (-1.0f / (e * q) + kk / (e * q * q)) / e, dcb_ds = -(1.0f / e) / (q * q) * (DT / (2.0f * e));
    ge = gca * dca_de + gcb * dcb_de;
    gs = gca * dca_ds + gcb * dcb_ds;
}

// chain rule for TEz: CaX, CbX of the 2-point x averages of eps = eps_r eps0
// and sigma (CaY, CbY along y); iMxy = 1 / (4-point average of mu = mu_r mu0)
// (0 where invalid)
__global__ void adj_te_final(PrepParams G, const StepParams P, const AdjShot A, float DT, float* geps, float* gsig, float* gmu,
                             int accumulate)
{
    const float eps0 = 8.8541878176e-12f, mu0 = 1.2566370614e-6f;
    const float* er = P.m[M_EPSR];
    const float* sg = P.m[M_SIG];
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < G.N; k += (long long)gridDim.x * blockDim.x) {
        const int kx = static_cast<int>(k % G.NX), ky = static_cast<int>(k / G.NX);
        float ge = 0.0f, gs = 0.0f;
        // rows (kx, ky) and (kx-1, ky) of the x averages, (kx, ky) and (kx, ky-1) of the y averages
        for (int d = 0; d <= 1; ++d) {
            if (kx - d >= 0) {
                const long long r = k - d;
                const bool pair = kx - d + 1 < G.NX;
                if (d == 0 || pair) {
                    const float w = pair ? 0.5f : 1.0f;
                    const float e = pair ? 0.5f * (er[r] * eps0) + 0.5f * (er[r + 1] * eps0) : er[r] * eps0;
                    const float s = pair ? 0.5f * sg[r] + 0.5f * sg[r + 1] : sg[r];
                    float a, b;
                    cacb_adj(e, s, DT, A.g[0][r], A.g[1][r], a, b);
                    ge += w * a;
                    gs += w * b;
                }
            }
            if (ky - d >= 0) {
                const long long r = k - d * (long long)G.NX;
                const bool pair = ky - d + 1 < G.NY;
                if (d == 0 || pair) {
                    const float w = pair ? 0.5f : 1.0f;
                    const float e = pair ? 0.5f * (er[r] * eps0) + 0.5f * (er[r + G.NX] * eps0) : er[r] * eps0;
                    const float s = pair ? 0.5f * sg[r] + 0.5f * sg[r + G.NX] : sg[r];
                    float a, b;
                    cacb_adj(e, s, DT, A.g[2][r], A.g[3][r], a, b);
                    ge += w * a;
                    gs += w * b;
                }
            }
        }
        float gm = 0.0f;
        for (int dy = 0; dy <= 1; ++dy)
            for (int dx = 0; dx <= 1; ++dx) {
                const int x = kx - dx, y = ky - dy;
                if (x < 0 || y < 0) continue;
                const long long r = x + (long long)G.NX * y;
                const float im = P.m[M_IMUXY][r];
                if (im == 0.0f) continue;
                const float w = w4(x, y, kx, ky, G.NX, G.NY);
                if (w != 0.0f) gm -= A.g[4][r] * im * im * w;
            }
        ge *= eps0;
        gm *= mu0;
        if (accumulate) { geps[k] += ge; gsig[k] += gs; gmu[k] += gm; }
        else { geps[k] = ge; gsig[k] = gs; gmu[k] = gm; }
    }
}

template <int H>
void launch_adj_h(int pass, const StepParams* Ps, const AdjShot* As, const BatchTile* W, const BatchSched& S, int grid, int vn,
                  int pending, cudaStream_t s)
{
    const dim3 block(32, 8, 1);
    switch (pass) {
    case 0: adj_pass<H, 0><<<grid, block, 0, s>>>(Ps, As, W, S, vn, pending); break;
    case 1: adj_pass<H, 1><<<grid, block, 0, s>>>(Ps, As, W, S, vn, pending); break;
    case 3: adj_pass<H, 3><<<grid, block, 0, s>>>(Ps, As, W, S, vn, pending); break;
    case 4: adj_pass<H, 4><<<grid, block, 0, s>>>(Ps, As, W, S, vn, pending); break;
    case 5: adj_pass<H, 5><<<grid, block, 0, s>>>(Ps, As, W, S, vn, pending); break;
    case 6: adj_pass<H, 6><<<grid, block, 0, s>>>(Ps, As, W, S, vn, pending); break;
    case 7: adj_pass<H, 7><<<grid, block, 0, s>>>(Ps, As, W, S, vn, pending); break;
    default: adj_pass<H, 8><<<grid, block, 0, s>>>(Ps, As, W, S, vn, pending); break;
    }
}

void launch_adj(int H, int pass, const StepParams* Ps, const AdjShot* As, const BatchTile* W, const BatchSched& S, int grid, int vn,
                int pending, cudaStream_t s)
{
    switch (H) {
    case 1: launch_adj_h<1>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    case 2: launch_adj_h<2>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    case 3: launch_adj_h<3>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    case 4: launch_adj_h<4>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    case 5: launch_adj_h<5>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    default: launch_adj_h<6>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    }
}

void ck(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// device allocations of one adjoint run, freed on scope exit
struct DevPool {
    std::vector<void*> ptrs;
    cudaStream_t s = nullptr;
    template <class T>
    T* get(size_t n)
    {
        void* p = nullptr;
        ck(cudaMallocAsync(&p, (n > 0 ? n : 1) * sizeof(T), s), "cudaMallocAsync");
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    ~DevPool()
    {
        for (void* p : ptrs) cudaFreeAsync(p, s);
        if (s) cudaStreamSynchronize(s);
    }
};

} // namespace

// Checks that a handle can run the adjoint; returns an error message or "".
std::string adjoint_supported(const wave_handle* h)
{
    const wave_config& c = h->cfg;
    if (c.dimension != 2 ||
        (c.equation != WAVE_EQ_ELASTIC && c.equation != WAVE_EQ_TMEM && c.equation != WAVE_EQ_SH && c.equation != WAVE_EQ_EMEM))
        return "the adjoint gradient is implemented for 2-D elastic, 2-D SH and lossless 2-D TMz and TEz modelling";
    if (c.equation == WAVE_EQ_TMEM) {
        for (int t : h->hRecType)
            if (t != WAVE_TYPE_EZ) return "the TMz adjoint takes Ez receivers only";
        for (int t : h->hSrcType)
            if (t != WAVE_TYPE_EZ) return "the TMz adjoint takes Ez sources only";
    }
    if (h->vg) return "the adjoint gradient is implemented on regular grids";
    if (!h->modelSet) return "set the model first";
    if (!h->seis || h->nrec < 1) return "set receivers first";
    return "";
}

// Runs forward + checkpoints, residuals, and the backward sweep for the shots.
// dobs[s] and the gradient outputs are device pointers; with `sum` the
// gradients of all shots are added into output 0.
void adjoint_run(const std::vector<wave_handle*>& shots, const AdjStepper& S, const float* const* dobs, int K, double* misfit,
                 float* const* gvp, float* const* gvs, float* const* grho, bool sum)
{
    const int ns = static_cast<int>(shots.size());
    const int NT = shots[0]->NT;
    const int H = shots[0]->H;
    cudaStream_t st = S.stream;
    DevPool pool;
    pool.s = st;
    std::vector<AdjShot> A(ns);
    std::vector<StepParams> Ps(ns);
    std::vector<CopyPart> toView, toCkpt, fromCkpt;
    std::vector<BatchTile> tiles;
    std::vector<float*> ckpt(ns);
    std::vector<long long> stride(ns);
    const int nck = (NT + K - 1) / K;
    double* dMisfit = pool.get<double>(ns);
    ck(cudaMemsetAsync(dMisfit, 0, ns * sizeof(double), st), "memset");
    for (int s = 0; s < ns; ++s) {
        wave_handle* h = shots[s];
        const long long N = h->N;
        // state layout: 5 field parts then 8 psi parts (absent parts: length 0);
        // TMz: hx, hy, ez and the psi of ezy, ezx, hyx, hxy
        // SH: vz, -, sxz, syz and the psi of sxz_x, syz_y, -, -, vzx, vzy
        const bool tm = h->cfg.equation == WAVE_EQ_TMEM;
        const bool sh = h->cfg.equation == WAVE_EQ_SH;
        long long off[AV_COUNT], len[AV_COUNT], o = 0;
        const int elasticFields[5] = {F_VX, F_VY, F_SXX, F_SYY, F_SXY};
        const int tmFields[5] = {F_HX, F_HY, F_EZ, -1, -1};
        const int tmPsi[8] = {PS_EZY, PS_EZX, PS_HYX, PS_HXY, -1, -1, -1, -1};
        // TEz: hz, -, ex, ey and the psi of eyx, exy, -, -, hzy, hzx
        const bool te = h->cfg.equation == WAVE_EQ_EMEM;
        const int shFields[5] = {F_VZ, -1, F_SXZ, F_SYZ, -1};
        const int shPsi[8] = {PS_SXZ_X, PS_SYZ_Y, -1, -1, PS_VZX, PS_VZY, -1, -1};
        const int teFields[5] = {F_HZ, -1, F_EX, F_EY, -1};
        const int tePsi[8] = {PS_EYX, PS_EXY, -1, -1, PS_HZY, PS_HZX, -1, -1};
        const int* fields = tm ? tmFields : sh ? shFields : te ? teFields : elasticFields;
        const int* psiSlot = tm ? tmPsi : sh ? shPsi : te ? tePsi : kAdjPsiSlot;
        for (int k = 0; k < 5; ++k) { off[k] = o; len[k] = fields[k] >= 0 ? N : 0; o += len[k]; }
        for (int k = 0; k < 8; ++k) {
            const int slot = psiSlot[k];
            off[5 + k] = o;
            len[5 + k] = (slot >= 0 && h->psi[slot]) ? h->psiLen[slot] : 0;
            o += len[5 + k];
        }
        stride[s] = o;
        AdjShot& a = A[s];
        a.tm = tm ? 1 : 0;
        a.sh = sh ? 1 : 0;
        a.te = te ? 1 : 0;
        a.view = pool.get<float>(static_cast<size_t>(o) * (K + 1));
        a.stride = o;
        for (int k = 0; k < AV_COUNT; ++k) a.off[k] = off[k];
        float* lstate = pool.get<float>(o);
        ck(cudaMemsetAsync(lstate, 0, o * sizeof(float), st), "memset");
        for (int k = 0; k < 5; ++k) a.lf[k] = lstate + off[k];
        for (int k = 0; k < 8; ++k) a.lpsi[k] = lstate + off[5 + k];
        float* temps = pool.get<float>(8 * N);
        for (int k = 0; k < 8; ++k) a.T[k] = temps + k * N;
        float* grads = pool.get<float>(5 * N);
        ck(cudaMemsetAsync(grads, 0, 5 * N * sizeof(float), st), "memset");
        for (int k = 0; k < 5; ++k) a.g[k] = grads + k * N;
        a.ridx = h->ridx;
        a.rtype = h->rtype;
        a.nrec = h->nrec;
        a.nt = NT;
        float* res = pool.get<float>(static_cast<size_t>(h->nrec) * NT);
        a.res = res;
        bool velocitySources = false;
        for (int t : h->hSrcType)
            velocitySources |= te ? t == WAVE_TYPE_HZ : sh ? t == WAVE_TYPE_VZ : (t == WAVE_TYPE_VX || t == WAVE_TYPE_VY);
        a.vprime[0] = a.vprime[1] = nullptr;
        if (h->cfg.DampingBoundary == 1 || velocitySources) {
            a.vprime[0] = pool.get<float>(2 * N);
            a.vprime[1] = a.vprime[0] + N;
        }
        a.sidx = h->sidx;
        a.stype = h->stype;
        a.signals = h->signals;
        a.nsrc = h->nsrc;
        ckpt[s] = pool.get<float>(static_cast<size_t>(o) * nck);
        for (int k = 0; k < AV_COUNT; ++k) {
            if (len[k] == 0) continue;
            float* live = k < 5 ? h->f[fields[k]] : h->psi[psiSlot[k - 5]];
            toView.push_back({live, a.view + off[k], len[k], 0, o});
            toCkpt.push_back({live, ckpt[s] + off[k], len[k], 0, o});
            fromCkpt.push_back({ckpt[s] + off[k], live, len[k], o, 0});
        }
        Ps[s] = h->sp;
        const int rows = h->NY * h->NZ;
        for (int r0 = 0; r0 < rows; r0 += S.rows)
            for (int x0 = 0; x0 < h->NX; x0 += S.cols) tiles.push_back({s, x0, r0, 0});
    }
    auto upload = [&](auto& v) {
        using T = typename std::decay_t<decltype(v)>::value_type;
        T* d = pool.get<T>(v.size());
        ck(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st), "upload");
        return d;
    };
    const StepParams* dP = upload(Ps);
    const AdjShot* dA = upload(A);
    const BatchTile* dT = upload(tiles);
    const CopyPart* dToView = upload(toView);
    const CopyPart* dToCkpt = upload(toCkpt);
    const CopyPart* dFromCkpt = upload(fromCkpt);
    const int ntiles = static_cast<int>(tiles.size());
    const BatchSched sched{ntiles, S.cols, S.rows, 0};
    const int grid = S.blocks > 0 ? std::min(ntiles, S.blocks) : ntiles;
    bool anyVprime = false;
    for (const AdjShot& a : A) anyVprime |= a.vprime[0] != nullptr;
    const dim3 cgrid(64, 1, 1);
    auto copy = [&](const CopyPart* parts, size_t nparts, long long si, long long di) {
        copy_parts<<<dim3(cgrid.x, static_cast<unsigned>(nparts), 1), 256, 0, st>>>(parts, si, di);
    };
    // the shots' own streams may still hold work: order them before this run
    for (auto* h : shots) ck(cudaStreamSynchronize(h->stream), "shot sync");

    // 1. forward with checkpoints (state zeroed first)
    for (auto* h : shots) {
        for (int f : h->fields) ck(cudaMemsetAsync(h->f[f], 0, h->N * sizeof(float), st), "memset");
        for (int k = 0; k < PS_COUNT; ++k)
            if (h->psi[k]) ck(cudaMemsetAsync(h->psi[k], 0, h->psiLen[k] * sizeof(float), st), "memset");
        ck(cudaMemsetAsync(h->seis, 0, static_cast<size_t>(h->nrec) * NT * sizeof(float), st), "memset");
    }
    S.set_counter(0);
    for (int n = 0; n < NT; ++n) {
        if (n % K == 0) copy(dToCkpt, toCkpt.size(), 0, n / K);
        S.step();
    }
    // 2. residuals and misfits
    for (int s = 0; s < ns; ++s) {
        const long long n = static_cast<long long>(shots[s]->nrec) * NT;
        residual_kernel<<<256, 256, 0, st>>>(shots[s]->seis, dobs[s], const_cast<float*>(A[s].res), n, dMisfit + s);
    }
    // 3. backward sweep over the checkpoint segments
    for (int seg = nck - 1; seg >= 0; --seg) {
        const int n0 = seg * K, n1 = n0 + K < NT ? n0 + K : NT;
        copy(dFromCkpt, fromCkpt.size(), seg, 0);
        copy(dToView, toView.size(), 0, 0);
        S.set_counter(n0);
        for (int n = n0; n < n1; ++n) {
            S.step();
            copy(dToView, toView.size(), 0, n - n0 + 1);
        }
        for (int n = n1 - 1; n >= n0; --n) {
            if (anyVprime) {
                adj_vprime<<<grid, dim3(32, 8, 1), 0, st>>>(dP, dA, dT, sched, n - n0);
                adj_vprime_sources<<<ns, 128, 0, st>>>(dP, dA, n);
            }
            adj_inject<<<ns, 256, 0, st>>>(dA, n);
            // two kernels per step: the third stage of step n (the transposed
            // derivatives of the first-pass inputs) runs inside the first kernel
            // of step n - 1; after step 0 it is not needed
            const int first = A[0].tm ? 3 : A[0].sh ? 5 : A[0].te ? 7 : 0;
            const int pending = n < NT - 1 ? 1 : 0;
            launch_adj(H, first, dP, dA, dT, sched, grid, n - n0, pending, st);
            launch_adj(H, first + 1, dP, dA, dT, sched, grid, n - n0, pending, st);
        }
        ck(cudaGetLastError(), "adjoint launch");
    }
    // 4. chain rule to vp, vs, rho
    for (int s = 0; s < ns; ++s) {
        wave_handle* h = shots[s];
        PrepParams G{h->NX, h->NY, h->NZ, h->N};
        const int o = sum ? 0 : s;
        if (A[s].tm)
            adj_tm_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], static_cast<float>(h->cfg.DT), gvp[o], gvs[o], grho[o],
                                               sum && s > 0 ? 1 : 0);
        else if (A[s].sh)
            adj_sh_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], gvp[o], gvs[o], grho[o], sum && s > 0 ? 1 : 0);
        else if (A[s].te)
            adj_te_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], static_cast<float>(h->cfg.DT), gvp[o], gvs[o], grho[o],
                                               sum && s > 0 ? 1 : 0);
        else
            adj_grad_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], gvp[o], gvs[o], grho[o], sum && s > 0 ? 1 : 0);
    }
    ck(cudaGetLastError(), "gradient launch");
    ck(cudaMemcpyAsync(misfit, dMisfit, ns * sizeof(double), cudaMemcpyDeviceToHost, st), "misfit copy");
    ck(cudaStreamSynchronize(st), "adjoint");
    for (auto* h : shots) h->stepsSinceReset = NT;
}

} // namespace wave

using namespace wave;

extern "C" int wave_adjoint_gradient(wave_handle* h, const float* dobs, int dobs_mem, int checkpoint_every, double* misfit,
                                     float* grad_vp, float* grad_vs, float* grad_rho, int grad_mem)
{
    if (!h) return WAVE_ERR_ARG;
    if (!dobs || !misfit || !grad_vp || !grad_vs || !grad_rho || checkpoint_every < 1) {
        h->err = "wave_adjoint_gradient: invalid argument";
        return WAVE_ERR_ARG;
    }
    const std::string why = adjoint_supported(h);
    if (!why.empty()) {
        h->err = "wave_adjoint_gradient: " + why;
        return WAVE_ERR_UNSUPPORTED;
    }
    try {
        const size_t nd = static_cast<size_t>(h->nrec) * h->NT;
        const size_t N = static_cast<size_t>(h->N);
        std::vector<void*> tmp;
        auto dev = [&](size_t n) {
            void* p = nullptr;
            ck(cudaMalloc(&p, n * sizeof(float)), "cudaMalloc");
            tmp.push_back(p);
            return static_cast<float*>(p);
        };
        struct Free {
            std::vector<void*>& v;
            ~Free() { for (void* p : v) cudaFree(p); }
        } freeTmp{tmp};
        const float* dDobs = dobs;
        if (dobs_mem != WAVE_MEM_DEVICE) {
            float* d = dev(nd);
            ck(cudaMemcpy(d, dobs, nd * sizeof(float), cudaMemcpyHostToDevice), "dobs upload");
            dDobs = d;
        }
        float* out[3] = {grad_vp, grad_vs, grad_rho};
        float* dOut[3];
        for (int k = 0; k < 3; ++k) dOut[k] = grad_mem == WAVE_MEM_DEVICE ? out[k] : dev(N);
        AdjStepper S;
        S.stream = h->stream;
        S.set_counter = [h](int n) { launch_set_counter(h->tcounter, n, h->stream); };
        S.step = [h]() { step_once(h); };
        adjoint_run({h}, S, &dDobs, checkpoint_every, misfit, &dOut[0], &dOut[1], &dOut[2], false);
        if (grad_mem != WAVE_MEM_DEVICE)
            for (int k = 0; k < 3; ++k) ck(cudaMemcpy(out[k], dOut[k], N * sizeof(float), cudaMemcpyDeviceToHost), "gradient copy");
    } catch (std::exception& e) {
        h->err = std::string("wave_adjoint_gradient: ") + e.what();
        return WAVE_ERR_CUDA;
    }
    return WAVE_OK;
}
