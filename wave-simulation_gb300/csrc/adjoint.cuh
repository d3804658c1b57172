// adjoint.cuh — the adjoint's saved-state layout, per-shot descriptor and
// per-point transposed step bodies, shared by the host driver (adjoint.cu)
// and the translation units that instantiate the per-pass kernels
// (adjoint_pass2d.cu, adjoint_pass3d.cu).
#pragma once

#include "handle.h"
#include "stencil.cuh"

namespace wave {

// parts of one saved state, in view order (2-D: five field parts, then eight
// psi parts; absent parts have length 0)
enum AdjPart { AV_VX, AV_VY, AV_SXX, AV_SYY, AV_SXY, AV_P1, AV_P2, AV_P3, AV_P4, AV_Q1, AV_Q2, AV_Q3, AV_Q4, AV_COUNT };
// 3-D elastic: nine field parts, the nine velocity-pass psi (P0..P8) and the
// nine stress-pass psi (Q0..Q8)
enum Adj3Part {
    E3_VX, E3_VY, E3_VZ, E3_SXX, E3_SYY, E3_SZZ, E3_SXY, E3_SXZ, E3_SYZ,
    E3_P0, E3_Q0 = E3_P0 + 9, E3_COUNT = E3_Q0 + 9
};
constexpr int kAdjMaxParts = E3_COUNT + 6 * kMaxL;   // 3-D visco-elastic: six memory variables per mechanism

// psi slot of each psi part: velocity pass P1..P4, stress pass Q1..Q4
static const int kAdjPsiSlot[8] = {PS_SXX_X, PS_SXY_Y, PS_SXY_X, PS_SYY_Y, PS_VXX, PS_VYY, PS_VXY, PS_VYX};

struct AdjShot {
    float* view;                 // recompute buffer: K+1 states
    long long stride;            // floats per state
    long long off[kAdjMaxParts]; // part offsets within a state (0 = absent psi)
    float* lf[9];                // adjoint fields (2-D elastic: vx, vy, sxx, syy, sxy)
    float* lpsi[18];             // adjoint psi (slab layout of the forward psi)
    float* T[18];                // adjoints of the raw derivatives (2-D elastic: c1..c4, a1..a4)
    float* g[9 + 3 * kMaxL];     // material adjoints (2-D elastic: dJ/dM, dJ/dmu, dJ/dmu_xy, dJ/dirx, dJ/diry)
    const long long* ridx;
    const int* rtype;
    const float* res;            // residual d - d_obs, nrec x nt
    int nrec, nt;
    int tm;                      // 1: lossless 2-D TMz (parts: hx, hy, ez; psi ezy, ezx, hyx, hxy)
    int sh;                      // 1: 2-D SH (parts: vz, sxz, syz; psi sxz_x, syz_y, vzx, vzy)
    int te;                      // 1: lossless 2-D TEz (parts: hz, ex, ey; psi eyx, exy, hzy, hzx)
    int e3;                      // 1: 3-D elastic (Adj3Part layout)
    int visco;                   // 1: visco-elastic (the elastic parts, then the memory variables per mechanism)
    int ac;                      // 1: acoustic, 2-D or 3-D (parts: p, vx, vy, vz; psi p_x, p_y, p_z, vxx, vyy, vzz)
    int em3;                     // 1: lossless 3-D EM (parts: hx, hy, hz, ex, ey, ez; psi of the six E and six H derivatives)
    float* lr[6 * kMaxL];        // adjoint memory variables of mechanism l at [k * kMaxL + l]: 2-D rxx, ryy, rxy;
                                 // 3-D rxx, ryy, rzz, rxy, rxz, ryz
    float* vprime[3];            // vx', vy' [, vz'] (TMz: hx', hy') of the current step (null: the saved state's are they)
    const long long* sidx;       // sources (velocity sources are taken out of v')
    const int* stype;
    const float* signals;        // nsrc x nt
    int nsrc;
};

// launches one adjoint pass over the (shot, tile) work list: 2-D passes 0, 1
// (elastic and visco-elastic), 3, 4 (TMz), 5, 6 (SH), 7, 8 (TEz); 3-D passes
// 9, 10 (elastic and visco-elastic); acoustic passes 11, 12; 3-D EM passes 13, 14
void launch_adj_pass2d(int H, int pass, const StepParams* Ps, const AdjShot* As, const BatchTile* W, const BatchSched& S, int grid,
                       int vn, int pending, cudaStream_t s);
void launch_adj_pass3d(int H, int pass, const StepParams* Ps, const AdjShot* As, const BatchTile* W, const BatchSched& S, int grid,
                       int vn, int pending, cudaStream_t s);
// acoustic passes 11, 12 (2-D and 3-D)
void launch_adj_pass_acoustic(int H, int pass, const StepParams* Ps, const AdjShot* As, const BatchTile* W, const BatchSched& S,
                              int grid, int vn, int pending, cudaStream_t s);
// lossless 3-D EM passes 13, 14
void launch_adj_pass_em3d(int H, int pass, const StepParams* Ps, const AdjShot* As, const BatchTile* W, const BatchSched& S, int grid,
                          int vn, int pending, cudaStream_t s);

namespace adj {


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
    int sx, sy, sz;
    long long px, py, pz;
};

__device__ __forceinline__ Slabs slabs_of(const StepParams& P, const Pt& p)
{
    Slabs S;
    S.sx = P.useCpml ? slab(p.x, P.cx) : -1;
    S.sy = P.useCpml ? slab(p.y, P.cy) : -1;
    S.sz = (P.useCpml && P.is3d) ? slab(p.z, P.cz) : -1;
    S.px = S.sx >= 0 ? pix(P, p, S.sx) : 0;
    S.py = S.sy >= 0 ? piy(P, p, S.sy) : 0;
    S.pz = S.sz >= 0 ? piz(P, p, S.sz) : 0;
    return S;
}

// transpose of the visco free-surface exchange at a surface point
// (FreeSurface2Dviscoelastic.cpp / FreeSurface3Dviscoelastic.cpp) for one
// horizontal normal stress: S' += sH h - sV v + DT/2 sum_l dR_l, R_l' += dR_l =
// rh_l h - rv_l v, with h the horizontal strain sum, v = vyy, sV = M opP -
// 2 mu opS, sH = -sV^2 / (M opP), rv_l = t3 c2_l / tau_l, rh_l = t3 ratio c2_l /
// tau_l, t3 = 2 mu tauS - M tauP, ratio = 2 mu opS / (M opP) - 1. lS is the
// adjoint of S's final value, LR[l] that of R_l after the regular update
// (its final adjoint plus DT/2 lS); adds to the adjoints of h and v and to
// dJ/dM, dJ/dmu
__device__ __forceinline__ void visco_fs_transpose(const StepParams& P, float M, float mu, float tP, float tS, float opP, float opS,
                                                   float lS, const float* LR, float h, float v, float& lh, float& lv, float& gM,
                                                   float& gMu)
{
    const float mp = M * opP, sV = mp - 2.0f * mu * opS, sH = -sV * sV / mp;
    const float t3 = 2.0f * mu * tS - M * tP, ratio = 2.0f * mu * opS / mp - 1.0f;
    float lhh = sH * lS, lvv = -sV * lS, grh = 0.0f, grv = 0.0f;
    for (int l = 0; l < P.L; ++l) {
        const float kk = P.c2[l] / P.relaxTime[l];
        lhh += t3 * ratio * kk * LR[l];
        lvv -= t3 * kk * LR[l];
        grh += LR[l] * h * kk;
        grv -= LR[l] * v * kk;
    }
    lh += lhh;
    lv += lvv;
    const float gsH = lS * h, gsV = -lS * v;
    const float dsH_dsV = -2.0f * sV / mp, dsH_dM = sV * sV / (mp * mp) * opP;
    gM += gsV * opP + gsH * (dsH_dsV * opP + dsH_dM);
    gMu += gsV * (-2.0f * opS) + gsH * dsH_dsV * (-2.0f * opS);
    const float dr_dM = -2.0f * mu * opS / (M * mp), dr_dmu = 2.0f * opS / mp;
    gM += grv * (-tP) + grh * (-tP * ratio + t3 * dr_dM);
    gMu += grv * (2.0f * tS) + grh * (2.0f * tS * ratio + t3 * dr_dmu);
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
    if (A.visco) {
        // per mechanism l, with e = c1' + c2', q = c2' (sxx) or c1' (syy), m = mu_xy (c3' + c4'):
        //   Rk' = c2_l (c1_l Rk - tauP M e / tau_l + tauS 2 mu q / tau_l)
        //   Sk' = Sk + DT/2 sum_l (Rk + Rk') + (1 + L tauP) M e - (1 + L tauS) 2 mu q
        //   Rxy' = c2_l (c1_l Rxy - tauSxy m / tau_l),  Sxy' = Sxy + DT/2 sum_l (Rxy + Rxy') + (1 + L tauS) m
        // (ForwardSolver2Dviscoelastic.cpp:218-316); the memory variables are not tapered
        const float e = c1 + c2, DTh = P.DThalf;
        const float tP = __ldg(P.m[M_TAUP] + i), tS = __ldg(P.m[M_TAUS] + i);
        const float opP = __ldg(P.m[M_OPLTP] + i), opS = __ldg(P.m[M_OPLTS] + i), tSxy = __ldg(P.m[M_TAUSXY] + i);
        float le = 0.0f, lq[2] = {0.0f, 0.0f}, gM = 0.0f, gMu = 0.0f;
        float LRx[kMaxL];
        if (fsRow)   // syy and ryy are zeroed on the surface row: their adjoints do not flow back
            for (int l = 0; l < P.L; ++l) A.lr[kMaxL + l][i] = 0.0f;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const float lS = k == 0 ? lxx : lyy, q = k == 0 ? c2 : c1;
            le += opP * M * lS;
            lq[k] -= opS * 2.0f * mu * lS;
            gM += opP * e * lS;
            gMu -= opS * 2.0f * q * lS;
            for (int l = 0; l < P.L; ++l) {
                const float cc = P.c2[l] * P.invRelax[l];
                float* r = A.lr[k * kMaxL + l] + i;
                const float LR = *r + DTh * lS;   // adjoint of Rk'
                if (k == 0) LRx[l] = LR;
                *r = P.c2[l] * P.c1[l] * LR + DTh * lS;
                le -= cc * tP * M * LR;
                lq[k] += cc * tS * 2.0f * mu * LR;
                gM -= cc * tP * e * LR;
                gMu += cc * tS * 2.0f * q * LR;
            }
        }
        l1 = le + lq[1];
        l2 = le + lq[0];
        if (fsRow) visco_fs_transpose(P, M, mu, tP, tS, opP, opS, lxx, LRx, c1, c2, l1, l2, gM, gMu);
        float lm = opS * lxy;
        for (int l = 0; l < P.L; ++l) {
            float* r = A.lr[2 * kMaxL + l] + i;
            const float LR = *r + DTh * lxy;
            *r = P.c2[l] * P.c1[l] * LR + DTh * lxy;
            lm -= P.c2[l] * P.invRelax[l] * tSxy * LR;
        }
        l3 = l4 = mxy * lm;
        A.g[0][i] += gM;
        A.g[1][i] += gMu;
        A.g[2][i] += lm * (c3 + c4);
    }
    if (fsRow && !A.visco) {
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
    if (!A.visco) {
        A.g[0][i] += (lxx + lyy) * (c1 + c2);
        A.g[1][i] += -2.0f * (lxx * c2 + lyy * c1);
        A.g[2][i] += lxy * (c3 + c4);
    }
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
    const float ez0 = X0[A.off[AV_SXX] + i];
    float l1 = cb * lez, l2 = -l1;
    float u = c1 - c2, ln = ca * lez;
    if (A.visco) {
        // visco-TMz (ForwardSolver2Dviscotmem.cpp:175-200): rz_l' = Cc_l rz_l + Cd_l ez and
        // ez' = Ca ez + Cb (c1' - c2' - DT sum_l rz_l'); rz_l' is state part 13 + l of X_{n+1}
        for (int l = 0; l < P.L; ++l) {
            u -= P.DT * X1[A.off[13 + l] + i];
            float* r = A.lr[l] + i;
            const float LR = *r - P.DT * cb * lez;   // adjoint of rz_l'
            ln += __ldg(P.m[M_CDZ0 + l] + i) * LR;
            A.g[4 + l][i] += LR * ez0;
            *r = P.Cc[l] * LR;
        }
    }
    A.g[0][i] += lez * ez0;
    A.g[1][i] += lez * u;
    A.lf[2][i] = ln;
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
    float lm[2] = {lxz, lyz};
    if (A.visco) {
        // visco-SH, per mechanism l with m = mu_k c': Rk' = c2_l (c1_l Rk - tauS_k m / tau_l),
        // Sk' = Sk + DT/2 sum_l (Rk + Rk') + (1 + L tauS) m (ForwardSolver2Dviscosh.cpp:180-240)
        const float opS = __ldg(P.m[M_OPLTS] + i);
        const float tS[2] = {__ldg(P.m[M_TAUSXZ] + i), __ldg(P.m[M_TAUSYZ] + i)};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const float lS = lm[q];
            lm[q] = opS * lS;
            for (int m = 0; m < P.L; ++m) {
                float* r = A.lr[q * kMaxL + m] + i;
                const float LR = *r + P.DThalf * lS;
                *r = P.c2[m] * P.c1[m] * LR + P.DThalf * lS;
                lm[q] -= P.c2[m] * P.invRelax[m] * tS[q] * LR;
            }
        }
    }
    float l1 = __ldg(P.m[M_MUXZ] + i) * lm[0], l2 = __ldg(P.m[M_MUYZ] + i) * lm[1];
    A.g[0][i] += lm[0] * c1;
    A.g[1][i] += lm[1] * c2;
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
    const float ex0 = X0[A.off[AV_SXX] + i], ey0 = X0[A.off[AV_SYY] + i];
    float ux = c1, uy = -c2, lnx = cax * lex, lny = cay * ley;
    if (A.visco) {
        // visco-TEz (ForwardSolver2Dviscoemem.cpp:176-220): r_l' = Cc_l r_l + Cd_l e per component, and
        // ex' = CaX ex + CbX (c1' - DT sum_l rx_l'), ey' = CaY ey + CbY (-c2' - DT sum_l ry_l');
        // rx_l', ry_l' are state parts 13 + l, 13 + L + l of X_{n+1}; dJ/dCd in g[5 + l], g[5 + L + l]
        for (int l = 0; l < P.L; ++l) {
            ux -= P.DT * X1[A.off[13 + l] + i];
            uy -= P.DT * X1[A.off[13 + P.L + l] + i];
            float* rx = A.lr[l] + i;
            float* ry = A.lr[kMaxL + l] + i;
            const float LX = *rx - P.DT * cbx * lex, LY = *ry - P.DT * cby * ley;   // adjoints of rx_l', ry_l'
            lnx += __ldg(P.m[M_CDX0 + l] + i) * LX;
            lny += __ldg(P.m[M_CDY0 + l] + i) * LY;
            A.g[5 + l][i] += LX * ex0;
            A.g[5 + P.L + l][i] += LY * ey0;
            *rx = P.Cc[l] * LX;
            *ry = P.Cc[l] * LY;
        }
    }
    A.g[0][i] += lex * ex0;
    A.g[1][i] += lex * ux;
    A.g[2][i] += ley * ey0;
    A.g[3][i] += ley * uy;
    float l1 = cbx * lex, l2 = -cby * ley;
    A.lf[2][i] = lnx;
    A.lf[3][i] = lny;
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


// ---- 3-D elastic -------------------------------------------------------------
// lf[0..8] = adjoints of vx, vy, vz, sxx, syy, szz, sxy, sxz, syz; lpsi[0..8]
// of the velocity-pass psi P0..P8 (sxx_x, sxy_y, sxz_z, sxy_x, syy_y, syz_z,
// sxz_x, syz_y, szz_z), lpsi[9..17] of the stress-pass psi Q0..Q8 (vxx, vyy,
// vzz, vxy, vyx, vxz, vzx, vyz, vzy); T[0..8] = adjoints of the stress-pass
// derivatives c0..c8, T[9..17] of the velocity-pass ones a0..a8; g[0..7] =
// dJ/dM, dJ/dmu, dJ/dmuXY, dJ/dmuXZ, dJ/dmuYZ, dJ/dirx, dJ/diry, dJ/dirz

// psi of the x, y or z slab at this point (0 outside the slabs or when absent)
__device__ __forceinline__ float psi_at(const float* X, const AdjShot& A, int part, const Slabs& S, int axis)
{
    if (axis == 0) return S.sx >= 0 ? X[A.off[part] + S.px] : 0.0f;
    if (axis == 1) return S.sy >= 0 ? X[A.off[part] + S.py] : 0.0f;
    return S.sz >= 0 ? X[A.off[part] + S.pz] : 0.0f;
}

__device__ __forceinline__ void cpml_adj_axis(const StepParams& P, const Pt& p, const Slabs& S, float& l, float* lpsi, int axis,
                                              bool half)
{
    if (axis == 0) {
        if (S.sx >= 0) cpml_adj(l, lpsi + S.px, half ? P.cx.a_half[p.x] : P.cx.a_full[p.x], half ? P.cx.b_half[p.x] : P.cx.b_full[p.x]);
    } else if (axis == 1) {
        if (S.sy >= 0) cpml_adj(l, lpsi + S.py, half ? P.cy.a_half[p.y] : P.cy.a_full[p.y], half ? P.cy.b_half[p.y] : P.cy.b_full[p.y]);
    } else {
        if (S.sz >= 0) cpml_adj(l, lpsi + S.pz, half ? P.cz.a_half[p.z] : P.cz.a_full[p.z], half ? P.cz.b_half[p.z] : P.cz.b_full[p.z]);
    }
}

// axis and half-grid profile of each velocity-pass derivative a0..a8 and the
// axis of each stress-pass derivative c0..c8 (forward derivatives on the half grid)
__host__ __device__ constexpr int e3_a_axis(int k) { return k % 3; }
__host__ __device__ constexpr bool e3_a_half(int k) { return k == 0 || k == 4 || k == 8; }
__host__ __device__ constexpr int e3_c_axis(int k) { return k == 0 || k == 4 || k == 6 ? 0 : k == 1 || k == 3 || k == 8 ? 1 : 2; }

// stress-update transpose at step n
template <int H>
__device__ __forceinline__ void adj_e3_s_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn, bool pending)
{
    const float* X1 = A.view + (long long)(vn + 1) * A.stride;
    const long long i = p.i, sy = (long long)P.NX * P.NZ, sz = P.NX;
    const float* vx1 = A.vprime[0] ? A.vprime[0] : X1 + A.off[E3_VX];
    const float* vy1 = A.vprime[0] ? A.vprime[1] : X1 + A.off[E3_VY];
    const float* vz1 = A.vprime[0] ? A.vprime[2] : X1 + A.off[E3_VZ];
    const Slabs S = slabs_of(P, p);
    float c[9];
    c[0] = deriv<H, false>(vx1, i, 1, p.x, P.Dxb);
    c[1] = deriv<H, false>(vy1, i, sy, p.y, P.Dyb);
    c[2] = deriv<H, false>(vz1, i, sz, p.z, P.Dzb);
    c[3] = deriv<H, true>(vx1, i, sy, p.y, P.Dyf);
    c[4] = deriv<H, true>(vy1, i, 1, p.x, P.Dxf);
    c[5] = deriv<H, true>(vx1, i, sz, p.z, P.Dzf);
    c[6] = deriv<H, true>(vz1, i, 1, p.x, P.Dxf);
    c[7] = deriv<H, true>(vy1, i, sz, p.z, P.Dzf);
    c[8] = deriv<H, true>(vz1, i, sy, p.y, P.Dyf);
#pragma unroll
    for (int k = 0; k < 9; ++k) c[k] += psi_at(X1, A, E3_Q0 + k, S, e3_c_axis(k));
    float lxx = A.lf[3][i], lyy = A.lf[4][i], lzz = A.lf[5][i], lxy = A.lf[6][i], lxz = A.lf[7][i], lyz = A.lf[8][i];
    if (pending) {
        // the transposed velocity-pass derivatives of the stresses from the step after this one
        const Op1D& DybS = P.fs ? P.DybS : P.Dyb;
        const Op1D& DyfS = P.fs ? P.DyfS : P.Dyf;
        lxx += derivT<H, true>(A.T[9], i, 1, p.x, P.Dxf);
        lxy += derivT<H, false>(A.T[10], i, sy, p.y, DybS);
        lxz += derivT<H, false>(A.T[11], i, sz, p.z, P.Dzb);
        lxy += derivT<H, false>(A.T[12], i, 1, p.x, P.Dxb);
        lyy += derivT<H, true>(A.T[13], i, sy, p.y, DyfS);
        lyz += derivT<H, false>(A.T[14], i, sz, p.z, P.Dzb);
        lxz += derivT<H, false>(A.T[15], i, 1, p.x, P.Dxb);
        lyz += derivT<H, false>(A.T[16], i, sy, p.y, DybS);
        lzz += derivT<H, true>(A.T[17], i, sz, p.z, P.Dzf);
    }
    if (P.abs) {
        // the taper multiplied all nine fields last: their adjoints first
        const float d = absDamp(P, p);
        lxx *= d; lyy *= d; lzz *= d; lxy *= d; lxz *= d; lyz *= d;
        A.lf[0][i] *= d;
        A.lf[1][i] *= d;
        A.lf[2][i] *= d;
    }
    const bool fsRow = P.fs && p.y == 0;
    if (fsRow) lyy = 0.0f;   // syy' = 0 on the surface
    A.lf[3][i] = lxx;
    A.lf[4][i] = lyy;
    A.lf[5][i] = lzz;
    A.lf[6][i] = lxy;
    A.lf[7][i] = lxz;
    A.lf[8][i] = lyz;
    const float M = __ldg(P.m[M_M] + i), mu = __ldg(P.m[M_MU] + i);
    const float ls = lxx + lyy + lzz;
    const float muP[3] = {__ldg(P.m[M_MUXY] + i), __ldg(P.m[M_MUXZ] + i), __ldg(P.m[M_MUYZ] + i)};
    float l[9];
    if (A.visco) {
        // per mechanism l, with e = c0' + c1' + c2', q the normal stress's partner sum and m = mu_plane (its
        // cross derivatives): Rk' = c2_l (c1_l Rk - tauP M e / tau_l + tauS 2 mu q / tau_l),
        // Sk' = Sk + DT/2 sum_l (Rk + Rk') + (1 + L tauP) M e - (1 + L tauS) 2 mu q;
        // Rs' = c2_l (c1_l Rs - tauS_plane m / tau_l), Ss' = Ss + DT/2 sum_l (Rs + Rs') + (1 + L tauS) m
        // (ForwardSolver3Dviscoelastic.cpp:283-452); the memory variables are not tapered
        const float e = c[0] + c[1] + c[2], DTh = P.DThalf;
        const float tP = __ldg(P.m[M_TAUP] + i), tS = __ldg(P.m[M_TAUS] + i);
        const float opP = __ldg(P.m[M_OPLTP] + i), opS = __ldg(P.m[M_OPLTS] + i);
        const float q[3] = {c[1] + c[2], c[0] + c[2], c[0] + c[1]};
        const float lS3[3] = {lxx, lyy, lzz};
        float le = 0.0f, lq[3] = {0.0f, 0.0f, 0.0f}, gM = 0.0f, gMu = 0.0f;
        float LRh[2][kMaxL];   // sxx's and szz's memory adjoints, for the free-surface exchange
        if (fsRow)   // syy and ryy are zeroed on the surface row: their adjoints do not flow back
            for (int m = 0; m < P.L; ++m) A.lr[kMaxL + m][i] = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float lS = lS3[k];
            le += opP * M * lS;
            lq[k] -= opS * 2.0f * mu * lS;
            gM += opP * e * lS;
            gMu -= opS * 2.0f * q[k] * lS;
            for (int m = 0; m < P.L; ++m) {
                const float cc = P.c2[m] * P.invRelax[m];
                float* r = A.lr[k * kMaxL + m] + i;
                const float LR = *r + DTh * lS;   // adjoint of Rk'
                if (k != 1) LRh[k / 2][m] = LR;
                *r = P.c2[m] * P.c1[m] * LR + DTh * lS;
                le -= cc * tP * M * LR;
                lq[k] += cc * tS * 2.0f * mu * LR;
                gM -= cc * tP * e * LR;
                gMu += cc * tS * 2.0f * q[k] * LR;
            }
        }
        l[0] = le + lq[1] + lq[2];
        l[1] = le + lq[0] + lq[2];
        l[2] = le + lq[0] + lq[1];
        if (fsRow) {
            // sxx and szz exchange with the horizontal sum c0' + c2' and vyy = c1'
            float lh = 0.0f, lv = 0.0f;
            visco_fs_transpose(P, M, mu, tP, tS, opP, opS, lxx, LRh[0], c[0] + c[2], c[1], lh, lv, gM, gMu);
            visco_fs_transpose(P, M, mu, tP, tS, opP, opS, lzz, LRh[1], c[0] + c[2], c[1], lh, lv, gM, gMu);
            l[0] += lh;
            l[2] += lh;
            l[1] += lv;
        }
        const float lSh[3] = {lxy, lxz, lyz};
        const float tPl[3] = {__ldg(P.m[M_TAUSXY] + i), __ldg(P.m[M_TAUSXZ] + i), __ldg(P.m[M_TAUSYZ] + i)};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float lS = lSh[k];
            float lm = opS * lS;
            for (int m = 0; m < P.L; ++m) {
                float* r = A.lr[(3 + k) * kMaxL + m] + i;
                const float LR = *r + DTh * lS;
                *r = P.c2[m] * P.c1[m] * LR + DTh * lS;
                lm -= P.c2[m] * P.invRelax[m] * tPl[k] * LR;
            }
            A.g[2 + k][i] += lm * (c[3 + 2 * k] + c[4 + 2 * k]);
            l[3 + 2 * k] = l[4 + 2 * k] = muP[k] * lm;
        }
        A.g[0][i] += gM;
        A.g[1][i] += gMu;
    } else {
        l[0] = M * ls - 2.0f * mu * (lyy + lzz);
        l[1] = M * ls - 2.0f * mu * (lxx + lzz);
        l[2] = M * ls - 2.0f * mu * (lxx + lyy);
        l[3] = l[4] = muP[0] * lxy;
        l[5] = l[6] = muP[1] * lxz;
        l[7] = l[8] = muP[2] * lyz;
        A.g[0][i] += ls * (c[0] + c[1] + c[2]);
        A.g[1][i] += -2.0f * (lxx * (c[1] + c[2]) + lyy * (c[0] + c[2]) + lzz * (c[0] + c[1]));
        A.g[2][i] += lxy * (c[3] + c[4]);
        A.g[3][i] += lxz * (c[5] + c[6]);
        A.g[4][i] += lyz * (c[7] + c[8]);
    }
    if (fsRow && !A.visco) {
        // sxx', szz' += sh (c0' + c2') - sv c1' with sv = M - 2 mu, sh = -sv^2 / M
        const float sv = M - 2.0f * mu, sh = -(sv * sv) / M, hs = lxx + lzz;
        l[0] += sh * hs;
        l[2] += sh * hs;
        l[1] -= sv * hs;
        const float gh = hs * (c[0] + c[2]), gv = -hs * c[1];
        A.g[0][i] += gv - gh * (2.0f * sv / M - (sv * sv) / (M * M));
        A.g[1][i] += -2.0f * gv + gh * 4.0f * sv / M;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        // stress-pass psi: backward derivatives (c0..c2) on the full grid, the cross ones on the half grid
        cpml_adj_axis(P, p, S, l[k], A.lpsi[9 + k], e3_c_axis(k), k >= 3);
        A.T[k][i] = l[k];
    }
}

// velocity-update transpose at step n (after the stress transpose of every point)
template <int H>
__device__ __forceinline__ void adj_e3_v_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn)
{
    const float* X0 = A.view + (long long)vn * A.stride;
    const float* X1 = X0 + A.stride;
    const long long i = p.i, sy = (long long)P.NX * P.NZ, sz = P.NX;
    float lvx = A.lf[0][i], lvy = A.lf[1][i], lvz = A.lf[2][i];
    lvx += derivT<H, false>(A.T[0], i, 1, p.x, P.Dxb);
    lvx += derivT<H, true>(A.T[3], i, sy, p.y, P.Dyf);
    lvx += derivT<H, true>(A.T[5], i, sz, p.z, P.Dzf);
    lvy += derivT<H, false>(A.T[1], i, sy, p.y, P.Dyb);
    lvy += derivT<H, true>(A.T[4], i, 1, p.x, P.Dxf);
    lvy += derivT<H, true>(A.T[7], i, sz, p.z, P.Dzf);
    lvz += derivT<H, false>(A.T[2], i, sz, p.z, P.Dzb);
    lvz += derivT<H, true>(A.T[6], i, 1, p.x, P.Dxf);
    lvz += derivT<H, true>(A.T[8], i, sy, p.y, P.Dyf);
    const Slabs S = slabs_of(P, p);
    const Op1D& DybS = P.fs ? P.DybS : P.Dyb;
    const Op1D& DyfS = P.fs ? P.DyfS : P.Dyf;
    const float *sxx = X0 + A.off[E3_SXX], *syy = X0 + A.off[E3_SYY], *szz = X0 + A.off[E3_SZZ];
    const float *sxy = X0 + A.off[E3_SXY], *sxz = X0 + A.off[E3_SXZ], *syz = X0 + A.off[E3_SYZ];
    float a[9];
    a[0] = deriv<H, true>(sxx, i, 1, p.x, P.Dxf);
    a[1] = deriv<H, false>(sxy, i, sy, p.y, DybS);
    a[2] = deriv<H, false>(sxz, i, sz, p.z, P.Dzb);
    a[3] = deriv<H, false>(sxy, i, 1, p.x, P.Dxb);
    a[4] = deriv<H, true>(syy, i, sy, p.y, DyfS);
    a[5] = deriv<H, false>(syz, i, sz, p.z, P.Dzb);
    a[6] = deriv<H, false>(sxz, i, 1, p.x, P.Dxb);
    a[7] = deriv<H, false>(syz, i, sy, p.y, DybS);
    a[8] = deriv<H, true>(szz, i, sz, p.z, P.Dzf);
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] += psi_at(X1, A, E3_P0 + k, S, e3_a_axis(k));
    const float irx = __ldg(P.m[M_IRX] + i), iry = __ldg(P.m[M_IRY] + i), irz = __ldg(P.m[M_IRZ] + i);
    A.g[5][i] += lvx * (a[0] + a[1] + a[2]);
    A.g[6][i] += lvy * (a[3] + a[4] + a[5]);
    A.g[7][i] += lvz * (a[6] + a[7] + a[8]);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        float l = (k < 3 ? irx * lvx : k < 6 ? iry * lvy : irz * lvz);
        cpml_adj_axis(P, p, S, l, A.lpsi[k], e3_a_axis(k), e3_a_half(k));
        A.T[9 + k][i] = l;
    }
    A.lf[0][i] = lvx;
    A.lf[1][i] = lvy;
    A.lf[2][i] = lvz;
}


// ---- acoustic (2-D and 3-D) ----------------------------------------------------
// lf[0..3] = adjoints of p, vx, vy, vz; lpsi[0..2] of the velocity-pass psi
// p_x, p_y, p_z, lpsi[3..5] of the pressure-pass psi vxx, vyy, vzz; T[0..2] =
// adjoints of the pressure-pass derivatives c0..c2, T[3..5] of the
// velocity-pass ones a0..a2; g[0..3] = dJ/dM, dJ/dirx, dJ/diry, dJ/dirz

// pressure-update transpose at step n
template <int H>
__device__ __forceinline__ void adj_ac_p_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn, bool pending)
{
    const float* X1 = A.view + (long long)(vn + 1) * A.stride;
    const long long i = p.i, sy = (long long)P.NX * P.NZ, sz = P.NX;
    const float* v1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) v1[k] = A.vprime[0] ? A.vprime[k] : X1 + A.off[1 + k];
    const Slabs S = slabs_of(P, p);
    float c0 = deriv<H, false>(v1[0], i, 1, p.x, P.Dxb) + psi_at(X1, A, 7, S, 0);
    float c1 = deriv<H, false>(v1[1], i, sy, p.y, P.Dyb) + psi_at(X1, A, 8, S, 1);
    float c2 = P.is3d ? deriv<H, false>(v1[2], i, sz, p.z, P.Dzb) + psi_at(X1, A, 9, S, 2) : 0.0f;
    float lp = A.lf[0][i];
    if (pending) {
        // the transposed velocity-update derivatives of p from the step after this one
        lp += derivT<H, true>(A.T[3], i, 1, p.x, P.Dxf);
        lp += derivT<H, true>(A.T[4], i, sy, p.y, P.fs ? P.DyfS : P.Dyf);
        if (P.is3d) lp += derivT<H, true>(A.T[5], i, sz, p.z, P.Dzf);
    }
    if (P.fs && p.y == 0) lp = 0.0f;   // p = 0 on the surface, after the taper
    if (P.abs) {
        const float d = absDamp(P, p);
        lp *= d;
        A.lf[1][i] *= d;
        A.lf[2][i] *= d;
        if (P.is3d) A.lf[3][i] *= d;
    }
    A.lf[0][i] = lp;
    A.g[0][i] += lp * (c0 + c1 + c2);
    const float l = __ldg(P.m[M_M] + i) * lp;
    float l0 = l, l1 = l, l2 = l;
    cpml_adj_axis(P, p, S, l0, A.lpsi[3], 0, false);   // vxx: x, full profile
    cpml_adj_axis(P, p, S, l1, A.lpsi[4], 1, false);   // vyy: y, full profile
    if (P.is3d) cpml_adj_axis(P, p, S, l2, A.lpsi[5], 2, false);   // vzz: z, full profile
    A.T[0][i] = l0;
    A.T[1][i] = l1;
    if (P.is3d) A.T[2][i] = l2;
}

// velocity-update transpose at step n (after the pressure transpose of every point)
template <int H>
__device__ __forceinline__ void adj_ac_v_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn)
{
    const float* X0 = A.view + (long long)vn * A.stride;
    const float* X1 = X0 + A.stride;
    const long long i = p.i, sy = (long long)P.NX * P.NZ, sz = P.NX;
    const float* p0 = X0 + A.off[0];
    const Slabs S = slabs_of(P, p);
    const int nd = P.is3d ? 3 : 2;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (k >= nd) break;
        float lv = A.lf[1 + k][i];
        float a;
        if (k == 0) {
            lv += derivT<H, false>(A.T[0], i, 1, p.x, P.Dxb);
            a = deriv<H, true>(p0, i, 1, p.x, P.Dxf);
        } else if (k == 1) {
            lv += derivT<H, false>(A.T[1], i, sy, p.y, P.Dyb);
            a = deriv<H, true>(p0, i, sy, p.y, P.fs ? P.DyfS : P.Dyf);
        } else {
            lv += derivT<H, false>(A.T[2], i, sz, p.z, P.Dzb);
            a = deriv<H, true>(p0, i, sz, p.z, P.Dzf);
        }
        a += psi_at(X1, A, 4 + k, S, k);
        const float ir = __ldg(P.m[M_IRX + k] + i);
        A.g[1 + k][i] += lv * a;
        float l = ir * lv;
        cpml_adj_axis(P, p, S, l, A.lpsi[k], k, true);   // p_x, p_y, p_z: half profile
        A.T[3 + k][i] = l;
        A.lf[1 + k][i] = lv;
    }
}


// ---- lossless 3-D EM ----------------------------------------------------------
// parts: 0..5 = hx, hy, hz, ex, ey, ez; 6..11 = psi of the H-update derivatives
// a0..a5 (ezy, eyz, exz, ezx, eyx, exy), 12..17 = psi of the E-update ones c0..c5
// (hzy, hyz, hxz, hzx, hyx, hxy); lf[0..5] the field adjoints, lpsi[0..11] the
// psi adjoints in part order; T[0..5] = adjoints of c0..c5, T[6..11] of a0..a5;
// g[0..5] = dJ/dCaX, dJ/dCbX, dJ/dCaY, dJ/dCbY, dJ/dCaZ, dJ/dCbZ, g[6..8] =
// dJ/diMyz, dJ/diMxz, dJ/diMxy

// E-update transpose at step n:  ex' = CaX ex + CbX (c0' - c1'), ey' = CaY ey + CbY (c2' - c3'),
// ez' = CaZ ez + CbZ (c4' - c5') with c0 = Dyb hz, c1 = Dzb hy, c2 = Dzb hx, c3 = Dxb hz, c4 = Dxb hy, c5 = Dyb hx
template <int H>
__device__ __forceinline__ void adj_em3_e_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn, bool pending)
{
    const float* X0 = A.view + (long long)vn * A.stride;
    const float* X1 = X0 + A.stride;
    const long long i = p.i, sy = (long long)P.NX * P.NZ, sz = P.NX;
    const float* h1[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) h1[k] = A.vprime[0] ? A.vprime[k] : X1 + A.off[k];
    const Slabs S = slabs_of(P, p);
    float c[6];
    c[0] = deriv<H, false>(h1[2], i, sy, p.y, P.Dyb) + psi_at(X1, A, 12, S, 1);
    c[1] = deriv<H, false>(h1[1], i, sz, p.z, P.Dzb) + psi_at(X1, A, 13, S, 2);
    c[2] = deriv<H, false>(h1[0], i, sz, p.z, P.Dzb) + psi_at(X1, A, 14, S, 2);
    c[3] = deriv<H, false>(h1[2], i, 1, p.x, P.Dxb) + psi_at(X1, A, 15, S, 0);
    c[4] = deriv<H, false>(h1[1], i, 1, p.x, P.Dxb) + psi_at(X1, A, 16, S, 0);
    c[5] = deriv<H, false>(h1[0], i, sy, p.y, P.Dyb) + psi_at(X1, A, 17, S, 1);
    float le[3] = {A.lf[3][i], A.lf[4][i], A.lf[5][i]};
    if (pending) {
        // the transposed H-update derivatives of the E fields from the step after this one
        le[2] += derivT<H, true>(A.T[6], i, sy, p.y, P.Dyf) + derivT<H, true>(A.T[9], i, 1, p.x, P.Dxf);
        le[1] += derivT<H, true>(A.T[7], i, sz, p.z, P.Dzf) + derivT<H, true>(A.T[10], i, 1, p.x, P.Dxf);
        le[0] += derivT<H, true>(A.T[8], i, sz, p.z, P.Dzf) + derivT<H, true>(A.T[11], i, sy, p.y, P.Dyf);
    }
    if (P.abs) {
        // the taper multiplied all six fields last: their adjoints first
        const float d = absDamp(P, p);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            le[q] *= d;
            A.lf[q][i] *= d;
        }
    }
    float l[6];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float ca = __ldg(P.m[M_CAX + 2 * q] + i), cb = __ldg(P.m[M_CBX + 2 * q] + i);
        const float e0 = X0[A.off[3 + q] + i];
        float u = c[2 * q] - c[2 * q + 1], ln = ca * le[q];
        if (A.visco) {
            // 3-D visco-EM (ForwardSolver3Dviscoemem.cpp:215-300): r_l' = Cc_l r_l + Cd_l e and
            // e' = Ca e + Cb (c' - c'' - DT sum_l r_l'); r_l' of component q is state part 18 + q L + l,
            // dJ/dCd in g[9 + q L + l]
            for (int m = 0; m < P.L; ++m) {
                u -= P.DT * X1[A.off[18 + q * P.L + m] + i];
                float* r = A.lr[q * kMaxL + m] + i;
                const float LR = *r - P.DT * cb * le[q];
                ln += __ldg(P.m[M_CDX0 + q * kMaxL + m] + i) * LR;
                A.g[9 + q * P.L + m][i] += LR * e0;
                *r = P.Cc[m] * LR;
            }
        }
        A.g[2 * q][i] += le[q] * e0;
        A.g[2 * q + 1][i] += le[q] * u;
        l[2 * q] = cb * le[q];
        l[2 * q + 1] = -cb * le[q];
        A.lf[3 + q][i] = ln;
    }
    // H-derivative psi: full profiles except hyx (CPMLEM3D.cpp:67-70)
    cpml_adj_axis(P, p, S, l[0], A.lpsi[6], 1, false);    // hzy
    cpml_adj_axis(P, p, S, l[1], A.lpsi[7], 2, false);    // hyz
    cpml_adj_axis(P, p, S, l[2], A.lpsi[8], 2, false);    // hxz
    cpml_adj_axis(P, p, S, l[3], A.lpsi[9], 0, false);    // hzx
    cpml_adj_axis(P, p, S, l[4], A.lpsi[10], 0, true);    // hyx
    cpml_adj_axis(P, p, S, l[5], A.lpsi[11], 1, false);   // hxy
#pragma unroll
    for (int k = 0; k < 6; ++k) A.T[k][i] = l[k];
}

// H-update transpose at step n (after the E transpose of every point):
// hx' = hx - iMyz (a0' - a1'), hy' = hy - iMxz (a2' - a3'), hz' = hz - iMxy (a4' - a5')
// with a0 = Dyf ez, a1 = Dzf ey, a2 = Dzf ex, a3 = Dxf ez, a4 = Dxf ey, a5 = Dyf ex
template <int H>
__device__ __forceinline__ void adj_em3_h_body(const StepParams& P, const AdjShot& A, const Pt& p, int vn)
{
    const float* X0 = A.view + (long long)vn * A.stride;
    const float* X1 = X0 + A.stride;
    const long long i = p.i, sy = (long long)P.NX * P.NZ, sz = P.NX;
    float lh[3];
    lh[0] = A.lf[0][i] + derivT<H, false>(A.T[2], i, sz, p.z, P.Dzb) + derivT<H, false>(A.T[5], i, sy, p.y, P.Dyb);
    lh[1] = A.lf[1][i] + derivT<H, false>(A.T[1], i, sz, p.z, P.Dzb) + derivT<H, false>(A.T[4], i, 1, p.x, P.Dxb);
    lh[2] = A.lf[2][i] + derivT<H, false>(A.T[0], i, sy, p.y, P.Dyb) + derivT<H, false>(A.T[3], i, 1, p.x, P.Dxb);
    const Slabs S = slabs_of(P, p);
    const float *ex0 = X0 + A.off[3], *ey0 = X0 + A.off[4], *ez0 = X0 + A.off[5];
    float a[6];
    a[0] = deriv<H, true>(ez0, i, sy, p.y, P.Dyf) + psi_at(X1, A, 6, S, 1);
    a[1] = deriv<H, true>(ey0, i, sz, p.z, P.Dzf) + psi_at(X1, A, 7, S, 2);
    a[2] = deriv<H, true>(ex0, i, sz, p.z, P.Dzf) + psi_at(X1, A, 8, S, 2);
    a[3] = deriv<H, true>(ez0, i, 1, p.x, P.Dxf) + psi_at(X1, A, 9, S, 0);
    a[4] = deriv<H, true>(ey0, i, 1, p.x, P.Dxf) + psi_at(X1, A, 10, S, 0);
    a[5] = deriv<H, true>(ex0, i, sy, p.y, P.Dyf) + psi_at(X1, A, 11, S, 1);
    const int slot[3] = {M_IMUYZ, M_IMUXZ, M_IMUXY};
    const int axis[6] = {1, 2, 2, 0, 0, 1};
    float l[6];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const float im = __ldg(P.m[slot[q]] + i);
        A.g[6 + q][i] -= lh[q] * (a[2 * q] - a[2 * q + 1]);
        l[2 * q] = -im * lh[q];
        l[2 * q + 1] = im * lh[q];
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        cpml_adj_axis(P, p, S, l[k], A.lpsi[k], axis[k], true);   // E-derivative psi: half profiles
        A.T[6 + k][i] = l[k];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) A.lf[q][i] = lh[q];
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
        else if (PASS == 8) adj_te_h_body<H>(P, A, p, vn);
        else if (PASS == 9) adj_e3_s_body<H>(P, A, p, vn, pending != 0);
        else if (PASS == 10) adj_e3_v_body<H>(P, A, p, vn);
        else if (PASS == 11) adj_ac_p_body<H>(P, A, p, vn, pending != 0);
        else if (PASS == 12) adj_ac_v_body<H>(P, A, p, vn);
        else if (PASS == 13) adj_em3_e_body<H>(P, A, p, vn, pending != 0);
        else adj_em3_h_body<H>(P, A, p, vn);
    });
}

} // namespace adj
} // namespace wave
