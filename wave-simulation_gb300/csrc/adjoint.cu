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
// The 3-D elastic step (FD3Delastic::run, ForwardSolver3Delastic.cpp:120-414)
// has the same three stages over nine fields and eighteen psi arrays:
//   vx' = vx + irx (Dxf sxx + DybS sxy + Dzb sxz)',  vy', vz' likewise,
//   normal stresses from c0' = Dxb vx', c1' = Dyb vy', c2' = Dzb vz' with M, 2 mu;
//   sxy, sxz, syz from the forward cross derivatives with muXY, muXZ, muYZ;
// then at y = 0 with the free surface syy' = 0 and sxx', szz' += sh (c0' + c2')
// - sv c1' (FreeSurface3Delastic.cpp:15-47), then the ABS taper on all nine
// fields; the last kernel maps dJ/dM, dJ/dmu, dJ/dmuXY, dJ/dmuXZ, dJ/dmuYZ and
// dJ/dirx, dJ/diry, dJ/dirz to vp, vs and rho through the harmonic 4-point
// averages in the xy, xz and yz planes and the 2-point inverse density
// averages (Modelparameter.cpp:336-639).
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

#include "adjoint.cuh"
#include "trace.h"

namespace wave {

struct CopyPart {
    const float* src;
    float* dst;
    long long n;
    long long srcStride, dstStride;   // per state index
};
namespace {

using namespace adj;

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
        if (A.e3) {
            for (int k = 0; k < 3; ++k) A.vprime[k][p.i] = X1[A.off[E3_VX + k] + p.i] / d;
            return;
        }
        if (A.ac) {
            for (int k = 0; k < (P.is3d ? 3 : 2); ++k) A.vprime[k][p.i] = X1[A.off[1 + k] + p.i] / d;
            return;
        }
        if (A.em3) {
            for (int k = 0; k < 3; ++k) A.vprime[k][p.i] = X1[A.off[k] + p.i] / d;
            return;
        }
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
        if (A.em3 ? t != WAVE_TYPE_HZ : (A.e3 || A.ac) ? (t != WAVE_TYPE_VX && t != WAVE_TYPE_VY && t != WAVE_TYPE_VZ)
                 : A.te ? t != WAVE_TYPE_HZ : A.sh ? t != WAVE_TYPE_VZ : (t != WAVE_TYPE_VX && t != WAVE_TYPE_VY))
            continue;
        const long long i = A.sidx[k];
        Pt p;
        p.i = i;
        p.x = static_cast<int>(i % P.NX);
        const long long r = i / P.NX;   // z + NZ y
        p.y = static_cast<int>(r / P.NZ);
        p.z = static_cast<int>(r - (long long)p.y * P.NZ);
        const float d = P.abs ? absDamp(P, p) : 1.0f;
        const int v = A.em3 ? 2 : (A.e3 || A.ac) ? t - WAVE_TYPE_VX : (A.sh || A.te || t == WAVE_TYPE_VX) ? 0 : 1;
        atomicAdd(A.vprime[v] + i, -A.signals[(long long)k * A.nt + n] / d);
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
        if (A.em3) {   // Ez, Ex, Ey, Hz receivers
            const int t = A.rtype[r];
            atomicAdd(A.lf[t == WAVE_TYPE_EZ ? 5 : t == WAVE_TYPE_EX ? 3 : t == WAVE_TYPE_EY ? 4 : 2] + i, v);
            continue;
        }
        if (A.ac) {   // p, vx, vy, vz receivers
            const int t = A.rtype[r];
            atomicAdd(A.lf[t == WAVE_TYPE_P ? 0 : 1 + t - WAVE_TYPE_VX] + i, v);
            continue;
        }
        if (A.e3) {   // a pressure trace is (sxx + syy + szz) / 3 (FDTD3Delastic)
            const int t = A.rtype[r];
            if (t == WAVE_TYPE_P) {
                for (int k = 3; k < 6; ++k) atomicAdd(A.lf[k] + i, v / 3.0f);
            } else {
                atomicAdd(A.lf[t - WAVE_TYPE_VX] + i, v);
            }
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
__global__ void adj_grad_final(PrepParams G, const StepParams P, const AdjShot A, float vsum, float* gvp, float* gvs, float* grho,
                               int accumulate)
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
        // visco: M = rho vp^2 / fP, mu = max(rho vs^2 / fS, 1) with f = 1 + sum tau (the relaxation times held fixed)
        const float fP = A.visco ? 1.0f + vsum * P.m[M_TAUP][k] : 1.0f, fS = A.visco ? 1.0f + vsum * P.m[M_TAUS][k] : 1.0f;
        float raw = rho;
        raw *= vs;
        raw *= vs;
        if (A.visco) raw = raw / fS;
        const bool unclamped = raw >= 1.0f;
        float gr = A.g[0][k] * vp * vp / fP;
        if (unclamped) gr += gmu * vs * vs / fS;
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
        const float gp = A.g[0][k] * 2.0f * rho * vp / fP;
        const float gs = unclamped ? gmu * 2.0f * rho * vs / fS : 0.0f;
        if (accumulate) { gvp[k] += gp; gvs[k] += gs; grho[k] += gr; }
        else { gvp[k] = gp; gvs[k] = gs; grho[k] = gr; }
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

// chain rule for TMz: Ca = (1 - k) / (1 + k), Cb = (1 / eps) / (1 + k) with
// k = sigma DT / (2 eps), eps = eps_r eps0; iMxz, iMyz = 1 / (2-point average of
// mu = mu_r mu0) along x, y (0 where invalid)
__global__ void adj_tm_final(PrepParams G, const StepParams P, const AdjShot A, float DT, ViscoEmCoef vc, float* geps, float* gsig,
                             float* gmu, int accumulate)
{
    const float eps0 = 8.8541878176e-12f, mu0 = 1.2566370614e-6f;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < G.N; k += (long long)gridDim.x * blockDim.x) {
        const int kx = static_cast<int>(k % G.NX), ky = static_cast<int>(k / G.NX);
        const float e0 = P.m[M_EPSR][k] * eps0, sg0 = P.m[M_SIG][k];
        // visco: Ca, Cb of eo = max((1 - te) e + s ts, eps0) and so = te sumInv e + s; Cd_l = -DT te cdScale_l e
        // (prep_visco_em, ForwardSolverEM.cpp:68-152), tau_eps (te) and tau_sigma (ts) held fixed
        float e = e0, sg = sg0, de_de = 1.0f, de_ds = 0.0f, ds_de = 0.0f, te = 0.0f;
        if (A.visco) {
            te = P.m[M_TAUP][k];
            const float ts = P.m[M_TAUS][k];
            const float eo = (1.0f - te) * e0 + sg0 * ts;
            const bool clamp = eo < eps0;
            e = clamp ? eps0 : eo;
            de_de = clamp ? 0.0f : 1.0f - te;
            de_ds = clamp ? 0.0f : ts;
            sg = te * vc.sumInv * e0 + sg0;
            ds_de = te * vc.sumInv;
        }
        float gE, gS;
        cacb_adj(e, sg, DT, A.g[0][k], A.g[1][k], gE, gS);
        float ged = gE * de_de + gS * ds_de;
        const float gs = gE * de_ds + gS;
        if (A.visco)
            for (int l = 0; l < vc.L; ++l) ged += A.g[4 + l][k] * (-DT) * te * vc.cdScale[l];
        const float ge = eps0 * ged;
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
__global__ void adj_sh_final(PrepParams G, const StepParams P, const AdjShot A, float vsum, float* gvp, float* gvs, float* grho,
                             int accumulate)
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
        // visco-SH: mu = max(rho vs^2 / fS, 1), fS = 1 + sum tauS (the relaxation times held fixed)
        const float fS = A.visco ? 1.0f + vsum * P.m[M_TAUS][k] : 1.0f;
        float raw = rho;
        raw *= vs;
        raw *= vs;
        if (A.visco) raw = raw / fS;
        const bool unclamped = raw >= 1.0f;
        const float ir = P.m[M_IR][k];
        const float gs = unclamped ? gmu * 2.0f * rho * vs / fS : 0.0f;
        const float gr = (unclamped ? gmu * vs * vs / fS : 0.0f) - A.g[2][k] * ir * ir;
        if (accumulate) { gvs[k] += gs; grho[k] += gr; }
        else { gvp[k] = 0.0f; gvs[k] = gs; grho[k] = gr; }
    }
}


// chain rule for TEz: CaX, CbX of the 2-point x averages of eps = eps_r eps0
// and sigma (CaY, CbY along y); iMxy = 1 / (4-point average of mu = mu_r mu0)
// (0 where invalid)
__global__ void adj_te_final(PrepParams G, const StepParams P, const AdjShot A, float DT, ViscoEmCoef vc, float* geps, float* gsig,
                             float* gmu, int accumulate)
{
    const float eps0 = 8.8541878176e-12f, mu0 = 1.2566370614e-6f;
    const float* er = P.m[M_EPSR];
    const float* sg = P.m[M_SIG];
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < G.N; k += (long long)gridDim.x * blockDim.x) {
        const int kx = static_cast<int>(k % G.NX), ky = static_cast<int>(k / G.NX);
        float ge = 0.0f, gs = 0.0f;
        // rows (kx, ky) and (kx-1, ky) of the x averages, (kx, ky) and (kx, ky-1) of the y averages
        for (int d = 0; d <= 1; ++d) {
            for (int q = 0; q < 2; ++q) {
                const int c = q == 0 ? kx : ky, Nc = q == 0 ? static_cast<int>(G.NX) : static_cast<int>(G.NY);
                const long long st = q == 0 ? 1 : G.NX;
                if (c - d < 0) continue;
                const long long r = k - d * st;
                const bool pair = c - d + 1 < Nc;
                if (!(d == 0 || pair)) continue;
                const float w = pair ? 0.5f : 1.0f;
                const float e0 = pair ? 0.5f * (er[r] * eps0) + 0.5f * (er[r + st] * eps0) : er[r] * eps0;
                const float s0 = pair ? 0.5f * sg[r] + 0.5f * sg[r + st] : sg[r];
                // visco: Ca, Cb of the optical permittivity / conductivity of the averaged eps, sigma,
                // tau_eps, tau_sigma; Cd_l = -DT te cdScale_l e (prep_visco_em), the taus held fixed
                float e = e0, s = s0, de_de = 1.0f, de_ds = 0.0f, ds_de = 0.0f, tq = 0.0f;
                if (A.visco) {
                    const float* te = P.m[M_TAUP];
                    const float* ts = P.m[M_TAUS];
                    tq = pair ? 0.5f * te[r] + 0.5f * te[r + st] : te[r];
                    const float sq = pair ? 0.5f * ts[r] + 0.5f * ts[r + st] : ts[r];
                    const float eo = (1.0f - tq) * e0 + s0 * sq;
                    const bool clamp = eo < eps0;
                    e = clamp ? eps0 : eo;
                    de_de = clamp ? 0.0f : 1.0f - tq;
                    de_ds = clamp ? 0.0f : sq;
                    s = tq * vc.sumInv * e0 + s0;
                    ds_de = tq * vc.sumInv;
                }
                float a, b;
                cacb_adj(e, s, DT, A.g[2 * q][r], A.g[2 * q + 1][r], a, b);
                float ga = a * de_de + b * ds_de;
                const float gb = a * de_ds + b;
                if (A.visco)
                    for (int l = 0; l < vc.L; ++l) ga += A.g[5 + q * vc.L + l][r] * (-DT) * tq * vc.cdScale[l];
                ge += w * ga;
                gs += w * gb;
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

// chain rule for the acoustic equations: M = rho vp^2; irx, iry, irz = 1 / (2-point
// average of rho along x, y, z) (0 where invalid); grad_vs is zero
__global__ void adj_ac_final(PrepParams G, const StepParams P, const AdjShot A, float* gvp, float* gvs, float* grho, int accumulate)
{
    const long long sy = (long long)G.NX * G.NZ, sz = G.NX;
    const int nd = G.NZ > 1 ? 3 : 2;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < G.N; k += (long long)gridDim.x * blockDim.x) {
        const int kx = static_cast<int>(k % G.NX);
        const long long rest = k / G.NX;
        const int kz = static_cast<int>(rest % G.NZ), ky = static_cast<int>(rest / G.NZ);
        const float rho = P.m[M_RHO][k], vp = P.m[M_VP][k];
        float gr = A.g[0][k] * vp * vp;
        const int kc[3] = {kx, ky, kz};
        const int Nc[3] = {static_cast<int>(G.NX), static_cast<int>(G.NY), static_cast<int>(G.NZ)};
        const long long st[3] = {1, sy, sz};
        for (int ax = 0; ax < nd; ++ax)
            for (int d = 0; d <= 1; ++d) {
                if (kc[ax] - d < 0) continue;
                const long long r = k - d * st[ax];
                const float ir = P.m[M_IRX + ax][r];
                const float w = (kc[ax] - d + 1 < Nc[ax]) ? 0.5f : 1.0f;
                if (ir != 0.0f && (d == 0 || w == 0.5f)) gr -= A.g[1 + ax][r] * ir * ir * w;
            }
        const float gp = A.g[0][k] * 2.0f * rho * vp;
        if (accumulate) { gvp[k] += gp; grho[k] += gr; }
        else { gvp[k] = gp; gvs[k] = 0.0f; grho[k] = gr; }
    }
}

// chain rule for lossless 3-D EM: CaQ, CbQ of the 2-point averages of eps = eps_r
// eps0 and sigma along axis Q; iMyz, iMxz, iMxy = 1 / (4-point average of mu = mu_r
// mu0 in the yz, xz, xy plane) (0 where invalid)
__global__ void adj_em3_final(PrepParams G, const StepParams P, const AdjShot A, float DT, ViscoEmCoef vc, float* geps, float* gsig,
                              float* gmu, int accumulate)
{
    const float eps0 = 8.8541878176e-12f, mu0 = 1.2566370614e-6f;
    const float* er = P.m[M_EPSR];
    const float* sg = P.m[M_SIG];
    const long long sy = (long long)G.NX * G.NZ, sz = G.NX;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < G.N; k += (long long)gridDim.x * blockDim.x) {
        const int kx = static_cast<int>(k % G.NX);
        const long long rest = k / G.NX;
        const int kz = static_cast<int>(rest % G.NZ), ky = static_cast<int>(rest / G.NZ);
        const int kc[3] = {kx, ky, kz};
        const int Nc[3] = {static_cast<int>(G.NX), static_cast<int>(G.NY), static_cast<int>(G.NZ)};
        const long long st[3] = {1, sy, sz};
        float ge = 0.0f, gs = 0.0f;
        for (int q = 0; q < 3; ++q)
            for (int d = 0; d <= 1; ++d) {
                if (kc[q] - d < 0) continue;
                const long long r = k - d * st[q];
                const bool pair = kc[q] - d + 1 < Nc[q];
                if (d == 1 && !pair) continue;
                const float w = pair ? 0.5f : 1.0f;
                const float e0 = pair ? 0.5f * (er[r] * eps0) + 0.5f * (er[r + st[q]] * eps0) : er[r] * eps0;
                const float s0 = pair ? 0.5f * sg[r] + 0.5f * sg[r + st[q]] : sg[r];
                // visco: the optical permittivity / conductivity of the averaged eps, sigma, tau_eps,
                // tau_sigma and Cd_l = -DT te cdScale_l e (prep_visco_em), the taus held fixed
                float e = e0, s = s0, de_de = 1.0f, de_ds = 0.0f, ds_de = 0.0f, tq = 0.0f;
                if (A.visco) {
                    const float* te = P.m[M_TAUP];
                    const float* ts = P.m[M_TAUS];
                    tq = pair ? 0.5f * te[r] + 0.5f * te[r + st[q]] : te[r];
                    const float sq = pair ? 0.5f * ts[r] + 0.5f * ts[r + st[q]] : ts[r];
                    const float eo = (1.0f - tq) * e0 + s0 * sq;
                    const bool clamp = eo < eps0;
                    e = clamp ? eps0 : eo;
                    de_de = clamp ? 0.0f : 1.0f - tq;
                    de_ds = clamp ? 0.0f : sq;
                    s = tq * vc.sumInv * e0 + s0;
                    ds_de = tq * vc.sumInv;
                }
                float a, b;
                cacb_adj(e, s, DT, A.g[2 * q][r], A.g[2 * q + 1][r], a, b);
                float ga = a * de_de + b * ds_de;
                const float gb = a * de_ds + b;
                if (A.visco)
                    for (int m = 0; m < vc.L; ++m) ga += A.g[9 + q * vc.L + m][r] * (-DT) * tq * vc.cdScale[m];
                ge += w * ga;
                gs += w * gb;
            }
        // plane rows that read point k: yz (iMyz, g[6]), xz (iMxz, g[7]), xy (iMxy, g[8])
        float gm = 0.0f;
        for (int db = 0; db <= 1; ++db)
            for (int da = 0; da <= 1; ++da) {
                if (ky - da >= 0 && kz - db >= 0) {
                    const long long r = k - da * sy - db * sz;
                    const float im = P.m[M_IMUYZ][r];
                    const float w = im != 0.0f ? w4(ky - da, kz - db, ky, kz, G.NY, G.NZ) : 0.0f;
                    if (w != 0.0f) gm -= A.g[6][r] * im * im * w;
                }
                if (kx - da >= 0 && kz - db >= 0) {
                    const long long r = k - da - db * sz;
                    const float im = P.m[M_IMUXZ][r];
                    const float w = im != 0.0f ? w4(kx - da, kz - db, kx, kz, G.NX, G.NZ) : 0.0f;
                    if (w != 0.0f) gm -= A.g[7][r] * im * im * w;
                }
                if (kx - da >= 0 && ky - db >= 0) {
                    const long long r = k - da - db * sy;
                    const float im = P.m[M_IMUXY][r];
                    const float w = im != 0.0f ? w4(kx - da, ky - db, kx, ky, G.NX, G.NY) : 0.0f;
                    if (w != 0.0f) gm -= A.g[8][r] * im * im * w;
                }
            }
        ge *= eps0;
        gm *= mu0;
        if (accumulate) { geps[k] += ge; gsig[k] += gs; gmu[k] += gm; }
        else { geps[k] = ge; gsig[k] = gs; gmu[k] = gm; }
    }
}

// weight of point (ka, kb) in the 4-point row at (a, b) of a plane average,
// by its two in-plane coordinates (the edge fallbacks of
// calc4PointAverageMatrixRow, Modelparameter.cpp:448-527)
__device__ __forceinline__ float w4p(int a, int b, int ka, int kb, int Na, int Nb) { return w4(a, b, ka, kb, Na, Nb); }

// chain rule for 3-D elastic: M = rho vp^2; mu = max(rho vs^2, 1); muXY, muXZ,
// muYZ = 1 / (4-point average of 1 / mu in the xy, xz, yz planes) (0 below 4);
// irx, iry, irz = 1 / (2-point average of rho along x, y, z) (0 where invalid)
__global__ void adj_e3_final(PrepParams G, const StepParams P, const AdjShot A, float vsum, float* gvp, float* gvs, float* grho,
                             int accumulate)
{
    const long long sy = (long long)G.NX * G.NZ, sz = G.NX;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < G.N; k += (long long)gridDim.x * blockDim.x) {
        const int kx = static_cast<int>(k % G.NX);
        const long long rest = k / G.NX;
        const int kz = static_cast<int>(rest % G.NZ), ky = static_cast<int>(rest / G.NZ);
        const float rho = P.m[M_RHO][k], vp = P.m[M_VP][k], vs = P.m[M_VS][k];
        const float muk = P.m[M_MU][k];
        float gmu = A.g[1][k];
        // rows of the plane averages that read point k: (x, y) - {0, 1}^2 in the xy plane, etc.
        for (int db = 0; db <= 1; ++db)
            for (int da = 0; da <= 1; ++da) {
                // xy plane
                if (kx - da >= 0 && ky - db >= 0) {
                    const long long r = k - da - db * sy;
                    const float m = P.m[M_MUXY][r];
                    const float w = m != 0.0f ? w4p(kx - da, ky - db, kx, ky, G.NX, G.NY) : 0.0f;
                    if (w != 0.0f) gmu += A.g[2][r] * w * (m / muk) * (m / muk);
                }
                // xz plane
                if (kx - da >= 0 && kz - db >= 0) {
                    const long long r = k - da - db * sz;
                    const float m = P.m[M_MUXZ][r];
                    const float w = m != 0.0f ? w4p(kx - da, kz - db, kx, kz, G.NX, G.NZ) : 0.0f;
                    if (w != 0.0f) gmu += A.g[3][r] * w * (m / muk) * (m / muk);
                }
                // yz plane
                if (ky - da >= 0 && kz - db >= 0) {
                    const long long r = k - da * sy - db * sz;
                    const float m = P.m[M_MUYZ][r];
                    const float w = m != 0.0f ? w4p(ky - da, kz - db, ky, kz, G.NY, G.NZ) : 0.0f;
                    if (w != 0.0f) gmu += A.g[4][r] * w * (m / muk) * (m / muk);
                }
            }
        // visco: M = rho vp^2 / fP, mu = max(rho vs^2 / fS, 1) with f = 1 + sum tau (the relaxation times held fixed)
        const float fP = A.visco ? 1.0f + vsum * P.m[M_TAUP][k] : 1.0f, fS = A.visco ? 1.0f + vsum * P.m[M_TAUS][k] : 1.0f;
        float raw = rho;
        raw *= vs;
        raw *= vs;
        if (A.visco) raw = raw / fS;
        const bool unclamped = raw >= 1.0f;
        float gr = A.g[0][k] * vp * vp / fP;
        if (unclamped) gr += gmu * vs * vs / fS;
        // inverse density averages: rows k and k - 1 along each axis
        const int kc[3] = {kx, ky, kz};
        const int Nc[3] = {static_cast<int>(G.NX), static_cast<int>(G.NY), static_cast<int>(G.NZ)};
        const long long st[3] = {1, sy, sz};
        const int slot[3] = {M_IRX, M_IRY, M_IRZ};
        for (int ax = 0; ax < 3; ++ax)
            for (int d = 0; d <= 1; ++d) {
                if (kc[ax] - d < 0) continue;
                const long long r = k - d * st[ax];
                const float ir = P.m[slot[ax]][r];
                const float w = (kc[ax] - d + 1 < Nc[ax]) ? 0.5f : 1.0f;
                if (ir != 0.0f && (d == 0 || w == 0.5f)) gr -= A.g[5 + ax][r] * ir * ir * w;
            }
        const float gp = A.g[0][k] * 2.0f * rho * vp / fP;
        const float gs = unclamped ? gmu * 2.0f * rho * vs / fS : 0.0f;
        if (accumulate) { gvp[k] += gp; gvs[k] += gs; grho[k] += gr; }
        else { gvp[k] = gp; gvs[k] = gs; grho[k] = gr; }
    }
}

void launch_adj(int H, int pass, const StepParams* Ps, const AdjShot* As, const BatchTile* W, const BatchSched& S, int grid, int vn,
                int pending, cudaStream_t s)
{
    if (pass >= 13) launch_adj_pass_em3d(H, pass, Ps, As, W, S, grid, vn, pending, s);
    else if (pass >= 11) launch_adj_pass_acoustic(H, pass, Ps, As, W, S, grid, vn, pending, s);
    else if (pass >= 9) launch_adj_pass3d(H, pass, Ps, As, W, S, grid, vn, pending, s);
    else launch_adj_pass2d(H, pass, Ps, As, W, S, grid, vn, pending, s);
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
    const bool ok2 = c.dimension == 2 && (c.equation == WAVE_EQ_ELASTIC || c.equation == WAVE_EQ_TMEM || c.equation == WAVE_EQ_SH ||
                                          c.equation == WAVE_EQ_EMEM || c.equation == WAVE_EQ_VISCOELASTIC ||
                                          c.equation == WAVE_EQ_VISCOSH || c.equation == WAVE_EQ_VISCOTMEM ||
                                          c.equation == WAVE_EQ_VISCOEMEM);
    const bool ok3 = c.dimension == 3 && (c.equation == WAVE_EQ_ELASTIC || c.equation == WAVE_EQ_VISCOELASTIC || c.equation == WAVE_EQ_EMEM ||
                                          c.equation == WAVE_EQ_VISCOEMEM);
    const bool okAc = c.equation == WAVE_EQ_ACOUSTIC;
    if (!ok2 && !ok3 && !okAc)
        return "the adjoint gradient is implemented for 2-D and 3-D acoustic, elastic and visco-elastic, 2-D SH and visco-SH, "
               "lossless 2-D TMz and TEz and lossless 3-D EM modelling";
    if (c.equation == WAVE_EQ_TMEM || c.equation == WAVE_EQ_VISCOTMEM) {
        for (int t : h->hRecType)
            if (t != WAVE_TYPE_EZ) return "the TMz adjoint takes Ez receivers only";
        for (int t : h->hSrcType)
            if (t != WAVE_TYPE_EZ) return "the TMz adjoint takes Ez sources only";
    }
    if (h->vg && c.equation != WAVE_EQ_ACOUSTIC && c.equation != WAVE_EQ_ELASTIC)
        return "the adjoint gradient on a variable grid is implemented for the acoustic and elastic equations";
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
        // 3-D elastic: the Adj3Part layout
        const bool tm = h->cfg.equation == WAVE_EQ_TMEM || h->cfg.equation == WAVE_EQ_VISCOTMEM;
        const bool sh = h->cfg.equation == WAVE_EQ_SH || h->cfg.equation == WAVE_EQ_VISCOSH;
        const bool ac = h->cfg.equation == WAVE_EQ_ACOUSTIC;
        const bool em3 = h->sp.is3d && (h->cfg.equation == WAVE_EQ_EMEM || h->cfg.equation == WAVE_EQ_VISCOEMEM);
        const bool e3 = h->sp.is3d && !ac && !em3;
        long long off[kAdjMaxParts], len[kAdjMaxParts], o = 0;
        const int elasticFields[5] = {F_VX, F_VY, F_SXX, F_SYY, F_SXY};
        const int tmFields[5] = {F_HX, F_HY, F_EZ, -1, -1};
        const int tmPsi[8] = {PS_EZY, PS_EZX, PS_HYX, PS_HXY, -1, -1, -1, -1};
        // TEz: hz, -, ex, ey and the psi of eyx, exy, -, -, hzy, hzx
        const bool te = !h->sp.is3d && (h->cfg.equation == WAVE_EQ_EMEM || h->cfg.equation == WAVE_EQ_VISCOEMEM);
        const int shFields[5] = {F_VZ, -1, F_SXZ, F_SYZ, -1};
        const int shPsi[8] = {PS_SXZ_X, PS_SYZ_Y, -1, -1, PS_VZX, PS_VZY, -1, -1};
        const int teFields[5] = {F_HZ, -1, F_EX, F_EY, -1};
        const int tePsi[8] = {PS_EYX, PS_EXY, -1, -1, PS_HZY, PS_HZX, -1, -1};
        const int e3Fields[9] = {F_VX, F_VY, F_VZ, F_SXX, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ};
        const int e3Psi[18] = {PS_SXX_X, PS_SXY_Y, PS_SXZ_Z, PS_SXY_X, PS_SYY_Y, PS_SYZ_Z, PS_SXZ_X, PS_SYZ_Y, PS_SZZ_Z,
                               PS_VXX,   PS_VYY,   PS_VZZ,   PS_VXY,   PS_VYX,   PS_VXZ,   PS_VZX,   PS_VYZ,   PS_VZY};
        // acoustic: p, vx, vy, vz and the psi of p_x, p_y, p_z, vxx, vyy, vzz (2-D: no vz, p_z, vzz)
        const int acFields[4] = {F_P, F_VX, F_VY, h->sp.is3d ? F_VZ : -1};
        const int acPsi[6] = {PS_P_X, PS_P_Y, PS_P_Z, PS_VXX, PS_VYY, PS_VZZ};
        // lossless 3-D EM: hx, hy, hz, ex, ey, ez and the psi of the H-update then the E-update derivatives
        const int em3Fields[6] = {F_HX, F_HY, F_HZ, F_EX, F_EY, F_EZ};
        const int em3Psi[12] = {PS_EZY, PS_EYZ, PS_EXZ, PS_EZX, PS_EYX, PS_EXY, PS_HZY, PS_HYZ, PS_HXZ, PS_HZX, PS_HYX, PS_HXY};
        const int* fields = em3 ? em3Fields : ac ? acFields : e3 ? e3Fields : tm ? tmFields : sh ? shFields : te ? teFields
                                                                                                  : elasticFields;
        const int* psiSlot = em3 ? em3Psi : ac ? acPsi : e3 ? e3Psi : tm ? tmPsi : sh ? shPsi : te ? tePsi : kAdjPsiSlot;
        // visco-elastic: the elastic parts, then rxx, ryy, rxy of each mechanism
        const bool visco = h->cfg.equation == WAVE_EQ_VISCOELASTIC || h->cfg.equation == WAVE_EQ_VISCOSH ||
                           h->cfg.equation == WAVE_EQ_VISCOTMEM || h->cfg.equation == WAVE_EQ_VISCOEMEM;
        const int ncomp = e3 ? 6 : (sh || te) ? 2 : tm ? 1 : 3;   // memory-variable components per mechanism (3-D EM: 3)
        const int nr = visco ? ncomp * h->L : 0;
        const int nf = em3 ? 6 : ac ? 4 : e3 ? 9 : 5, np = em3 ? 12 : ac ? 6 : e3 ? 18 : 8, nparts = nf + np + nr;
        for (int k = 0; k < nf; ++k) { off[k] = o; len[k] = fields[k] >= 0 ? N : 0; o += len[k]; }
        for (int k = 0; k < np; ++k) {
            const int slot = psiSlot[k];
            off[nf + k] = o;
            len[nf + k] = (slot >= 0 && h->psi[slot]) ? h->psiLen[slot] : 0;
            o += len[nf + k];
        }
        const int memVar2[3] = {R_XX, R_YY, R_XY};
        const int memVar3[6] = {R_XX, R_YY, R_ZZ, R_XY, R_XZ, R_YZ};
        const int memVarSH[2] = {R_XZ, R_YZ};
        const int memVarTM[1] = {R_EZ};
        const int memVarTE[2] = {R_EX, R_EY};
        const int memVarEM3[3] = {R_EX, R_EY, R_EZ};
        const int* memVar = e3 ? memVar3 : sh ? memVarSH : tm ? memVarTM : te ? memVarTE : em3 ? memVarEM3 : memVar2;
        auto rpart = [&](int j) { return h->r[memVar[j / h->L]][j % h->L]; };
        for (int j = 0; j < nr; ++j) { off[nf + np + j] = o; len[nf + np + j] = N; o += N; }
        stride[s] = o;
        AdjShot& a = A[s];
        a.tm = tm ? 1 : 0;
        a.sh = sh ? 1 : 0;
        a.te = te ? 1 : 0;
        a.e3 = e3 ? 1 : 0;
        a.visco = visco ? 1 : 0;
        a.ac = ac ? 1 : 0;
        a.em3 = em3 ? 1 : 0;
        a.view = pool.get<float>(static_cast<size_t>(o) * (K + 1));
        a.stride = o;
        for (int k = 0; k < kAdjMaxParts; ++k) a.off[k] = k < nparts ? off[k] : 0;
        float* lstate = pool.get<float>(o);
        ck(cudaMemsetAsync(lstate, 0, o * sizeof(float), st), "memset");
        for (int k = 0; k < nf; ++k) a.lf[k] = lstate + off[k];
        for (int k = 0; k < np; ++k) a.lpsi[k] = lstate + off[nf + k];
        for (int k = 0; k < 6 * kMaxL; ++k) a.lr[k] = nullptr;
        for (int j = 0; j < nr; ++j) a.lr[(j / h->L) * kMaxL + j % h->L] = lstate + off[nf + np + j];
        // acoustic: 6 and 4 of them; visco-TMz: dJ/dCd_l in g[4 + l]
        const int ntemp = e3 ? 18 : em3 ? 12 : 8;
        const int ngrad = e3 ? 8 : em3 ? 9 + (visco ? 3 * h->L : 0) : (tm && visco) ? 4 + h->L : (te && visco) ? 5 + 2 * h->L : 5;
        float* temps = pool.get<float>(static_cast<size_t>(ntemp) * N);
        for (int k = 0; k < ntemp; ++k) a.T[k] = temps + k * N;
        float* grads = pool.get<float>(static_cast<size_t>(ngrad) * N);
        ck(cudaMemsetAsync(grads, 0, ngrad * N * sizeof(float), st), "memset");
        for (int k = 0; k < ngrad; ++k) a.g[k] = grads + k * N;
        a.ridx = h->ridx;
        a.rtype = h->rtype;
        a.nrec = h->nrec;
        a.nt = NT;
        float* res = pool.get<float>(static_cast<size_t>(h->nrec) * NT);
        a.res = res;
        bool velocitySources = false;
        for (int t : h->hSrcType)
            velocitySources |= em3 ? t == WAVE_TYPE_HZ : (e3 || ac) ? (t == WAVE_TYPE_VX || t == WAVE_TYPE_VY || t == WAVE_TYPE_VZ)
                             : te ? t == WAVE_TYPE_HZ : sh ? t == WAVE_TYPE_VZ : (t == WAVE_TYPE_VX || t == WAVE_TYPE_VY);
        a.vprime[0] = a.vprime[1] = a.vprime[2] = nullptr;
        if (h->cfg.DampingBoundary == 1 || velocitySources) {
            const int nv = (e3 || ac || em3) ? 3 : 2;
            a.vprime[0] = pool.get<float>(static_cast<size_t>(nv) * N);
            for (int k = 1; k < nv; ++k) a.vprime[k] = a.vprime[0] + k * N;
        }
        a.sidx = h->sidx;
        a.stype = h->stype;
        a.signals = h->signals;
        a.nsrc = h->nsrc;
        ckpt[s] = pool.get<float>(static_cast<size_t>(o) * nck);
        for (int k = 0; k < nparts; ++k) {
            if (len[k] == 0) continue;
            float* live = k < nf ? h->f[fields[k]] : k < nf + np ? h->psi[psiSlot[k - nf]] : rpart(k - nf - np);
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
    TraceRange phase("adjoint.forward");
    for (auto* h : shots) {
        for (int f : h->fields) ck(cudaMemsetAsync(h->f[f], 0, h->N * sizeof(float), st), "memset");
        for (int k = 0; k < PS_COUNT; ++k)
            if (h->psi[k]) ck(cudaMemsetAsync(h->psi[k], 0, h->psiLen[k] * sizeof(float), st), "memset");
        for (int rr = 0; rr < R_COUNT; ++rr)
            for (int l = 0; l < kMaxL; ++l)
                if (h->r[rr][l]) ck(cudaMemsetAsync(h->r[rr][l], 0, h->N * sizeof(float), st), "memset");
        ck(cudaMemsetAsync(h->seis, 0, static_cast<size_t>(h->nrec) * NT * sizeof(float), st), "memset");
    }
    S.set_counter(0);
    for (int n = 0; n < NT; ++n) {
        if (n % K == 0) copy(dToCkpt, toCkpt.size(), 0, n / K);
        S.step();
    }
    // 2. residuals and misfits
    phase.next("adjoint.residuals");
    for (int s = 0; s < ns; ++s) {
        const long long n = static_cast<long long>(shots[s]->nrec) * NT;
        residual_kernel<<<256, 256, 0, st>>>(shots[s]->seis, dobs[s], const_cast<float*>(A[s].res), n, dMisfit + s);
    }
    // 3. backward sweep over the checkpoint segments
    phase.next("adjoint.backward");
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
            const int first = A[0].em3 ? 13 : A[0].ac ? 11 : A[0].e3 ? 9 : A[0].tm ? 3 : A[0].sh ? 5 : A[0].te ? 7 : 0;
            const int pending = n < NT - 1 ? 1 : 0;
            launch_adj(H, first, dP, dA, dT, sched, grid, n - n0, pending, st);
            launch_adj(H, first + 1, dP, dA, dT, sched, grid, n - n0, pending, st);
        }
        ck(cudaGetLastError(), "adjoint launch");
    }
    // 4. chain rule to vp, vs, rho
    phase.next("adjoint.chainRule");
    for (int s = 0; s < ns; ++s) {
        wave_handle* h = shots[s];
        PrepParams G{h->NX, h->NY, h->NZ, h->N};
        const int o = sum ? 0 : s;
        if (A[s].em3)
            adj_em3_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], static_cast<float>(h->cfg.DT), h->vemc, gvp[o], gvs[o], grho[o],
                                                sum && s > 0 ? 1 : 0);
        else if (A[s].ac)
            adj_ac_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], gvp[o], gvs[o], grho[o], sum && s > 0 ? 1 : 0);
        else if (A[s].e3)
            adj_e3_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], A[s].visco ? visco_modulus_sum(h->cfg, h->L) : 0.0f, gvp[o], gvs[o],
                                               grho[o], sum && s > 0 ? 1 : 0);
        else if (A[s].tm)
            adj_tm_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], static_cast<float>(h->cfg.DT), h->vemc, gvp[o], gvs[o], grho[o],
                                               sum && s > 0 ? 1 : 0);
        else if (A[s].sh)
            adj_sh_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], A[s].visco ? visco_modulus_sum(h->cfg, h->L) : 0.0f, gvp[o], gvs[o],
                                               grho[o], sum && s > 0 ? 1 : 0);
        else if (A[s].te)
            adj_te_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], static_cast<float>(h->cfg.DT), h->vemc, gvp[o], gvs[o], grho[o],
                                               sum && s > 0 ? 1 : 0);
        else
            adj_grad_final<<<1216, 256, 0, st>>>(G, Ps[s], A[s], A[s].visco ? visco_modulus_sum(h->cfg, h->L) : 0.0f, gvp[o],
                                                 gvs[o], grho[o], sum && s > 0 ? 1 : 0);
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
    wave::TraceRange region("adjoint.gradient");
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
        if (h->vg) {
            vargrid_adjoint(h, dDobs, checkpoint_every, misfit, dOut[0], dOut[1], dOut[2]);
        } else {
            AdjStepper S;
            S.stream = h->stream;
            S.set_counter = [h](int n) { launch_set_counter(h->tcounter, n, h->stream); };
            S.step = [h]() { step_once(h); };
            adjoint_run({h}, S, &dDobs, checkpoint_every, misfit, &dOut[0], &dOut[1], &dOut[2], false);
        }
        if (grad_mem != WAVE_MEM_DEVICE)
            for (int k = 0; k < 3; ++k) ck(cudaMemcpy(out[k], dOut[k], N * sizeof(float), cudaMemcpyDeviceToHost), "gradient copy");
    } catch (std::exception& e) {
        h->err = std::string("wave_adjoint_gradient: ") + e.what();
        return WAVE_ERR_CUDA;
    }
    return WAVE_OK;
}
