// adjoint_impl.hpp — TEST INFRASTRUCTURE ONLY (the oracle).
//
// Discrete adjoint of the oracle's 2-D elastic step (Sim<T>::stepElastic,
// restating FD2Delastic::run, ForwardSolver2Delastic.cpp:117-297, with CPML
// CPML.cpp:84-95, the free surface FreeSurface2Delastic.cpp:14-45 and the ABS
// taper ABS2D.cpp:14-50): the gradient of J = 1/2 sum (d - d_obs)^2 over all
// receivers and samples with respect to vp, vs and rho, in the oracle's value
// type (double: the FP64 gradient the CUDA adjoint is checked against).
//
// The reference has no adjoint; this is an independent restatement on the
// oracle's CSR operators (transposed explicitly), written from the forward
// operation list, not from the CUDA adjoint.
//
// Per step t the forward maps state X_t = (vx, vy, sxx, syy, sxy, psi) to
// X_{t+1}; the receivers read X_{t+1}. Intermediates of step t are formed
// from X_t and X_{t+1}:
//   a1' = Dxf sxx + P1   a2' = DybS sxy + P2   a3' = Dxb sxy + P3   a4' = DyfS syy + P4
//   vx' = vx + irx (a1' + a2')                  vy' = vy + iry (a3' + a4')
//   c1' = Dxb vx' + Q1   c2' = Dyb vy' + Q2   c3' = Dyf vx' + Q3   c4' = Dxf vy' + Q4
// (P, Q: the psi arrays of X_{t+1}; vx', vy' are the velocities before the
// ABS taper and the sources). Checkpoints every K steps; each segment is
// recomputed with the oracle's own step and walked backwards.
#pragma once

#include <cmath>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "refcpu.hpp"

namespace refcpu {

template <class T>
CSR<T> transpose(const CSR<T>& A)
{
    CSR<T> B;
    B.n = A.n;
    B.ptr.assign(A.n + 1, 0);
    for (idx_t k = 0; k < A.ptr[A.n]; ++k) ++B.ptr[A.col[k] + 1];
    for (idx_t r = 0; r < A.n; ++r) B.ptr[r + 1] += B.ptr[r];
    B.col.resize(A.ptr[A.n]);
    B.val.resize(A.ptr[A.n]);
    std::vector<idx_t> fill(B.ptr.begin(), B.ptr.end() - 1);
    for (idx_t r = 0; r < A.n; ++r)
        for (idx_t k = A.ptr[r]; k < A.ptr[r + 1]; ++k) {
            const idx_t d = fill[A.col[k]]++;
            B.col[d] = r;
            B.val[d] = A.val[k];
        }
    return B;
}

// y += A x
template <class T>
void spmv_add(const CSR<T>& A, const std::vector<T>& x, std::vector<T>& y)
{
#pragma omp parallel for schedule(static)
    for (idx_t r = 0; r < A.n; ++r) {
        T s = 0;
        for (idx_t k = A.ptr[r]; k < A.ptr[r + 1]; ++k) s += A.val[k] * x[A.col[k]];
        y[r] += s;
    }
}

template <class T>
struct AverageTranspose {
    const Sim<T>& s;
    const idx_t N;
    explicit AverageTranspose(const Sim<T>& sim) : s(sim), N(sim.g.N()) {}
    // A^T y for the averaging operator `avg` (out = avg(in)), whose row r reads
    // at most the 2 x 2 x 2 block at r (x, x+1) x (y, y+1) x (z, z+1): probed
    // with one unit pattern per (x mod 2, y mod 2, z mod 2) colour, so the edge
    // fallbacks come from the oracle's own averaging code.
    template <class Avg>
    void avgT(Avg avg, const std::vector<T>& y, std::vector<T>& out) const
    {
        std::vector<T> e(N), col(N);
        const int ncz = s.g.NZ > 1 ? 2 : 1;
        for (int cx = 0; cx < 2; ++cx)
            for (int cy = 0; cy < 2; ++cy)
                for (int cz = 0; cz < ncz; ++cz) {
                    for (idx_t k = 0; k < N; ++k) {
                        idx_t x, yy, z;
                        s.g.coord(k, x, yy, z);
                        e[k] = (x % 2 == cx && yy % 2 == cy && z % 2 == cz) ? T(1) : T(0);
                    }
                    avg(e.data(), col.data());   // col[r] = A[r, k_c(r)]
                    for (idx_t r = 0; r < N; ++r) {
                        if (col[r] == T(0)) continue;
                        idx_t x, yy, z;
                        s.g.coord(r, x, yy, z);
                        const idx_t kx = (x % 2 == cx) ? x : x + 1, ky = (yy % 2 == cy) ? yy : yy + 1;
                        const idx_t kz = (z % 2 == cz) ? z : z + 1;
                        out[s.g.index(kx, ky, kz)] += col[r] * y[r];
                    }
                }
    }

};

template <class T>
struct ElasticAdjoint2D {
    Sim<T>& s;
    const idx_t N;
    CSR<T> DxfT, DxbT, DyfT, DybT, DyfST, DybST;
    // psi names and (a, b) profiles, in the forward's order (stepElastic 2-D)
    static constexpr const char* kP[4] = {"sxx_x", "sxy_y", "sxy_x", "syy_y"};
    static constexpr const char* kQ[4] = {"vxx", "vyy", "vxy", "vyx"};

    const bool visco;   // 2-D visco-elastic (FD2Dviscoelastic::run, ForwardSolver2Dviscoelastic.cpp:130-321)

    explicit ElasticAdjoint2D(Sim<T>& sim) : s(sim), N(sim.g.N()), visco(sim.eq == WAVE_EQ_VISCOELASTIC)
    {
        if (s.is3d || (s.eq != WAVE_EQ_ELASTIC && s.eq != WAVE_EQ_VISCOELASTIC))
            throw std::invalid_argument("oracle adjoint: 2-D elastic or visco-elastic only");
        DxfT = transpose(s.Dxf);
        DxbT = transpose(s.Dxb);
        DyfT = transpose(s.Dyf);
        DybT = transpose(s.Dyb);
        DyfST = transpose(s.fs ? s.DyfFS : s.Dyf);
        DybST = transpose(s.fs ? s.DybFS : s.Dyb);
    }

    struct State {
        std::map<std::string, std::vector<T>> F, psi;
        std::map<std::string, std::vector<std::vector<T>>> R;
    };
    State save() const { return {s.F, s.psi, s.R}; }
    void load(const State& x)
    {
        s.F = x.F;
        s.psi = x.psi;
        s.R = x.R;
    }
    const std::vector<T>& psiOf(const State& x, const char* n, const std::vector<T>& zero) const
    {
        auto it = x.psi.find(n);
        return it == x.psi.end() ? zero : it->second;
    }
    std::pair<const std::vector<T>*, const std::vector<T>*> prof(const char* n) const
    {
        const std::string k(n);
        if (k == "sxx_x" || k == "vyx") return {&s.axh, &s.bxh};
        if (k == "sxy_y" || k == "vyy") return {&s.ay, &s.by};
        if (k == "sxy_x" || k == "vxx") return {&s.ax, &s.bx};
        return {&s.ayh, &s.byh};   // syy_y, vxy
    }

    // adjoint of (c, psi) -> (c' = (1 + a) c + b psi, psi' = a c + b psi) at every point:
    // in: lc = adjoint of c', lp = adjoint of psi'; out: lc = adjoint of c, lp = adjoint of psi
    void cpmlT(std::vector<T>& lc, std::vector<T>& lp, const char* n) const
    {
        if (!s.useCpml) return;
        auto ab = prof(n);
        const std::vector<T>& a = *ab.first;
        const std::vector<T>& b = *ab.second;
        for_n(N, [&](idx_t i) {
            const T c = (T(1) + a[i]) * lc[i] + a[i] * lp[i];
            lp[i] = b[i] * (lc[i] + lp[i]);
            lc[i] = c;
        });
    }

    // transpose of the visco free-surface exchange at one surface point for one
    // horizontal normal stress S with the adjoint lS of its final value and LR[l]
    // the adjoints of its memory variables after the regular update (lR + DT/2 lS):
    // adds to the adjoints of the horizontal strain sum (h) and of vyy (v) and to
    // dJ/dM, dJ/dmu
    static void fsExchangeT(const Sim<T>& s, idx_t i, T lS, const T* LR, T h, T v, T& lh, T& lv, T& gM, T& gMu)
    {
        const T M = s.M[i], mu = s.mu[i], tP = s.tauP[i], tS = s.tauS[i], opP = s.onePlusLtauP[i], opS = s.onePlusLtauS[i];
        const T mp = M * opP, sV = mp - T(2) * mu * opS, sH = -sV * sV / mp;
        const T t3 = T(2) * mu * tS - M * tP, ratio = T(2) * mu * opS / mp - T(1);
        T lhh = sH * lS, lvv = -sV * lS;
        // dJ/dsH = lS h, dJ/dsV = -lS v; dJ/drh_l = LR_l h, dJ/drv_l = -LR_l v
        const T gsH = lS * h, gsV = -lS * v;
        T grh = 0, grv = 0;   // summed over l with the factor c2_l / tau_l
        for (int l = 0; l < s.L; ++l) {
            const T kk = s.viscoC2[l] / s.relaxTime[l];
            lhh += t3 * ratio * kk * LR[l];
            lvv -= t3 * kk * LR[l];
            grh += LR[l] * h * kk;
            grv += -LR[l] * v * kk;
        }
        lh += lhh;
        lv += lvv;
        // sV = M opP - 2 mu opS; sH = -sV^2 / (M opP)
        const T dsH_dsV = -T(2) * sV / mp, dsH_dM = sV * sV / (mp * mp) * opP;
        gM += gsV * opP + gsH * (dsH_dsV * opP + dsH_dM);
        gMu += gsV * (-T(2) * opS) + gsH * dsH_dsV * (-T(2) * opS);
        // rv = t3 k, rh = t3 ratio k: dt3/dM = -tauP, dt3/dmu = 2 tauS; dratio/dM = -2 mu opS / (M^2 opP),
        // dratio/dmu = 2 opS / (M opP)
        const T dr_dM = -T(2) * mu * opS / (M * mp), dr_dmu = T(2) * opS / mp;
        gM += grv * (-tP) + grh * (-tP * ratio + t3 * dr_dM);
        gMu += grv * (T(2) * tS) + grh * (T(2) * tS * ratio + t3 * dr_dmu);
    }

    // Returns the misfit; writes the gradients with respect to vp, vs, rho.
    double run(const std::vector<T>& vp, const std::vector<T>& vs, const std::vector<T>& rho, const T* dobs, int K,
               T* gvp, T* gvs, T* grho)
    {
        const int NT = s.NT;
        const size_t nrec = s.rec.idx.size();
        const std::vector<T> zero(N, T(0));
        // 1. forward with checkpoints
        s.reset();
        std::vector<State> ck;
        for (int t = 0; t < NT; ++t) {
            if (t % K == 0) ck.push_back(save());
            s.step(t);
        }
        std::vector<T> res(nrec * static_cast<size_t>(NT));
        double J = 0;
        for (size_t k = 0; k < res.size(); ++k) {
            res[k] = s.seis[k] - dobs[k];
            J += 0.5 * static_cast<double>(res[k]) * static_cast<double>(res[k]);
        }
        // adjoint state and material gradients
        std::map<std::string, std::vector<T>> lF, lpsi;
        for (const char* n : {"vx", "vy", "sxx", "syy", "sxy"}) lF[n].assign(N, 0);
        for (int k = 0; k < 4; ++k) { lpsi[kP[k]].assign(N, 0); lpsi[kQ[k]].assign(N, 0); }
        // adjoint memory variables rxx, ryy, rxy per mechanism (visco)
        std::vector<std::vector<std::vector<T>>> lR(3, std::vector<std::vector<T>>(visco ? s.L : 0, std::vector<T>(N, 0)));
        std::vector<T> gM(N, 0), gMu(N, 0), gMuXY(N, 0), gIrx(N, 0), gIry(N, 0);
        std::vector<T> a[4], c[4], vxp(N), vyp(N), la[4], lc[4];
        for (int k = 0; k < 4; ++k) { a[k].assign(N, 0); c[k].assign(N, 0); la[k].assign(N, 0); lc[k].assign(N, 0); }
        // 2. backward over the segments
        const int nseg = static_cast<int>(ck.size());
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const int t0 = seg * K, t1 = std::min(NT, t0 + K);
            std::vector<State> X;
            load(ck[seg]);
            X.push_back(save());
            for (int t = t0; t < t1; ++t) {
                s.step(t);
                X.push_back(save());
            }
            for (int t = t1 - 1; t >= t0; --t) {
                const State& X0 = X[t - t0];
                const State& X1 = X[t - t0 + 1];
                // intermediates of step t
                const CSR<T>& DybS = s.fs ? s.DybFS : s.Dyb;
                const CSR<T>& DyfS = s.fs ? s.DyfFS : s.Dyf;
                s.Dxf.spmv(X0.F.at("sxx").data(), a[0].data());
                DybS.spmv(X0.F.at("sxy").data(), a[1].data());
                s.Dxb.spmv(X0.F.at("sxy").data(), a[2].data());
                DyfS.spmv(X0.F.at("syy").data(), a[3].data());
                for (int k = 0; k < 4; ++k) {
                    const std::vector<T>& p = psiOf(X1, kP[k], zero);
                    for_n(N, [&](idx_t i) { a[k][i] += p[i]; });
                }
                const std::vector<T>& vx0 = X0.F.at("vx");
                const std::vector<T>& vy0 = X0.F.at("vy");
                for_n(N, [&](idx_t i) {
                    vxp[i] = vx0[i] + s.invRhoX[i] * (a[0][i] + a[1][i]);
                    vyp[i] = vy0[i] + s.invRhoY[i] * (a[2][i] + a[3][i]);
                });
                s.Dxb.spmv(vxp.data(), c[0].data());
                s.Dyb.spmv(vyp.data(), c[1].data());
                s.Dyf.spmv(vxp.data(), c[2].data());
                s.Dxf.spmv(vyp.data(), c[3].data());
                for (int k = 0; k < 4; ++k) {
                    const std::vector<T>& q = psiOf(X1, kQ[k], zero);
                    for_n(N, [&](idx_t i) { c[k][i] += q[i]; });
                }
                // receivers read X_{t+1}: gather^T of the residual
                for (size_t r = 0; r < nrec; ++r) {
                    const idx_t i = s.rec.idx[r];
                    const T v = res[r * NT + t];
                    switch (s.rec.type[r]) {
                    case WAVE_TYPE_P: lF["sxx"][i] += T(0.5) * v; lF["syy"][i] += T(0.5) * v; break;
                    case WAVE_TYPE_VX: lF["vx"][i] += v; break;
                    default: lF["vy"][i] += v; break;
                    }
                }
                auto& lvx = lF["vx"];
                auto& lvy = lF["vy"];
                auto& lxx = lF["sxx"];
                auto& lyy = lF["syy"];
                auto& lxy = lF["sxy"];
                // ABS taper on all five fields (after the free surface)
                if (s.useAbs)
                    for (auto* v : {&lxx, &lyy, &lxy, &lvx, &lvy}) {
                        auto& w = *v;
                        for_n(N, [&](idx_t i) { w[i] *= s.damping[i]; });
                    }
                for (int k = 0; k < 4; ++k) std::fill(lc[k].begin(), lc[k].end(), T(0));
                if (s.fs && !visco) {
                    // sxx += scaleH c1' - scaleV c2'; syy *= fsZero
                    for_n(N, [&](idx_t i) {
                        lyy[i] *= s.fsZero[i];
                        lc[0][i] += s.scaleH[i] * lxx[i];
                        lc[1][i] -= s.scaleV[i] * lxx[i];
                        // scaleV = sel (M - 2 mu), scaleH = -sel (M - 2 mu)^2 / M
                        const T sel = s.fsSelect[i];
                        if (sel != T(0)) {
                            const T gH = lxx[i] * c[0][i], gV = -lxx[i] * c[1][i];
                            const T sv = s.M[i] - T(2) * s.mu[i];
                            gM[i] += gV * sel - gH * sel * (T(2) * sv / s.M[i] - sv * sv / (s.M[i] * s.M[i]));
                            gMu[i] += -T(2) * gV * sel + gH * sel * T(4) * sv / s.M[i];
                        }
                    });
                }
                if (visco) {
                    // per mechanism l, with e = c1' + c2', q = c2' (sxx) or c1' (syy), m = muXY (c3' + c4'):
                    //   Rk' = c2_l (c1_l Rk - tauP M e / tau_l + tauS 2 mu q / tau_l)
                    //   Sk' = Sk + DT/2 sum_l (Rk + Rk') + (1 + L tauP) M e - (1 + L tauS) 2 mu q
                    //   Rxy' = c2_l (c1_l Rxy - tauSXY m / tau_l)
                    //   Sxy' = Sxy + DT/2 sum_l (Rxy + Rxy') + (1 + L tauS) m
                    const T DTh = s.DThalf;
                    for_n(N, [&](idx_t i) {
                        const T e = c[0][i] + c[1][i], M = s.M[i], mu = s.mu[i];
                        const T tP = s.tauP[i], tS = s.tauS[i], opP = s.onePlusLtauP[i], opS = s.onePlusLtauS[i];
                        // free surface (FreeSurface2Dviscoelastic.cpp): syy and ryy are zeroed on the
                        // surface row, so their adjoints do not flow back
                        const bool surf = s.fs && s.fsSelect[i] != T(0);
                        if (surf) {
                            lyy[i] = 0;
                            for (int l = 0; l < s.L; ++l) lR[1][l][i] = 0;
                        }
                        T LRx[8] = {0, 0, 0, 0, 0, 0, 0, 0};
                        T le = 0, lq[2] = {0, 0};
                        for (int k = 0; k < 2; ++k) {
                            const T lS = k == 0 ? lxx[i] : lyy[i];
                            const T q = k == 0 ? c[1][i] : c[0][i];
                            le += opP * M * lS;
                            lq[k] -= opS * T(2) * mu * lS;
                            gM[i] += opP * e * lS;
                            gMu[i] -= opS * T(2) * q * lS;
                            auto& lRk = lR[k];
                            for (int l = 0; l < s.L; ++l) {
                                const T c1 = s.viscoC1[l], c2 = s.viscoC2[l], irt = s.invRelaxTime[l];
                                const T LR = lRk[l][i] + DTh * lS;   // adjoint of Rk'
                                if (k == 0) LRx[l] = LR;
                                lRk[l][i] = c2 * c1 * LR + DTh * lS;
                                le -= c2 * irt * tP * M * LR;
                                lq[k] += c2 * irt * tS * T(2) * mu * LR;
                                gM[i] -= c2 * irt * tP * e * LR;
                                gMu[i] += c2 * irt * tS * T(2) * q * LR;
                            }
                        }
                        lc[0][i] += le + lq[1];
                        lc[1][i] += le + lq[0];
                        if (surf) {
                            // on the surface row: Sxx' += sH c1' - sV c2' + DT/2 sum_l dR_l,
                            // Rxx_l' += dR_l = rh_l c1' - rv_l c2' with sV = M opP - 2 mu opS,
                            // sH = -sV^2 / (M opP), rv_l = t3 c2_l / tau_l, rh_l = t3 ratio c2_l / tau_l,
                            // t3 = 2 mu tauS - M tauP, ratio = 2 mu opS / (M opP) - 1
                            fsExchangeT(s, i, lxx[i], LRx, c[0][i], c[1][i], lc[0][i], lc[1][i], gM[i], gMu[i]);
                        }
                        const T lS = lxy[i], sh = c[2][i] + c[3][i];
                        T lm = opS * lS;
                        for (int l = 0; l < s.L; ++l) {
                            const T c1 = s.viscoC1[l], c2 = s.viscoC2[l], irt = s.invRelaxTime[l];
                            const T LR = lR[2][l][i] + DTh * lS;
                            lR[2][l][i] = c2 * c1 * LR + DTh * lS;
                            lm -= c2 * irt * s.tauSXY[i] * LR;
                        }
                        gMuXY[i] += sh * lm;
                        lc[2][i] += s.muXY[i] * lm;
                        lc[3][i] += s.muXY[i] * lm;
                    });
                } else {
                    // sxy += muXY (c3' + c4')
                    for_n(N, [&](idx_t i) {
                        lc[2][i] += s.muXY[i] * lxy[i];
                        lc[3][i] += s.muXY[i] * lxy[i];
                        gMuXY[i] += lxy[i] * (c[2][i] + c[3][i]);
                    });
                    // sxx += M (c1' + c2') - 2 mu c2', syy += M (c1' + c2') - 2 mu c1'
                    for_n(N, [&](idx_t i) {
                        lc[0][i] += s.M[i] * (lxx[i] + lyy[i]) - T(2) * s.mu[i] * lyy[i];
                        lc[1][i] += s.M[i] * (lxx[i] + lyy[i]) - T(2) * s.mu[i] * lxx[i];
                        gM[i] += (lxx[i] + lyy[i]) * (c[0][i] + c[1][i]);
                        gMu[i] += -T(2) * (lxx[i] * c[1][i] + lyy[i] * c[0][i]);
                    });
                }
                for (int k = 0; k < 4; ++k) cpmlT(lc[k], lpsi[kQ[k]], kQ[k]);
                // the undamped velocities vx', vy' feed c1..c4
                spmv_add(DxbT, lc[0], lvx);
                spmv_add(DyfT, lc[2], lvx);
                spmv_add(DybT, lc[1], lvy);
                spmv_add(DxfT, lc[3], lvy);
                // vx' = vx + irx (a1' + a2'), vy' = vy + iry (a3' + a4')
                for_n(N, [&](idx_t i) {
                    la[0][i] = la[1][i] = s.invRhoX[i] * lvx[i];
                    la[2][i] = la[3][i] = s.invRhoY[i] * lvy[i];
                    gIrx[i] += lvx[i] * (a[0][i] + a[1][i]);
                    gIry[i] += lvy[i] * (a[2][i] + a[3][i]);
                });
                for (int k = 0; k < 4; ++k) cpmlT(la[k], lpsi[kP[k]], kP[k]);
                spmv_add(DxfT, la[0], lxx);
                spmv_add(DybST, la[1], lxy);
                spmv_add(DxbT, la[2], lxy);
                spmv_add(DyfST, la[3], lyy);
            }
        }
        chain(vp, vs, rho, gM, gMu, gMuXY, gIrx, gIry, gvp, gvs, grho);
        return J;
    }

    template <class Avg>
    void avgT(Avg avg, const std::vector<T>& y, std::vector<T>& out) const { AverageTranspose<T>(s).avgT(avg, y, out); }

    // the model preparation's transpose: (M, mu, muXY, irx, iry) -> (vp, vs, rho)
    void chain(const std::vector<T>& vp, const std::vector<T>& vs, const std::vector<T>& rho, const std::vector<T>& gM,
               const std::vector<T>& gMu, const std::vector<T>& gMuXY, const std::vector<T>& gIrx, const std::vector<T>& gIry,
               T* gvp, T* gvs, T* grho) const
    {
        // muXY = 1 / A4 (1 / mu_c) (0 below 4): d muXY_r / d mu_c,k = muXY_r^2 A4[r, k] / mu_c,k^2
        std::vector<T> y(N), gmuc(gMu);
        for_n(N, [&](idx_t r) { y[r] = gMuXY[r] * s.muXY[r] * s.muXY[r]; });
        std::vector<T> t(N, 0);
        avgT([&](const T* in, T* out) { average4<T>(s.g, 0, in, out); }, y, t);
        for_n(N, [&](idx_t k) { gmuc[k] += t[k] / (s.mu[k] * s.mu[k]); });
        // irx = 1 / A2x(rho) (0 where invalid): d irx_r / d rho_k = -irx_r^2 A2x[r, k]; the same along y
        std::vector<T> grhoAvg(N, 0);
        for_n(N, [&](idx_t r) { y[r] = -gIrx[r] * s.invRhoX[r] * s.invRhoX[r]; });
        avgT([&](const T* in, T* out) { average2<T>(s.g, Axis::X, in, out); }, y, grhoAvg);
        for_n(N, [&](idx_t r) { y[r] = -gIry[r] * s.invRhoY[r] * s.invRhoY[r]; });
        avgT([&](const T* in, T* out) { average2<T>(s.g, Axis::Y, in, out); }, y, grhoAvg);
        // visco: M = rho vp^2 / (1 + sum tauP), mu = rho vs^2 / (1 + sum tauS)
        // (Viscoelastic.cpp:650-715), the relaxation times held fixed
        T sum = 0;
        if (visco) {
            const T w_ref = static_cast<T>(2.0 * M_PI * s.cfg.CenterFrequencyCPML);
            for (int l = 0; l < s.L; ++l) {
                const T ts = static_cast<T>(1.0 / (2.0 * M_PI * static_cast<T>(s.cfg.relaxationFrequency[l])));
                sum += w_ref * w_ref * ts * ts / (T(1.0) + w_ref * w_ref * ts * ts);
            }
        }
        for (idx_t k = 0; k < N; ++k) {
            // M = rho vp^2 / fP; mu_c = max(rho vs^2 / fS, 1) (clamped values do not move)
            const T fP = visco ? T(1) + sum * s.tauP[k] : T(1), fS = visco ? T(1) + sum * s.tauS[k] : T(1);
            T raw = rho[k];
            raw *= vs[k];
            raw *= vs[k];
            if (visco) raw = raw / fS;
            const bool unclamped = raw >= T(1);
            gvp[k] = gM[k] * T(2) * rho[k] * vp[k] / fP;
            gvs[k] = unclamped ? gmuc[k] * T(2) * rho[k] * vs[k] / fS : T(0);
            grho[k] = gM[k] * vp[k] * vp[k] / fP + (unclamped ? gmuc[k] * vs[k] * vs[k] / fS : T(0)) + grhoAvg[k];
        }
    }
};


// Discrete adjoint of the oracle's lossless 2-D TMz step (Sim<T>::stepTM,
// restating FD2Dtmem::run, ForwardSolver2Dtmem.cpp:108-174, with CPML and the
// ABS taper): the gradient of J = 1/2 sum (d - d_obs)^2 (Ez receivers) with
// respect to eps_r, sigma and mu_r. Per step, from X_t and X_{t+1}:
//   a1' = Dyf ez + P(ezy)   a2' = Dxf ez + P(ezx)
//   hx' = hx - iMyz a1'     hy' = hy + iMxz a2'          (before the taper)
//   c1' = Dxb hy' + P(hyx)  c2' = Dyb hx' + P(hxy)
//   ez  <- Ca ez + Cb (c1' - c2'), then the taper on ez, hx, hy
// with Ca = (1 - k) / (1 + k), Cb = (1 / eps) / (1 + k), k = sigma DT / (2 eps),
// eps = eps_r eps0 (TMEM.cpp:230-241, ForwardSolverEM.cpp:14-67) and
// iMxz, iMyz the inverse 2-point averages of mu = mu_r mu0 (TMEM.cpp:366-374).
template <class T>
struct TMAdjoint2D {
    Sim<T>& s;
    const idx_t N;
    CSR<T> DxfT, DxbT, DyfT, DybT;
    const bool visco;   // 2-D visco-TMz (FD2Dviscotmem::run, ForwardSolver2Dviscotmem.cpp:130-205)

    explicit TMAdjoint2D(Sim<T>& sim) : s(sim), N(sim.g.N()), visco(sim.eq == WAVE_EQ_VISCOTMEM)
    {
        if (s.is3d || (s.eq != WAVE_EQ_TMEM && s.eq != WAVE_EQ_VISCOTMEM)) throw std::invalid_argument("oracle adjoint: 2-D TMz only");
        DxfT = transpose(s.Dxf);
        DxbT = transpose(s.Dxb);
        DyfT = transpose(s.Dyf);
        DybT = transpose(s.Dyb);
    }
    struct State {
        std::map<std::string, std::vector<T>> F, psi;
        std::map<std::string, std::vector<std::vector<T>>> R;
    };
    const std::vector<T>& psiOf(const State& x, const char* n, const std::vector<T>& zero) const
    {
        auto it = x.psi.find(n);
        return it == x.psi.end() ? zero : it->second;
    }
    void cpmlT(std::vector<T>& lc, std::vector<T>& lp, const std::vector<T>& a, const std::vector<T>& b) const
    {
        if (!s.useCpml) return;
        for_n(N, [&](idx_t i) {
            const T c = (T(1) + a[i]) * lc[i] + a[i] * lp[i];
            lp[i] = b[i] * (lc[i] + lp[i]);
            lc[i] = c;
        });
    }

    double run(const std::vector<T>& epsr, const std::vector<T>& sigma, const std::vector<T>& mur, const T* dobs, int K,
               T* geps, T* gsig, T* gmu)
    {
        const int NT = s.NT;
        const size_t nrec = s.rec.idx.size();
        for (size_t r = 0; r < nrec; ++r)
            if (s.rec.type[r] != WAVE_TYPE_EZ) throw std::invalid_argument("oracle TMz adjoint: Ez receivers only");
        const std::vector<T> zero(N, T(0));
        s.reset();
        std::vector<State> ck;
        for (int t = 0; t < NT; ++t) {
            if (t % K == 0) ck.push_back({s.F, s.psi, s.R});
            s.step(t);
        }
        std::vector<T> res(nrec * static_cast<size_t>(NT));
        double J = 0;
        for (size_t k = 0; k < res.size(); ++k) {
            res[k] = s.seis[k] - dobs[k];
            J += 0.5 * static_cast<double>(res[k]) * static_cast<double>(res[k]);
        }
        std::vector<T> lhx(N, 0), lhy(N, 0), lez(N, 0);
        std::map<std::string, std::vector<T>> lp;
        for (const char* n : {"ezy", "ezx", "hyx", "hxy"}) lp[n].assign(N, 0);
        std::vector<T> gCa(N, 0), gCb(N, 0), gMxz(N, 0), gMyz(N, 0);
        // visco: adjoints of the memory variables rz_l and the material adjoints of Cd_l
        const int L = visco ? s.L : 0;
        std::vector<std::vector<T>> lR(L, std::vector<T>(N, 0)), gCd(L, std::vector<T>(N, 0));
        std::vector<T> a1(N), a2(N), c1(N), c2(N), hxp(N), hyp(N), la1(N), la2(N), lc1(N), lc2(N);
        const int nseg = static_cast<int>(ck.size());
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const int t0 = seg * K, t1 = std::min(NT, t0 + K);
            std::vector<State> X;
            s.F = ck[seg].F;
            s.psi = ck[seg].psi;
            s.R = ck[seg].R;
            X.push_back({s.F, s.psi, s.R});
            for (int t = t0; t < t1; ++t) {
                s.step(t);
                X.push_back({s.F, s.psi, s.R});
            }
            for (int t = t1 - 1; t >= t0; --t) {
                const State& X0 = X[t - t0];
                const State& X1 = X[t - t0 + 1];
                s.Dyf.spmv(X0.F.at("ez").data(), a1.data());
                s.Dxf.spmv(X0.F.at("ez").data(), a2.data());
                const auto& pezy = psiOf(X1, "ezy", zero);
                const auto& pezx = psiOf(X1, "ezx", zero);
                const auto& hx1 = X1.F.at("hx");
                const auto& hy1 = X1.F.at("hy");
                for_n(N, [&](idx_t i) {
                    a1[i] += pezy[i];
                    a2[i] += pezx[i];
                    const T d = s.useAbs ? s.damping[i] : T(1);
                    hxp[i] = hx1[i] / d;
                    hyp[i] = hy1[i] / d;
                });
                s.Dxb.spmv(hyp.data(), c1.data());
                s.Dyb.spmv(hxp.data(), c2.data());
                const auto& phyx = psiOf(X1, "hyx", zero);
                const auto& phxy = psiOf(X1, "hxy", zero);
                for_n(N, [&](idx_t i) { c1[i] += phyx[i]; c2[i] += phxy[i]; });
                for (size_t r = 0; r < nrec; ++r) lez[s.rec.idx[r]] += res[r * NT + t];
                if (s.useAbs)
                    for (auto* v : {&lez, &lhx, &lhy}) {
                        auto& w = *v;
                        for_n(N, [&](idx_t i) { w[i] *= s.damping[i]; });
                    }
                // ez <- Ca ez + Cb (c1' - c2' - DT sum_l rz_l'), rz_l' = Cc_l rz_l + Cd_l ez (visco)
                const auto& ez0 = X0.F.at("ez");
                for_n(N, [&](idx_t i) {
                    T u = c1[i] - c2[i];
                    for (int l = 0; l < L; ++l) u -= s.DT * X1.R.at("rz")[l][i];
                    lc1[i] = s.CbZ[i] * lez[i];
                    lc2[i] = -s.CbZ[i] * lez[i];
                    gCa[i] += lez[i] * ez0[i];
                    gCb[i] += lez[i] * u;
                    T ln = s.CaZ[i] * lez[i];
                    for (int l = 0; l < L; ++l) {
                        const T LR = lR[l][i] - s.DT * s.CbZ[i] * lez[i];   // adjoint of rz_l'
                        ln += s.CdZ[l][i] * LR;
                        gCd[l][i] += LR * ez0[i];
                        lR[l][i] = s.emCc[l] * LR;
                    }
                    lez[i] = ln;
                });
                cpmlT(lc1, lp["hyx"], s.ax, s.bx);
                cpmlT(lc2, lp["hxy"], s.ay, s.by);
                spmv_add(DxbT, lc1, lhy);
                spmv_add(DybT, lc2, lhx);
                // hx' = hx - iMyz a1', hy' = hy + iMxz a2'
                for_n(N, [&](idx_t i) {
                    la1[i] = -s.invMuYZ[i] * lhx[i];
                    la2[i] = s.invMuXZ[i] * lhy[i];
                    gMyz[i] -= lhx[i] * a1[i];
                    gMxz[i] += lhy[i] * a2[i];
                });
                cpmlT(la1, lp["ezy"], s.ayh, s.byh);
                cpmlT(la2, lp["ezx"], s.axh, s.bxh);
                spmv_add(DyfT, la1, lez);
                spmv_add(DxfT, la2, lez);
            }
        }
        // Ca, Cb -> eps, sigma; iMxz, iMyz -> mu
        const T eps0 = static_cast<T>(8.8541878176e-12), mu0 = static_cast<T>(1.2566370614e-6);
        const T DT = s.DT;
        // visco: Ca, Cb of the effective optical permittivity eo = max((1 - te) e + s ts, eps0)
        // and conductivity so = te sumInv e + s; Cd_l = -DT te cdScale_l e (ForwardSolverEM.cpp:68-152),
        // tau_eps (te) and tau_sigma (ts, times 1 / (2 pi f_CPML)) held fixed
        T sumInv = 0;
        std::vector<T> cdScale(L);
        if (visco) {
            for (int l = 0; l < L; ++l) {
                const double r = 1.0 / (2.0 * M_PI * static_cast<double>(static_cast<T>(s.cfg.relaxationFrequency[l])));
                const T rt = static_cast<T>(r);
                sumInv = static_cast<T>(static_cast<double>(sumInv) + 1.0 / static_cast<double>(rt));
                T tv = static_cast<T>(1 / (1 + 0.5 * static_cast<double>(DT) / static_cast<double>(rt)));
                tv /= (static_cast<T>(L) * rt * rt);
                cdScale[l] = tv;
            }
            sumInv /= static_cast<T>(L);
        }
        for (idx_t i = 0; i < N; ++i) {
            const T e0 = epsr[i] * eps0, sg0 = sigma[i];
            T e = e0, sg = sg0, de_de = 1, de_ds = 0, ds_de = 0, ds_ds = 1;
            if (visco) {
                const T te = s.emTauE[i], ts = s.emTauS[i];
                const T eo = (T(1) - te) * e0 + sg0 * ts;
                const bool clamp = eo < eps0;
                e = clamp ? eps0 : eo;
                de_de = clamp ? T(0) : T(1) - te;
                de_ds = clamp ? T(0) : ts;
                sg = te * sumInv * e0 + sg0;
                ds_de = te * sumInv;
            }
            const T k = sg * DT / (T(2) * e), q = T(1) + k;
            const T dCa_de = T(2) * k / (e * q * q), dCa_ds = -T(2) / (q * q) * DT / (T(2) * e);
            const T dCb_de = -T(1) / (e * e * q) + k / (e * e * q * q), dCb_ds = -(T(1) / e) / (q * q) * DT / (T(2) * e);
            const T gE = gCa[i] * dCa_de + gCb[i] * dCb_de, gS = gCa[i] * dCa_ds + gCb[i] * dCb_ds;
            T ge = gE * de_de + gS * ds_de, gs = gE * de_ds + gS * ds_ds;
            for (int l = 0; l < L; ++l) ge += gCd[l][i] * (-DT) * s.emTauE[i] * cdScale[l];
            geps[i] = eps0 * ge;
            gsig[i] = gs;
        }
        std::vector<T> y(N), gm(N, 0);
        AverageTranspose<T> probe(s);
        for_n(N, [&](idx_t r) { y[r] = -gMxz[r] * s.invMuXZ[r] * s.invMuXZ[r]; });
        probe.avgT([&](const T* in, T* out) { average2<T>(s.g, Axis::X, in, out); }, y, gm);
        for_n(N, [&](idx_t r) { y[r] = -gMyz[r] * s.invMuYZ[r] * s.invMuYZ[r]; });
        probe.avgT([&](const T* in, T* out) { average2<T>(s.g, Axis::Y, in, out); }, y, gm);
        for (idx_t i = 0; i < N; ++i) gmu[i] = gm[i] * mu0;
        (void)mur;
        return J;
    }
};

// Discrete adjoint of the oracle's 2-D SH step (Sim<T>::stepSH, restating
// FD2Dsh::run, ForwardSolver2Dsh.cpp:108-196, with CPML, the ABS taper and the
// free surface's image operator on syz): the gradient of J = 1/2 sum
// (d - d_obs)^2 (vz receivers) with respect to vs and rho. Per step, from X_t
// and X_{t+1}:
//   a1' = Dxb sxz + P(sxz_x)   a2' = DybS syz + P(syz_y)
//   vz' = vz + irho (a1' + a2')                        (before the taper)
//   c1' = Dxf vz' + P(vzx)     c2' = Dyf vz' + P(vzy)
//   sxz <- sxz + muXZ c1',  syz <- syz + muYZ c2', then the taper on sxz, syz, vz
// with irho = 1 / rho and muXZ, muYZ the harmonic 2-point averages of
// mu = max(rho vs^2, 1) along x and y (0 below 4; SH.cpp:424-431,
// ModelparameterSeismic.cpp:421-432).
template <class T>
struct SHAdjoint2D {
    Sim<T>& s;
    const idx_t N;
    CSR<T> DxfT, DxbT, DyfT, DybST;
    const bool visco;   // 2-D visco-SH (FD2Dviscosh::run, ForwardSolver2Dviscosh.cpp:126-244)

    explicit SHAdjoint2D(Sim<T>& sim) : s(sim), N(sim.g.N()), visco(sim.eq == WAVE_EQ_VISCOSH)
    {
        if (s.is3d || (s.eq != WAVE_EQ_SH && s.eq != WAVE_EQ_VISCOSH)) throw std::invalid_argument("oracle adjoint: 2-D SH only");
        DxfT = transpose(s.Dxf);
        DxbT = transpose(s.Dxb);
        DyfT = transpose(s.Dyf);
        DybST = transpose(s.fs ? s.DybFS : s.Dyb);
    }
    struct State {
        std::map<std::string, std::vector<T>> F, psi;
        std::map<std::string, std::vector<std::vector<T>>> R;
    };
    const std::vector<T>& psiOf(const State& x, const char* n, const std::vector<T>& zero) const
    {
        auto it = x.psi.find(n);
        return it == x.psi.end() ? zero : it->second;
    }
    void cpmlT(std::vector<T>& lc, std::vector<T>& lp, const std::vector<T>& a, const std::vector<T>& b) const
    {
        if (!s.useCpml) return;
        for_n(N, [&](idx_t i) {
            const T c = (T(1) + a[i]) * lc[i] + a[i] * lp[i];
            lp[i] = b[i] * (lc[i] + lp[i]);
            lc[i] = c;
        });
    }

    double run(const std::vector<T>& vs, const std::vector<T>& rho, const T* dobs, int K, T* gvs, T* grho)
    {
        const int NT = s.NT;
        const size_t nrec = s.rec.idx.size();
        for (size_t r = 0; r < nrec; ++r)
            if (s.rec.type[r] != WAVE_TYPE_VZ) throw std::invalid_argument("oracle SH adjoint: vz receivers only");
        const std::vector<T> zero(N, T(0));
        s.reset();
        std::vector<State> ck;
        for (int t = 0; t < NT; ++t) {
            if (t % K == 0) ck.push_back({s.F, s.psi, s.R});
            s.step(t);
        }
        std::vector<T> res(nrec * static_cast<size_t>(NT));
        double J = 0;
        for (size_t k = 0; k < res.size(); ++k) {
            res[k] = s.seis[k] - dobs[k];
            J += 0.5 * static_cast<double>(res[k]) * static_cast<double>(res[k]);
        }
        std::vector<T> lvz(N, 0), lxz(N, 0), lyz(N, 0);
        std::map<std::string, std::vector<T>> lp;
        for (const char* n : {"sxz_x", "syz_y", "vzx", "vzy"}) lp[n].assign(N, 0);
        std::vector<T> gMuXZ(N, 0), gMuYZ(N, 0), gIr(N, 0);
        // adjoint memory variables rxz, ryz per mechanism (visco-SH)
        std::vector<std::vector<std::vector<T>>> lR(2, std::vector<std::vector<T>>(visco ? s.L : 0, std::vector<T>(N, 0)));
        std::vector<T> a1(N), a2(N), c1(N), c2(N), vzp(N), la1(N), la2(N), lc1(N), lc2(N);
        const int nseg = static_cast<int>(ck.size());
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const int t0 = seg * K, t1 = std::min(NT, t0 + K);
            std::vector<State> X;
            s.F = ck[seg].F;
            s.psi = ck[seg].psi;
            s.R = ck[seg].R;
            X.push_back({s.F, s.psi, s.R});
            for (int t = t0; t < t1; ++t) {
                s.step(t);
                X.push_back({s.F, s.psi, s.R});
            }
            for (int t = t1 - 1; t >= t0; --t) {
                const State& X0 = X[t - t0];
                const State& X1 = X[t - t0 + 1];
                s.Dxb.spmv(X0.F.at("sxz").data(), a1.data());
                (s.fs ? s.DybFS : s.Dyb).spmv(X0.F.at("syz").data(), a2.data());
                const auto& p1 = psiOf(X1, "sxz_x", zero);
                const auto& p2 = psiOf(X1, "syz_y", zero);
                const auto& vz0 = X0.F.at("vz");
                for_n(N, [&](idx_t i) {
                    a1[i] += p1[i];
                    a2[i] += p2[i];
                    vzp[i] = vz0[i] + s.invRho[i] * (a1[i] + a2[i]);
                });
                s.Dxf.spmv(vzp.data(), c1.data());
                s.Dyf.spmv(vzp.data(), c2.data());
                const auto& q1 = psiOf(X1, "vzx", zero);
                const auto& q2 = psiOf(X1, "vzy", zero);
                for_n(N, [&](idx_t i) { c1[i] += q1[i]; c2[i] += q2[i]; });
                // receivers read X_{t+1}
                for (size_t r = 0; r < nrec; ++r) lvz[s.rec.idx[r]] += res[r * NT + t];
                if (s.useAbs)
                    for (auto* v : {&lxz, &lyz, &lvz}) {
                        auto& w = *v;
                        for_n(N, [&](idx_t i) { w[i] *= s.damping[i]; });
                    }
                // sxz += muXZ c1', syz += muYZ c2'; visco-SH, per mechanism l with m = mu_k c':
                // Rk' = c2_l (c1_l Rk - tauS_k m / tau_l), Sk' = Sk + DT/2 sum_l (Rk + Rk') + (1 + L tauS) m
                for_n(N, [&](idx_t i) {
                    T lm[2] = {lxz[i], lyz[i]};
                    if (visco) {
                        const T tS[2] = {s.tauSXZ[i], s.tauSYZ[i]};
                        for (int q = 0; q < 2; ++q) {
                            const T lS = lm[q];
                            lm[q] = s.onePlusLtauS[i] * lS;
                            for (int l = 0; l < s.L; ++l) {
                                const T cc1 = s.viscoC1[l], cc2 = s.viscoC2[l], irt = s.invRelaxTime[l];
                                const T LR = lR[q][l][i] + s.DThalf * lS;
                                lR[q][l][i] = cc2 * cc1 * LR + s.DThalf * lS;
                                lm[q] -= cc2 * irt * tS[q] * LR;
                            }
                        }
                    }
                    lc1[i] = s.muXZ[i] * lm[0];
                    lc2[i] = s.muYZ[i] * lm[1];
                    gMuXZ[i] += lm[0] * c1[i];
                    gMuYZ[i] += lm[1] * c2[i];
                });
                cpmlT(lc1, lp["vzx"], s.axh, s.bxh);
                cpmlT(lc2, lp["vzy"], s.ayh, s.byh);
                spmv_add(DxfT, lc1, lvz);
                spmv_add(DyfT, lc2, lvz);
                // vz' = vz + irho (a1' + a2')
                for_n(N, [&](idx_t i) {
                    la1[i] = la2[i] = s.invRho[i] * lvz[i];
                    gIr[i] += lvz[i] * (a1[i] + a2[i]);
                });
                cpmlT(la1, lp["sxz_x"], s.ax, s.bx);
                cpmlT(la2, lp["syz_y"], s.ay, s.by);
                spmv_add(DxbT, la1, lxz);
                spmv_add(DybST, la2, lyz);
            }
        }
        // muXZ = 1 / A2x(1 / mu) (0 below 4): d muXZ_r / d mu_k = muXZ_r^2 A2x[r, k] / mu_k^2; the same along y
        std::vector<T> y(N), gmu(N, 0);
        AverageTranspose<T> probe(s);
        for_n(N, [&](idx_t r) { y[r] = gMuXZ[r] * s.muXZ[r] * s.muXZ[r]; });
        probe.avgT([&](const T* in, T* out) { average2<T>(s.g, Axis::X, in, out); }, y, gmu);
        for_n(N, [&](idx_t r) { y[r] = gMuYZ[r] * s.muYZ[r] * s.muYZ[r]; });
        probe.avgT([&](const T* in, T* out) { average2<T>(s.g, Axis::Y, in, out); }, y, gmu);
        // visco-SH: mu = rho vs^2 / (1 + sum tauS) with the relaxation times fixed
        T sum = 0;
        if (visco) {
            const T w_ref = static_cast<T>(2.0 * M_PI * s.cfg.CenterFrequencyCPML);
            for (int l = 0; l < s.L; ++l) {
                const T ts = static_cast<T>(1.0 / (2.0 * M_PI * static_cast<T>(s.cfg.relaxationFrequency[l])));
                sum += w_ref * w_ref * ts * ts / (T(1.0) + w_ref * w_ref * ts * ts);
            }
        }
        for (idx_t k = 0; k < N; ++k) {
            // mu = max(rho vs^2 / fS, 1) (clamped values do not move); irho = 1 / rho
            const T fS = visco ? T(1) + sum * s.tauS[k] : T(1);
            T raw = rho[k];
            raw *= vs[k];
            raw *= vs[k];
            if (visco) raw = raw / fS;
            const bool unclamped = raw >= T(1);
            const T gm = gmu[k] / (s.mu[k] * s.mu[k]);
            gvs[k] = unclamped ? gm * T(2) * rho[k] * vs[k] / fS : T(0);
            grho[k] = (unclamped ? gm * vs[k] * vs[k] / fS : T(0)) - gIr[k] * s.invRho[k] * s.invRho[k];
        }
        return J;
    }
};

// Discrete adjoint of the oracle's lossless 2-D TEz step (Sim<T>::stepTE,
// restating FD2Demem::run, ForwardSolver2Demem.cpp:112-185, with CPML and the
// ABS taper): the gradient of J = 1/2 sum (d - d_obs)^2 (Ex, Ey and Hz
// receivers) with respect to eps_r, sigma and mu_r. Per step, from X_t and
// X_{t+1}:
//   a1' = Dxf ey + P(eyx)   a2' = Dyf ex + P(exy)
//   hz' = hz - iMxy (a1' - a2')                          (before the taper)
//   c1' = Dyb hz' + P(hzy)  c2' = Dxb hz' + P(hzx)
//   ex <- CaX ex + CbX c1',  ey <- CaY ey - CbY c2', then the taper on ey, ex, hz
// with CaX, CbX of the 2-point x averages of eps = eps_r eps0 and sigma (CaY,
// CbY along y; ForwardSolverEM.cpp:14-67, EMEM.cpp:378-392) and iMxy the
// inverse 4-point average of mu = mu_r mu0.
template <class T>
struct TEAdjoint2D {
    Sim<T>& s;
    const idx_t N;
    CSR<T> DxfT, DxbT, DyfT, DybT;
    const bool visco;   // 2-D visco-TEz (FD2Dviscoemem::run, ForwardSolver2Dviscoemem.cpp:142-228)

    explicit TEAdjoint2D(Sim<T>& sim) : s(sim), N(sim.g.N()), visco(sim.eq == WAVE_EQ_VISCOEMEM)
    {
        if (s.is3d || (s.eq != WAVE_EQ_EMEM && s.eq != WAVE_EQ_VISCOEMEM)) throw std::invalid_argument("oracle adjoint: 2-D TEz only");
        DxfT = transpose(s.Dxf);
        DxbT = transpose(s.Dxb);
        DyfT = transpose(s.Dyf);
        DybT = transpose(s.Dyb);
    }
    struct State {
        std::map<std::string, std::vector<T>> F, psi;
        std::map<std::string, std::vector<std::vector<T>>> R;
    };
    const std::vector<T>& psiOf(const State& x, const char* n, const std::vector<T>& zero) const
    {
        auto it = x.psi.find(n);
        return it == x.psi.end() ? zero : it->second;
    }
    void cpmlT(std::vector<T>& lc, std::vector<T>& lp, const std::vector<T>& a, const std::vector<T>& b) const
    {
        if (!s.useCpml) return;
        for_n(N, [&](idx_t i) {
            const T c = (T(1) + a[i]) * lc[i] + a[i] * lp[i];
            lp[i] = b[i] * (lc[i] + lp[i]);
            lc[i] = c;
        });
    }

    double run(const std::vector<T>& epsr, const std::vector<T>& sigma, const std::vector<T>& mur, const T* dobs, int K,
               T* geps, T* gsig, T* gmu)
    {
        const int NT = s.NT;
        const size_t nrec = s.rec.idx.size();
        const std::vector<T> zero(N, T(0));
        s.reset();
        std::vector<State> ck;
        for (int t = 0; t < NT; ++t) {
            if (t % K == 0) ck.push_back({s.F, s.psi, s.R});
            s.step(t);
        }
        std::vector<T> res(nrec * static_cast<size_t>(NT));
        double J = 0;
        for (size_t k = 0; k < res.size(); ++k) {
            res[k] = s.seis[k] - dobs[k];
            J += 0.5 * static_cast<double>(res[k]) * static_cast<double>(res[k]);
        }
        std::vector<T> lhz(N, 0), lex(N, 0), ley(N, 0);
        std::map<std::string, std::vector<T>> lp;
        for (const char* n : {"eyx", "exy", "hzy", "hzx"}) lp[n].assign(N, 0);
        std::vector<T> gCaX(N, 0), gCbX(N, 0), gCaY(N, 0), gCbY(N, 0), gMxy(N, 0);
        // visco: adjoints of the memory variables rx_l, ry_l and of Cd_x,l, Cd_y,l
        const int L = visco ? s.L : 0;
        std::vector<std::vector<T>> lR[2], gCd[2];
        for (int q = 0; q < 2; ++q) { lR[q].assign(L, std::vector<T>(N, 0)); gCd[q].assign(L, std::vector<T>(N, 0)); }
        std::vector<T> a1(N), a2(N), c1(N), c2(N), hzp(N), la1(N), la2(N), lc1(N), lc2(N);
        const int nseg = static_cast<int>(ck.size());
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const int t0 = seg * K, t1 = std::min(NT, t0 + K);
            std::vector<State> X;
            s.F = ck[seg].F;
            s.psi = ck[seg].psi;
            s.R = ck[seg].R;
            X.push_back({s.F, s.psi, s.R});
            for (int t = t0; t < t1; ++t) {
                s.step(t);
                X.push_back({s.F, s.psi, s.R});
            }
            for (int t = t1 - 1; t >= t0; --t) {
                const State& X0 = X[t - t0];
                const State& X1 = X[t - t0 + 1];
                const auto& ex0 = X0.F.at("ex");
                const auto& ey0 = X0.F.at("ey");
                const auto& hz0 = X0.F.at("hz");
                s.Dxf.spmv(ey0.data(), a1.data());
                s.Dyf.spmv(ex0.data(), a2.data());
                const auto& peyx = psiOf(X1, "eyx", zero);
                const auto& pexy = psiOf(X1, "exy", zero);
                for_n(N, [&](idx_t i) {
                    a1[i] += peyx[i];
                    a2[i] += pexy[i];
                    hzp[i] = hz0[i] - s.invMuXY[i] * (a1[i] - a2[i]);
                });
                s.Dyb.spmv(hzp.data(), c1.data());
                s.Dxb.spmv(hzp.data(), c2.data());
                const auto& phzy = psiOf(X1, "hzy", zero);
                const auto& phzx = psiOf(X1, "hzx", zero);
                for_n(N, [&](idx_t i) { c1[i] += phzy[i]; c2[i] += phzx[i]; });
                for (size_t r = 0; r < nrec; ++r) {
                    const idx_t i = s.rec.idx[r];
                    const T v = res[r * NT + t];
                    switch (s.rec.type[r]) {
                    case WAVE_TYPE_EX: lex[i] += v; break;
                    case WAVE_TYPE_EY: ley[i] += v; break;
                    case WAVE_TYPE_HZ: lhz[i] += v; break;
                    default: throw std::invalid_argument("oracle TEz adjoint: Ex, Ey and Hz receivers only");
                    }
                }
                if (s.useAbs)
                    for (auto* v : {&ley, &lex, &lhz}) {
                        auto& w = *v;
                        for_n(N, [&](idx_t i) { w[i] *= s.damping[i]; });
                    }
                // ex <- CaX ex + CbX (c1' - DT sum_l rx_l'), ey <- CaY ey + CbY (-c2' - DT sum_l ry_l'),
                // r_l' = Cc_l r_l + Cd_l e (visco)
                for_n(N, [&](idx_t i) {
                    T ux = c1[i], uy = -c2[i];
                    for (int l = 0; l < L; ++l) {
                        ux -= s.DT * X1.R.at("rx")[l][i];
                        uy -= s.DT * X1.R.at("ry")[l][i];
                    }
                    lc1[i] = s.CbX[i] * lex[i];
                    lc2[i] = -s.CbY[i] * ley[i];
                    gCaX[i] += lex[i] * ex0[i];
                    gCbX[i] += lex[i] * ux;
                    gCaY[i] += ley[i] * ey0[i];
                    gCbY[i] += ley[i] * uy;
                    T nx = s.CaX[i] * lex[i], ny = s.CaY[i] * ley[i];
                    for (int l = 0; l < L; ++l) {
                        const T LX = lR[0][l][i] - s.DT * s.CbX[i] * lex[i], LY = lR[1][l][i] - s.DT * s.CbY[i] * ley[i];
                        nx += s.CdX[l][i] * LX;
                        ny += s.CdY[l][i] * LY;
                        gCd[0][l][i] += LX * ex0[i];
                        gCd[1][l][i] += LY * ey0[i];
                        lR[0][l][i] = s.emCc[l] * LX;
                        lR[1][l][i] = s.emCc[l] * LY;
                    }
                    lex[i] = nx;
                    ley[i] = ny;
                });
                cpmlT(lc1, lp["hzy"], s.ay, s.by);
                cpmlT(lc2, lp["hzx"], s.ax, s.bx);
                spmv_add(DybT, lc1, lhz);
                spmv_add(DxbT, lc2, lhz);
                // hz' = hz - iMxy (a1' - a2')
                for_n(N, [&](idx_t i) {
                    la1[i] = -s.invMuXY[i] * lhz[i];
                    la2[i] = s.invMuXY[i] * lhz[i];
                    gMxy[i] -= lhz[i] * (a1[i] - a2[i]);
                });
                cpmlT(la1, lp["eyx"], s.axh, s.bxh);
                cpmlT(la2, lp["exy"], s.ayh, s.byh);
                spmv_add(DxfT, la1, ley);
                spmv_add(DyfT, la2, lex);
            }
        }
        // CaX, CbX -> the x averages of eps and sigma -> eps_r, sigma (the same along y)
        const T eps0 = static_cast<T>(8.8541878176e-12), mu0 = static_cast<T>(1.2566370614e-6);
        const T DT = s.DT;
        std::vector<T> eps(N), ge(N, 0), gs(N, 0), ye(N), ys(N), avE(N), avS(N);
        for (idx_t i = 0; i < N; ++i) eps[i] = epsr[i] * eps0;
        AverageTranspose<T> probe(s);
        // visco: Ca, Cb of the effective optical permittivity and conductivity of the averaged
        // eps, sigma, tau_eps, tau_sigma; Cd_l = -DT te cdScale_l e (ForwardSolverEM.cpp:68-152)
        T sumInv = 0;
        std::vector<T> cdScale(L), avTe(N), avTs(N);
        for (int l = 0; l < L; ++l) {
            const double r = 1.0 / (2.0 * M_PI * static_cast<double>(static_cast<T>(s.cfg.relaxationFrequency[l])));
            const T rt = static_cast<T>(r);
            sumInv = static_cast<T>(static_cast<double>(sumInv) + 1.0 / static_cast<double>(rt));
            T tv = static_cast<T>(1 / (1 + 0.5 * static_cast<double>(DT) / static_cast<double>(rt)));
            tv /= (static_cast<T>(L) * rt * rt);
            cdScale[l] = tv;
        }
        if (L > 0) sumInv /= static_cast<T>(L);
        for (Axis a : {Axis::X, Axis::Y}) {
            average2<T>(s.g, a, eps.data(), avE.data());
            average2<T>(s.g, a, sigma.data(), avS.data());
            if (visco) {
                average2<T>(s.g, a, s.emTauE.data(), avTe.data());
                average2<T>(s.g, a, s.emTauS.data(), avTs.data());
            }
            const std::vector<T>& gCa = a == Axis::X ? gCaX : gCaY;
            const std::vector<T>& gCb = a == Axis::X ? gCbX : gCbY;
            const auto& gCdA = gCd[a == Axis::X ? 0 : 1];
            for (idx_t i = 0; i < N; ++i) {
                T e = avE[i], sg = avS[i], de_de = 1, de_ds = 0, ds_de = 0;
                if (visco) {
                    const T te = avTe[i], ts = avTs[i];
                    const T eo = (T(1) - te) * avE[i] + avS[i] * ts;
                    const bool clamp = eo < eps0;
                    e = clamp ? eps0 : eo;
                    de_de = clamp ? T(0) : T(1) - te;
                    de_ds = clamp ? T(0) : ts;
                    sg = te * sumInv * avE[i] + avS[i];
                    ds_de = te * sumInv;
                }
                const T k = sg * DT / (T(2) * e), q = T(1) + k;
                const T dCa_de = T(2) * k / (e * q * q), dCa_ds = -T(2) / (q * q) * DT / (T(2) * e);
                const T dCb_de = -T(1) / (e * e * q) + k / (e * e * q * q), dCb_ds = -(T(1) / e) / (q * q) * DT / (T(2) * e);
                const T gE = gCa[i] * dCa_de + gCb[i] * dCb_de, gS = gCa[i] * dCa_ds + gCb[i] * dCb_ds;
                ye[i] = gE * de_de + gS * ds_de;
                ys[i] = gE * de_ds + gS;
                for (int l = 0; l < L; ++l) ye[i] += gCdA[l][i] * (-DT) * avTe[i] * cdScale[l];
            }
            probe.avgT([&](const T* in, T* out) { average2<T>(s.g, a, in, out); }, ye, ge);
            probe.avgT([&](const T* in, T* out) { average2<T>(s.g, a, in, out); }, ys, gs);
        }
        std::vector<T> y(N), gm(N, 0);
        for_n(N, [&](idx_t r) { y[r] = -gMxy[r] * s.invMuXY[r] * s.invMuXY[r]; });
        probe.avgT([&](const T* in, T* out) { average4<T>(s.g, 0, in, out); }, y, gm);
        for (idx_t i = 0; i < N; ++i) {
            geps[i] = eps0 * ge[i];
            gsig[i] = gs[i];
            gmu[i] = mu0 * gm[i];
        }
        (void)mur;
        return J;
    }
};

// Discrete adjoint of the oracle's 3-D elastic step (Sim<T>::stepElastic,
// restating FD3Delastic::run, ForwardSolver3Delastic.cpp:120-414, with CPML
// CPML3D.cpp:31-371, the free surface FreeSurface3Delastic.cpp:15-47 and the
// ABS taper ABS3D.cpp:14-60): the gradient of J = 1/2 sum (d - d_obs)^2 with
// respect to vp, vs and rho. Per step, from X_t and X_{t+1}:
//   a0' = Dxf sxx  a1' = DybS sxy  a2' = Dzb sxz  -> vx' = vx + irx (a0' + a1' + a2')
//   a3' = Dxb sxy  a4' = DyfS syy  a5' = Dzb syz  -> vy' = vy + iry (a3' + a4' + a5')
//   a6' = Dxb sxz  a7' = DybS syz  a8' = Dzf szz  -> vz' = vz + irz (a6' + a7' + a8')
//   c0' = Dxb vx'  c1' = Dyb vy'  c2' = Dzb vz'    (normal stresses with M and 2 mu)
//   c3' = Dyf vx'  c4' = Dxf vy' (sxy, muXY)  c5' = Dzf vx'  c6' = Dxf vz' (sxz, muXZ)
//   c7' = Dzf vy'  c8' = Dyf vz' (syz, muYZ)
// each with its psi of X_{t+1}; then at y = 0 with the free surface syy' = 0,
// sxx' and szz' += sh (c0' + c2') - sv c1' (sv = M - 2 mu, sh = -sv^2 / M), then
// the taper on all nine fields.
template <class T>
struct ElasticAdjoint3D {
    Sim<T>& s;
    const idx_t N;
    CSR<T> DxfT, DxbT, DyfT, DybT, DzfT, DzbT, DyfST, DybST;
    static constexpr const char* kP[9] = {"sxx_x", "sxy_y", "sxz_z", "sxy_x", "syy_y", "syz_z", "sxz_x", "syz_y", "szz_z"};
    static constexpr const char* kQ[9] = {"vxx", "vyy", "vzz", "vxy", "vyx", "vxz", "vzx", "vyz", "vzy"};

    const bool visco;   // 3-D visco-elastic (FD3Dviscoelastic::run, ForwardSolver3Dviscoelastic.cpp:132-457)

    explicit ElasticAdjoint3D(Sim<T>& sim) : s(sim), N(sim.g.N()), visco(sim.eq == WAVE_EQ_VISCOELASTIC)
    {
        if (!s.is3d || (s.eq != WAVE_EQ_ELASTIC && s.eq != WAVE_EQ_VISCOELASTIC))
            throw std::invalid_argument("oracle adjoint: 3-D elastic or visco-elastic only");
        DxfT = transpose(s.Dxf);
        DxbT = transpose(s.Dxb);
        DyfT = transpose(s.Dyf);
        DybT = transpose(s.Dyb);
        DzfT = transpose(s.Dzf);
        DzbT = transpose(s.Dzb);
        DyfST = transpose(s.fs ? s.DyfFS : s.Dyf);
        DybST = transpose(s.fs ? s.DybFS : s.Dyb);
    }
    struct State {
        std::map<std::string, std::vector<T>> F, psi;
        std::map<std::string, std::vector<std::vector<T>>> R;
    };
    const std::vector<T>& psiOf(const State& x, const char* n, const std::vector<T>& zero) const
    {
        auto it = x.psi.find(n);
        return it == x.psi.end() ? zero : it->second;
    }
    // (a, b) profile of a psi array: forward derivatives on the half grid
    std::pair<const std::vector<T>*, const std::vector<T>*> prof(const std::string& n) const
    {
        if (n == "sxx_x" || n == "vyx" || n == "vzx") return {&s.axh, &s.bxh};
        if (n == "sxy_x" || n == "sxz_x" || n == "vxx") return {&s.ax, &s.bx};
        if (n == "syy_y" || n == "vxy" || n == "vzy") return {&s.ayh, &s.byh};
        if (n == "sxy_y" || n == "syz_y" || n == "vyy") return {&s.ay, &s.by};
        if (n == "szz_z" || n == "vxz" || n == "vyz") return {&s.azh, &s.bzh};
        return {&s.az, &s.bz};   // sxz_z, syz_z, vzz
    }
    void cpmlT(std::vector<T>& lc, std::vector<T>& lp, const char* n) const
    {
        if (!s.useCpml) return;
        auto ab = prof(n);
        const std::vector<T>& a = *ab.first;
        const std::vector<T>& b = *ab.second;
        for_n(N, [&](idx_t i) {
            const T c = (T(1) + a[i]) * lc[i] + a[i] * lp[i];
            lp[i] = b[i] * (lc[i] + lp[i]);
            lc[i] = c;
        });
    }

    double run(const std::vector<T>& vp, const std::vector<T>& vs, const std::vector<T>& rho, const T* dobs, int K,
               T* gvp, T* gvs, T* grho)
    {
        const int NT = s.NT;
        const size_t nrec = s.rec.idx.size();
        const std::vector<T> zero(N, T(0));
        s.reset();
        std::vector<State> ck;
        for (int t = 0; t < NT; ++t) {
            if (t % K == 0) ck.push_back({s.F, s.psi, s.R});
            s.step(t);
        }
        std::vector<T> res(nrec * static_cast<size_t>(NT));
        double J = 0;
        for (size_t k = 0; k < res.size(); ++k) {
            res[k] = s.seis[k] - dobs[k];
            J += 0.5 * static_cast<double>(res[k]) * static_cast<double>(res[k]);
        }
        std::map<std::string, std::vector<T>> lF, lpsi;
        for (const char* n : {"vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz"}) lF[n].assign(N, 0);
        for (int k = 0; k < 9; ++k) { lpsi[kP[k]].assign(N, 0); lpsi[kQ[k]].assign(N, 0); }
        std::vector<T> gM(N, 0), gMu(N, 0), gMuXY(N, 0), gMuXZ(N, 0), gMuYZ(N, 0), gIrx(N, 0), gIry(N, 0), gIrz(N, 0);
        // adjoint memory variables rxx, ryy, rzz, rxy, rxz, ryz per mechanism (visco)
        std::vector<std::vector<std::vector<T>>> lR(6, std::vector<std::vector<T>>(visco ? s.L : 0, std::vector<T>(N, 0)));
        std::vector<T> a[9], c[9], la[9], lc[9], vxp(N), vyp(N), vzp(N);
        for (int k = 0; k < 9; ++k) { a[k].assign(N, 0); c[k].assign(N, 0); la[k].assign(N, 0); lc[k].assign(N, 0); }
        const CSR<T>& DybS = s.fs ? s.DybFS : s.Dyb;
        const CSR<T>& DyfS = s.fs ? s.DyfFS : s.Dyf;
        const int nseg = static_cast<int>(ck.size());
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const int t0 = seg * K, t1 = std::min(NT, t0 + K);
            std::vector<State> X;
            s.F = ck[seg].F;
            s.psi = ck[seg].psi;
            s.R = ck[seg].R;
            X.push_back({s.F, s.psi, s.R});
            for (int t = t0; t < t1; ++t) {
                s.step(t);
                X.push_back({s.F, s.psi, s.R});
            }
            for (int t = t1 - 1; t >= t0; --t) {
                const State& X0 = X[t - t0];
                const State& X1 = X[t - t0 + 1];
                auto f0 = [&](const char* n) { return X0.F.at(n).data(); };
                s.Dxf.spmv(f0("sxx"), a[0].data());
                DybS.spmv(f0("sxy"), a[1].data());
                s.Dzb.spmv(f0("sxz"), a[2].data());
                s.Dxb.spmv(f0("sxy"), a[3].data());
                DyfS.spmv(f0("syy"), a[4].data());
                s.Dzb.spmv(f0("syz"), a[5].data());
                s.Dxb.spmv(f0("sxz"), a[6].data());
                DybS.spmv(f0("syz"), a[7].data());
                s.Dzf.spmv(f0("szz"), a[8].data());
                for (int k = 0; k < 9; ++k) {
                    const std::vector<T>& p = psiOf(X1, kP[k], zero);
                    for_n(N, [&](idx_t i) { a[k][i] += p[i]; });
                }
                const auto& vx0 = X0.F.at("vx");
                const auto& vy0 = X0.F.at("vy");
                const auto& vz0 = X0.F.at("vz");
                for_n(N, [&](idx_t i) {
                    vxp[i] = vx0[i] + s.invRhoX[i] * (a[0][i] + a[1][i] + a[2][i]);
                    vyp[i] = vy0[i] + s.invRhoY[i] * (a[3][i] + a[4][i] + a[5][i]);
                    vzp[i] = vz0[i] + s.invRhoZ[i] * (a[6][i] + a[7][i] + a[8][i]);
                });
                s.Dxb.spmv(vxp.data(), c[0].data());
                s.Dyb.spmv(vyp.data(), c[1].data());
                s.Dzb.spmv(vzp.data(), c[2].data());
                s.Dyf.spmv(vxp.data(), c[3].data());
                s.Dxf.spmv(vyp.data(), c[4].data());
                s.Dzf.spmv(vxp.data(), c[5].data());
                s.Dxf.spmv(vzp.data(), c[6].data());
                s.Dzf.spmv(vyp.data(), c[7].data());
                s.Dyf.spmv(vzp.data(), c[8].data());
                for (int k = 0; k < 9; ++k) {
                    const std::vector<T>& q = psiOf(X1, kQ[k], zero);
                    for_n(N, [&](idx_t i) { c[k][i] += q[i]; });
                }
                // receivers read X_{t+1}: a pressure trace is (sxx + syy + szz) / 3
                for (size_t r = 0; r < nrec; ++r) {
                    const idx_t i = s.rec.idx[r];
                    const T v = res[r * NT + t];
                    switch (s.rec.type[r]) {
                    case WAVE_TYPE_P:
                        lF["sxx"][i] += v / T(3);
                        lF["syy"][i] += v / T(3);
                        lF["szz"][i] += v / T(3);
                        break;
                    case WAVE_TYPE_VX: lF["vx"][i] += v; break;
                    case WAVE_TYPE_VY: lF["vy"][i] += v; break;
                    default: lF["vz"][i] += v; break;
                    }
                }
                auto& lvx = lF["vx"];
                auto& lvy = lF["vy"];
                auto& lvz = lF["vz"];
                auto& lxx = lF["sxx"];
                auto& lyy = lF["syy"];
                auto& lzz = lF["szz"];
                auto& lxy = lF["sxy"];
                auto& lxz = lF["sxz"];
                auto& lyz = lF["syz"];
                if (s.useAbs)
                    for (auto* v : {&lxx, &lyy, &lzz, &lxy, &lxz, &lyz, &lvx, &lvy, &lvz}) {
                        auto& w = *v;
                        for_n(N, [&](idx_t i) { w[i] *= s.damping[i]; });
                    }
                for (int k = 0; k < 9; ++k) std::fill(lc[k].begin(), lc[k].end(), T(0));
                if (s.fs && !visco) {
                    // syy *= fsZero; sxx, szz += scaleH (c0' + c2') - scaleV c1'
                    for_n(N, [&](idx_t i) {
                        lyy[i] *= s.fsZero[i];
                        const T hs = lxx[i] + lzz[i];
                        lc[0][i] += s.scaleH[i] * hs;
                        lc[2][i] += s.scaleH[i] * hs;
                        lc[1][i] -= s.scaleV[i] * hs;
                        const T sel = s.fsSelect[i];
                        if (sel != T(0)) {
                            const T gH = hs * (c[0][i] + c[2][i]), gV = -hs * c[1][i];
                            const T sv = s.M[i] - T(2) * s.mu[i];
                            gM[i] += gV * sel - gH * sel * (T(2) * sv / s.M[i] - sv * sv / (s.M[i] * s.M[i]));
                            gMu[i] += -T(2) * gV * sel + gH * sel * T(4) * sv / s.M[i];
                        }
                    });
                }
                if (visco) {
                    // per mechanism l, with e = c0' + c1' + c2' and q the normal stress's
                    // partner sum (c1' + c2', c0' + c2', c0' + c1'), and for the shear
                    // stresses m = mu_plane (its two cross derivatives):
                    //   Rk' = c2_l (c1_l Rk - tauP M e / tau_l + tauS 2 mu q / tau_l)
                    //   Sk' = Sk + DT/2 sum_l (Rk + Rk') + (1 + L tauP) M e - (1 + L tauS) 2 mu q
                    //   Rs' = c2_l (c1_l Rs - tauS_plane m / tau_l), Ss' = Ss + DT/2 sum_l (Rs + Rs') + (1 + L tauS) m
                    const T DTh = s.DThalf;
                    for_n(N, [&](idx_t i) {
                        const T e = c[0][i] + c[1][i] + c[2][i], M = s.M[i], mu = s.mu[i];
                        const T tP = s.tauP[i], tS = s.tauS[i], opP = s.onePlusLtauP[i], opS = s.onePlusLtauS[i];
                        const T q[3] = {c[1][i] + c[2][i], c[0][i] + c[2][i], c[0][i] + c[1][i]};
                        // free surface (FreeSurface3Dviscoelastic.cpp): syy and ryy zeroed on the surface row
                        const bool surf = s.fs && s.fsSelect[i] != T(0);
                        if (surf) {
                            lyy[i] = 0;
                            for (int l = 0; l < s.L; ++l) lR[1][l][i] = 0;
                        }
                        const T lS3[3] = {lxx[i], lyy[i], lzz[i]};
                        T LRk[3][8] = {};
                        T le = 0, lq[3] = {0, 0, 0};
                        for (int k = 0; k < 3; ++k) {
                            const T lS = lS3[k];
                            le += opP * M * lS;
                            lq[k] -= opS * T(2) * mu * lS;
                            gM[i] += opP * e * lS;
                            gMu[i] -= opS * T(2) * q[k] * lS;
                            for (int l = 0; l < s.L; ++l) {
                                const T c1 = s.viscoC1[l], c2 = s.viscoC2[l], irt = s.invRelaxTime[l];
                                const T LR = lR[k][l][i] + DTh * lS;
                                LRk[k][l] = LR;
                                lR[k][l][i] = c2 * c1 * LR + DTh * lS;
                                le -= c2 * irt * tP * M * LR;
                                lq[k] += c2 * irt * tS * T(2) * mu * LR;
                                gM[i] -= c2 * irt * tP * e * LR;
                                gMu[i] += c2 * irt * tS * T(2) * q[k] * LR;
                            }
                        }
                        lc[0][i] += le + lq[1] + lq[2];
                        lc[1][i] += le + lq[0] + lq[2];
                        lc[2][i] += le + lq[0] + lq[1];
                        if (surf) {
                            // sxx and szz: the exchange with the horizontal sum c0' + c2' and vyy = c1'
                            T lh = 0, lv = 0;
                            for (int k = 0; k < 3; k += 2)
                                ElasticAdjoint2D<T>::fsExchangeT(s, i, lS3[k], LRk[k], c[0][i] + c[2][i], c[1][i], lh, lv, gM[i], gMu[i]);
                            lc[0][i] += lh;
                            lc[2][i] += lh;
                            lc[1][i] += lv;
                        }
                        const T lSh[3] = {lxy[i], lxz[i], lyz[i]};
                        const T muP[3] = {s.muXY[i], s.muXZ[i], s.muYZ[i]};
                        const T tauPl[3] = {s.tauSXY[i], s.tauSXZ[i], s.tauSYZ[i]};
                        std::vector<T>* gP[3] = {&gMuXY, &gMuXZ, &gMuYZ};
                        for (int k = 0; k < 3; ++k) {
                            const T lS = lSh[k], sh = c[3 + 2 * k][i] + c[4 + 2 * k][i];
                            T lm = opS * lS;
                            for (int l = 0; l < s.L; ++l) {
                                const T c1 = s.viscoC1[l], c2 = s.viscoC2[l], irt = s.invRelaxTime[l];
                                const T LR = lR[3 + k][l][i] + DTh * lS;
                                lR[3 + k][l][i] = c2 * c1 * LR + DTh * lS;
                                lm -= c2 * irt * tauPl[k] * LR;
                            }
                            (*gP[k])[i] += sh * lm;
                            lc[3 + 2 * k][i] += muP[k] * lm;
                            lc[4 + 2 * k][i] += muP[k] * lm;
                        }
                    });
                } else
                for_n(N, [&](idx_t i) {
                    const T ls = lxx[i] + lyy[i] + lzz[i];
                    lc[0][i] += s.M[i] * ls - T(2) * s.mu[i] * (lyy[i] + lzz[i]);
                    lc[1][i] += s.M[i] * ls - T(2) * s.mu[i] * (lxx[i] + lzz[i]);
                    lc[2][i] += s.M[i] * ls - T(2) * s.mu[i] * (lxx[i] + lyy[i]);
                    gM[i] += ls * (c[0][i] + c[1][i] + c[2][i]);
                    gMu[i] += -T(2) * (lxx[i] * (c[1][i] + c[2][i]) + lyy[i] * (c[0][i] + c[2][i]) + lzz[i] * (c[0][i] + c[1][i]));
                    lc[3][i] += s.muXY[i] * lxy[i];
                    lc[4][i] += s.muXY[i] * lxy[i];
                    gMuXY[i] += lxy[i] * (c[3][i] + c[4][i]);
                    lc[5][i] += s.muXZ[i] * lxz[i];
                    lc[6][i] += s.muXZ[i] * lxz[i];
                    gMuXZ[i] += lxz[i] * (c[5][i] + c[6][i]);
                    lc[7][i] += s.muYZ[i] * lyz[i];
                    lc[8][i] += s.muYZ[i] * lyz[i];
                    gMuYZ[i] += lyz[i] * (c[7][i] + c[8][i]);
                });
                for (int k = 0; k < 9; ++k) cpmlT(lc[k], lpsi[kQ[k]], kQ[k]);
                spmv_add(DxbT, lc[0], lvx);
                spmv_add(DyfT, lc[3], lvx);
                spmv_add(DzfT, lc[5], lvx);
                spmv_add(DybT, lc[1], lvy);
                spmv_add(DxfT, lc[4], lvy);
                spmv_add(DzfT, lc[7], lvy);
                spmv_add(DzbT, lc[2], lvz);
                spmv_add(DxfT, lc[6], lvz);
                spmv_add(DyfT, lc[8], lvz);
                for_n(N, [&](idx_t i) {
                    la[0][i] = la[1][i] = la[2][i] = s.invRhoX[i] * lvx[i];
                    la[3][i] = la[4][i] = la[5][i] = s.invRhoY[i] * lvy[i];
                    la[6][i] = la[7][i] = la[8][i] = s.invRhoZ[i] * lvz[i];
                    gIrx[i] += lvx[i] * (a[0][i] + a[1][i] + a[2][i]);
                    gIry[i] += lvy[i] * (a[3][i] + a[4][i] + a[5][i]);
                    gIrz[i] += lvz[i] * (a[6][i] + a[7][i] + a[8][i]);
                });
                for (int k = 0; k < 9; ++k) cpmlT(la[k], lpsi[kP[k]], kP[k]);
                spmv_add(DxfT, la[0], lxx);
                spmv_add(DybST, la[1], lxy);
                spmv_add(DzbT, la[2], lxz);
                spmv_add(DxbT, la[3], lxy);
                spmv_add(DyfST, la[4], lyy);
                spmv_add(DzbT, la[5], lyz);
                spmv_add(DxbT, la[6], lxz);
                spmv_add(DybST, la[7], lyz);
                spmv_add(DzfT, la[8], lzz);
            }
        }
        // the model preparation's transpose
        AverageTranspose<T> probe(s);
        std::vector<T> y(N), gmuc(gMu), t(N, 0);
        const std::vector<T>* gPlane[3] = {&gMuXY, &gMuXZ, &gMuYZ};
        const std::vector<T>* muPlane[3] = {&s.muXY, &s.muXZ, &s.muYZ};
        for (int plane = 0; plane < 3; ++plane) {
            const std::vector<T>& gp = *gPlane[plane];
            const std::vector<T>& mp = *muPlane[plane];
            for_n(N, [&](idx_t r) { y[r] = gp[r] * mp[r] * mp[r]; });
            std::fill(t.begin(), t.end(), T(0));
            probe.avgT([&](const T* in, T* out) { average4<T>(s.g, plane, in, out); }, y, t);
            for_n(N, [&](idx_t k) { gmuc[k] += t[k] / (s.mu[k] * s.mu[k]); });
        }
        std::vector<T> grhoAvg(N, 0);
        const std::vector<T>* gIr[3] = {&gIrx, &gIry, &gIrz};
        const std::vector<T>* ir[3] = {&s.invRhoX, &s.invRhoY, &s.invRhoZ};
        const Axis axes[3] = {Axis::X, Axis::Y, Axis::Z};
        for (int a3 = 0; a3 < 3; ++a3) {
            for_n(N, [&](idx_t r) { y[r] = -(*gIr[a3])[r] * (*ir[a3])[r] * (*ir[a3])[r]; });
            probe.avgT([&](const T* in, T* out) { average2<T>(s.g, axes[a3], in, out); }, y, grhoAvg);
        }
        // visco: M = rho vp^2 / (1 + sum tauP), mu = rho vs^2 / (1 + sum tauS), relaxation times fixed
        T sum = 0;
        if (visco) {
            const T w_ref = static_cast<T>(2.0 * M_PI * s.cfg.CenterFrequencyCPML);
            for (int l = 0; l < s.L; ++l) {
                const T ts = static_cast<T>(1.0 / (2.0 * M_PI * static_cast<T>(s.cfg.relaxationFrequency[l])));
                sum += w_ref * w_ref * ts * ts / (T(1.0) + w_ref * w_ref * ts * ts);
            }
        }
        for (idx_t k = 0; k < N; ++k) {
            const T fP = visco ? T(1) + sum * s.tauP[k] : T(1), fS = visco ? T(1) + sum * s.tauS[k] : T(1);
            T raw = rho[k];
            raw *= vs[k];
            raw *= vs[k];
            if (visco) raw = raw / fS;
            const bool unclamped = raw >= T(1);
            gvp[k] = gM[k] * T(2) * rho[k] * vp[k] / fP;
            gvs[k] = unclamped ? gmuc[k] * T(2) * rho[k] * vs[k] / fS : T(0);
            grho[k] = gM[k] * vp[k] * vp[k] / fP + (unclamped ? gmuc[k] * vs[k] * vs[k] / fS : T(0)) + grhoAvg[k];
        }
        return J;
    }
};

// Discrete adjoint of the oracle's acoustic step in 2-D and 3-D
// (Sim<T>::stepAcoustic, restating FD2Dacoustic::run,
// ForwardSolver2Dacoustic.cpp:91-194, and FD3Dacoustic::run,
// ForwardSolver3Dacoustic.cpp:91-233, with CPML, the ABS taper and the free
// surface's image operator and p = 0 on the surface row): the gradient of
// J = 1/2 sum (d - d_obs)^2 with respect to vp and rho. Per step, from X_t and
// X_{t+1}:
//   a0' = Dxf p + P(p_x)  a1' = DyfS p + P(p_y)  [a2' = Dzf p + P(p_z)]
//   vx' = vx + irx a0',  vy' = vy + iry a1'  [, vz' = vz + irz a2']
//   c0' = Dxb vx' + P(vxx)  c1' = Dyb vy' + P(vyy)  [c2' = Dzb vz' + P(vzz)]
//   p <- (p + M (c0' + c1' + c2')) d, v <- v' d, then p = 0 on the surface
// with M = rho vp^2 and irx, iry, irz the inverse 2-point density averages.
template <class T>
struct AcousticAdjoint {
    Sim<T>& s;
    const idx_t N;
    const bool d3;
    CSR<T> DxfT, DxbT, DyfST, DybT, DzfT, DzbT;
    explicit AcousticAdjoint(Sim<T>& sim) : s(sim), N(sim.g.N()), d3(sim.is3d)
    {
        if (s.eq != WAVE_EQ_ACOUSTIC) throw std::invalid_argument("oracle adjoint: acoustic only");
        DxfT = transpose(s.Dxf);
        DxbT = transpose(s.Dxb);
        DyfST = transpose(s.fs ? s.DyfFS : s.Dyf);
        DybT = transpose(s.Dyb);
        if (d3) {
            DzfT = transpose(s.Dzf);
            DzbT = transpose(s.Dzb);
        }
    }
    struct State {
        std::map<std::string, std::vector<T>> F, psi;
    };
    const std::vector<T>& psiOf(const State& x, const char* n, const std::vector<T>& zero) const
    {
        auto it = x.psi.find(n);
        return it == x.psi.end() ? zero : it->second;
    }
    void cpmlT(std::vector<T>& lc, std::vector<T>& lp, const std::vector<T>& a, const std::vector<T>& b) const
    {
        if (!s.useCpml) return;
        for_n(N, [&](idx_t i) {
            const T c = (T(1) + a[i]) * lc[i] + a[i] * lp[i];
            lp[i] = b[i] * (lc[i] + lp[i]);
            lc[i] = c;
        });
    }

    double run(const std::vector<T>& vp, const std::vector<T>& rho, const T* dobs, int K, T* gvp, T* grho)
    {
        const int NT = s.NT;
        const size_t nrec = s.rec.idx.size();
        const std::vector<T> zero(N, T(0));
        const int nd = d3 ? 3 : 2;
        s.reset();
        std::vector<State> ck;
        for (int t = 0; t < NT; ++t) {
            if (t % K == 0) ck.push_back({s.F, s.psi});
            s.step(t);
        }
        std::vector<T> res(nrec * static_cast<size_t>(NT));
        double J = 0;
        for (size_t k = 0; k < res.size(); ++k) {
            res[k] = s.seis[k] - dobs[k];
            J += 0.5 * static_cast<double>(res[k]) * static_cast<double>(res[k]);
        }
        const char* vn[3] = {"vx", "vy", "vz"};
        const char* pP[3] = {"p_x", "p_y", "p_z"};
        const char* pQ[3] = {"vxx", "vyy", "vzz"};
        const std::vector<T>* aH[3] = {&s.axh, &s.ayh, &s.azh};
        const std::vector<T>* bH[3] = {&s.bxh, &s.byh, &s.bzh};
        const std::vector<T>* aF[3] = {&s.ax, &s.ay, &s.az};
        const std::vector<T>* bF[3] = {&s.bx, &s.by, &s.bz};
        const std::vector<T>* ir[3] = {&s.invRhoX, &s.invRhoY, &s.invRhoZ};
        std::vector<T> lp(N, 0), lv[3], lP[3], lQ[3], a[3], c[3], vpr[3], la[3], lc[3], gIr[3];
        for (int k = 0; k < 3; ++k) {
            lv[k].assign(N, 0); lP[k].assign(N, 0); lQ[k].assign(N, 0); a[k].assign(N, 0); c[k].assign(N, 0);
            vpr[k].assign(N, 0); la[k].assign(N, 0); lc[k].assign(N, 0); gIr[k].assign(N, 0);
        }
        std::vector<T> gM(N, 0);
        const int nseg = static_cast<int>(ck.size());
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const int t0 = seg * K, t1 = std::min(NT, t0 + K);
            std::vector<State> X;
            s.F = ck[seg].F;
            s.psi = ck[seg].psi;
            X.push_back({s.F, s.psi});
            for (int t = t0; t < t1; ++t) {
                s.step(t);
                X.push_back({s.F, s.psi});
            }
            for (int t = t1 - 1; t >= t0; --t) {
                const State& X0 = X[t - t0];
                const State& X1 = X[t - t0 + 1];
                const auto& p0 = X0.F.at("p");
                s.Dxf.spmv(p0.data(), a[0].data());
                (s.fs ? s.DyfFS : s.Dyf).spmv(p0.data(), a[1].data());
                if (d3) s.Dzf.spmv(p0.data(), a[2].data());
                for (int k = 0; k < nd; ++k) {
                    const auto& ps = psiOf(X1, pP[k], zero);
                    const auto& v0 = X0.F.at(vn[k]);
                    const auto& irk = *ir[k];
                    for_n(N, [&](idx_t i) {
                        a[k][i] += ps[i];
                        vpr[k][i] = v0[i] + irk[i] * a[k][i];
                    });
                }
                s.Dxb.spmv(vpr[0].data(), c[0].data());
                s.Dyb.spmv(vpr[1].data(), c[1].data());
                if (d3) s.Dzb.spmv(vpr[2].data(), c[2].data());
                for (int k = 0; k < nd; ++k) {
                    const auto& q = psiOf(X1, pQ[k], zero);
                    for_n(N, [&](idx_t i) { c[k][i] += q[i]; });
                }
                for (size_t r = 0; r < nrec; ++r) {
                    const idx_t i = s.rec.idx[r];
                    const T v = res[r * NT + t];
                    switch (s.rec.type[r]) {
                    case WAVE_TYPE_P: lp[i] += v; break;
                    case WAVE_TYPE_VX: lv[0][i] += v; break;
                    case WAVE_TYPE_VY: lv[1][i] += v; break;
                    default: lv[2][i] += v; break;
                    }
                }
                // p = 0 on the surface (after the taper), the taper on p and v
                if (s.fs) for_n(N, [&](idx_t i) { lp[i] *= s.fsZero[i]; });
                if (s.useAbs) {
                    for_n(N, [&](idx_t i) { lp[i] *= s.damping[i]; });
                    for (int k = 0; k < nd; ++k) for_n(N, [&](idx_t i) { lv[k][i] *= s.damping[i]; });
                }
                // p <- p + M (c0' + c1' + c2')
                for_n(N, [&](idx_t i) {
                    T cs = 0;
                    for (int k = 0; k < nd; ++k) cs += c[k][i];
                    gM[i] += lp[i] * cs;
                    for (int k = 0; k < nd; ++k) lc[k][i] = s.M[i] * lp[i];
                });
                for (int k = 0; k < nd; ++k) cpmlT(lc[k], lQ[k], *aF[k], *bF[k]);
                spmv_add(DxbT, lc[0], lv[0]);
                spmv_add(DybT, lc[1], lv[1]);
                if (d3) spmv_add(DzbT, lc[2], lv[2]);
                // v' = v + ir a'
                for (int k = 0; k < nd; ++k) {
                    const auto& irk = *ir[k];
                    for_n(N, [&](idx_t i) {
                        la[k][i] = irk[i] * lv[k][i];
                        gIr[k][i] += lv[k][i] * a[k][i];
                    });
                    cpmlT(la[k], lP[k], *aH[k], *bH[k]);
                }
                spmv_add(DxfT, la[0], lp);
                spmv_add(DyfST, la[1], lp);
                if (d3) spmv_add(DzfT, la[2], lp);
            }
        }
        // M = rho vp^2; ir = 1 / A2(rho) (0 where invalid)
        AverageTranspose<T> probe(s);
        std::vector<T> y(N), grhoAvg(N, 0);
        const Axis axes[3] = {Axis::X, Axis::Y, Axis::Z};
        for (int k = 0; k < nd; ++k) {
            const auto& irk = *ir[k];
            for_n(N, [&](idx_t r) { y[r] = -gIr[k][r] * irk[r] * irk[r]; });
            probe.avgT([&](const T* in, T* out) { average2<T>(s.g, axes[k], in, out); }, y, grhoAvg);
        }
        for (idx_t k = 0; k < N; ++k) {
            gvp[k] = gM[k] * T(2) * rho[k] * vp[k];
            grho[k] = gM[k] * vp[k] * vp[k] + grhoAvg[k];
        }
        return J;
    }
};

// Discrete adjoint of the oracle's lossless 3-D EM step (Sim<T>::stepEM3D,
// restating FD3Demem::run, ForwardSolver3Demem.cpp:119-237, with CPMLEM3D
// and the ABS taper): the gradient of J = 1/2 sum (d - d_obs)^2 with respect
// to eps_r, sigma and mu_r. Per step, from X_t and X_{t+1} (all E derivatives
// forward on the half profile; H derivatives backward on the full profile
// except hyx, which uses the half one, CPMLEM3D.cpp:67-70):
//   hx' = hx - iMyz (a0' - a1'),  a0' = Dyf ez, a1' = Dzf ey
//   hy' = hy - iMxz (a2' - a3'),  a2' = Dzf ex, a3' = Dxf ez
//   hz' = hz - iMxy (a4' - a5'),  a4' = Dxf ey, a5' = Dyf ex
//   ex' = CaX ex + CbX (c0' - c1'),  c0' = Dyb hz', c1' = Dzb hy'
//   ey' = CaY ey + CbY (c2' - c3'),  c2' = Dzb hx', c3' = Dxb hz'
//   ez' = CaZ ez + CbZ (c4' - c5'),  c4' = Dxb hy', c5' = Dyb hx'
// then the taper on all six fields; Ca, Cb of the 2-point averages of
// eps = eps_r eps0 and sigma along each E component's axis, iM the inverse
// 4-point averages of mu = mu_r mu0 in the yz, xz and xy planes (EMEM.cpp:378-392).
template <class T>
struct EM3Adjoint {
    Sim<T>& s;
    const idx_t N;
    CSR<T> DxfT, DyfT, DzfT, DxbT, DybT, DzbT;
    static constexpr const char* kA[6] = {"ezy", "eyz", "exz", "ezx", "eyx", "exy"};
    static constexpr const char* kC[6] = {"hzy", "hyz", "hxz", "hzx", "hyx", "hxy"};
    const bool visco;   // 3-D visco-EM (FD3Dviscoemem::run, ForwardSolver3Dviscoemem.cpp:161-309)

    explicit EM3Adjoint(Sim<T>& sim) : s(sim), N(sim.g.N()), visco(sim.eq == WAVE_EQ_VISCOEMEM)
    {
        if (!s.is3d || (s.eq != WAVE_EQ_EMEM && s.eq != WAVE_EQ_VISCOEMEM)) throw std::invalid_argument("oracle adjoint: 3-D EM only");
        DxfT = transpose(s.Dxf);
        DyfT = transpose(s.Dyf);
        DzfT = transpose(s.Dzf);
        DxbT = transpose(s.Dxb);
        DybT = transpose(s.Dyb);
        DzbT = transpose(s.Dzb);
    }
    struct State {
        std::map<std::string, std::vector<T>> F, psi;
        std::map<std::string, std::vector<std::vector<T>>> R;
    };
    const std::vector<T>& psiOf(const State& x, const char* n, const std::vector<T>& zero) const
    {
        auto it = x.psi.find(n);
        return it == x.psi.end() ? zero : it->second;
    }
    std::pair<const std::vector<T>*, const std::vector<T>*> prof(const std::string& n) const
    {
        if (n == "ezx" || n == "eyx" || n == "hyx") return {&s.axh, &s.bxh};
        if (n == "ezy" || n == "exy") return {&s.ayh, &s.byh};
        if (n == "eyz" || n == "exz") return {&s.azh, &s.bzh};
        if (n == "hzx") return {&s.ax, &s.bx};
        if (n == "hzy" || n == "hxy") return {&s.ay, &s.by};
        return {&s.az, &s.bz};   // hyz, hxz
    }
    void cpmlT(std::vector<T>& lc, std::vector<T>& lp, const char* n) const
    {
        if (!s.useCpml) return;
        auto ab = prof(n);
        const std::vector<T>& a = *ab.first;
        const std::vector<T>& b = *ab.second;
        for_n(N, [&](idx_t i) {
            const T c = (T(1) + a[i]) * lc[i] + a[i] * lp[i];
            lp[i] = b[i] * (lc[i] + lp[i]);
            lc[i] = c;
        });
    }

    double run(const std::vector<T>& epsr, const std::vector<T>& sigma, const std::vector<T>& mur, const T* dobs, int K,
               T* geps, T* gsig, T* gmu)
    {
        const int NT = s.NT;
        const size_t nrec = s.rec.idx.size();
        const std::vector<T> zero(N, T(0));
        s.reset();
        std::vector<State> ck;
        for (int t = 0; t < NT; ++t) {
            if (t % K == 0) ck.push_back({s.F, s.psi, s.R});
            s.step(t);
        }
        std::vector<T> res(nrec * static_cast<size_t>(NT));
        double J = 0;
        for (size_t k = 0; k < res.size(); ++k) {
            res[k] = s.seis[k] - dobs[k];
            J += 0.5 * static_cast<double>(res[k]) * static_cast<double>(res[k]);
        }
        std::map<std::string, std::vector<T>> lF, lp;
        for (const char* n : {"hx", "hy", "hz", "ex", "ey", "ez"}) lF[n].assign(N, 0);
        for (int k = 0; k < 6; ++k) { lp[kA[k]].assign(N, 0); lp[kC[k]].assign(N, 0); }
        std::vector<T> gCa[3], gCb[3], gM[3], a[6], c[6], la[6], lc[6], hp[3];
        for (int k = 0; k < 3; ++k) { gCa[k].assign(N, 0); gCb[k].assign(N, 0); gM[k].assign(N, 0); hp[k].assign(N, 0); }
        for (int k = 0; k < 6; ++k) { a[k].assign(N, 0); c[k].assign(N, 0); la[k].assign(N, 0); lc[k].assign(N, 0); }
        const std::vector<T>* iM[3] = {&s.invMuYZ, &s.invMuXZ, &s.invMuXY};
        const std::vector<T>* Ca[3] = {&s.CaX, &s.CaY, &s.CaZ};
        const std::vector<T>* Cb[3] = {&s.CbX, &s.CbY, &s.CbZ};
        const char* hn[3] = {"hx", "hy", "hz"};
        const char* en[3] = {"ex", "ey", "ez"};
        const char* rn[3] = {"rx", "ry", "rz"};
        // visco: adjoints of the memory variables and of Cd per component and mechanism
        const int L = visco ? s.L : 0;
        std::vector<std::vector<T>> lR[3], gCd[3];
        for (int q = 0; q < 3; ++q) { lR[q].assign(L, std::vector<T>(N, 0)); gCd[q].assign(L, std::vector<T>(N, 0)); }
        const std::vector<std::vector<T>>* Cd[3] = {&s.CdX, &s.CdY, &s.CdZ};
        const int nseg = static_cast<int>(ck.size());
        for (int seg = nseg - 1; seg >= 0; --seg) {
            const int t0 = seg * K, t1 = std::min(NT, t0 + K);
            std::vector<State> X;
            s.F = ck[seg].F;
            s.psi = ck[seg].psi;
            s.R = ck[seg].R;
            X.push_back({s.F, s.psi, s.R});
            for (int t = t0; t < t1; ++t) {
                s.step(t);
                X.push_back({s.F, s.psi, s.R});
            }
            for (int t = t1 - 1; t >= t0; --t) {
                const State& X0 = X[t - t0];
                const State& X1 = X[t - t0 + 1];
                auto f0 = [&](const char* n) { return X0.F.at(n).data(); };
                s.Dyf.spmv(f0("ez"), a[0].data());
                s.Dzf.spmv(f0("ey"), a[1].data());
                s.Dzf.spmv(f0("ex"), a[2].data());
                s.Dxf.spmv(f0("ez"), a[3].data());
                s.Dxf.spmv(f0("ey"), a[4].data());
                s.Dyf.spmv(f0("ex"), a[5].data());
                for (int k = 0; k < 6; ++k) {
                    const auto& p = psiOf(X1, kA[k], zero);
                    for_n(N, [&](idx_t i) { a[k][i] += p[i]; });
                }
                for (int q = 0; q < 3; ++q) {
                    const auto& h0 = X0.F.at(hn[q]);
                    const auto& im = *iM[q];
                    for_n(N, [&](idx_t i) { hp[q][i] = h0[i] - im[i] * (a[2 * q][i] - a[2 * q + 1][i]); });
                }
                s.Dyb.spmv(hp[2].data(), c[0].data());
                s.Dzb.spmv(hp[1].data(), c[1].data());
                s.Dzb.spmv(hp[0].data(), c[2].data());
                s.Dxb.spmv(hp[2].data(), c[3].data());
                s.Dxb.spmv(hp[1].data(), c[4].data());
                s.Dyb.spmv(hp[0].data(), c[5].data());
                for (int k = 0; k < 6; ++k) {
                    const auto& p = psiOf(X1, kC[k], zero);
                    for_n(N, [&](idx_t i) { c[k][i] += p[i]; });
                }
                for (size_t r = 0; r < nrec; ++r) {
                    const idx_t i = s.rec.idx[r];
                    const T v = res[r * NT + t];
                    const int ty = s.rec.type[r];
                    lF[ty == WAVE_TYPE_EZ ? "ez" : ty == WAVE_TYPE_EX ? "ex" : ty == WAVE_TYPE_EY ? "ey" : "hz"][i] += v;
                }
                if (s.useAbs)
                    for (const char* n : {"hx", "hy", "hz", "ex", "ey", "ez"}) {
                        auto& w = lF[n];
                        for_n(N, [&](idx_t i) { w[i] *= s.damping[i]; });
                    }
                // E <- Ca E + Cb (c' - c'' - DT sum_l r_l'), r_l' = Cc_l r_l + Cd_l E (visco)
                for (int q = 0; q < 3; ++q) {
                    auto& le = lF[en[q]];
                    const auto& e0 = X0.F.at(en[q]);
                    const auto& ca = *Ca[q];
                    const auto& cb = *Cb[q];
                    for_n(N, [&](idx_t i) {
                        T u = c[2 * q][i] - c[2 * q + 1][i];
                        for (int l = 0; l < L; ++l) u -= s.DT * X1.R.at(rn[q])[l][i];
                        lc[2 * q][i] = cb[i] * le[i];
                        lc[2 * q + 1][i] = -cb[i] * le[i];
                        gCa[q][i] += le[i] * e0[i];
                        gCb[q][i] += le[i] * u;
                        T ln = ca[i] * le[i];
                        for (int l = 0; l < L; ++l) {
                            const T LR = lR[q][l][i] - s.DT * cb[i] * le[i];
                            ln += (*Cd[q])[l][i] * LR;
                            gCd[q][l][i] += LR * e0[i];
                            lR[q][l][i] = s.emCc[l] * LR;
                        }
                        le[i] = ln;
                    });
                }
                for (int k = 0; k < 6; ++k) cpmlT(lc[k], lp[kC[k]], kC[k]);
                spmv_add(DybT, lc[0], lF["hz"]);
                spmv_add(DzbT, lc[1], lF["hy"]);
                spmv_add(DzbT, lc[2], lF["hx"]);
                spmv_add(DxbT, lc[3], lF["hz"]);
                spmv_add(DxbT, lc[4], lF["hy"]);
                spmv_add(DybT, lc[5], lF["hx"]);
                // H' = H - iM (a' - a'')
                for (int q = 0; q < 3; ++q) {
                    const auto& lh = lF[hn[q]];
                    const auto& im = *iM[q];
                    for_n(N, [&](idx_t i) {
                        la[2 * q][i] = -im[i] * lh[i];
                        la[2 * q + 1][i] = im[i] * lh[i];
                        gM[q][i] -= lh[i] * (a[2 * q][i] - a[2 * q + 1][i]);
                    });
                }
                for (int k = 0; k < 6; ++k) cpmlT(la[k], lp[kA[k]], kA[k]);
                spmv_add(DyfT, la[0], lF["ez"]);
                spmv_add(DzfT, la[1], lF["ey"]);
                spmv_add(DzfT, la[2], lF["ex"]);
                spmv_add(DxfT, la[3], lF["ez"]);
                spmv_add(DxfT, la[4], lF["ey"]);
                spmv_add(DyfT, la[5], lF["ex"]);
            }
        }
        // Ca, Cb -> the 2-point averages of eps and sigma along x, y, z; iM -> the
        // inverse 4-point averages of mu in the yz, xz and xy planes
        const T eps0 = static_cast<T>(8.8541878176e-12), mu0 = static_cast<T>(1.2566370614e-6);
        const T DT = s.DT;
        std::vector<T> eps(N), ge(N, 0), gs(N, 0), ye(N), ys(N), avE(N), avS(N), y(N), gm(N, 0), avTe(N), avTs(N);
        for (idx_t i = 0; i < N; ++i) eps[i] = epsr[i] * eps0;
        // visco: the optical permittivity / conductivity of the averaged eps, sigma, tau_eps,
        // tau_sigma and Cd_l = -DT te cdScale_l e (ForwardSolverEM.cpp:68-152), the taus fixed
        T sumInv = 0;
        std::vector<T> cdScale(L);
        for (int l = 0; l < L; ++l) {
            const double r = 1.0 / (2.0 * M_PI * static_cast<double>(static_cast<T>(s.cfg.relaxationFrequency[l])));
            const T rt = static_cast<T>(r);
            sumInv = static_cast<T>(static_cast<double>(sumInv) + 1.0 / static_cast<double>(rt));
            T tv = static_cast<T>(1 / (1 + 0.5 * static_cast<double>(DT) / static_cast<double>(rt)));
            tv /= (static_cast<T>(L) * rt * rt);
            cdScale[l] = tv;
        }
        if (L > 0) sumInv /= static_cast<T>(L);
        AverageTranspose<T> probe(s);
        const Axis axes[3] = {Axis::X, Axis::Y, Axis::Z};
        for (int q = 0; q < 3; ++q) {
            average2<T>(s.g, axes[q], eps.data(), avE.data());
            average2<T>(s.g, axes[q], sigma.data(), avS.data());
            if (visco) {
                average2<T>(s.g, axes[q], s.emTauE.data(), avTe.data());
                average2<T>(s.g, axes[q], s.emTauS.data(), avTs.data());
            }
            for (idx_t i = 0; i < N; ++i) {
                T e = avE[i], sg = avS[i], de_de = 1, de_ds = 0, ds_de = 0;
                if (visco) {
                    const T te = avTe[i], ts = avTs[i];
                    const T eo = (T(1) - te) * avE[i] + avS[i] * ts;
                    const bool clamp = eo < eps0;
                    e = clamp ? eps0 : eo;
                    de_de = clamp ? T(0) : T(1) - te;
                    de_ds = clamp ? T(0) : ts;
                    sg = te * sumInv * avE[i] + avS[i];
                    ds_de = te * sumInv;
                }
                const T k = sg * DT / (T(2) * e), qq = T(1) + k;
                const T dCa_de = T(2) * k / (e * qq * qq), dCa_ds = -T(2) / (qq * qq) * DT / (T(2) * e);
                const T dCb_de = -T(1) / (e * e * qq) + k / (e * e * qq * qq), dCb_ds = -(T(1) / e) / (qq * qq) * DT / (T(2) * e);
                const T gE = gCa[q][i] * dCa_de + gCb[q][i] * dCb_de, gS = gCa[q][i] * dCa_ds + gCb[q][i] * dCb_ds;
                ye[i] = gE * de_de + gS * ds_de;
                ys[i] = gE * de_ds + gS;
                for (int l = 0; l < L; ++l) ye[i] += gCd[q][l][i] * (-DT) * avTe[i] * cdScale[l];
            }
            probe.avgT([&](const T* in, T* out) { average2<T>(s.g, axes[q], in, out); }, ye, ge);
            probe.avgT([&](const T* in, T* out) { average2<T>(s.g, axes[q], in, out); }, ys, gs);
        }
        const int plane[3] = {2, 1, 0};   // iMyz, iMxz, iMxy
        for (int q = 0; q < 3; ++q) {
            const auto& im = *iM[q];
            for_n(N, [&](idx_t r) { y[r] = -gM[q][r] * im[r] * im[r]; });
            probe.avgT([&](const T* in, T* out) { average4<T>(s.g, plane[q], in, out); }, y, gm);
        }
        for (idx_t i = 0; i < N; ++i) {
            geps[i] = eps0 * ge[i];
            gsig[i] = gs[i];
            gmu[i] = mu0 * gm[i];
        }
        (void)mur;
        return J;
    }
};

template <class T>
constexpr const char* ElasticAdjoint2D<T>::kP[4];
template <class T>
constexpr const char* ElasticAdjoint2D<T>::kQ[4];
template <class T>
constexpr const char* ElasticAdjoint3D<T>::kP[9];
template <class T>
constexpr const char* ElasticAdjoint3D<T>::kQ[9];
template <class T>
constexpr const char* EM3Adjoint<T>::kA[6];
template <class T>
constexpr const char* EM3Adjoint<T>::kC[6];

} // namespace refcpu
