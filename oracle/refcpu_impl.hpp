// refcpu_impl.hpp — TEST INFRASTRUCTURE ONLY (the oracle). Implementation of
// refcpu::Sim<T>; see refcpu.hpp for what this file restates and why.
#pragma once

namespace refcpu {

template <class F>
inline void for_n(idx_t n, F&& f)
{
#pragma omp parallel for schedule(static)
    for (idx_t i = 0; i < n; ++i) f(i);
}

inline bool eq_seismic(int eq) { return eq <= WAVE_EQ_VISCOSH; }
inline bool eq_visco(int eq) { return eq == WAVE_EQ_VISCOELASTIC || eq == WAVE_EQ_VISCOSH || eq == WAVE_EQ_VISCOTMEM || eq == WAVE_EQ_VISCOEMEM; }
inline bool eq_elasticlike(int eq) { return eq == WAVE_EQ_ELASTIC || eq == WAVE_EQ_VISCOELASTIC || eq == WAVE_EQ_SH || eq == WAVE_EQ_VISCOSH; }

template <class T>
void Sim<T>::setup(const wave_config& c, const Model<T>& m)
{
    cfg = c;
    g.NX = c.NX; g.NY = c.NY; g.NZ = c.dimension == 2 ? 1 : c.NZ;
    is3d = c.dimension == 3;
    eq = c.equation;
    order = c.spatialFDorder;
    stencil = c.useStencilMatrix != 0;
    DT = static_cast<T>(c.DT);
    DH = static_cast<T>(c.DH);
    // NT = int(T/DT + 0.5) in the value type (Common.hpp:240-243)
    NT = static_cast<int>(static_cast<T>(c.T) / DT + T(0.5));
    fs = c.FreeSurface == 1;
    useAbs = c.DampingBoundary == 1;
    useCpml = c.DampingBoundary == 2;
    L = eq_visco(eq) ? c.numRelaxationMechanisms : 0;
    fd_coef_d(order); // validates the order
    buildOperators();
    prepareModel(m);
    buildBoundaries();
    reset();
}

template <class T>
void Sim<T>::buildOperators()
{
    // Stencil matrices and sparse matrices without edge-order reduction drop
    // neighbours outside the grid; only the value scaling differs
    // (c*(DT/DH) vs (c/DH)*DT), far below the parity tolerance.
    auto make = [&](Axis a, idx_t n, bool fwd) {
        std::vector<Row1D<T>> rows(n);
        for (idx_t c = 0; c < n; ++c) {
            if (stencil || !cfg.edgeOrderReduction) rows[c] = stencil_row<T>(c, n, order, fwd, DH, DT);
            else rows[c] = fwd ? sparse_row_forward<T>(c, n, order, DH, DT) : sparse_row_backward<T>(c, n, order, DH, DT);
        }
        return kron_axis<T>(g, a, rows);
    };
    Dxf = make(Axis::X, g.NX, true);
    Dxb = make(Axis::X, g.NX, false);
    Dyf = make(Axis::Y, g.NY, true);
    Dyb = make(Axis::Y, g.NY, false);
    if (is3d) {
        Dzf = make(Axis::Z, g.NZ, true);
        Dzb = make(Axis::Z, g.NZ, false);
    }
    if (fs) { // FDTD3D::initializeFreeSurfaceMatrices (FDTD3D.cpp:312-343)
        std::vector<Row1D<T>> rf(g.NY), rb(g.NY);
        for (idx_t y = 0; y < g.NY; ++y) {
            rf[y] = fs_row<T>(y, g.NY, order, true, DH, DT);
            rb[y] = fs_row<T>(y, g.NY, order, false, DH, DT);
        }
        DyfFS = kron_axis<T>(g, Axis::Y, rf);
        DybFS = kron_axis<T>(g, Axis::Y, rb);
    }
}

template <class T>
void Sim<T>::prepareModel(const Model<T>& m)
{
    const idx_t N = g.N();
    auto inv_avg = [&](const std::vector<T>& p, Axis a, std::vector<T>& out) {
        // calcInverseAveragedParameter (Modelparameter.cpp:633-639)
        out.assign(N, 0);
        average2<T>(g, a, p.data(), out.data());
        for_n(N, [&](idx_t i) { T v = T(1) / out[i]; out[i] = is_invalid(v) ? T(0) : v; });
    };
    auto harmonic = [&](std::vector<T>& mod, int plane, bool twoPointAxis, Axis a, std::vector<T>& out) {
        // calcAveragedSWaveModulus (ModelparameterSeismic.cpp:421-432)
        for_n(N, [&](idx_t i) { if (mod[i] < T(1.0)) mod[i] = T(1.0); });
        std::vector<T> inv(N), av(N);
        for_n(N, [&](idx_t i) { inv[i] = T(1) / mod[i]; });
        if (twoPointAxis) average2<T>(g, a, inv.data(), av.data());
        else average4<T>(g, plane, inv.data(), av.data());
        out.assign(N, 0);
        for_n(N, [&](idx_t i) { T v = T(1) / av[i]; out[i] = v < T(4.0) ? T(0) : v; });
    };
    auto modulus = [&](const std::vector<T>& v, const std::vector<T>& rho, std::vector<T>& out) {
        // calcModulusFromVelocity (ModelparameterSeismic.cpp:131-136)
        out.assign(N, 0);
        for_n(N, [&](idx_t i) { T s = rho[i]; s *= v[i]; s *= v[i]; out[i] = s; });
    };

    if (eq_seismic(eq)) {
        if (eq != WAVE_EQ_SH && eq != WAVE_EQ_VISCOSH) modulus(m.vp, m.rho, M);
        if (eq != WAVE_EQ_ACOUSTIC) modulus(m.vs, m.rho, mu);
        if (eq_visco(eq)) {
            // Viscoelastic::getPWaveModulus/getSWaveModulus (Viscoelastic.cpp:650-715)
            T w_ref = static_cast<T>(2.0 * M_PI * cfg.CenterFrequencyCPML);
            T sum = 0;
            for (int l = 0; l < L; ++l) {
                T tauSigma = static_cast<T>(1.0 / (2.0 * M_PI * static_cast<T>(cfg.relaxationFrequency[l])));
                sum += w_ref * w_ref * tauSigma * tauSigma / (T(1.0) + w_ref * w_ref * tauSigma * tauSigma);
            }
            if (eq == WAVE_EQ_VISCOELASTIC)
                for_n(N, [&](idx_t i) { M[i] = M[i] / (T(1.0) + sum * m.taup[i]); });
            for_n(N, [&](idx_t i) { mu[i] = mu[i] / (T(1.0) + sum * m.taus[i]); });
            tauS = m.taus;
            if (eq == WAVE_EQ_VISCOELASTIC) tauP = m.taup;
        }
        if (eq == WAVE_EQ_SH || eq == WAVE_EQ_VISCOSH) {
            // SH::calculateAveraging (SH.cpp:424-431), ViscoSH.cpp:450-459
            invRho.assign(N, 0);
            for_n(N, [&](idx_t i) { invRho[i] = T(1) / m.rho[i]; });
            harmonic(mu, 0, true, Axis::X, muXZ);
            harmonic(mu, 0, true, Axis::Y, muYZ);
            if (eq == WAVE_EQ_VISCOSH) {
                tauSXZ.assign(N, 0); tauSYZ.assign(N, 0);
                average2<T>(g, Axis::X, tauS.data(), tauSXZ.data());
                average2<T>(g, Axis::Y, tauS.data(), tauSYZ.data());
            }
        } else {
            // Elastic/Acoustic/Viscoelastic::calculateAveraging (Elastic.cpp:576-588)
            inv_avg(m.rho, Axis::X, invRhoX);
            inv_avg(m.rho, Axis::Y, invRhoY);
            if (is3d) inv_avg(m.rho, Axis::Z, invRhoZ);
            if (eq != WAVE_EQ_ACOUSTIC) {
                harmonic(mu, 0, false, Axis::X, muXY);
                if (is3d) {
                    harmonic(mu, 1, false, Axis::X, muXZ);
                    harmonic(mu, 2, false, Axis::X, muYZ);
                }
            }
            if (eq == WAVE_EQ_VISCOELASTIC) {
                tauSXY.assign(N, 0);
                average4<T>(g, 0, tauS.data(), tauSXY.data());
                if (is3d) {
                    tauSXZ.assign(N, 0); tauSYZ.assign(N, 0);
                    average4<T>(g, 1, tauS.data(), tauSXZ.data());
                    average4<T>(g, 2, tauS.data(), tauSYZ.data());
                }
            }
        }
        if (eq_visco(eq)) {
            // initForwardSolver coefficients (ForwardSolver3Dviscoelastic.cpp:56-66)
            relaxTime.clear(); invRelaxTime.clear(); viscoC1.clear(); viscoC2.clear();
            for (int l = 0; l < L; ++l) {
                relaxTime.push_back(static_cast<T>(1.0 / (2.0 * M_PI * static_cast<T>(cfg.relaxationFrequency[l]))));
                invRelaxTime.push_back(T(1.0) / relaxTime[l]);
                viscoC1.push_back(T(1.0) - DT / (T(2.0) * relaxTime[l]));
                viscoC2.push_back(T(1.0) / (T(1.0) + DT / (T(2.0) * relaxTime[l])));
            }
            DThalf = DT / T(2.0);
            // prepareForModelling (ForwardSolver3Dviscoelastic.cpp:103-118)
            onePlusLtauS.assign(N, 0);
            for_n(N, [&](idx_t i) { onePlusLtauS[i] = T(1.0) + T(L) * tauS[i]; });
            if (eq == WAVE_EQ_VISCOELASTIC) {
                onePlusLtauP.assign(N, 0);
                for_n(N, [&](idx_t i) { onePlusLtauP[i] = T(1.0) + T(L) * tauP[i]; });
            }
        }
    } else {
        // EM: TMEM::init (TMEM.cpp:230-241), ViscoTMEM::init (ViscoTMEM.cpp:274-292) with
        // eps = eps_r*eps0, mu = mu_r*mu0 and tau_sigma times tau_ref = 1/(2 pi f_c);
        // calculateAveraging (TMEM.cpp:366-374, EMEM.cpp:378-392, ViscoTMEM.cpp:442-450,
        // ViscoEMEM.cpp:409-432); coefficients ForwardSolverEM.cpp:14-152.
        const T eps0 = static_cast<T>(8.8541878176e-12), mu0 = static_cast<T>(1.2566370614e-6);
        const bool visco = eq == WAVE_EQ_VISCOTMEM || eq == WAVE_EQ_VISCOEMEM;
        std::vector<T> eps(N), sig(m.sigma), muv(N), tauE, tauSg;
        for_n(N, [&](idx_t i) { eps[i] = m.eps_r[i] * eps0; muv[i] = m.mu_r[i] * mu0; });
        std::vector<T> relax;   // 1 / (2 pi f_l)
        if (visco) {
            if (m.tau_eps.size() != static_cast<size_t>(N) || m.tau_sigma.size() != static_cast<size_t>(N))
                throw std::invalid_argument("visco-EM needs tau_eps and tau_sigma");
            tauE = m.tau_eps;
            tauSg = m.tau_sigma;
            const T tauRef = static_cast<T>(1.0 / (2.0 * M_PI * static_cast<T>(cfg.CenterFrequencyCPML)));
            for_n(N, [&](idx_t i) { tauSg[i] *= tauRef; });
            emTauE = tauE;
            emTauS = tauSg;
            for (int l = 0; l < L; ++l) relax.push_back(static_cast<T>(1.0 / (2.0 * M_PI * static_cast<T>(cfg.relaxationFrequency[l]))));
        }
        auto Cinv = [&](T e, T s) { T c = T(0.5) / e; c *= s; c *= DT; c += T(1); return T(1) / c; };
        auto Ca = [&](T e, T s) { T c = T(0.5) / e; c *= s; c *= DT; c = T(1) - c; return c * Cinv(e, s); };
        auto Cb = [&](T e, T s) { T c = T(1) / e; return c * Cinv(e, s); };
        // getDielectricPermittivityEffectiveOptical (ForwardSolverEM.cpp:140-152), clamped below at eps0
        auto epsOpt = [&](T es, T ss, T te, T ts) {
            T e = T(1) - te; e *= es; T tmp = ss * ts; e += tmp;
            return e < eps0 ? eps0 : e;
        };
        // getElectricConductivityEffectiveOptical (ForwardSolverEM.cpp:118-133)
        T sumInv = 0;
        for (int l = 0; l < L && visco; ++l) sumInv = static_cast<T>(static_cast<double>(sumInv) + 1.0 / static_cast<double>(relax[l]));
        if (visco) sumInv /= static_cast<T>(L);
        auto sigOpt = [&](T es, T ss, T te) { T s = te * sumInv; s *= es; s += ss; return s; };
        // getCc / getAveragedCd (ForwardSolverEM.cpp:68-109)
        emCc.clear();
        std::vector<T> cdScale;
        for (int l = 0; l < L && visco; ++l) {
            const double r = static_cast<double>(relax[l]);
            emCc.push_back(static_cast<T>((1 - 0.5 * static_cast<double>(DT) / r) / (1 + 0.5 * static_cast<double>(DT) / r)));
            T tv = static_cast<T>(1 / (1 + 0.5 * static_cast<double>(DT) / r));
            tv /= (static_cast<T>(L) * relax[l] * relax[l]);
            cdScale.push_back(tv);
        }
        // coefficients of one E component from its (averaged) material values
        auto coeffs = [&](const std::vector<T>& e, const std::vector<T>& s, const std::vector<T>* te, const std::vector<T>* ts,
                          std::vector<T>& ca, std::vector<T>& cb, std::vector<std::vector<T>>& cd) {
            ca.assign(N, 0); cb.assign(N, 0);
            for_n(N, [&](idx_t i) {
                T ee = e[i], ss = s[i];
                if (visco) { T eo = epsOpt(e[i], s[i], (*te)[i], (*ts)[i]); ss = sigOpt(e[i], s[i], (*te)[i]); ee = eo; }
                ca[i] = Ca(ee, ss); cb[i] = Cb(ee, ss);
            });
            cd.assign(visco ? L : 0, std::vector<T>(N, 0));
            for (int l = 0; l < L && visco; ++l)
                for_n(N, [&](idx_t i) { T c = (*te)[i] * cdScale[l]; c *= e[i]; c *= -DT; cd[l][i] = c; });
        };
        auto inv4 = [&](int plane, std::vector<T>& out) {
            out.assign(N, 0);
            average4<T>(g, plane, muv.data(), out.data());
            for_n(N, [&](idx_t i) { T v = T(1) / out[i]; out[i] = is_invalid(v) ? T(0) : v; });
        };
        auto avg = [&](const std::vector<T>& in, Axis a) { std::vector<T> o(N); average2<T>(g, a, in.data(), o.data()); return o; };
        if (eq == WAVE_EQ_TMEM || eq == WAVE_EQ_VISCOTMEM) {
            if (is3d) throw std::invalid_argument("TM modelling is 2-D only");
            inv_avg(muv, Axis::X, invMuXZ);
            inv_avg(muv, Axis::Y, invMuYZ);
            coeffs(eps, sig, visco ? &tauE : nullptr, visco ? &tauSg : nullptr, CaZ, CbZ, CdZ);
        } else if (eq == WAVE_EQ_EMEM || eq == WAVE_EQ_VISCOEMEM) {
            inv4(0, invMuXY);
            if (is3d) { inv4(1, invMuXZ); inv4(2, invMuYZ); }
            std::vector<Axis> axes = {Axis::X, Axis::Y};
            if (is3d) axes.push_back(Axis::Z);
            for (Axis a : axes) {
                auto e = avg(eps, a), s = avg(sig, a);
                std::vector<T> te, ts;
                if (visco) { te = avg(tauE, a); ts = avg(tauSg, a); }
                auto& ca = a == Axis::X ? CaX : (a == Axis::Y ? CaY : CaZ);
                auto& cb = a == Axis::X ? CbX : (a == Axis::Y ? CbY : CbZ);
                auto& cd = a == Axis::X ? CdX : (a == Axis::Y ? CdY : CdZ);
                coeffs(e, s, visco ? &te : nullptr, visco ? &ts : nullptr, ca, cb, cd);
            }
        } else {
            throw std::invalid_argument("equation not available in the oracle");
        }
    }
}

template <class T>
void Sim<T>::buildBoundaries()
{
    const idx_t N = g.N();
    const int w = cfg.BoundaryWidth;
    if (useAbs) {
        // ABS2D::init (ABS2D.cpp:110-180), ABS3D::init (ABS3D.cpp:154-220)
        damping.assign(N, T(1.0));
        T amp = T(1.0) - static_cast<T>(cfg.DampingCoeff) / T(100.0);
        T a = std::sqrt(-std::log(amp) / T(w * w));
        std::vector<T> coeff(w);
        for (int j = 0; j < w; ++j) coeff[j] = std::exp(-(a * a * T(w - j) * T(w - j)));
        for (idx_t r = 0; r < N; ++r) {
            idx_t x, y, z;
            g.coord(r, x, y, z);
            idx_t dx = Grid::edge(x, g.NX), dy = Grid::edge(y, g.NY), dz = Grid::edge(z, g.NZ);
            if (!is3d) {
                idx_t mn = dx < dy ? dx : dy;
                if (!fs) { if (mn < w) damping[r] = coeff[mn]; }
                else {
                    if (y < w) { if (dx < w) damping[r] = coeff[dx]; }
                    else if (mn < w) damping[r] = coeff[mn];
                }
            } else {
                idx_t mn = std::min(dx, std::min(dy, dz));
                if (!fs) { if (mn < w) damping[r] = coeff[mn]; }
                else {
                    idx_t xz = !(dx < dz) ? dz : dx;
                    if (y < w) { if (dz < w || dx < w) damping[r] = coeff[xz]; }
                    else if (mn < w) damping[r] = coeff[mn];
                }
            }
        }
    }
    if (useCpml) {
        std::vector<T> a(w), b(w), ah(w), bh(w);
        T np = static_cast<T>(cfg.NPower), fc = static_cast<T>(cfg.CenterFrequencyCPML), vm = static_cast<T>(cfg.VMaxCPML);
        cpml_coeff<T>(a, b, np, fc, vm, DT, DH, false);
        cpml_coeff<T>(ah, bh, np, fc, vm, DT, DH, true);
        auto PX = cpml_axis<T>(g.NX, w, a, b, ah, bh, false);
        auto PY = cpml_axis<T>(g.NY, w, a, b, ah, bh, cfg.FreeSurface != 0);
        auto PZ = cpml_axis<T>(g.NZ, w, a, b, ah, bh, false);
        auto expand = [&](const CpmlAxis<T>& P, Axis ax_, std::vector<T>& A, std::vector<T>& B, std::vector<T>& Ah, std::vector<T>& Bh) {
            A.assign(N, 0); B.assign(N, 0); Ah.assign(N, 0); Bh.assign(N, 0);
            for_n(N, [&](idx_t r) {
                idx_t x, y, z;
                g.coord(r, x, y, z);
                idx_t c = ax_ == Axis::X ? x : (ax_ == Axis::Y ? y : z);
                A[r] = P.a_full[c]; B[r] = P.b_full[c]; Ah[r] = P.a_half[c]; Bh[r] = P.b_half[c];
            });
        };
        expand(PX, Axis::X, ax, bx, axh, bxh);
        expand(PY, Axis::Y, ay, by, ayh, byh);
        if (is3d) expand(PZ, Axis::Z, az, bz, azh, bzh);
    }
    if (fs) {
        // FreeSurfaceAcoustic/Elastic::init (FreeSurfaceElastic.cpp:58-88)
        fsZero.assign(N, T(1)); fsSelect.assign(N, T(0));
        for (idx_t r = 0; r < N; ++r) {
            idx_t x, y, z;
            g.coord(r, x, y, z);
            if (y == 0) { fsZero[r] = 0; fsSelect[r] = 1; }
        }
        if (eq == WAVE_EQ_ELASTIC) {
            // FreeSurfaceElastic::setModelparameter (FreeSurfaceElastic.cpp:11-47)
            scaleH.assign(N, 0); scaleV.assign(N, 0);
            for_n(N, [&](idx_t i) {
                T t = M[i] - T(2) * mu[i];
                scaleV[i] = fsSelect[i] * t;
                T t2 = t * t; t2 /= M[i]; t2 *= T(-1);
                scaleH[i] = fsSelect[i] * t2;
            });
        } else if (eq == WAVE_EQ_VISCOELASTIC) {
            // FreeSurfaceViscoelastic::setModelparameter (FreeSurfaceViscoelastic.cpp:12-97)
            scaleH.assign(N, 0); scaleV.assign(N, 0);
            scaleRelH.assign(L, std::vector<T>(N, 0)); scaleRelV.assign(L, std::vector<T>(N, 0));
            for_n(N, [&](idx_t i) {
                T temp = T(-2) * mu[i] * onePlusLtauS[i];
                T temp2 = M[i] * onePlusLtauP[i];
                temp += temp2;
                temp2 = T(1) / temp2;
                scaleV[i] = fsSelect[i] * temp;
                T h = T(-1) * fsSelect[i];
                h *= temp; h *= temp; h *= temp2;
                scaleH[i] = h;
            });
            for (int l = 0; l < L; ++l) {
                T rt = relaxTime[l];
                T vc2 = viscoC2[l];
                for_n(N, [&](idx_t i) {
                    T temp = T(2) * mu[i];
                    T temp2 = M[i];
                    T temp3 = temp * tauS[i];
                    temp3 -= temp2 * tauP[i];
                    T sv = fsSelect[i]; sv *= temp3; sv *= vc2; sv /= rt;
                    scaleRelV[l][i] = sv;
                    temp *= onePlusLtauS[i];
                    temp2 *= onePlusLtauP[i];
                    temp /= temp2;
                    temp -= T(1);
                    T sh = fsSelect[i]; sh *= temp3; sh *= temp; sh *= vc2; sh /= rt;
                    scaleRelH[l][i] = sh;
                });
            }
        }
    }
}

template <class T>
void Sim<T>::reset()
{
    const idx_t N = g.N();
    F.clear(); R.clear(); psi.clear();
    std::vector<const char*> names;
    switch (eq) {
    case WAVE_EQ_ACOUSTIC: names = is3d ? std::vector<const char*>{"vx", "vy", "vz", "p"} : std::vector<const char*>{"vx", "vy", "p"}; break;
    case WAVE_EQ_ELASTIC:
    case WAVE_EQ_VISCOELASTIC:
        names = is3d ? std::vector<const char*>{"vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz"}
                     : std::vector<const char*>{"vx", "vy", "sxx", "syy", "sxy"};
        break;
    case WAVE_EQ_SH:
    case WAVE_EQ_VISCOSH: names = {"vz", "sxz", "syz"}; break;
    case WAVE_EQ_TMEM:
    case WAVE_EQ_VISCOTMEM: names = {"hx", "hy", "ez"}; break;
    case WAVE_EQ_EMEM:
    case WAVE_EQ_VISCOEMEM:
        names = is3d ? std::vector<const char*>{"hx", "hy", "hz", "ex", "ey", "ez"} : std::vector<const char*>{"hz", "ex", "ey"};
        break;
    }
    for (auto n : names) F[n].assign(N, 0);
    if (eq == WAVE_EQ_VISCOELASTIC) {
        std::vector<const char*> rn = is3d ? std::vector<const char*>{"rxx", "ryy", "rzz", "rxy", "rxz", "ryz"} : std::vector<const char*>{"rxx", "ryy", "rxy"};
        for (auto n : rn) R[n].assign(L, std::vector<T>(N, 0));
    }
    if (eq == WAVE_EQ_VISCOSH) {
        R["rxz"].assign(L, std::vector<T>(N, 0));
        R["ryz"].assign(L, std::vector<T>(N, 0));
    }
    if (eq == WAVE_EQ_VISCOTMEM) R["rz"].assign(L, std::vector<T>(N, 0));
    if (eq == WAVE_EQ_VISCOEMEM) {
        R["rx"].assign(L, std::vector<T>(N, 0));
        R["ry"].assign(L, std::vector<T>(N, 0));
        if (is3d) R["rz"].assign(L, std::vector<T>(N, 0));
    }
    upd.assign(N, 0); updt.assign(N, 0); upd2.assign(N, 0); vxx.assign(N, 0); vyy.assign(N, 0); vzz.assign(N, 0); tmp.assign(N, 0);
    seis.assign(rec.idx.size() * static_cast<size_t>(NT), 0);
}

// CPML::applyCPML (CPML.cpp:84-95): Psi = b*Psi + a*Vec; Vec += Psi.
template <class T>
void Sim<T>::cpml(std::vector<T>& d, const char* name, const std::vector<T>& a, const std::vector<T>& b)
{
    auto& p = psi[name];
    if (p.empty()) p.assign(g.N(), 0);
    T* P = p.data();
    T* D = d.data();
    const T* A = a.data();
    const T* B = b.data();
    for_n(g.N(), [&](idx_t i) {
        T ps = P[i] * B[i];
        ps += A[i] * D[i];
        P[i] = ps;
        D[i] += ps;
    });
}

// SourceReceiverImpl::applySource (SourceReceiverImplSeismic.cpp:80-105, FDTD*.cpp,
// SourceReceiverImplEM.cpp:95-165): per component type in order 1..4, raw sample added.
template <class T>
void Sim<T>::applySources(int t)
{
    for (int type = 1; type <= 4; ++type) {
        for (size_t s = 0; s < src.idx.size(); ++s) {
            if (src.type[s] != type) continue;
            T v = signals[s * NT + t];
            idx_t i = src.idx[s];
            if (eq_seismic(eq)) {
                if (type == WAVE_TYPE_P) {
                    if (eq == WAVE_EQ_ACOUSTIC) F["p"][i] += v;
                    else if (eq == WAVE_EQ_ELASTIC || eq == WAVE_EQ_VISCOELASTIC) {
                        F["sxx"][i] += v; F["syy"][i] += v;
                        if (is3d) F["szz"][i] += v;
                    } else throw std::invalid_argument("pressure sources are not available in SH modelling");
                } else if (type == WAVE_TYPE_VX) F["vx"][i] += v;
                else if (type == WAVE_TYPE_VY) F["vy"][i] += v;
                else F["vz"][i] += v;
            } else {
                const char* n = type == WAVE_TYPE_EZ ? "ez" : type == WAVE_TYPE_EX ? "ex" : type == WAVE_TYPE_EY ? "ey" : "hz";
                if (!F.count(n)) throw std::invalid_argument("source component not available for this EM equation");
                F[n][i] += v;
            }
        }
    }
}

template <class T>
void Sim<T>::gather(int t)
{
    for (size_t r = 0; r < rec.idx.size(); ++r) {
        idx_t i = rec.idx[r];
        int type = rec.type[r];
        T v = 0;
        if (eq_seismic(eq)) {
            if (type == WAVE_TYPE_P) {
                if (eq == WAVE_EQ_ACOUSTIC) v = F["p"][i];
                else if (is3d) { v = F["sxx"][i]; v += F["syy"][i]; v += F["szz"][i]; v /= T(3); }
                else { v = F["sxx"][i]; v += F["syy"][i]; v *= T(0.5); }
            } else if (type == WAVE_TYPE_VX) v = F["vx"][i];
            else if (type == WAVE_TYPE_VY) v = F["vy"][i];
            else v = F["vz"][i];
        } else {
            const char* n = type == WAVE_TYPE_EZ ? "ez" : type == WAVE_TYPE_EX ? "ex" : type == WAVE_TYPE_EY ? "ey" : "hz";
            v = F[n][i];
        }
        seis[r * NT + t] = v;
    }
}

template <class T>
void Sim<T>::step(int t)
{
    if (copyStateEachStep) Fcopy = F; // Simulation.cpp:450
    switch (eq) {
    case WAVE_EQ_ACOUSTIC: stepAcoustic(t); break;
    case WAVE_EQ_ELASTIC: stepElastic(t); break;
    case WAVE_EQ_VISCOELASTIC: stepVisco(t); break;
    case WAVE_EQ_SH:
    case WAVE_EQ_VISCOSH: stepSH(t); break;
    case WAVE_EQ_TMEM:
    case WAVE_EQ_VISCOTMEM: stepTM(t); break;
    case WAVE_EQ_EMEM:
    case WAVE_EQ_VISCOEMEM:
        if (is3d) stepEM3D(t);
        else stepTE(t);
        break;
    default: throw std::invalid_argument("equation not available in the oracle");
    }
}

#define VEC_OP(expr) for_n(N, [&](idx_t i) { expr; })

// FD2Dacoustic::run (ForwardSolver2Dacoustic.cpp:91-194), FD3Dacoustic::run (ForwardSolver3Dacoustic.cpp:91-233)
template <class T>
void Sim<T>::stepAcoustic(int t)
{
    const idx_t N = g.N();
    auto& vX = F["vx"]; auto& vY = F["vy"]; auto& p = F["p"];
    Dxf.spmv(p.data(), upd.data());
    if (useCpml) cpml(upd, "p_x", axh, bxh);
    VEC_OP(upd[i] *= invRhoX[i]);
    VEC_OP(vX[i] += upd[i]);
    (fs ? DyfFS : Dyf).spmv(p.data(), upd.data());
    if (useCpml) cpml(upd, "p_y", ayh, byh);
    VEC_OP(upd[i] *= invRhoY[i]);
    VEC_OP(vY[i] += upd[i]);
    if (is3d) {
        auto& vZ = F["vz"];
        Dzf.spmv(p.data(), upd.data());
        if (useCpml) cpml(upd, "p_z", azh, bzh);
        VEC_OP(upd[i] *= invRhoZ[i]);
        VEC_OP(vZ[i] += upd[i]);
    }
    Dxb.spmv(vX.data(), upd.data());
    if (useCpml) cpml(upd, "vxx", ax, bx);
    Dyb.spmv(vY.data(), updt.data());
    if (useCpml) cpml(updt, "vyy", ay, by);
    VEC_OP(upd[i] += updt[i]);
    if (is3d) {
        Dzb.spmv(F["vz"].data(), updt.data());
        if (useCpml) cpml(updt, "vzz", az, bz);
        VEC_OP(upd[i] += updt[i]);
    }
    VEC_OP(upd[i] *= M[i]);
    VEC_OP(p[i] += upd[i]);
    if (useAbs) {
        VEC_OP(p[i] *= damping[i]);
        VEC_OP(vX[i] *= damping[i]);
        VEC_OP(vY[i] *= damping[i]);
        if (is3d) { auto& vZ = F["vz"]; VEC_OP(vZ[i] *= damping[i]); }
    }
    if (fs) VEC_OP(p[i] *= fsZero[i]);
    applySources(t);
    gather(t);
}

// FD2Delastic::run (ForwardSolver2Delastic.cpp:117-297), FD3Delastic::run (ForwardSolver3Delastic.cpp:120-414)
template <class T>
void Sim<T>::stepElastic(int t)
{
    const idx_t N = g.N();
    auto& vX = F["vx"]; auto& vY = F["vy"];
    auto& Sxx = F["sxx"]; auto& Syy = F["syy"]; auto& Sxy = F["sxy"];
    const CSR<T>& DybS = fs ? DybFS : Dyb;
    const CSR<T>& DyfS = fs ? DyfFS : Dyf;
    if (!is3d) {
        Dxf.spmv(Sxx.data(), upd.data());
        if (useCpml) cpml(upd, "sxx_x", axh, bxh);
        DybS.spmv(Sxy.data(), updt.data());
        if (useCpml) cpml(updt, "sxy_y", ay, by);
        VEC_OP(upd[i] += updt[i]);
        VEC_OP(upd[i] *= invRhoX[i]);
        VEC_OP(vX[i] += upd[i]);
        Dxb.spmv(Sxy.data(), upd.data());
        if (useCpml) cpml(upd, "sxy_x", ax, bx);
        DyfS.spmv(Syy.data(), updt.data());
        if (useCpml) cpml(updt, "syy_y", ayh, byh);
        VEC_OP(upd[i] += updt[i]);
        VEC_OP(upd[i] *= invRhoY[i]);
        VEC_OP(vY[i] += upd[i]);
        Dxb.spmv(vX.data(), vxx.data());
        Dyb.spmv(vY.data(), vyy.data());
        if (useCpml) { cpml(vxx, "vxx", ax, bx); cpml(vyy, "vyy", ay, by); }
        VEC_OP(upd[i] = vxx[i]);
        VEC_OP(upd[i] += vyy[i]);
        VEC_OP(upd[i] *= M[i]);
        VEC_OP(Sxx[i] += upd[i]);
        VEC_OP(Syy[i] += upd[i]);
        VEC_OP(upd[i] = vyy[i]);
        VEC_OP(upd[i] *= mu[i]);
        VEC_OP(Sxx[i] -= T(2.0) * upd[i]);
        VEC_OP(upd[i] = vxx[i]);
        VEC_OP(upd[i] *= mu[i]);
        VEC_OP(Syy[i] -= T(2.0) * upd[i]);
        Dyf.spmv(vX.data(), upd.data());
        if (useCpml) cpml(upd, "vxy", ayh, byh);
        Dxf.spmv(vY.data(), updt.data());
        if (useCpml) cpml(updt, "vyx", axh, bxh);
        VEC_OP(upd[i] += updt[i]);
        VEC_OP(upd[i] *= muXY[i]);
        VEC_OP(Sxy[i] += upd[i]);
        if (fs) {
            // FreeSurface2Delastic::exchangeHorizontalUpdate (FreeSurface2Delastic.cpp:14-45)
            VEC_OP(Sxx[i] += scaleH[i] * vxx[i]);
            VEC_OP(Sxx[i] -= scaleV[i] * vyy[i]);
            VEC_OP(Syy[i] *= fsZero[i]);
        }
        if (useAbs) {
            for (auto* v : {&Sxx, &Syy, &Sxy, &vX, &vY}) { auto& w = *v; VEC_OP(w[i] *= damping[i]); }
        }
    } else {
        auto& vZ = F["vz"]; auto& Szz = F["szz"]; auto& Sxz = F["sxz"]; auto& Syz = F["syz"];
        // vx
        Dxf.spmv(Sxx.data(), upd.data());
        if (useCpml) cpml(upd, "sxx_x", axh, bxh);
        DybS.spmv(Sxy.data(), updt.data());
        if (useCpml) cpml(updt, "sxy_y", ay, by);
        VEC_OP(upd[i] += updt[i]);
        Dzb.spmv(Sxz.data(), updt.data());
        if (useCpml) cpml(updt, "sxz_z", az, bz);
        VEC_OP(upd[i] += updt[i]);
        VEC_OP(upd[i] *= invRhoX[i]);
        VEC_OP(vX[i] += upd[i]);
        // vy
        Dxb.spmv(Sxy.data(), upd.data());
        if (useCpml) cpml(upd, "sxy_x", ax, bx);
        DyfS.spmv(Syy.data(), updt.data());
        if (useCpml) cpml(updt, "syy_y", ayh, byh);
        VEC_OP(upd[i] += updt[i]);
        Dzb.spmv(Syz.data(), updt.data());
        if (useCpml) cpml(updt, "syz_z", az, bz);
        VEC_OP(upd[i] += updt[i]);
        VEC_OP(upd[i] *= invRhoY[i]);
        VEC_OP(vY[i] += upd[i]);
        // vz
        Dxb.spmv(Sxz.data(), upd.data());
        if (useCpml) cpml(upd, "sxz_x", ax, bx);
        DybS.spmv(Syz.data(), updt.data());
        if (useCpml) cpml(updt, "syz_y", ay, by);
        VEC_OP(upd[i] += updt[i]);
        Dzf.spmv(Szz.data(), updt.data());
        if (useCpml) cpml(updt, "szz_z", azh, bzh);
        VEC_OP(upd[i] += updt[i]);
        VEC_OP(upd[i] *= invRhoZ[i]);
        VEC_OP(vZ[i] += upd[i]);
        // normal stress
        Dxb.spmv(vX.data(), vxx.data());
        Dyb.spmv(vY.data(), vyy.data());
        Dzb.spmv(vZ.data(), vzz.data());
        if (useCpml) { cpml(vxx, "vxx", ax, bx); cpml(vyy, "vyy", ay, by); cpml(vzz, "vzz", az, bz); }
        VEC_OP(upd[i] = vxx[i]);
        VEC_OP(upd[i] += vyy[i]);
        VEC_OP(upd[i] += vzz[i]);
        VEC_OP(upd[i] *= M[i]);
        VEC_OP(Sxx[i] += upd[i]);
        VEC_OP(Syy[i] += upd[i]);
        VEC_OP(Szz[i] += upd[i]);
        VEC_OP(upd[i] = vyy[i] + vzz[i]);
        VEC_OP(upd[i] *= mu[i]);
        VEC_OP(Sxx[i] -= T(2.0) * upd[i]);
        VEC_OP(upd[i] = vxx[i] + vzz[i]);
        VEC_OP(upd[i] *= mu[i]);
        VEC_OP(Syy[i] -= T(2.0) * upd[i]);
        VEC_OP(upd[i] = vxx[i] + vyy[i]);
        VEC_OP(upd[i] *= mu[i]);
        VEC_OP(Szz[i] -= T(2.0) * upd[i]);
        // shear
        Dyf.spmv(vX.data(), upd.data());
        if (useCpml) cpml(upd, "vxy", ayh, byh);
        Dxf.spmv(vY.data(), updt.data());
        if (useCpml) cpml(updt, "vyx", axh, bxh);
        VEC_OP(upd[i] += updt[i]);
        VEC_OP(upd[i] *= muXY[i]);
        VEC_OP(Sxy[i] += upd[i]);
        Dzf.spmv(vX.data(), upd.data());
        if (useCpml) cpml(upd, "vxz", azh, bzh);
        Dxf.spmv(vZ.data(), updt.data());
        if (useCpml) cpml(updt, "vzx", axh, bxh);
        VEC_OP(upd[i] += updt[i]);
        VEC_OP(upd[i] *= muXZ[i]);
        VEC_OP(Sxz[i] += upd[i]);
        Dzf.spmv(vY.data(), upd.data());
        if (useCpml) cpml(upd, "vyz", azh, bzh);
        Dyf.spmv(vZ.data(), updt.data());
        if (useCpml) cpml(updt, "vzy", ayh, byh);
        VEC_OP(upd[i] += updt[i]);
        VEC_OP(upd[i] *= muYZ[i]);
        VEC_OP(Syz[i] += upd[i]);
        if (fs) {
            // FreeSurface3Delastic::exchangeHorizontalUpdate (FreeSurface3Delastic.cpp:15-47),
            // setSurfaceZero(Syy) first (ForwardSolver3Delastic.cpp:400-404)
            VEC_OP(upd[i] = vxx[i] + vzz[i]);
            VEC_OP(Syy[i] *= fsZero[i]);
            VEC_OP(tmp[i] = scaleH[i] * upd[i]);
            VEC_OP(Sxx[i] += tmp[i]);
            VEC_OP(Szz[i] += tmp[i]);
            VEC_OP(tmp[i] = scaleV[i] * vyy[i]);
            VEC_OP(Sxx[i] -= tmp[i]);
            VEC_OP(Szz[i] -= tmp[i]);
        }
        if (useAbs) {
            for (auto* v : {&Sxx, &Syy, &Szz, &Sxy, &Sxz, &Syz, &vX, &vY, &vZ}) { auto& w = *v; VEC_OP(w[i] *= damping[i]); }
        }
    }
    applySources(t);
    gather(t);
}

// FD2Dviscoelastic::run (ForwardSolver2Dviscoelastic.cpp:130-321),
// FD3Dviscoelastic::run (ForwardSolver3Dviscoelastic.cpp:132-457)
template <class T>
void Sim<T>::stepVisco(int t)
{
    const idx_t N = g.N();
    auto& vX = F["vx"]; auto& vY = F["vy"];
    auto& Sxx = F["sxx"]; auto& Syy = F["syy"]; auto& Sxy = F["sxy"];
    auto& Rxx = R["rxx"]; auto& Ryy = R["ryy"]; auto& Rxy = R["rxy"];
    const CSR<T>& DybS = fs ? DybFS : Dyb;
    const CSR<T>& DyfS = fs ? DyfFS : Dyf;
    const T DTh = DThalf;
    // velocities
    Dxf.spmv(Sxx.data(), upd.data());
    if (useCpml) cpml(upd, "sxx_x", axh, bxh);
    DybS.spmv(Sxy.data(), updt.data());
    if (useCpml) cpml(updt, "sxy_y", ay, by);
    VEC_OP(upd[i] += updt[i]);
    if (is3d) {
        Dzb.spmv(F["sxz"].data(), updt.data());
        if (useCpml) cpml(updt, "sxz_z", az, bz);
        VEC_OP(upd[i] += updt[i]);
    }
    VEC_OP(upd[i] *= invRhoX[i]);
    VEC_OP(vX[i] += upd[i]);
    Dxb.spmv(Sxy.data(), upd.data());
    if (useCpml) cpml(upd, "sxy_x", ax, bx);
    DyfS.spmv(Syy.data(), updt.data());
    if (useCpml) cpml(updt, "syy_y", ayh, byh);
    VEC_OP(upd[i] += updt[i]);
    if (is3d) {
        Dzb.spmv(F["syz"].data(), updt.data());
        if (useCpml) cpml(updt, "syz_z", az, bz);
        VEC_OP(upd[i] += updt[i]);
    }
    VEC_OP(upd[i] *= invRhoY[i]);
    VEC_OP(vY[i] += upd[i]);
    if (is3d) {
        auto& vZ = F["vz"];
        Dxb.spmv(F["sxz"].data(), upd.data());
        if (useCpml) cpml(upd, "sxz_x", ax, bx);
        DybS.spmv(F["syz"].data(), updt.data());
        if (useCpml) cpml(updt, "syz_y", ay, by);
        VEC_OP(upd[i] += updt[i]);
        Dzf.spmv(F["szz"].data(), updt.data());
        if (useCpml) cpml(updt, "szz_z", azh, bzh);
        VEC_OP(upd[i] += updt[i]);
        VEC_OP(upd[i] *= invRhoZ[i]);
        VEC_OP(vZ[i] += upd[i]);
    }
    // normal stresses
    Dxb.spmv(vX.data(), vxx.data());
    Dyb.spmv(vY.data(), vyy.data());
    if (is3d) Dzb.spmv(F["vz"].data(), vzz.data());
    if (useCpml) {
        cpml(vxx, "vxx", ax, bx);
        cpml(vyy, "vyy", ay, by);
        if (is3d) cpml(vzz, "vzz", az, bz);
    }
    VEC_OP(upd[i] = vxx[i]);
    VEC_OP(upd[i] += vyy[i]);
    if (is3d) VEC_OP(upd[i] += vzz[i]);
    VEC_OP(upd[i] *= M[i]);
    std::vector<std::vector<T>*> Sn = {&Sxx, &Syy};
    std::vector<std::vector<std::vector<T>>*> Rn = {&Rxx, &Ryy};
    if (is3d) { Sn.push_back(&F["szz"]); Rn.push_back(&R["rzz"]); }
    for (int l = 0; l < L; ++l) {
        T irt = invRelaxTime[l], c1 = viscoC1[l];
        VEC_OP(upd2[i] = irt * upd[i]);
        VEC_OP(upd2[i] *= tauP[i]);
        for (size_t k = 0; k < Sn.size(); ++k) {
            auto& S = *Sn[k]; auto& Rl = (*Rn[k])[l];
            VEC_OP(S[i] += DTh * Rl[i]);
            VEC_OP(Rl[i] *= c1);
            VEC_OP(Rl[i] -= upd2[i]);
        }
    }
    VEC_OP(upd[i] *= onePlusLtauP[i]);
    for (auto* S : Sn) { auto& s = *S; VEC_OP(s[i] += upd[i]); }
    auto shearPart = [&](std::vector<T>& S, std::vector<std::vector<T>>& Rr, auto sumFn) {
        VEC_OP(upd[i] = sumFn(i));
        VEC_OP(upd[i] *= mu[i]);
        VEC_OP(upd[i] *= T(2.0));
        for (int l = 0; l < L; ++l) {
            T irt = invRelaxTime[l], c2 = viscoC2[l];
            VEC_OP(upd2[i] = irt * upd[i]);
            VEC_OP(upd2[i] *= tauS[i]);
            VEC_OP(Rr[l][i] += upd2[i]);
            VEC_OP(Rr[l][i] *= c2);
            VEC_OP(S[i] += DTh * Rr[l][i]);
        }
        VEC_OP(upd[i] *= onePlusLtauS[i]);
        VEC_OP(S[i] -= upd[i]);
    };
    if (is3d) {
        shearPart(Sxx, Rxx, [&](idx_t i) { return vyy[i] + vzz[i]; });
        shearPart(Syy, Ryy, [&](idx_t i) { return vxx[i] + vzz[i]; });
        shearPart(F["szz"], R["rzz"], [&](idx_t i) { return vxx[i] + vyy[i]; });
    } else {
        shearPart(Sxx, Rxx, [&](idx_t i) { return vyy[i]; });
        shearPart(Syy, Ryy, [&](idx_t i) { return vxx[i]; });
    }
    // shear stresses
    auto shearStress = [&](std::vector<T>& S, std::vector<std::vector<T>>& Rr, const std::vector<T>& muAv, const std::vector<T>& tauAv) {
        VEC_OP(upd[i] *= muAv[i]);
        for (int l = 0; l < L; ++l) {
            T irt = invRelaxTime[l], c1 = viscoC1[l], c2 = viscoC2[l];
            VEC_OP(S[i] += DTh * Rr[l][i]);
            VEC_OP(Rr[l][i] *= c1);
            VEC_OP(upd2[i] = irt * upd[i]);
            VEC_OP(upd2[i] *= tauAv[i]);
            VEC_OP(Rr[l][i] -= upd2[i]);
            VEC_OP(Rr[l][i] *= c2);
            VEC_OP(S[i] += DTh * Rr[l][i]);
        }
        VEC_OP(upd[i] *= onePlusLtauS[i]);
        VEC_OP(S[i] += upd[i]);
    };
    Dyf.spmv(vX.data(), upd.data());
    if (useCpml) cpml(upd, "vxy", ayh, byh);
    Dxf.spmv(vY.data(), updt.data());
    if (useCpml) cpml(updt, "vyx", axh, bxh);
    VEC_OP(upd[i] += updt[i]);
    shearStress(Sxy, Rxy, muXY, tauSXY);
    if (is3d) {
        auto& vZ = F["vz"];
        Dzf.spmv(vX.data(), upd.data());
        if (useCpml) cpml(upd, "vxz", azh, bzh);
        Dxf.spmv(vZ.data(), updt.data());
        if (useCpml) cpml(updt, "vzx", axh, bxh);
        VEC_OP(upd[i] += updt[i]);
        shearStress(F["sxz"], R["rxz"], muXZ, tauSXZ);
        Dzf.spmv(vY.data(), upd.data());
        if (useCpml) cpml(upd, "vyz", azh, bzh);
        Dyf.spmv(vZ.data(), updt.data());
        if (useCpml) cpml(updt, "vzy", ayh, byh);
        VEC_OP(upd[i] += updt[i]);
        shearStress(F["syz"], R["ryz"], muYZ, tauSYZ);
    }
    if (fs) {
        // FreeSurface2Dviscoelastic / FreeSurface3Dviscoelastic::exchangeHorizontalUpdate
        if (is3d) VEC_OP(upd[i] = vxx[i] + vzz[i]);
        else VEC_OP(upd[i] = vxx[i]);
        std::vector<std::vector<T>*> SH = {&Sxx};
        std::vector<std::vector<std::vector<T>>*> RH = {&Rxx};
        if (is3d) { SH.push_back(&F["szz"]); RH.push_back(&R["rzz"]); }
        for (int l = 0; l < L; ++l)
            for (size_t k = 0; k < SH.size(); ++k) { auto& S = *SH[k]; auto& Rl = (*RH[k])[l]; VEC_OP(S[i] -= DTh * (fsSelect[i] * Rl[i])); }
        VEC_OP(tmp[i] = scaleH[i] * upd[i]);
        for (auto* S : SH) { auto& s = *S; VEC_OP(s[i] += tmp[i]); }
        VEC_OP(tmp[i] = scaleV[i] * vyy[i]);
        for (auto* S : SH) { auto& s = *S; VEC_OP(s[i] -= tmp[i]); }
        for (int l = 0; l < L; ++l) {
            VEC_OP(tmp[i] = scaleRelH[l][i] * upd[i]);
            for (auto* Rr : RH) { auto& Rl = (*Rr)[l]; VEC_OP(Rl[i] += tmp[i]); }
            VEC_OP(tmp[i] = scaleRelV[l][i] * vyy[i]);
            for (auto* Rr : RH) { auto& Rl = (*Rr)[l]; VEC_OP(Rl[i] -= tmp[i]); }
            for (size_t k = 0; k < SH.size(); ++k) { auto& S = *SH[k]; auto& Rl = (*RH[k])[l]; VEC_OP(S[i] += DTh * (fsSelect[i] * Rl[i])); }
        }
        VEC_OP(Syy[i] *= fsZero[i]);
        for (int l = 0; l < L; ++l) { auto& Rl = Ryy[l]; VEC_OP(Rl[i] *= fsZero[i]); }
    }
    if (useAbs) {
        std::vector<std::vector<T>*> all = {&Sxx, &Syy, &Sxy, &vX, &vY};
        if (is3d) all = {&Sxx, &Syy, &F["szz"], &Sxy, &F["sxz"], &F["syz"], &vX, &vY, &F["vz"]};
        for (auto* v : all) { auto& w = *v; VEC_OP(w[i] *= damping[i]); }
    }
    applySources(t);
    gather(t);
}

// FD2Dsh::run (ForwardSolver2Dsh.cpp:108-196), FD2Dviscosh::run (ForwardSolver2Dviscosh.cpp:126-244)
template <class T>
void Sim<T>::stepSH(int t)
{
    const idx_t N = g.N();
    auto& vZ = F["vz"]; auto& Sxz = F["sxz"]; auto& Syz = F["syz"];
    Dxb.spmv(Sxz.data(), upd.data());
    (fs ? DybFS : Dyb).spmv(Syz.data(), updt.data());
    if (useCpml) { cpml(upd, "sxz_x", ax, bx); cpml(updt, "syz_y", ay, by); }
    VEC_OP(upd[i] += updt[i]);
    VEC_OP(upd[i] *= invRho[i]);
    VEC_OP(vZ[i] += upd[i]);
    auto stress = [&](const CSR<T>& D, const char* pname, const std::vector<T>& a, const std::vector<T>& b,
                      std::vector<T>& S, const std::vector<T>& muAv, const char* rname, const std::vector<T>& tauAv) {
        D.spmv(vZ.data(), upd.data());
        if (useCpml) cpml(upd, pname, a, b);
        VEC_OP(upd[i] *= muAv[i]);
        if (eq == WAVE_EQ_VISCOSH) {
            auto& Rr = R[rname];
            for (int l = 0; l < L; ++l) {
                T irt = invRelaxTime[l], c1 = viscoC1[l], c2 = viscoC2[l], DTh = DThalf;
                VEC_OP(S[i] += DTh * Rr[l][i]);
                VEC_OP(Rr[l][i] *= c1);
                VEC_OP(upd2[i] = irt * upd[i]);
                VEC_OP(upd2[i] *= tauAv[i]);
                VEC_OP(Rr[l][i] -= upd2[i]);
                VEC_OP(Rr[l][i] *= c2);
                VEC_OP(S[i] += DTh * Rr[l][i]);
            }
            VEC_OP(upd[i] *= onePlusLtauS[i]);
        }
        VEC_OP(S[i] += upd[i]);
    };
    stress(Dxf, "vzx", axh, bxh, Sxz, muXZ, "rxz", tauSXZ);
    stress(Dyf, "vzy", ayh, byh, Syz, muYZ, "ryz", tauSYZ);
    if (useAbs) {
        for (auto* v : {&Sxz, &Syz, &vZ}) { auto& w = *v; VEC_OP(w[i] *= damping[i]); }
    }
    applySources(t);
    gather(t);
}

// FD2Dtmem::run (ForwardSolverEM/ForwardSolver2Dtmem.cpp:108-174)
template <class T>
void Sim<T>::stepTM(int t)
{
    const idx_t N = g.N();
    auto& hX = F["hx"]; auto& hY = F["hy"]; auto& eZ = F["ez"];
    Dyf.spmv(eZ.data(), upd.data());
    if (useCpml) cpml(upd, "ezy", ayh, byh);
    VEC_OP(upd[i] *= invMuYZ[i]);
    VEC_OP(hX[i] -= upd[i]);
    Dxf.spmv(eZ.data(), updt.data());
    if (useCpml) cpml(updt, "ezx", axh, bxh);
    VEC_OP(upd[i] = -updt[i]);
    VEC_OP(upd[i] *= invMuXZ[i]);
    VEC_OP(hY[i] -= upd[i]);
    // visco-TM memory variables (ForwardSolver2Dviscotmem.cpp:175-182)
    for (int l = 0; l < L; ++l) {
        auto& r = R["rz"][l];
        const T cc = emCc[l];
        const auto& cd = CdZ[l];
        VEC_OP(T u = cc * r[i]; T ut = cd[i] * eZ[i]; r[i] = ut + u);
    }
    Dxb.spmv(hY.data(), upd.data());
    Dyb.spmv(hX.data(), updt.data());
    if (useCpml) { cpml(upd, "hyx", ax, bx); cpml(updt, "hxy", ay, by); }
    VEC_OP(upd[i] -= updt[i]);
    for (int l = 0; l < L; ++l) { const auto& r = R["rz"][l]; VEC_OP(upd[i] -= DT * r[i]); }
    VEC_OP(upd[i] *= CbZ[i]);
    VEC_OP(updt[i] = CaZ[i] * eZ[i]);
    VEC_OP(eZ[i] = updt[i] + upd[i]);
    if (useAbs) {
        for (auto* v : {&eZ, &hX, &hY}) { auto& w = *v; VEC_OP(w[i] *= damping[i]); }
    }
    applySources(t);
    gather(t);
}

// FD2Demem::run (ForwardSolverEM/ForwardSolver2Demem.cpp:112-185),
// FD2Dviscoemem::run (ForwardSolverEM/ForwardSolver2Dviscoemem.cpp:154-228)
template <class T>
void Sim<T>::stepTE(int t)
{
    const idx_t N = g.N();
    auto& hZ = F["hz"]; auto& eX = F["ex"]; auto& eY = F["ey"];
    Dxf.spmv(eY.data(), upd.data());
    Dyf.spmv(eX.data(), updt.data());
    if (useCpml) { cpml(upd, "eyx", axh, bxh); cpml(updt, "exy", ayh, byh); }
    VEC_OP(upd[i] -= updt[i]);
    VEC_OP(upd[i] *= invMuXY[i]);
    VEC_OP(hZ[i] -= upd[i]);
    for (int l = 0; l < L; ++l) {
        const T cc = emCc[l];
        auto& rx = R["rx"][l];
        auto& ry = R["ry"][l];
        const auto& cdx = CdX[l];
        const auto& cdy = CdY[l];
        VEC_OP(T u = cc * rx[i]; T ut = cdx[i] * eX[i]; rx[i] = ut + u);
        VEC_OP(T u = cc * ry[i]; T ut = cdy[i] * eY[i]; ry[i] = ut + u);
    }
    Dyb.spmv(hZ.data(), upd.data());
    if (useCpml) cpml(upd, "hzy", ay, by);
    for (int l = 0; l < L; ++l) { const auto& r = R["rx"][l]; VEC_OP(upd[i] -= DT * r[i]); }
    VEC_OP(upd[i] *= CbX[i]);
    VEC_OP(updt[i] = CaX[i] * eX[i]);
    VEC_OP(eX[i] = updt[i] + upd[i]);
    Dxb.spmv(hZ.data(), updt.data());
    if (useCpml) cpml(updt, "hzx", ax, bx);
    VEC_OP(upd[i] = -updt[i]);
    for (int l = 0; l < L; ++l) { const auto& r = R["ry"][l]; VEC_OP(upd[i] -= DT * r[i]); }
    VEC_OP(upd[i] *= CbY[i]);
    VEC_OP(updt[i] = CaY[i] * eY[i]);
    VEC_OP(eY[i] = updt[i] + upd[i]);
    if (useAbs) {
        for (auto* v : {&eY, &eX, &hZ}) { auto& w = *v; VEC_OP(w[i] *= damping[i]); }
    }
    applySources(t);
    gather(t);
}

// FD3Demem::run (ForwardSolverEM/ForwardSolver3Demem.cpp:140-237) and
// FD3Dviscoemem::run (ForwardSolverEM/ForwardSolver3Dviscoemem.cpp:186-309).
// CPML as CPMLEM3D.cpp:25-108: E derivatives use the half profile, H
// derivatives the full one, except hyx, which uses the half profile there.
template <class T>
void Sim<T>::stepEM3D(int t)
{
    const idx_t N = g.N();
    auto& hX = F["hx"]; auto& hY = F["hy"]; auto& hZ = F["hz"];
    auto& eX = F["ex"]; auto& eY = F["ey"]; auto& eZ = F["ez"];
    Dyf.spmv(eZ.data(), upd.data());
    Dzf.spmv(eY.data(), updt.data());
    if (useCpml) { cpml(upd, "ezy", ayh, byh); cpml(updt, "eyz", azh, bzh); }
    VEC_OP(upd[i] -= updt[i]);
    VEC_OP(upd[i] *= invMuYZ[i]);
    VEC_OP(hX[i] -= upd[i]);
    Dzf.spmv(eX.data(), upd.data());
    Dxf.spmv(eZ.data(), updt.data());
    if (useCpml) { cpml(upd, "exz", azh, bzh); cpml(updt, "ezx", axh, bxh); }
    VEC_OP(upd[i] -= updt[i]);
    VEC_OP(upd[i] *= invMuXZ[i]);
    VEC_OP(hY[i] -= upd[i]);
    Dxf.spmv(eY.data(), upd.data());
    Dyf.spmv(eX.data(), updt.data());
    if (useCpml) { cpml(upd, "eyx", axh, bxh); cpml(updt, "exy", ayh, byh); }
    VEC_OP(upd[i] -= updt[i]);
    VEC_OP(upd[i] *= invMuXY[i]);
    VEC_OP(hZ[i] -= upd[i]);
    for (int l = 0; l < L; ++l) {
        const T cc = emCc[l];
        for (auto [rn, cdv, e] : {std::make_tuple("rx", &CdX, &eX), std::make_tuple("ry", &CdY, &eY), std::make_tuple("rz", &CdZ, &eZ)}) {
            auto& r = R[rn][l];
            const auto& cd = (*cdv)[l];
            const auto& ef = *e;
            VEC_OP(T u = cc * r[i]; T ut = cd[i] * ef[i]; r[i] = ut + u);
        }
    }
    // ex
    Dyb.spmv(hZ.data(), upd.data());
    Dzb.spmv(hY.data(), updt.data());
    if (useCpml) { cpml(upd, "hzy", ay, by); cpml(updt, "hyz", az, bz); }
    VEC_OP(upd[i] -= updt[i]);
    for (int l = 0; l < L; ++l) { const auto& r = R["rx"][l]; VEC_OP(upd[i] -= DT * r[i]); }
    VEC_OP(upd[i] *= CbX[i]);
    VEC_OP(updt[i] = CaX[i] * eX[i]);
    VEC_OP(eX[i] = updt[i] + upd[i]);
    // ey
    Dzb.spmv(hX.data(), upd.data());
    Dxb.spmv(hZ.data(), updt.data());
    if (useCpml) { cpml(upd, "hxz", az, bz); cpml(updt, "hzx", ax, bx); }
    VEC_OP(upd[i] -= updt[i]);
    for (int l = 0; l < L; ++l) { const auto& r = R["ry"][l]; VEC_OP(upd[i] -= DT * r[i]); }
    VEC_OP(upd[i] *= CbY[i]);
    VEC_OP(updt[i] = CaY[i] * eY[i]);
    VEC_OP(eY[i] = updt[i] + upd[i]);
    // ez
    Dxb.spmv(hY.data(), upd.data());
    Dyb.spmv(hX.data(), updt.data());
    if (useCpml) { cpml(upd, "hyx", axh, bxh); cpml(updt, "hxy", ay, by); }
    VEC_OP(upd[i] -= updt[i]);
    for (int l = 0; l < L; ++l) { const auto& r = R["rz"][l]; VEC_OP(upd[i] -= DT * r[i]); }
    VEC_OP(upd[i] *= CbZ[i]);
    VEC_OP(updt[i] = CaZ[i] * eZ[i]);
    VEC_OP(eZ[i] = updt[i] + upd[i]);
    if (useAbs) {
        for (auto* v : {&eZ, &eY, &eX, &hX, &hY, &hZ}) { auto& w = *v; VEC_OP(w[i] *= damping[i]); }
    }
    applySources(t);
    gather(t);
}

// snapType 3 energies: FD2Delastic::getCurl/getDiv (Wavefields2Delastic.cpp:218-250),
// FD3Delastic::getCurl/getDiv (Wavefields3Delastic.cpp:197-240)
template <class T>
void Sim<T>::curlDiv(std::vector<T>& curl, std::vector<T>& div)
{
    const idx_t N = g.N();
    curl.assign(N, 0);
    div.assign(N, 0);
    auto& vX = F["vx"];
    auto& vY = F["vy"];
    std::vector<T> a(N), b(N);
    if (!is3d) {
        Dyf.spmv(vX.data(), a.data());
        Dxf.spmv(vY.data(), b.data());
        VEC_OP(T c = a[i]; c -= b[i]; c *= std::sqrt(mu[i]); curl[i] = c);
        Dxb.spmv(vX.data(), a.data());
        Dyb.spmv(vY.data(), b.data());
        VEC_OP(T d = a[i]; d += b[i]; d *= std::sqrt(M[i]); div[i] = d);
        return;
    }
    auto& vZ = F["vz"];
    Dyf.spmv(vZ.data(), a.data());
    Dzf.spmv(vY.data(), b.data());
    VEC_OP(T u = a[i] - b[i]; curl[i] = u * u);
    Dzf.spmv(vX.data(), a.data());
    Dxf.spmv(vZ.data(), b.data());
    VEC_OP(T u = a[i] - b[i]; curl[i] += u * u);
    Dxf.spmv(vY.data(), a.data());
    Dyf.spmv(vX.data(), b.data());
    VEC_OP(T u = a[i] - b[i]; curl[i] += u * u; curl[i] *= mu[i]; curl[i] = std::sqrt(curl[i]));
    Dxb.spmv(vX.data(), a.data());
    Dyb.spmv(vY.data(), b.data());
    VEC_OP(div[i] = a[i] + b[i]);
    Dzb.spmv(vZ.data(), a.data());
    VEC_OP(T d = div[i] + a[i]; d *= d; d *= M[i]; div[i] = std::sqrt(d));
}

#undef VEC_OP

} // namespace refcpu
