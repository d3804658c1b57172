// wavelets.cpp — source time functions of the reference's Sources::generateSyntheticSignal
// (Acquisition/Sources.cpp:157-215), evaluated in single precision at t = k*DT.
#include <cmath>
#include <vector>

#include "wave_internal.h"

namespace wave {

int make_wavelet(int shape, int nt, double dt_, double fc_, double amp_, double tshift_, float* out)
{
    if (nt <= 0 || dt_ <= 0 || !out) return WAVE_ERR_ARG;
    const float DT = static_cast<float>(dt_), FC = static_cast<float>(fc_);
    const float AMP = static_cast<float>(amp_), TS = static_cast<float>(tshift_);
    std::vector<float> s(nt, 0.0f);
    auto t_of = [&](int k) { return static_cast<float>(k) * DT; };
    switch (shape) {
    case 1: { // Ricker (SourceSignal/Ricker.cpp:29-53): AMP(1-2tau^2)exp(-tau^2), tau = pi fc (t - 1.5/fc - tshift)
        if (FC <= 0) return WAVE_ERR_ARG;
        const float h = 1.5f / FC + TS;
        const float pf = static_cast<float>(M_PI * FC);
        for (int k = 0; k < nt; ++k) {
            float tau = (t_of(k) - h) * pf;
            float t2 = tau * tau;
            s[k] = AMP * ((1.0f - 2.0f * t2) * std::exp(-1.0f * t2));
        }
        break;
    }
    case 2:   // SinW (SourceSignal/SinW.cpp): sin(tau) - 0.5 sin(2 tau) over one period after tshift
    case 3:   // SinThree (SourceSignal/SinThree.cpp): sin(pi fc (t - tshift))^3 over one period
    case 6: { // IntgSinThree (SourceSignal/IntgSinThree.cpp)
        if (FC <= 0) return WAVE_ERR_ARG;
        long long i1 = static_cast<long long>(std::floor(TS / DT));
        long long i2 = i1 + static_cast<long long>(std::floor(1.0 / FC / DT));
        if (i2 > nt) i2 = nt - 1;
        long long count = 0;
        for (long long i = i1; i <= i2 && i < nt; ++i, ++count) {
            if (i < 0) continue;
            if (shape == 2) {
                double a = 2.0 * count * DT * M_PI * FC;
                s[i] = AMP * static_cast<float>(std::sin(a) - std::sin(2.0 * a) / 2.0);
            } else if (shape == 3) {
                double a = count * DT * M_PI * FC;
                s[i] = AMP * static_cast<float>(std::pow(std::sin(a), 3));
            } else {
                double a = count * DT * M_PI * FC;
                double c = std::cos(a);
                double v = (0.5 + (0.25 * std::pow(c, 3) - 0.75 * c)) / FC / M_PI / 0.75;
                s[i] = AMP * static_cast<float>(v);
            }
        }
        if (shape == 6) {
            // IntgSinThree adds 0.5 at every sample before scaling (its "half"
            // vector spans the whole trace), so outside the pulse the signal is
            // the constant AMP*0.5/FC/pi/0.75.
            for (long long i = 0; i < nt; ++i) {
                if (i >= i1 && i <= i2) continue;
                s[i] = AMP * static_cast<float>(0.5 / FC / M_PI / 0.75);
            }
        }
        break;
    }
    case 4: { // FGaussian (SourceSignal/FGaussian.cpp): -2 AMP tau exp(-tau^2), tau = pi fc (t - 1.2/fc - tshift)
        if (FC <= 0) return WAVE_ERR_ARG;
        const float h = 1.2f / FC + TS;
        const float pf = static_cast<float>(M_PI * FC);
        for (int k = 0; k < nt; ++k) {
            float tau = (t_of(k) - h) * pf;
            s[k] = AMP * ((-2.0f * tau) * std::exp(-1.0f * tau * tau));
        }
        break;
    }
    case 5: { // Spike (SourceSignal/Spike.cpp)
        long long i = static_cast<long long>(std::floor(TS / DT));
        if (i < 0 || i >= nt) return WAVE_ERR_ARG;
        s[i] = AMP;
        break;
    }
    case 7: { // Ricker_GprMax (SourceSignal/Ricker_GprMax.cpp:29-59)
        if (FC <= 0) return WAVE_ERR_ARG;
        const float h = 1.0f / FC + TS;
        const float zeta = static_cast<float>(2.0 * M_PI * M_PI * FC * FC);
        const float scale = -2.0f * (zeta * std::exp((1.0f / zeta) / 4.0f));
        for (int k = 0; k < nt; ++k) {
            float tau = t_of(k) - h;
            float e = std::exp(-1.0f * (zeta * (tau * tau)));
            s[k] = AMP * (scale * (e * tau));
        }
        break;
    }
    case 8: { // Berlage (SourceSignal/Berlage.cpp): cos(2 pi fc t') t'^2 exp(-2 fc t') H(t'), normalised to AMP
        if (FC <= 0) return WAVE_ERR_ARG;
        const float h = 1.0f / FC + TS;
        float mx = 0.0f;
        for (int k = 0; k < nt; ++k) {
            float tau = t_of(k) - h;
            float v = std::cos(static_cast<float>(2.0 * M_PI * FC) * tau);
            v *= std::pow(tau, 2.0f);
            v *= std::exp(-(2.0f * FC) * tau);
            float hv = tau > 0.0f ? 1.0f : (tau == 0.0f ? 1.0f : 0.0f);
            v *= hv;
            s[k] = v;
            mx = std::fmax(mx, std::fabs(v));
        }
        if (mx > 0) for (int k = 0; k < nt; ++k) s[k] *= AMP / mx;
        break;
    }
    case 9: { // Sin (SourceSignal/Sin.cpp): AMP sin(2 pi fc (t - tshift))
        for (int k = 0; k < nt; ++k) {
            float tau = (t_of(k) - TS) * static_cast<float>(2.0 * M_PI * FC);
            s[k] = AMP * std::sin(tau);
        }
        break;
    }
    default: return WAVE_ERR_ARG;
    }
    for (int k = 0; k < nt; ++k) out[k] = s[k];
    return WAVE_OK;
}

} // namespace wave
