// tables.cpp — host-side builders for the 1-D tables the kernels read:
// derivative-operator weights (interior + edge rows), CPML profiles and the
// ABS taper. Runs once per solver; nothing here is on the time-step path.
#include <cmath>
#include <stdexcept>

#include "wave_internal.h"

namespace wave {

// Staggered-grid FD coefficient sets of orders 2..12, as defined by
// Derivatives::setFDCoef (ForwardSolver/Derivatives/Derivatives.cpp:2000-2042);
// orders 10 and 12 are given there as exact binary fractions.
bool fd_coefficients(int order, std::vector<double>& c)
{
    switch (order) {
    case 2: c = {-1.0, 1.0}; return true;
    case 4: c = {1.0 / 24.0, -9.0 / 8.0, 9.0 / 8.0, -1.0 / 24.0}; return true;
    case 6: c = {-3.0 / 640.0, 25.0 / 384.0, -75.0 / 64.0, 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0}; return true;
    case 8:
        c = {5.0 / 7168.0, -49.0 / 5120.0, 245.0 / 3072.0, -1225.0 / 1024.0,
             1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0};
        return true;
    case 10:
        c = {-8756999275442633.0 / 73786976294838206464.0, 8142668969129685.0 / 4611686018427387904.0,
             -567.0 / 40960.0, 735.0 / 8192.0, -19845.0 / 16384.0,
             19845.0 / 16384.0, -735.0 / 8192.0, 567.0 / 40960.0,
             -8142668969129685.0 / 4611686018427387904.0, 8756999275442633.0 / 73786976294838206464.0};
        return true;
    case 12:
        c = {6448335830095439.0 / 295147905179352825856.0, -1655620175512543.0 / 4611686018427387904.0,
             6842103786556949.0 / 2305843009213693952.0, -628618285389933.0 / 36028797018963968.0,
             436540475965291.0 / 4503599627370496.0, -2750204998582123.0 / 2251799813685248.0,
             2750204998582123.0 / 2251799813685248.0, -436540475965291.0 / 4503599627370496.0,
             628618285389933.0 / 36028797018963968.0, -6842103786556949.0 / 2305843009213693952.0,
             1655620175512543.0 / 4611686018427387904.0, -6448335830095439.0 / 295147905179352825856.0};
        return true;
    default: return false;
    }
}

namespace {

struct Coefs {
    std::vector<float> v[13];
    explicit Coefs()
    {
        for (int q = 2; q <= 12; q += 2) {
            std::vector<double> d;
            fd_coefficients(q, d);
            for (double x : d) v[q].push_back(static_cast<float>(x));
        }
    }
};
const Coefs& coefs()
{
    static Coefs c;
    return c;
}

// Offset of tap j of an order-q stencil: forward-type j - q/2 + 1,
// backward-type j - q/2 (Derivatives.cpp:149, 728).
inline int tap_offset(bool forward, int q, int j) { return forward ? j - q / 2 + 1 : j - q / 2; }

// Edge row of a sparse operator with edge-order reduction
// (Derivatives.cpp:166-179 forward, 743-756 backward): the order is lowered
// by twice the overhang until the stencil fits; an order that drops to zero
// becomes a second-order stencil moved one point inward.
void reduced_row(bool forward, int c, int n, int q0, int& q, int& shift)
{
    q = q0;
    shift = 0;
    for (int guard = 0; guard < 64; ++guard) {
        int cc = c + shift;
        int lo = cc + tap_offset(forward, q, 0);
        int hi = cc + tap_offset(forward, q, q - 1);
        if (lo < 0) {
            q += 2 * lo;
            if (!forward && q == 0) { q = 2; shift += 1; }
        } else if (hi >= n) {
            q -= 2 * (hi - n + 1);
            if (forward && q == 0) { q = 2; shift -= 1; }
        } else {
            return;
        }
    }
    throw std::runtime_error("edge-order reduction did not converge");
}

} // namespace

OpHost build_op(int n, int order, OpKind kind, int stencilMode, int edgeReduce, float DH, float DT)
{
    const auto& C = coefs();
    const int H = order / 2;
    const bool forward = (kind == OP_F || kind == OP_FS_F);
    const bool fsk = (kind == OP_FS_F || kind == OP_FS_B);
    OpHost op;
    op.n = n;
    op.E = H + 1;
    op.full = n < 2 * op.E ? 1 : 0;
    const int slots = op.full ? n : 2 * op.E;
    op.tab.assign(static_cast<size_t>(slots) * kTabW, 0.0f);
    const float s = DT / DH; // stencil-matrix scaling (FDTD3D.cpp:210-216)
    auto scaled = [&](float c) -> float {
        if (stencilMode && !fsk) return c * s;
        float v = c / DH;     // sparse rows: c/DH, then *= DT (FDTD3D.cpp:250-256)
        return v * DT;
    };
    // interior weights
    for (int j = 0; j < order; ++j)
        op.w[kMaxHalf + tap_offset(forward, order, j)] = scaled(C.v[order][j]);

    auto fill_row = [&](int slot, int c) {
        float* row = &op.tab[static_cast<size_t>(slot) * kTabW];
        if (fsk) {
            // image method along depth (DyfFreeSurface Derivatives.cpp:367-440,
            // DybFreeSurface :448-526): tap j gets c_j - c_img where the image
            // tap mirrors column Y about the surface; columns outside [0,n) dropped.
            for (int j = 0; j < order; ++j) {
                int Y = c + tap_offset(forward, order, j);
                float fd = C.v[order][j];
                float diff = 0.0f;
                int img = forward ? order - 2 - 2 * c - j : order - 1 - 2 * c - j;
                if (img >= 0) diff = C.v[order][img];
                if (Y >= 0 && Y < n) {
                    float v = (fd - diff) / DH;
                    row[kMaxHalf + (Y - c)] = v * DT;
                }
            }
            return;
        }
        if (stencilMode || !edgeReduce) {
            for (int j = 0; j < order; ++j) {
                int X = c + tap_offset(forward, order, j);
                if (X >= 0 && X < n) row[kMaxHalf + (X - c)] = scaled(C.v[order][j]);
            }
            return;
        }
        int q, shift;
        reduced_row(forward, c, n, order, q, shift);
        for (int j = 0; j < q; ++j) {
            int X = c + shift + tap_offset(forward, q, j);
            row[kMaxHalf + (X - c)] = scaled(C.v[q][j]);
        }
    };
    if (op.full) {
        for (int c = 0; c < n; ++c) fill_row(c, c);
    } else {
        for (int c = 0; c < op.E; ++c) fill_row(c, c);
        for (int c = n - op.E; c < n; ++c) fill_row(op.E + c - (n - op.E), c);
    }
    return op;
}

// CPML damping profile, CPML::calcCoeffCPML (BoundaryCondition/CPML.cpp:38-68):
// d = d0*((w-i-shift)/w)^N, alpha = pi*fc*(1-(w-i-shift)/w), b = exp(-(d+alpha)DT),
// a = d(b-1)/(d+alpha), shift 0.5 for the half-grid profile; the near slab
// uses (a, a_half) and the far slab swaps them (CPML3D.cpp:304-362); the top
// depth slab is left out with a free surface.
CpmlHost build_cpml(int n, int width, bool dropTop, float NPower, float fc, float vmax, float DT, float DH)
{
    CpmlHost P;
    P.a_full.assign(n, 0.f); P.b_full.assign(n, 0.f); P.a_half.assign(n, 0.f); P.b_half.assign(n, 0.f);
    // compact psi layout: both slabs, or only the far slab when the near (top)
    // slab has no coefficients
    P.lo = (dropTop && n > 2 * width) ? 0 : 1;
    P.ns = n <= 2 * width ? n : (P.lo ? 2 * width : width);
    if (width <= 0) { P.ns = 0; return P; }
    std::vector<float> a(width), b(width), ah(width), bh(width);
    auto prof = [&](std::vector<float>& A, std::vector<float>& B, float shift) {
        const float R = 0.0008f;
        const float alpha_max = static_cast<float>(2.0 * M_PI * (fc / 2.0));
        const float d0 = -(NPower + 1) * vmax * std::log(R) / (2.0f * width * DH);
        for (int i = 0; i < width; ++i) {
            float pn = (static_cast<float>(width - i) - shift) / width;
            float d = d0 * std::pow(pn, NPower);
            float al = alpha_max * (1.0f - pn);
            B[i] = std::exp(-(d + al) * DT);
            A[i] = std::fabs(d) > 1.0e-6f ? d * (B[i] - 1.0f) / (d + al) : 0.0f;
        }
    };
    prof(a, b, 0.0f);
    prof(ah, bh, 0.5f);
    for (int c = 0; c < n; ++c) {
        int d = (n - 1 - c) < c ? (n - 1 - c) : c;   // Coordinates::estimateDistanceToEdges3D
        if (d >= width) continue;
        if (c < width) {
            if (dropTop) continue;
            P.a_full[c] = a[d]; P.b_full[c] = b[d]; P.a_half[c] = ah[d]; P.b_half[c] = bh[d];
        } else {
            P.a_full[c] = ah[d]; P.b_full[c] = bh[d]; P.a_half[c] = a[d]; P.b_half[c] = b[d];
        }
    }
    return P;
}

// ABS taper, ABS2D::init / ABS3D::init (ABS2D.cpp:130-137): exp(-(a(w-j))^2),
// a = sqrt(-ln(1 - DampingCoeff/100))/w.
std::vector<float> build_abs_coeff(int width, float dampingCoeff)
{
    std::vector<float> c(width > 0 ? width : 0);
    if (width <= 0) return c;
    float amp = 1.0f - dampingCoeff / 100.0f;
    float a = std::sqrt(-std::log(amp) / static_cast<float>(width * width));
    for (int j = 0; j < width; ++j) c[j] = std::exp(-(a * a * (width - j) * (width - j)));
    return c;
}

} // namespace wave
