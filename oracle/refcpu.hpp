// refcpu.hpp — TEST INFRASTRUCTURE ONLY (the oracle).
//
// CPU restatement of WAVE-Simulation's forward time step, templated on the
// value type: refcpu<float> stands in for the reference's own FP32 CPU run,
// refcpu<double> is the FP64 oracle. It follows the reference formulation
// operation by operation: derivative operators assembled as CSR matrices
// (including the edge-order reduction of the sparse path and the image method
// of the free surface), one whole-array pass per vector operation, CPML as
// psi = b*psi + a*d on full-length coefficient vectors, source scatter and
// receiver gather, and the full state copy of Simulation.cpp:450 each step.
//
// Only tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
// this code, and only as the checker / the timed CPU baseline. The product
// library never links it.
//
// Parity is pinned against the reference's own golden seismograms
// (par/ci/seismogram.*.ref.*.mtx) with the reference's metric
// (src/Tests/IntegrationTest/Test_CompareSeismogram.cpp:57-88).
#pragma once

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <limits>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../include/wave.h"

namespace refcpu {

using idx_t = int64_t;

// ----------------------------------------------------------------------------
// FD coefficients, Derivatives::setFDCoef (ForwardSolver/Derivatives/Derivatives.cpp:2000-2042).
// Literals are double expressions converted to the value type, as there.
// ----------------------------------------------------------------------------
inline const std::vector<double>& fd_coef_d(int q)
{
    static const std::map<int, std::vector<double>> m = {
        {2, {-1.0, 1.0}},
        {4, {1.0 / 24.0, -9.0 / 8.0, 9.0 / 8.0, -1.0 / 24.0}},
        {6, {-3.0 / 640.0, 25.0 / 384.0, -75.0 / 64.0, 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0}},
        {8, {5.0 / 7168.0, -49.0 / 5120.0, 245.0 / 3072.0, -1225.0 / 1024.0, 1225.0 / 1024.0,
             -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0}},
        {10, {-8756999275442633.0 / 73786976294838206464.0, 8142668969129685.0 / 4611686018427387904.0,
              -567.0 / 40960.0, 735.0 / 8192.0, -19845.0 / 16384.0, 19845.0 / 16384.0, -735.0 / 8192.0,
              567.0 / 40960.0, -8142668969129685.0 / 4611686018427387904.0,
              8756999275442633.0 / 73786976294838206464.0}},
        {12, {6448335830095439.0 / 295147905179352825856.0, -1655620175512543.0 / 4611686018427387904.0,
              6842103786556949.0 / 2305843009213693952.0, -628618285389933.0 / 36028797018963968.0,
              436540475965291.0 / 4503599627370496.0, -2750204998582123.0 / 2251799813685248.0,
              2750204998582123.0 / 2251799813685248.0, -436540475965291.0 / 4503599627370496.0,
              628618285389933.0 / 36028797018963968.0, -6842103786556949.0 / 2305843009213693952.0,
              1655620175512543.0 / 4611686018427387904.0, -6448335830095439.0 / 295147905179352825856.0}}};
    auto it = m.find(q);
    if (it == m.end())
        throw std::invalid_argument("unsupported spatialFDorder");
    return it->second;
}

template <class T>
inline T fd_coef(int q, int j) { return static_cast<T>(fd_coef_d(q)[j]); }

// ----------------------------------------------------------------------------
// Grid, Coordinates::mapIndex2coordinate / map3Dcoordinate2index
// (Acquisition/Coordinates.cpp:598-700): idx = x + z*NX + y*NX*NZ.
// ----------------------------------------------------------------------------
struct Grid {
    idx_t NX = 1, NY = 1, NZ = 1;
    idx_t N() const { return NX * NY * NZ; }
    idx_t index(idx_t x, idx_t y, idx_t z) const { return x + z * NX + y * NX * NZ; }
    void coord(idx_t i, idx_t& x, idx_t& y, idx_t& z) const
    {
        y = i / (NX * NZ);
        i -= y * NX * NZ;
        z = i / NX;
        x = i - z * NX;
    }
    // Coordinates::estimateDistanceToEdges3D (Coordinates.cpp:734-750)
    static idx_t edge(idx_t c, idx_t n) { return !((n - 1 - c) < c) ? c : (n - 1 - c); }
};

// ----------------------------------------------------------------------------
// CSR matrix with the reference's row assembly order (MatrixAssembly::push).
// ----------------------------------------------------------------------------
template <class T>
struct CSR {
    idx_t n = 0;
    std::vector<idx_t> ptr;
    std::vector<idx_t> col;
    std::vector<T> val;
    bool empty() const { return n == 0; }
    void spmv(const T* x, T* y) const
    {
#pragma omp parallel for schedule(static)
        for (idx_t r = 0; r < n; ++r) {
            T s = 0;
            for (idx_t k = ptr[r]; k < ptr[r + 1]; ++k)
                s += val[k] * x[col[k]];
            y[r] = s;
        }
    }
};

// One row of a 1-D operator: (column coordinate along the axis, value).
template <class T>
using Row1D = std::vector<std::pair<idx_t, T>>;

enum class Axis { X, Y, Z };

// Builds an N x N CSR matrix whose row at point p only depends on p's
// coordinate along `axis`, from the 1-D rows rows1d[c].
template <class T>
CSR<T> kron_axis(const Grid& g, Axis axis, const std::vector<Row1D<T>>& rows1d)
{
    CSR<T> A;
    A.n = g.N();
    A.ptr.assign(A.n + 1, 0);
    for (idx_t r = 0; r < A.n; ++r) {
        idx_t x, y, z;
        g.coord(r, x, y, z);
        idx_t c = axis == Axis::X ? x : (axis == Axis::Y ? y : z);
        A.ptr[r + 1] = A.ptr[r] + static_cast<idx_t>(rows1d[c].size());
    }
    A.col.resize(A.ptr[A.n]);
    A.val.resize(A.ptr[A.n]);
#pragma omp parallel for schedule(static)
    for (idx_t r = 0; r < A.n; ++r) {
        idx_t x, y, z;
        g.coord(r, x, y, z);
        idx_t c = axis == Axis::X ? x : (axis == Axis::Y ? y : z);
        idx_t k = A.ptr[r];
        for (auto const& e : rows1d[c]) {
            idx_t cx = x, cy = y, cz = z;
            if (axis == Axis::X) cx = e.first;
            else if (axis == Axis::Y) cy = e.first;
            else cz = e.first;
            A.col[k] = g.index(cx, cy, cz);
            A.val[k] = e.second;
            ++k;
        }
    }
    return A;
}

// Sparse forward operator row with edge-order reduction
// (Derivatives::calcDxf/calcDyf/calcDzf, Derivatives.cpp:129-185, 210-270, 303-357).
// Values: (c_j / DH) then scaled by DT (FDTD3D.cpp:230-301, FDTD2D.cpp:194-230).
template <class T>
Row1D<T> sparse_row_forward(idx_t c, idx_t n, int order, T DH, T DT)
{
    Row1D<T> row;
    int q = order;
    for (int j = 0; j < q; ++j) {
        idx_t X = c + (j - q / 2 + 1);
        idx_t Xmin = c + (-q / 2 + 1);
        idx_t Xmax = c + q / 2;
        if (Xmin < 0) {
            q += 2 * static_cast<int>(Xmin);
            j--;
        } else if (Xmax >= n) {
            q -= 2 * static_cast<int>(Xmax - n + 1);
            if (q == 0) {
                q = 2;
                c -= 1;
            }
            j--;
        } else {
            T v = fd_coef<T>(q, j) / DH;
            row.emplace_back(X, static_cast<T>(v * DT));
        }
    }
    return row;
}

// Sparse backward operator row (Derivatives::calcDxb/Dyb/Dzb,
// Derivatives.cpp:706-760, 770-850, 1180-1234).
template <class T>
Row1D<T> sparse_row_backward(idx_t c, idx_t n, int order, T DH, T DT)
{
    Row1D<T> row;
    int q = order;
    for (int j = 0; j < q; ++j) {
        idx_t X = c + (j - q / 2);
        idx_t Xmin = c + (-q / 2);
        idx_t Xmax = c + (q / 2 - 1);
        if (Xmin < 0) {
            q += 2 * static_cast<int>(Xmin);
            if (q == 0) {
                q = 2;
                c += 1;
            }
            j--;
        } else if (Xmax >= n) {
            q -= 2 * static_cast<int>(Xmax - n + 1);
            j--;
        } else {
            T v = fd_coef<T>(q, j) / DH;
            row.emplace_back(X, static_cast<T>(v * DT));
        }
    }
    return row;
}

// Zero-padded operator row: the stencil-matrix path (useStencilMatrix=1) and
// the rule the reference's CI goldens were made with. Stencil1D with offsets
// j - q/2 + 1 (Dxf) and Dxb = -Dxf^T (FDTD3D.cpp:183-219, FDTD2D.cpp:156-180),
// scaled by DT/DH; LAMA's stencil matrix drops neighbours outside the grid.
template <class T>
Row1D<T> stencil_row(idx_t c, idx_t n, int q, bool forward, T DH, T DT)
{
    Row1D<T> row;
    T s = DT / DH;
    for (int j = 0; j < q; ++j) {
        idx_t X = forward ? c + (j - q / 2 + 1) : c + (j - q / 2);
        if (X < 0 || X >= n) continue;
        // Dxb = -(Dxf)^T: entry at offset (j - q/2) is -c_{q-1-j} = c_j
        row.emplace_back(X, static_cast<T>(fd_coef<T>(q, j) * s));
    }
    return row;
}

// Free-surface (image method) rows along depth: DyfFreeSurface
// (Derivatives.cpp:367-440) and DybFreeSurface (Derivatives.cpp:448-526);
// no edge-order reduction, columns outside [0, NY) are dropped.
template <class T>
Row1D<T> fs_row(idx_t y, idx_t n, int q, bool forward, T DH, T DT)
{
    Row1D<T> row;
    for (int j = 0; j < q; ++j) {
        idx_t Y = forward ? y + (j - q / 2 + 1) : y + (j - q / 2);
        T fdCoeff = fd_coef<T>(q, j);
        T diffCoeff = 0;
        if (forward) {
            if (q >= 2 + 2 * y + j) diffCoeff = fd_coef<T>(q, static_cast<int>(q - 2 - 2 * y - j));
        } else {
            if (q >= 1 + 2 * y + j) diffCoeff = fd_coef<T>(q, static_cast<int>(q - 1 - 2 * y - j));
        }
        if (Y >= 0 && Y < n) {
            T v = (fdCoeff - diffCoeff) / DH;
            row.emplace_back(Y, static_cast<T>(v * DT));
        }
    }
    return row;
}

// ----------------------------------------------------------------------------
// Averaging matrices (Modelparameter.cpp:336-624), applied matrix-free with
// the same row weights and the same far-edge fallbacks.
// ----------------------------------------------------------------------------
template <class T>
void average2(const Grid& g, Axis a, const T* in, T* out)
{
    const idx_t N = g.N();
#pragma omp parallel for schedule(static)
    for (idx_t r = 0; r < N; ++r) {
        idx_t x, y, z;
        g.coord(r, x, y, z);
        idx_t nx = x, ny = y, nz = z;
        bool ok;
        if (a == Axis::X) { nx = x + 1; ok = nx < g.NX; }
        else if (a == Axis::Y) { ny = y + 1; ok = ny < g.NY; }
        else { nz = z + 1; ok = nz < g.NZ; }
        if (ok) {
            T s = T(0.5) * in[r];
            s += T(0.5) * in[g.index(nx, ny, nz)];
            out[r] = s;
        } else {
            out[r] = T(1.0) * in[r];
        }
    }
}

// calc4PointAverageMatrixRow (Modelparameter.cpp:448-527) for the XY, XZ, YZ
// planes: pX/pY/pZ as in calcAverageMatrixXY/XZ/YZ (Modelparameter.cpp:533-624).
template <class T>
void average4(const Grid& g, int plane /*0=XY,1=XZ,2=YZ*/, const T* in, T* out)
{
    const idx_t N = g.N();
#pragma omp parallel for schedule(static)
    for (idx_t r = 0; r < N; ++r) {
        idx_t x, y, z;
        g.coord(r, x, y, z);
        idx_t pX[5], pY[5], pZ[5];
        if (plane == 0) {
            idx_t X[5] = {0, x, x + 1, x, x + 1}, Y[5] = {0, y, y, y + 1, y + 1}, Z[5] = {0, z, z, z, z};
            std::copy(X, X + 5, pX); std::copy(Y, Y + 5, pY); std::copy(Z, Z + 5, pZ);
        } else if (plane == 1) {
            idx_t X[5] = {0, x, x + 1, x, x + 1}, Y[5] = {0, y, y, y, y}, Z[5] = {0, z, z, z + 1, z + 1};
            std::copy(X, X + 5, pX); std::copy(Y, Y + 5, pY); std::copy(Z, Z + 5, pZ);
        } else {
            idx_t X[5] = {0, x, x, x, x}, Y[5] = {0, y, y + 1, y, y + 1}, Z[5] = {0, z, z, z + 1, z + 1};
            std::copy(X, X + 5, pX); std::copy(Y, Y + 5, pY); std::copy(Z, Z + 5, pZ);
        }
        idx_t maxX = *std::max_element(pX, pX + 5);
        idx_t maxY = *std::max_element(pY, pY + 5);
        idx_t maxZ = *std::max_element(pZ, pZ + 5);
        bool inX = maxX < g.NX, inY = maxY < g.NY, inZ = maxZ < g.NZ;
        T s = 0;
        bool any = false;
        if (inX && inY && inZ) {
            s = T(0.25) * in[r];
            s += T(0.25) * in[g.index(pX[2], pY[2], pZ[2])];
            s += T(0.25) * in[g.index(pX[3], pY[3], pZ[3])];
            s += T(0.25) * in[g.index(pX[4], pY[4], pZ[4])];
            any = true;
        }
        if (inX && !inY && inZ) { // bottom side
            s = T(0.5) * in[g.index(maxX, pY[1], maxZ)];
            s += T(0.5) * in[r];
            any = true;
        }
        if (!inX && inY && inZ) { // right side
            s = T(0.5) * in[g.index(pX[1], maxY, maxZ)];
            s += T(0.5) * in[r];
            any = true;
        }
        if (inX && inY && !inZ) { // back side
            s = T(0.5) * in[g.index(maxX, maxY, pZ[1])];
            s += T(0.5) * in[r];
            any = true;
        }
        if ((!inX && !inY && inZ) || (inX && !inY && !inZ) || (!inX && inY && !inZ)) {
            s = T(1.0) * in[r];
            any = true;
        }
        out[r] = any ? s : T(0);
    }
}

template <class T>
inline bool is_invalid(T v) { return std::isnan(v) || v == std::numeric_limits<T>::infinity() || -v == std::numeric_limits<T>::infinity(); }

// ----------------------------------------------------------------------------
// CPML coefficients, CPML::calcCoeffCPML (ForwardSolver/BoundaryCondition/CPML.cpp:38-68).
// ----------------------------------------------------------------------------
template <class T>
void cpml_coeff(std::vector<T>& a, std::vector<T>& b, T NPower, T fc, T vmax, T DT, T DH, bool shiftGrid)
{
    idx_t w = static_cast<idx_t>(a.size());
    T shift = shiftGrid ? T(0.5) : T(0);
    T RCoef = T(0.0008);
    T alpha_max = static_cast<T>(2.0 * M_PI * (fc / 2.0));
    T d0 = -(NPower + 1) * vmax * std::log(RCoef) / (T(2.0) * T(w) * DH);
    for (idx_t i = 0; i < w; ++i) {
        T pn = static_cast<T>(T(w - i) - shift) / T(w);
        T d = d0 * std::pow(pn, NPower);
        T alpha = alpha_max * (T(1.0) - pn);
        b[i] = std::exp(-(d + alpha) * DT);
        if (std::abs(d) > T(1.0e-6))
            a[i] = d * (b[i] - T(1.0)) / (d + alpha);
        else
            a[i] = T(0);
    }
}

// Per-axis full/half coefficient profile (CPML3D.cpp:222-371, CPML2D.cpp,
// CPML2DAcoustic.cpp:106-200): near slab uses (a, a_half), far slab swaps them;
// the top depth slab is dropped when the free surface is on.
template <class T>
struct CpmlAxis {
    std::vector<T> a_full, b_full, a_half, b_half; // length n along the axis
};

template <class T>
CpmlAxis<T> cpml_axis(idx_t n, int width, const std::vector<T>& a, const std::vector<T>& b,
                      const std::vector<T>& ah, const std::vector<T>& bh, bool dropTop)
{
    CpmlAxis<T> P;
    P.a_full.assign(n, 0); P.b_full.assign(n, 0); P.a_half.assign(n, 0); P.b_half.assign(n, 0);
    for (idx_t c = 0; c < n; ++c) {
        idx_t d = Grid::edge(c, n);
        if (d < width) {
            if (c < width) {
                if (dropTop) continue;
                P.a_full[c] = a[d]; P.b_full[c] = b[d]; P.a_half[c] = ah[d]; P.b_half[c] = bh[d];
            } else {
                P.a_full[c] = ah[d]; P.b_full[c] = bh[d]; P.a_half[c] = a[d]; P.b_half[c] = b[d];
            }
        }
    }
    return P;
}

// ----------------------------------------------------------------------------
// The simulation state and the per-equation time step.
// ----------------------------------------------------------------------------
template <class T>
struct Model {
    // seismic
    std::vector<T> rho, vp, vs, taup, taus;
    // EM
    std::vector<T> eps_r, sigma, mu_r, tau_eps, tau_sigma;
};

struct Acq {
    std::vector<idx_t> idx;
    std::vector<int> type;
};

template <class T>
class Sim {
  public:
    wave_config cfg{};
    Grid g;
    int NT = 0;
    int order = 2;
    bool is3d = false, stencil = false;
    int eq = 0;
    int L = 0;
    T DT = 0, DH = 0;
    bool fs = false, useAbs = false, useCpml = false;

    // operators
    CSR<T> Dxf, Dxb, Dyf, Dyb, Dzf, Dzb, DyfFS, DybFS;

    // material (prepared)
    std::vector<T> M, mu, invRhoX, invRhoY, invRhoZ, invRho, muXY, muXZ, muYZ;
    std::vector<T> tauP, tauS, tauSXY, tauSXZ, tauSYZ, onePlusLtauP, onePlusLtauS;
    std::vector<T> relaxTime, invRelaxTime, viscoC1, viscoC2;
    std::vector<T> emTauE, emTauS;   // visco-EM tau_eps and tau_sigma (times 1 / (2 pi f_CPML)), kept for the adjoint
    T DThalf = 0;
    // EM
    std::vector<T> CaZ, CbZ, CaX, CbX, CaY, CbY, invMuXZ, invMuYZ, invMuXY;
    std::vector<T> emCc;                              // visco EM: C_c per mechanism
    std::vector<std::vector<T>> CdX, CdY, CdZ;        // visco EM: C_d per mechanism (DT folded in)
    // boundaries
    std::vector<T> damping;                   // ABS (1 outside the frame)
    std::vector<T> fsZero, fsSelect, scaleH, scaleV;  // free surface
    std::vector<std::vector<T>> scaleRelH, scaleRelV; // visco free surface
    // CPML coefficient vectors (full grid, zero outside the slabs)
    std::vector<T> ax, bx, axh, bxh, ay, by, ayh, byh, az, bz, azh, bzh;

    // wavefields
    std::map<std::string, std::vector<T>> F;
    std::map<std::string, std::vector<std::vector<T>>> R; // memory variables
    std::map<std::string, std::vector<T>> psi;
    std::vector<T> upd, updt, upd2, vxx, vyy, vzz, tmp;
    std::map<std::string, std::vector<T>> Fcopy; // Simulation.cpp:450 state copy

    // acquisition
    Acq src, rec;
    std::vector<T> signals;   // nsrc x NT
    std::vector<T> seis;      // nrec x NT
    bool copyStateEachStep = true;

    void setup(const wave_config& c, const Model<T>& m);
    void step(int t);
    void reset();
    void curlDiv(std::vector<T>& curl, std::vector<T>& div);

  private:
    void buildOperators();
    void prepareModel(const Model<T>& m);
    void buildBoundaries();
    std::vector<T>& f(const char* name) { return F[name]; }
    void cpml(std::vector<T>& d, const char* name, const std::vector<T>& a, const std::vector<T>& b);
    void applySources(int t);
    void gather(int t);
    void stepAcoustic(int t);
    void stepElastic(int t);
    void stepVisco(int t);
    void stepSH(int t);
    void stepTM(int t);
    void stepTE(int t);
    void stepEM3D(int t);
};

} // namespace refcpu

#include "refcpu_impl.hpp"
