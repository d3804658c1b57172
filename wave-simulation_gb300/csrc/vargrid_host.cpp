// vargrid_host.cpp — host-side set-up of the variable grid: the layered index
// space (Acquisition/Coordinates.cpp:35-245, 381-513, 603-698), the sparse FD
// operators of the acoustic equations on it (ForwardSolver/Derivatives/
// Derivatives.cpp:129-188, 210-282, 304-362, 367-430, 706-845, 1177-1245,
// DT scaling FDTD2D.cpp:193-229 / FDTD3D.cpp:230-300), the interface
// interpolations (Derivatives.cpp:1252-1546), the per-layer CPML coefficients
// (CPML2DAcoustic.cpp:105-210, CPML3DAcoustic.cpp) and the density-average
// partners (Modelparameter.cpp:336-446).
//
// Every row follows the reference's per-row assembly rule; the rows are then
// packed into fixed-width ELL blocks for the device.
#include "vargrid.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <unordered_map>

#include "wave_internal.h"

namespace wave {

void VarGridLayout::coord(long long idx, int& x, int& y, int& z) const
{
    int l = 0;
    while (l < nl - 1 && idx >= offset[l + 1]) ++l;
    idx -= offset[l];
    const long long plane = static_cast<long long>(vnx[l]) * vnz[l];
    const long long yy = idx / plane;
    idx -= yy * plane;
    const long long zz = idx / vnx[l];
    const long long xx = idx - zz * vnx[l];
    x = static_cast<int>(xx * dhf[l]);
    z = static_cast<int>(zz * dhf[l]);
    y = static_cast<int>(yy * dhf[l] + start[l]);
}

long long VarGridLayout::index(long long X, long long Y, long long Z) const
{
    if (X < 0 || X >= NX || Y < 0 || Y >= NY || Z < 0 || Z >= NZ) return -1;
    for (int l = 0; l < nl; ++l) {
        if (Y < start[l] || Y > end[l]) continue;
        const long long f = dhf[l];
        return X / f + (Z / f) * vnx[l] + ((Y - start[l]) / f) * vnx[l] * vnz[l] + offset[l];
    }
    return -1;   // between the stored rows of two layers
}

int vargrid_layout(const wave_config& c, VarGridLayout& L, std::string& err)
{
    L = VarGridLayout{};
    const bool is3d = c.dimension == 3;
    long long NX = c.NX, NY = c.NY, NZ = is3d ? c.NZ : 1;
    L.DH = static_cast<float>(c.DH);
    L.varGrid = c.useVariableGrid != 0;
    L.varOrder = c.useVariableFDoperators != 0 && c.useStencilMatrix == 0;
    const int rows = c.gridLayers;
    if (rows < 1 || rows > WAVE_MAX_GRID_LAYERS) {
        err = "gridLayers must be 1.." + std::to_string(WAVE_MAX_GRID_LAYERS);
        return WAVE_ERR_ARG;
    }
    if (c.gridInterface[0] != 0) {
        err = "First interface must by at y=0";
        return WAVE_ERR_ARG;
    }
    std::vector<int> iface(c.gridInterface + 1, c.gridInterface + rows);
    std::vector<int> dhf;
    if (L.varGrid) {
        dhf.assign(c.gridDHFactor, c.gridDHFactor + rows);
    } else {
        dhf.assign(rows, 1);   // variable FD orders on a regular grid (Coordinates.cpp:80-90)
    }
    for (size_t i = 1; i < iface.size(); ++i)
        if (iface[i] <= iface[i - 1]) {
            err = "interface coordinates must increase";
            return WAVE_ERR_ARG;
        }
    for (size_t i = 1; i < dhf.size(); ++i)
        if (dhf[i] != dhf[i - 1] * 3 && dhf[i] != dhf[i - 1] / 3 && dhf[i] != dhf[i - 1]) {
            err = "Only gridspacing changes with factor 3 eg: 1<->3 or 9<->3 are alowed";
            return WAVE_ERR_ARG;
        }
    const int nl = static_cast<int>(dhf.size());
    int dhMax = 0;
    for (int f : dhf) {
        int g = f;
        while (g > 1 && g % 3 == 0) g /= 3;
        if (f < 1 || g != 1) {
            err = "incompatible dhFactor, dhFactor must be 3^n";
            return WAVE_ERR_ARG;
        }
        dhMax = std::max(dhMax, f);
    }
    iface.insert(iface.begin(), -1);
    iface.push_back(static_cast<int>(NY - 1));
    long long NXmax = NX, NZmax = NZ;
    if (dhMax != 1) {
        while (NXmax > 0 && NXmax != (NXmax / dhMax) * dhMax + 1 + dhMax / 2) --NXmax;
        while (NZ != 1 && NZmax > 0 && NZmax != (NZmax / dhMax) * dhMax + 1 + dhMax / 2) --NZmax;
        if (NXmax <= 0 || NZmax <= 0) {
            err = "grid too small for the variable grid";
            return WAVE_ERR_ARG;
        }
        NX = NXmax;
        NZ = NZmax;
        // move interfaces up until every layer holds whole coarse cells
        // (Coordinates.cpp:170-190)
        int guard = 0;
        for (int layer = 0; layer < 1;) {
            ++layer;
            const int d = iface[layer] - iface[layer - 1] - 1;
            if (d % dhf[layer - 1] != 0) {
                --iface[layer];
                --layer;
            }
            if (++guard > 1 << 20) break;
        }
        for (int layer = 1; layer < nl;) {
            ++layer;
            const int d = iface[layer] - iface[layer - 1];
            if (d % dhf[layer - 1] != 0) {
                --iface[layer];
                --layer;
            }
            if (++guard > 1 << 20) break;
        }
    }
    NY = iface[nl] + 1;
    L.nl = nl;
    L.dhf = dhf;
    L.iface = iface;
    L.start.assign(nl, 0);
    L.end.assign(nl, 0);
    L.trans.assign(nl, 0);
    for (int l = 0; l < nl - 1; ++l) {
        if (dhf[l] < dhf[l + 1]) {
            L.trans[l] = 1;
            L.end[l] = iface[l + 1];
            L.start[l + 1] = iface[l + 1] + dhf[l + 1];
        } else if (dhf[l] > dhf[l + 1]) {
            L.trans[l] = -1;
            L.end[l] = iface[l + 1] - dhf[l];
            L.start[l + 1] = iface[l + 1];
        } else {
            L.trans[l] = 0;
            L.end[l] = iface[l + 1] - dhf[l];
            L.start[l + 1] = iface[l + 1];
        }
    }
    L.end[nl - 1] = iface[nl];
    L.vnx.assign(nl, 0); L.vny.assign(nl, 0); L.vnz.assign(nl, 0);
    L.offset.assign(nl + 1, 0);
    for (int l = 0; l < nl; ++l) {
        if (L.end[l] < L.start[l]) {
            err = "layer " + std::to_string(l) + " of the variable grid is empty";
            return WAVE_ERR_ARG;
        }
        L.vny[l] = (L.end[l] - L.start[l]) / dhf[l] + 1;
        L.vnx[l] = static_cast<int>(NXmax / dhf[l]) + (dhf[l] > 1 ? 1 : 0);
        L.vnz[l] = static_cast<int>(NZmax / dhf[l]) + (dhf[l] > 1 ? 1 : 0);
        L.offset[l + 1] = L.offset[l] + static_cast<long long>(L.vnx[l]) * L.vny[l] * L.vnz[l];
    }
    L.N = L.offset[nl];
    L.NX = static_cast<int>(NX);
    L.NY = static_cast<int>(NY);
    L.NZ = static_cast<int>(NZ);
    // FD order per layer (Derivatives.cpp:1663-1702)
    std::vector<double> tmp;
    if (L.varOrder) {
        L.order.assign(c.gridFDOrder, c.gridFDOrder + nl);
    } else {
        L.order.assign(1, c.spatialFDorder);
    }
    for (int o : L.order)
        if (!fd_coefficients(o, tmp)) {
            err = "spatialFDorder = " + std::to_string(o) + " Unsupported spatialFDorder value.";
            return WAVE_ERR_ARG;
        }
    // functions of y (getLayer :381-397, locatedOnInterface :455-465,
    // getTransition :499-513, distToInterface :472-481)
    L.layerY.assign(L.NY, 0); L.transY.assign(L.NY, 0); L.distY.assign(L.NY, 0); L.onIfaceY.assign(L.NY, 0);
    for (int y = 0; y < L.NY; ++y) {
        int layer = 0;
        for (; layer < nl; ++layer) {
            if (y < iface[layer + 1] && y > iface[layer]) break;
            if (y == iface[layer + 1]) {
                if (L.trans[layer] > 0) ++layer;
                break;
            }
        }
        L.layerY[y] = layer;
        bool on = false;
        for (int l = 0; l < nl; ++l)
            if (y == iface[l]) on = true;
        L.onIfaceY[y] = on;
        int tr = 0;
        if (on)
            for (int l = 0; l < nl; ++l)
                if (y == iface[l + 1]) tr = L.trans[l];
        L.transY[y] = tr;
        int d = L.NY;
        for (int i = 1; i < nl; ++i) d = std::min(d, std::abs(y - iface[i]));
        L.distY[y] = d;
    }
    return WAVE_OK;
}

namespace {

struct Tap {
    long long col;
    float val;
};

struct Assembler {
    const VarGridLayout& L;
    float DT;
    bool edge;     // reduce the order at the grid edges (else drop taps outside the grid)
    std::vector<double> coef[13];

    Assembler(const VarGridLayout& L_, float DT_, bool edge_) : L(L_), DT(DT_), edge(edge_)
    {
        for (int o = 2; o <= 12; o += 2) fd_coefficients(o, coef[o]);
    }
    int order_of(int layer) const { return L.varOrder ? L.order[layer] : L.order[0]; }
    // stencil value / DH (ValueType), then times DT (FDTD2D.cpp:212-215)
    float value(int order, int j, int dhLayer, int image = -1) const
    {
        float c = static_cast<float>(coef[order][j]);
        if (image >= 0) c = c - static_cast<float>(coef[order][image]);
        const float v = c / L.dh(dhLayer);
        return v * DT;
    }
    int reduce_at_interface(int order, int y, int layer) const
    {
        if (!L.varGrid) return order;
        const int dist = L.distY[y] / L.dhf[layer];
        if (dist == 0) return 2;
        return order > 2 * dist ? 2 * dist : order;
    }

    // Dxf / Dxb (Derivatives.cpp:149-184, 726-761) and Dzf / Dzb (:323-358, :1196-1241)
    void axis_row(int x, int y, int z, int axis, bool backward, std::vector<Tap>& out) const
    {
        const int layer = L.layerY[y];
        const int f = L.dhf[layer];
        const bool on = L.onIfaceY[y] != 0;
        int order = order_of(layer);
        int c = axis == 0 ? x : z;
        const int n = axis == 0 ? L.NX : L.NZ;
        const int sh = on ? (backward ? f / 3 : -(f / 3)) : 0;
        for (int j = 0; j < order; ++j) {
            const int lo = backward ? -order / 2 : -order / 2 + 1;
            const int P = c + sh + f * (j + lo);
            if (!edge) {
                if (P >= 0 && P < n) out.push_back({axis == 0 ? L.index(P, y, z) : L.index(x, y, P), value(order, j, layer)});
                continue;
            }
            const int Pmin = c + sh + f * lo;
            const int Pmax = c + sh + f * (lo + order - 1);
            if (Pmin < 0) {
                order += 2 * Pmin;
                if (backward && order == 0) {
                    order = 2;
                    c += 1;
                }
                --j;
            } else if (Pmax >= n) {
                order -= 2 * (Pmax - n + 1);
                if (!backward && order == 0) {
                    order = 2;
                    c -= 1;
                }
                --j;
            } else {
                out.push_back({axis == 0 ? L.index(P, y, z) : L.index(x, y, P), value(order, j, layer)});
            }
        }
    }

    // Dyf (:227-276) or, with the mirror free surface, DyfFreeSurface (:380-425)
    void dyf_row(int x, int y, int z, bool fs, std::vector<Tap>& out) const
    {
        const int layer = L.layerY[y];
        const int order0 = reduce_at_interface(order_of(layer), y, layer);
        const bool coarseToFine = L.onIfaceY[y] && L.transY[y] == -1;
        const int dl = coarseToFine ? layer + 1 : layer;
        const int f = L.dhf[dl];
        int order = order0;
        if (fs) {
            for (int j = 0; j < order; ++j) {
                const int Y = y + f * (j - order / 2 + 1);
                int img = -1;
                if (order >= 2 + 2 * y / f + j) img = order - 2 - 2 * y / f - j;
                if (Y >= 0 && Y < L.NY) out.push_back({L.index(x, Y, z), value(order, j, dl, img)});
            }
            return;
        }
        int yy = y;
        for (int j = 0; j < order; ++j) {
            const int Y = yy + f * (j - order / 2 + 1);
            if (!edge) {
                if (Y >= 0 && Y < L.NY) out.push_back({L.index(x, Y, z), value(order, j, dl)});
                continue;
            }
            const int Ymin = yy + f * (-order / 2 + 1);
            const int Ymax = yy + f * (order / 2);
            if (Ymin < 0) {
                order += 2 * Ymin;
                --j;
            } else if (Ymax >= L.NY) {
                order -= 2 * (Ymax - L.NY + 1);
                if (order == 0) {
                    order = 2;
                    yy -= 1;
                }
                --j;
            } else {
                out.push_back({L.index(x, Y, z), value(order, j, dl)});
            }
        }
    }

    // DyfStaggeredX / DybStaggeredX (:852-1011): the y-derivatives of the
    // elastic step at x-staggered points. Near an interface the staggered
    // point of the coarse layer sits at another x, so single taps shift by
    // dhFactor/3; taps outside the grid are dropped (no edge rule).
    // zAxis: DyfStaggeredZ / DybStaggeredZ (:1012-1168), the same rule with
    // the taps shifting along z. fsImage (backward only): the free-surface
    // variants DybStaggeredX / ZFreeSurface (:533-704), the image coefficient
    // c[order - 1 - 2y/f - j] subtracted where it exists.
    void stag_row(int x, int y, int z, bool forward, std::vector<Tap>& out, bool zAxis = false, bool fsImage = false) const
    {
        const int layer = L.layerY[y];
        int order = order_of(layer);
        const int dist = L.distY[y] / L.dhf[layer];
        if (dist == 0) order = 2;
        else if (order > 2 * dist) order = 2 * dist;
        const bool on = L.onIfaceY[y] != 0;
        const int tr = L.transY[y];
        const int n = zAxis ? L.NZ : L.NX;
        auto iface = [&](long long yy) { return yy >= 0 && yy < L.NY && L.onIfaceY[yy]; };
        auto at = [&](int c, int Y) { return zAxis ? L.index(x, Y, c) : L.index(c, Y, z); };
        std::vector<int> C(order, zAxis ? z : x);
        if (forward) {
            const bool c2f = on && tr == -1;
            const int f = c2f ? L.dhf[layer + 1] : L.dhf[layer];
            const int dl = c2f ? layer + 1 : layer;
            if (on && tr == 1 && C[0] >= f / 3) C[1] -= f / 3;
            const long long yq = y + static_cast<long long>(order / 2) * f;
            if (iface(yq) && L.transY[yq] == -1 && C[0] < n - f / 3) C[order - 1] += f / 3;
            for (int j = 0; j < order; ++j) {
                const int Y = y + f * (j - order / 2 + 1);
                if (Y >= 0 && Y < L.NY) out.push_back({at(C[j], Y), value(order, j, dl)});
            }
            return;
        }
        const int f = L.dhf[layer];
        const long long yq = y - static_cast<long long>(order / 2) * f;
        if (iface(yq) && L.transY[yq] == 1 && C[1] < n - f / 3) C[0] += f / 3;
        if (on && tr == -1 && C[1] >= f / 3) C[0] -= f / 3;
        for (int j = 0; j < order; ++j) {
            int Y = y + f * (j - order / 2);
            if (on) {
                if (j == 0 && tr == 1) Y += L.dhf[layer - 1];
                if (j == 1 && tr == -1) Y += L.dhf[layer + 1];
            }
            const int img = fsImage && order >= 1 + 2 * y / f + j ? order - 1 - 2 * y / f - j : -1;
            if (Y >= 0 && Y < L.NY) out.push_back({at(C[j], Y), value(order, j, layer, img)});
        }
    }

    // Dyb (:790-840)
    void dyb_row(int x, int y, int z, std::vector<Tap>& out) const
    {
        const int layer = L.layerY[y];
        const int f = L.dhf[layer];
        int order = reduce_at_interface(order_of(layer), y, layer);
        int yy = y;
        for (int j = 0; j < order; ++j) {
            int Y = yy + f * (j - order / 2);
            const int Ymin = yy + f * (-order / 2);
            const int Ymax = yy + f * (order / 2 - 1);
            // staggered-grid correction on the interface rows (the current row)
            if (yy >= 0 && yy < L.NY && L.onIfaceY[yy]) {
                if (j == 0 && L.transY[yy] == 1) Y += L.dhf[layer - 1];
                if (j == 1 && L.transY[yy] == -1) Y += L.dhf[layer + 1];
            }
            const int dl = (yy >= 0 && yy < L.NY) ? L.layerY[yy] : layer;
            if (!edge) {
                if (Y >= 0 && Y < L.NY) out.push_back({L.index(x, Y, z), value(order, j, dl)});
                continue;
            }
            if (Ymin < 0) {
                order += 2 * Ymin;
                if (order == 0) {
                    order = 2;
                    yy += 1;
                }
                --j;
            } else if (Ymax >= L.NY) {
                order -= 2 * (Ymax - L.NY + 1);
                --j;
            } else {
                out.push_back({L.index(x, Y, z), value(order, j, dl)});
            }
        }
    }
};

// Rows are independent: contiguous row ranges are assembled on host threads
// (up to 16), each into its own tap lists, then packed into the ELL block.
template <class RowFn>
int build_ell(long long N, RowFn fn, EllHost& E, std::string& err, const char* name)
{
    unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (N < (1LL << 16)) nt = 1;
    struct Part {
        std::vector<int> cnt;
        std::vector<long long> cols;
        std::vector<float> vals;
        bool bad = false;
    };
    std::vector<Part> parts(nt);
    auto range = [&](unsigned t, long long& lo, long long& hi) {
        lo = N * t / nt;
        hi = N * (t + 1) / nt;
    };
    auto gather = [&](unsigned t) {
        long long lo, hi;
        range(t, lo, hi);
        Part& P = parts[t];
        P.cnt.resize(hi - lo);
        P.cols.reserve((hi - lo) * 6);
        P.vals.reserve((hi - lo) * 6);
        std::vector<Tap> taps;
        for (long long i = lo; i < hi; ++i) {
            taps.clear();
            fn(i, taps);
            P.cnt[i - lo] = static_cast<int>(taps.size());
            for (const Tap& tp : taps) {
                if (tp.col < 0) P.bad = true;
                P.cols.push_back(tp.col);
                P.vals.push_back(tp.val);
            }
        }
    };
    auto run = [&](auto&& f) {
        std::vector<std::thread> th;
        for (unsigned t = 1; t < nt; ++t) th.emplace_back(f, t);
        f(0u);
        for (auto& x : th) x.join();
    };
    run(gather);
    int W = 0;
    for (const Part& P : parts) {
        if (P.bad) {
            err = std::string(name) + ": a stencil tap falls between the stored rows of the variable grid";
            return WAVE_ERR_ARG;
        }
        for (int c : P.cnt) W = std::max(W, c);
    }
    E.W = W;
    E.col.assign(static_cast<size_t>(W) * N, 0);
    E.val.assign(static_cast<size_t>(W) * N, 0.0f);
    auto pack = [&](unsigned t) {
        long long lo, hi;
        range(t, lo, hi);
        const Part& P = parts[t];
        size_t at = 0;
        for (long long i = lo; i < hi; ++i) {
            const int n = P.cnt[i - lo];
            for (int k = 0; k < W; ++k) {
                const size_t o = static_cast<size_t>(k) * N + i;
                if (k < n) {
                    E.col[o] = static_cast<int>(P.cols[at + k]);
                    E.val[o] = P.vals[at + k];
                } else {
                    E.col[o] = static_cast<int>(i);   // padding: weight 0 on the row itself
                }
            }
            at += n;
        }
    };
    run(pack);
    return WAVE_OK;
}

// InterpolationFull / StaggeredX / StaggeredZ rows on the interfaces
// (Derivatives.cpp:1252-1335, 1356-1440, 1462-1546). kind 0 full, 1 x, 2 z.
int build_interp(const VarGridLayout& L, const std::vector<long long>& rows, int kind, InterpHost& I, std::string& err)
{
    for (long long i : rows) {
        int x, y, z;
        L.coord(i, x, y, z);
        const int layer = L.layerY[y];
        const int f = L.dhf[layer];
        int ff = f;
        if (L.transY[y] == 1) ff = L.dhf[layer - 1];
        else if (L.transY[y] == -1) ff = L.dhf[layer + 1];
        const float den = 1.0f / static_cast<float>(f * f);
        int mx, mz;   // C remainders (sign of the dividend)
        bool ok[4];
        if (kind == 0) {
            mx = x % f; mz = z % f;
            ok[0] = true;
            ok[1] = x + 2 * ff < L.NX;
            ok[2] = z + 2 * ff < L.NZ;
            ok[3] = ok[1] && ok[2];
        } else if (kind == 1) {
            mx = (x - f / 2) % f; mz = z % f;
            ok[0] = x >= mx;
            ok[1] = x + ff < L.NX;
            ok[2] = x >= mx && z + 2 * ff < L.NZ;
            ok[3] = x + ff < L.NX && z + 2 * ff < L.NZ;
        } else if (kind == 2) {
            mx = x % f; mz = (z - f / 2) % f;
            ok[0] = z >= mz;
            ok[1] = x + 2 * ff < L.NX;
            ok[2] = x >= mx && z + ff < L.NZ;
            ok[3] = x + 2 * ff < L.NX && z + ff < L.NZ;
        } else {   // staggered xz (:1568-1661)
            mx = (x - f / 2) % f; mz = (z - f / 2) % f;
            ok[0] = x >= mx && z >= mz;
            ok[1] = x + ff < L.NX;
            ok[2] = x >= mx && z + ff < L.NZ;
            ok[3] = x + ff < L.NX && z + ff < L.NZ;
        }
        const int X[4] = {x - mx, x + f - mx, x - mx, x + f - mx};
        const int Z[4] = {z - mz, z - mz, z + f - mz, z + f - mz};
        const int Wt[4] = {(f - mx) * (f - mz), mx * (f - mz), (f - mx) * mz, mx * mz};
        int cols[4];
        float w[4];
        int n = 0;
        bool identity = true;
        for (int k = 0; k < 4; ++k) {
            if (!ok[k]) continue;
            const long long cidx = L.index(X[k], y, Z[k]);
            if (cidx < 0) {
                err = "interface interpolation reads outside the grid";
                return WAVE_ERR_ARG;
            }
            cols[n] = static_cast<int>(cidx);
            w[n] = static_cast<float>(Wt[k]) * den;
            if (!((cidx == i && w[n] == 1.0f) || w[n] == 0.0f)) identity = false;
            ++n;
        }
        if (identity) continue;   // the coarse-aligned points keep their value
        I.row.push_back(static_cast<int>(i));
        for (int k = 0; k < 4; ++k) {
            I.col.push_back(k < n ? cols[k] : static_cast<int>(i));
            I.w.push_back(k < n ? w[k] : 0.0f);
        }
    }
    // in place only if the rewritten rows read no other rewritten row (true
    // for 1:3 steps; a 3:9 step's staggered rule reads rewritten points)
    std::vector<char> rewritten(L.N, 0);
    for (int r : I.row) rewritten[r] = 1;
    for (size_t k = 0; k < I.col.size(); ++k)
        if (I.w[k] != 0.0f && rewritten[I.col[k]] && I.col[k] != I.row[k / 4]) I.inplace = false;
    (void)err;
    return WAVE_OK;
}

// Groups the rows of one pass by their (offset, weight) entries. Gives up
// (ok = false) when the classes would not be much smaller than the ELL blocks.
void build_classes(long long N, const EllHost* const* ops, int nops, ClassHost& C)
{
    C = ClassHost{};
    int KW = 0;
    for (int q = 0; q < nops; ++q) {
        C.opBase[q] = KW;
        KW += ops[q]->W;
    }
    C.KW = KW;
    if (KW == 0) return;
    const long long cap = std::max<long long>(1024, N / 8);
    std::unordered_map<std::string, unsigned> index;
    index.reserve(4096);
    C.id.resize(N);
    std::string key(static_cast<size_t>(KW) * 8, '\0');
    for (long long i = 0; i < N; ++i) {
        char* k = &key[0];
        for (int q = 0; q < nops; ++q) {
            const EllHost& E = *ops[q];
            for (int e = 0; e < E.W; ++e) {
                const int off = static_cast<int>(E.col[static_cast<size_t>(e) * N + i] - i);
                const float w = E.val[static_cast<size_t>(e) * N + i];
                std::memcpy(k, &off, 4);
                std::memcpy(k + 4, &w, 4);
                k += 8;
            }
        }
        auto it = index.find(key);
        if (it == index.end()) {
            if (static_cast<long long>(index.size()) >= cap) {
                C = ClassHost{};
                return;
            }
            const unsigned cls = static_cast<unsigned>(index.size());
            index.emplace(key, cls);
            for (int e = 0; e < KW; ++e) {
                int off;
                float w;
                std::memcpy(&off, key.data() + 8 * e, 4);
                std::memcpy(&w, key.data() + 8 * e + 4, 4);
                C.off.push_back(off);
                C.w.push_back(w);
            }
            C.id[i] = cls;
        } else {
            C.id[i] = it->second;
        }
    }
    C.nClass = static_cast<int>(index.size());
    C.ok = true;
}

} // namespace

int vargrid_build(const wave_config& c, VarGridHost& G, std::string& err, bool elastic)
{
    int rc = vargrid_layout(c, G.L, err);
    if (rc != WAVE_OK) return rc;
    const VarGridLayout& L = G.L;
    const long long N = L.N;
    if (N >= (1LL << 31)) {
        err = "variable grid larger than 2^31 points";
        return WAVE_ERR_ARG;
    }
    const bool is3d = c.dimension == 3;
    Assembler A(L, static_cast<float>(c.DT), c.edgeOrderReduction != 0);
    std::vector<int> X(N), Y(N), Z(N);
    for (long long i = 0; i < N; ++i) L.coord(i, X[i], Y[i], Z[i]);
    auto axis = [&](int ax, bool bw) {
        return [&, ax, bw](long long i, std::vector<Tap>& t) { A.axis_row(X[i], Y[i], Z[i], ax, bw, t); };
    };
    const bool fs = c.FreeSurface == 1;
    if ((rc = build_ell(N, axis(0, false), G.Dxf, err, "Dxf")) != WAVE_OK) return rc;
    if ((rc = build_ell(N, axis(0, true), G.Dxb, err, "Dxb")) != WAVE_OK) return rc;
    if ((rc = build_ell(N, [&](long long i, std::vector<Tap>& t) { A.dyf_row(X[i], Y[i], Z[i], fs, t); }, G.Dyf, err, "Dyf")) != WAVE_OK) return rc;
    if ((rc = build_ell(N, [&](long long i, std::vector<Tap>& t) { A.dyb_row(X[i], Y[i], Z[i], t); }, G.Dyb, err, "Dyb")) != WAVE_OK) return rc;
    if (is3d) {
        if ((rc = build_ell(N, axis(2, false), G.Dzf, err, "Dzf")) != WAVE_OK) return rc;
        if ((rc = build_ell(N, axis(2, true), G.Dzb, err, "Dzb")) != WAVE_OK) return rc;
    }
    // with the free surface the backward staggered operators are their image
    // variants (the only ones the elastic step then uses)
    if (elastic) {
        if ((rc = build_ell(N, [&](long long i, std::vector<Tap>& t) { A.stag_row(X[i], Y[i], Z[i], true, t); }, G.DyfSX, err,
                            "DyfStaggeredX")) != WAVE_OK)
            return rc;
        if ((rc = build_ell(N, [&](long long i, std::vector<Tap>& t) { A.stag_row(X[i], Y[i], Z[i], false, t, false, fs); },
                            G.DybSX, err, "DybStaggeredX")) != WAVE_OK)
            return rc;
    }
    if (elastic && is3d) {
        if ((rc = build_ell(N, [&](long long i, std::vector<Tap>& t) { A.stag_row(X[i], Y[i], Z[i], true, t, true); }, G.DyfSZ,
                            err, "DyfStaggeredZ")) != WAVE_OK)
            return rc;
        if ((rc = build_ell(N, [&](long long i, std::vector<Tap>& t) { A.stag_row(X[i], Y[i], Z[i], false, t, true, fs); },
                            G.DybSZ, err, "DybStaggeredZ")) != WAVE_OK)
            return rc;
    }
    if (L.varGrid) {
        std::vector<long long> rows;
        for (long long i = 0; i < N; ++i)
            if (L.onIfaceY[Y[i]]) rows.push_back(i);
        if ((rc = build_interp(L, rows, 0, G.full, err)) != WAVE_OK) return rc;
        if ((rc = build_interp(L, rows, 1, G.stagX, err)) != WAVE_OK) return rc;
        if (is3d && (rc = build_interp(L, rows, 2, G.stagZ, err)) != WAVE_OK) return rc;
        if (is3d && elastic && (rc = build_interp(L, rows, 3, G.stagXZ, err)) != WAVE_OK) return rc;
    }
    // CPML coefficients per point (CPML2DAcoustic.cpp:140-205): the layer's
    // profile over ceil(BoundaryWidth / dhFactor) points at its own spacing
    if (c.DampingBoundary == 2) {
        const int naxes = is3d ? 3 : 2;
        const float np = static_cast<float>(c.NPower), fc = static_cast<float>(c.CenterFrequencyCPML);
        const float vm = static_cast<float>(c.VMaxCPML), DT = static_cast<float>(c.DT);
        std::vector<CpmlHost> prof(L.nl);
        std::vector<int> width(L.nl);
        for (int l = 0; l < L.nl; ++l) {
            width[l] = static_cast<int>(std::ceil(static_cast<float>(c.BoundaryWidth) / L.dhf[l]));
            prof[l] = build_cpml(2 * width[l] + 1, width[l], false, np, fc, vm, DT, L.dh(l));
        }
        for (int ax = 0; ax < naxes; ++ax) {
            for (int k = 0; k < 4; ++k) G.cpml[ax][k].assign(N, 0.0f);
            const int n = ax == 0 ? L.NX : ax == 1 ? L.NY : L.NZ;
            for (long long i = 0; i < N; ++i) {
                const int cc = ax == 0 ? X[i] : ax == 1 ? Y[i] : Z[i];
                const int layer = L.layerY[Y[i]];
                const int f = L.dhf[layer];
                const int gd = std::min(cc, n - 1 - cc);
                const int dist = gd / f;
                if (dist >= width[layer]) continue;
                const CpmlHost& P = prof[layer];
                // P.a_full[d] / P.a_half[d] (d < width) are the profile at distance d
                if (cc / f < width[layer]) {
                    if (ax == 1 && c.FreeSurface != 0) continue;
                    G.cpml[ax][0][i] = P.a_full[dist]; G.cpml[ax][1][i] = P.b_full[dist];
                    G.cpml[ax][2][i] = P.a_half[dist]; G.cpml[ax][3][i] = P.b_half[dist];
                } else {
                    G.cpml[ax][0][i] = P.a_half[dist]; G.cpml[ax][1][i] = P.b_half[dist];
                    G.cpml[ax][2][i] = P.a_full[dist]; G.cpml[ax][3][i] = P.b_full[dist];
                }
            }
        }
    }
    // coefficient codes: the distinct quadruples of each axis (a layer's
    // profile on the near and the far side), code 0 for none
    if (c.DampingBoundary == 2) {
        for (int ax = 0; ax < (is3d ? 3 : 2); ++ax) {
            std::unordered_map<std::string, unsigned short> codes;
            G.cpTab[ax].assign(4, 0.0f);
            G.cpCode[ax].assign(N, 0);
            std::string key(16, '\0');
            for (long long i = 0; i < N; ++i) {
                float q[4];
                for (int k = 0; k < 4; ++k) q[k] = G.cpml[ax][k][i];
                if (q[0] == 0.0f && q[1] == 0.0f && q[2] == 0.0f && q[3] == 0.0f) continue;
                std::memcpy(&key[0], q, 16);
                auto it = codes.find(key);
                if (it == codes.end()) {
                    if (codes.size() >= 65535) {
                        err = "too many distinct CPML coefficients";
                        return WAVE_ERR_ARG;
                    }
                    const unsigned short code = static_cast<unsigned short>(codes.size() + 1);
                    it = codes.emplace(key, code).first;
                    G.cpTab[ax].insert(G.cpTab[ax].end(), q, q + 4);
                }
                G.cpCode[ax][i] = it->second;
            }
        }
    }
    // density averaging partners (Modelparameter.cpp:336-446)
    for (int ax = 0; ax < (is3d ? 3 : 2); ++ax) {
        G.avgPartner[ax].assign(N, -1);
        for (long long i = 0; i < N; ++i) {
            const int layer = L.layerY[Y[i]];
            long long j = -1;
            if (ax == 0) {
                const long long Xn = X[i] + L.dhf[layer];
                if (Xn < L.NX) j = L.index(Xn, Y[i], Z[i]);
            } else if (ax == 2) {
                const long long Zn = Z[i] + L.dhf[layer];
                if (Zn < L.NZ) j = L.index(X[i], Y[i], Zn);
            } else {
                const bool t0 = L.onIfaceY[Y[i]] && L.transY[Y[i]] == 0;
                const long long Yn = Y[i] + (t0 ? L.dhf[std::min(layer + 1, L.nl - 1)] : L.dhf[layer]);
                if (Yn < L.NY) j = L.index(X[i], Yn, Z[i]);
            }
            G.avgPartner[ax][i] = static_cast<int>(j);
        }
    }
    if (elastic) {
        // calcAverageMatrixXY / XZ / YZ's 4-point partners (Modelparameter.cpp:
        // 449-624): per pair of axes (a, b) the neighbours f along a, along b
        // and along both, -1 where a coordinate passes the grid
        const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
        for (int q = 0; q < (is3d ? 3 : 1); ++q) {
            for (auto& v : G.shearPartner[q]) v.assign(N, -1);
            for (long long i = 0; i < N; ++i) {
                const int f = L.dhf[L.layerY[Y[i]]];
                const int c[3] = {X[i], Y[i], Z[i]}, n[3] = {L.NX, L.NY, L.NZ};
                const int a = pairs[q][0], b = pairs[q][1];
                const bool oka = c[a] + f < n[a], okb = c[b] + f < n[b];
                auto at = [&](int da, int db) {
                    int p[3] = {c[0], c[1], c[2]};
                    p[a] += da * f;
                    p[b] += db * f;
                    return static_cast<int>(L.index(p[0], p[1], p[2]));
                };
                if (oka) G.shearPartner[q][0][i] = at(1, 0);
                if (okb) G.shearPartner[q][1][i] = at(0, 1);
                if (oka && okb) G.shearPartner[q][2][i] = at(1, 1);
            }
        }
    }
    if (c.DampingBoundary == 1) {
        // ABS2D / ABS3D::init (ABS2D.cpp:110-180, ABS3D.cpp:154-220) at each
        // point's fine-grid coordinates (Coordinates::edgeDistance,
        // Coordinates.cpp:734-760); the top rows of a free surface take the
        // x (and z) distance only
        const int w = c.BoundaryWidth;
        const std::vector<float> coeff = build_abs_coeff(w, static_cast<float>(c.DampingCoeff));
        const bool fsTop = c.FreeSurface != 0;
        auto edge = [](int v, int n) { return !((n - 1 - v) < v) ? v : n - 1 - v; };
        G.absDamp.assign(N, 1.0f);
        for (long long i = 0; i < N; ++i) {
            const int dx = edge(X[i], L.NX), dy = edge(Y[i], L.NY), dz = edge(Z[i], L.NZ);
            int m = dx < dy ? dx : dy;
            if (is3d) m = m < dz ? m : dz;
            float f = 1.0f;
            if (fsTop && Y[i] < w) {
                const int xz = is3d ? (!(dx < dz) ? dz : dx) : dx;
                if (dx < w || (is3d && dz < w)) f = coeff[xz];
            } else if (m < w) {
                f = coeff[m];
            }
            G.absDamp[i] = f;
        }
    }
    G.nSurface = static_cast<long long>(L.vnx[0]) * L.vnz[0];   // layer 0 starts at y = 0
    const EllHost* vel[3] = {&G.Dxf, &G.Dyf, &G.Dzf};
    const EllHost* pres[3] = {&G.Dxb, &G.Dyb, &G.Dzb};
    build_classes(N, vel, is3d ? 3 : 2, G.cls[0]);
    build_classes(N, pres, is3d ? 3 : 2, G.cls[1]);
    return WAVE_OK;
}

} // namespace wave
