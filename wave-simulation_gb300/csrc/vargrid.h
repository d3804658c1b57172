// vargrid.h — the variable (discontinuous) grid: layered index space, its
// sparse operators in ELL form, and the device-side state of a handle that
// runs on it (vargrid_host.cpp builds, vargrid.cu launches).
//
// The grid is the reference's Coordinates with dhFactor layers
// (Acquisition/Coordinates.cpp:119-245): depth is cut into layers at the
// interfaces of gridConfigurationFilename, layer l has spacing DH*dhFactor[l]
// (dhFactor a power of 3) and its own box of varNX x varNY x varNZ points,
// stored layer after layer in the reference index order. The rows on an
// interface are stored at the fine spacing and filled from the coarse-aligned
// points by bilinear interpolation after each update.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/wave.h"

namespace wave {

struct VarGridLayout {
    int NX = 1, NY = 1, NZ = 1;        // fine-grid extents (NX, NZ, NY reduced to fit the coarse layers)
    float DH = 0.0f;
    int nl = 1;
    bool varGrid = false;              // layers of different spacing (interface order reduction + interpolation)
    bool varOrder = false;             // FD order per layer
    std::vector<int> dhf, order;       // per layer
    std::vector<int> iface;            // nl + 1 entries: -1, the interfaces, NY - 1
    std::vector<int> start, end, trans, vnx, vny, vnz;
    std::vector<long long> offset;     // nl + 1 entries: first index of each layer, N
    long long N = 0;
    // functions of the depth row y only
    std::vector<int> layerY, transY, distY;
    std::vector<char> onIfaceY;

    float dh(int layer) const { return DH * static_cast<float>(dhf[layer]); }
    // Coordinates::mapIndex2coordinate (Coordinates.cpp:603-634)
    void coord(long long idx, int& x, int& y, int& z) const;
    // Coordinates::map3Dcoordinate2index (Coordinates.cpp:668-698); -1 outside the grid
    long long index(long long X, long long Y, long long Z) const;
};

// ELL operator: W entries per row, stored entry-major (col[k*N + row]) so a
// warp reads consecutive rows; unused entries have col = row, val = 0.
struct EllHost {
    int W = 0;
    std::vector<int> col;
    std::vector<float> val;
};

// Interface rows that the interpolation rewrites: 4 (col, weight) pairs per row.
struct InterpHost {
    std::vector<int> row;
    std::vector<int> col;      // 4 per row
    std::vector<float> w;      // 4 per row
    bool inplace = true;       // no rewritten row reads another rewritten row
};

// Stencil classes of one pass (its three operators): rows whose entries have
// the same column offsets (col - row) and weights share a class. Per row a
// 32-bit class id; per class KW = sum of the operators' ELL widths (offset,
// weight) pairs, operator after operator, in ELL entry order.
struct ClassHost {
    bool ok = false;                   // false: too many classes, use the ELL blocks
    int KW = 0;
    int nClass = 0;
    int opBase[3] = {};                // first entry of each operator in a class row
    std::vector<unsigned> id;          // N
    std::vector<int> off;              // nClass x KW
    std::vector<float> w;              // nClass x KW
};

struct VarGridHost {
    VarGridLayout L;
    EllHost Dxf, Dxb, Dyf, Dyb, Dzf, Dzb;
    EllHost DyfSX, DybSX;              // staggered-x y-derivatives (elastic only)
    EllHost DyfSZ, DybSZ;              // staggered-z y-derivatives (3-D elastic only)
    ClassHost cls[2];                  // velocity pass (Dxf, Dyf, Dzf), pressure pass (Dxb, Dyb, Dzb)
    InterpHost full, stagX, stagZ, stagXZ;   // stagXZ: 3-D elastic only
    std::vector<float> cpml[3][4];     // per axis: a_full, b_full, a_half, b_half (N each; CPML only)
    // the same as a per-point code per axis into a table of (a_full, b_full,
    // a_half, b_half) quadruples; code 0 = no coefficients
    std::vector<unsigned short> cpCode[3];
    std::vector<float> cpTab[3];
    std::vector<int> avgPartner[3];    // averaging partner per axis (-1: the point alone)
    // elastic: the 4-point shear-modulus averages' partners per axis pair
    // (xy; 3-D also xz, yz): the neighbours f along the pair's first axis,
    // its second axis and both, f the layer's dhFactor (-1: outside the grid)
    std::vector<int> shearPartner[3][3];
    long long nSurface = 0;            // rows with y == 0 (the first rows of layer 0)
    std::vector<float> absDamp;        // ABS (DampingBoundary=1): the taper factor per point, else empty
};

// Coordinates set-up from the configuration (Coordinates.cpp:35-95, 119-245).
int vargrid_layout(const wave_config& c, VarGridLayout& L, std::string& err);
// Every operator, interpolation, CPML coefficient and averaging partner of
// the acoustic equations on the grid.
// elastic: also the staggered-x y-derivatives and the shear-average
// partners of the 2-D elastic step
int vargrid_build(const wave_config& c, VarGridHost& G, std::string& err, bool elastic = false);

// device side of a variable-grid handle (vargrid.cu)
struct VarGridDev {
    VarGridLayout L;                        // host copy of the index space
    long long N = 0;
    int is3d = 0;
    int elastic = 0;                        // 2-D elastic step (else acoustic)
    int nOps = 0;
    // Dxf, Dyf, Dzf, Dxb, Dyb, Dzb, DyfStaggeredX, DybStaggeredX, DyfStaggeredZ, DybStaggeredZ
    int W[10] = {};
    const int* col[10] = {};
    const float* val[10] = {};
    int nInterp[4] = {};                    // full, staggered x, staggered z, staggered xz
    const int* irow[4] = {};
    const int* icol[4] = {};
    const float* iw[4] = {};
    int inplace[4] = {1, 1, 1, 1};
    float* itmp = nullptr;                  // scratch of the two-phase interpolation (sum of the row counts)
    const unsigned short* cpCode[3] = {};   // CPML coefficient code per axis and point (null: no CPML)
    const float* cpTab[3] = {};             // 4 floats per code
    const int* partner[3] = {};
    const int* shear[3][3] = {};            // elastic: shear-average partners per axis pair
    long long nSurface = 0;
    int fs = 0;
    const float* absDamp = nullptr;         // ABS taper per point (null: no ABS)
    // transposes of the operators above as ELL blocks (the adjoint; built at
    // its first call)
    bool transposed = false;
    int WT[10] = {};
    const int* colT[10] = {};
    const float* valT[10] = {};
    // stencil classes per pass (null: not available)
    const unsigned* clsId[2] = {};
    const int* clsOff[2] = {};
    const float* clsW[2] = {};
    int clsKW[2] = {};
    int clsBase[2][3] = {};
};

} // namespace wave
