// wave_internal.h — data structures shared by the host orchestration
// (solver.cu, tables.cpp) and the sm_103a kernels (kernels_*.cu).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/wave.h"

namespace wave {

constexpr int kMaxHalf = 6;               // spatialFDorder 12 -> half width 6
constexpr int kTabW = 2 * kMaxHalf + 1;   // weights per edge-table row (offsets -H..H)
constexpr int kMaxL = 4;                  // relaxation mechanisms

// One 1-D derivative operator along an axis, already scaled by DT/DH.
// Rows c in [E, n-E) use the interior weights w (offsets -H..H; one end is
// zero); every other row uses tab[slot*(2H+1) + k+H].
struct Op1D {
    int n = 1;          // axis length
    int E = 0;          // edge band width
    int full = 0;       // 1: every row is a table row (slot = c)
    int pad = 0;
    const float* tab = nullptr;   // device pointer
    float w[kTabW] = {};
};

enum OpKind { OP_F = 0, OP_B = 1, OP_FS_F = 2, OP_FS_B = 3 };

// CPML profile along one axis: a/b for backward-type ("full") and
// forward-type ("half") derivatives, zero outside the slabs.
struct Cpml1D {
    int n = 1, w = 0, ns = 0;   // axis length, slab width, compact slab length
    int lo = 0;                 // 1: the near slab (c < w) is part of the compact layout
    int on = 0;
    const float* a_full = nullptr;
    const float* b_full = nullptr;
    const float* a_half = nullptr;
    const float* b_half = nullptr;
};

// Field slots (structure of arrays, one N-vector each).
enum Field {
    F_VX, F_VY, F_VZ, F_P, F_SXX, F_SYY, F_SZZ, F_SXY, F_SXZ, F_SYZ,
    F_HX, F_HY, F_HZ, F_EX, F_EY, F_EZ, F_COUNT
};
// Memory-variable slots (L arrays each).
enum MemVar { R_XX, R_YY, R_ZZ, R_XY, R_XZ, R_YZ, R_EZ, R_EX, R_EY, R_COUNT };
// CPML psi slots: one per (field, derivative direction), named as in the reference.
enum Psi {
    PS_P_X, PS_P_Y, PS_P_Z, PS_VXX, PS_VYY, PS_VZZ,
    PS_SXX_X, PS_SXY_Y, PS_SXZ_Z, PS_SXY_X, PS_SYY_Y, PS_SYZ_Z, PS_SXZ_X, PS_SYZ_Y, PS_SZZ_Z,
    PS_VXY, PS_VYX, PS_VXZ, PS_VZX, PS_VYZ, PS_VZY,
    PS_EZY, PS_EZX, PS_HYX, PS_HXY, PS_EYX, PS_EXY, PS_HZY, PS_HZX,
    PS_EZZ, PS_EXZ, PS_EYZ, PS_HXZ, PS_HYZ, PS_EXX_UNUSED,
    PS_COUNT
};
// Prepared material slots.
enum Mat {
    M_M, M_MU, M_IRX, M_IRY, M_IRZ, M_IR, M_MUXY, M_MUXZ, M_MUYZ,
    M_TAUP, M_TAUS, M_TAUSXY, M_TAUSXZ, M_TAUSYZ, M_OPLTP, M_OPLTS,
    M_CAX, M_CBX, M_CAY, M_CBY, M_CAZ, M_CBZ, M_IMUXY, M_IMUXZ, M_IMUYZ,
    M_CDX0, M_CDY0 = M_CDX0 + kMaxL, M_CDZ0 = M_CDY0 + kMaxL,   // visco-EM C_d per E component and mechanism
    M_RHO = M_CDZ0 + kMaxL,       // density, kept for kernels that average it in-kernel
    M_VP, M_VS,                   // base velocities, kept for the adjoint's chain rule (elastic, visco-elastic; vs for 2-D SH)
    M_EPSR, M_SIG, M_MUR,         // base EM parameters, kept for the adjoint's chain rule (TMz, TEz, 3-D EM)
    M_COUNT
};

// Sources and receivers handled inside the acoustic pressure kernel (small
// grids, pressure sources, no ABS): the thread that updates a marked point
// adds its sources and records its receivers; the velocity kernel advances
// the step counter.
struct SrFuse {
    int on, nt;
    int* tcounter;
    const int* map;        // N entries: -1, or the point's record
    const int* ptSrc;      // per record: first source at the point (-1: none)
    const int* ptRec;      // per record: first receiver at the point
    const int* srcNext;    // next source at the same point, in index order
    const int* recNext;
    const float* signals;  // nsrc x nt
    const int* rtype;
    float* seis;           // nrec x nt
};

// Everything a step kernel needs, passed by value.
struct StepParams {
    int NX, NY, NZ;
    int is3d;
    long long N;
    float* f[F_COUNT];
    float* r[R_COUNT][kMaxL];
    float* psi[PS_COUNT];
    const float* m[M_COUNT];
    // operators: x/y/z forward & backward, free-surface y forward & backward
    Op1D Dxf, Dxb, Dyf, Dyb, Dzf, Dzb, DyfS, DybS;
    Cpml1D cx, cy, cz;
    int useCpml;
    int fs;          // free surface (image method) on
    int abs;         // ABS damping frame on
    int absW;
    const float* absCoeff;  // BoundaryWidth entries
    int L;
    float scale;            // DT/DH: interior FD taps use compile-time coefficients times this
    float DT;
    float DThalf;
    float invRelax[kMaxL], c1[kMaxL], c2[kMaxL], Cc[kMaxL], relaxTime[kMaxL];
    SrFuse sr;
};

struct SrcRecParams {
    int nsrc, nrec, nt, t;
    const long long* sidx;
    const int* stype;
    const float* signals;   // nsrc x nt
    const long long* ridx;
    const int* rtype;
    float* seis;            // nrec x nt
    int eq, is3d;
    float* f[F_COUNT];
};

// one block of a batched launch: shot index and tile origin (x0, row r0 = z + NZ*y);
// a tile is 32 points along x by kTileRows rows, a 32 x 8 block covering it in 4 passes
constexpr int kTileRows = 32;
// BatchTile::flags: the tile lies wholly inside its shot's grid, away from
// the operators' edge bands, the CPML slabs and the ABS frame (set by the
// host for the lossless 2-D TMz batch, whose kernels then skip every
// per-point boundary test on it)
constexpr int kTileInterior = 1;
struct BatchTile {
    int shot, x0, r0, flags;
};
// kTileInterior for the tile [x0, x0+cols) x [r0, r0+rows) of a shot
bool batch_tile_interior(const StepParams& P, int x0, int r0, int cols, int rows);
// Schedule of a batched launch: the work list holds `ntiles` tiles of
// `cols` (a multiple of 32) x `rows` (a multiple of 8) points; the launch's
// blocks walk the list with a grid stride (one block per tile when the grid
// equals ntiles, persistent blocks when it is smaller).
// `smem`: dynamic shared memory of the launch, the staging area of an
// interior tile (lossless 2-D TMz passes; 0 otherwise).
struct BatchSched {
    int ntiles, cols, rows, smem;
};

struct PrepParams {
    int NX, NY, NZ;
    long long N;
};

// kernel launchers (kernels.cu). The kernel tables take the equation code,
// with kEm3d added for the 3-D EM solvers (FD3Demem, FD3Dviscoemem).
constexpr int kEm3d = 100;
inline int kernel_eq(int eq, bool is3d) { return (is3d && eq >= WAVE_EQ_TMEM) ? eq + kEm3d : eq; }
using StepKernel = void (*)(StepParams);
StepKernel kernel_for(int eq, int pass, int H);
using BatchKernel = void (*)(const StepParams*, const BatchTile*, BatchSched);
// the EM equations' kernels (kernels_em.cu)
StepKernel em_kernel_for(int eq, int pass, int H);
BatchKernel em_batch_kernel_for(int eq, int pass, int H);
// dep: programmatic dependent launch (the kernel waits for its predecessor in-kernel)
cudaError_t launch_step_kernel(StepKernel k, dim3 grid, dim3 block, const StepParams& P, bool dep, cudaStream_t s);
// sources and receivers of one step; returns the launches made (2 when the
// receivers, more than kSplitReceivers, get a grid of their own)
constexpr int kSplitReceivers = 1024;
int launch_srcrec(const SrcRecParams& Q, int* tcounter, cudaStream_t s, bool dep = false);
void launch_set_counter(int* c, int v, cudaStream_t s);
void launch_set_counters(int* c, int n, int v, cudaStream_t s);
void launch_batch_pass(int eq, int pass, int H, const StepParams* Ps, const BatchTile* tiles, const BatchSched& S, int grid,
                       cudaStream_t s);
void launch_batch_aux(const StepParams* Ps, const BatchTile* tiles, const BatchSched& S, int grid, int f0, int f1, int f2,
                      const SrcRecParams* Qs, int* counters, int nshots, bool abs, cudaStream_t s);
// resident blocks per SM of the batched kernels of an equation (the smaller of the two passes)
int batch_blocks_per_sm(int eq, int H, int smem = 0);
// Staging bytes of an interior tile of the batched passes of `eq` for a
// cols x rows tile (0: no staged path for it), with the passes' dynamic
// shared-memory limit raised to them.
int batch_tile_smem(int eq, int H, int cols, int rows);
void launch_abs_frame(const StepParams& P, dim3 grid, dim3 block, int f0, int f1, int f2, cudaStream_t s, bool dep = false);
void launch_finite(const float* a, long long n, int* flag, cudaStream_t s);
void k_modulus(PrepParams G, const float* rho, const float* v, const float* tau, float sum, int clamp, float* out, cudaStream_t s);
void k_inverse(PrepParams G, const float* a, float* out, cudaStream_t s);
void k_inv_avg2(PrepParams G, const float* a, int axis, float* out, cudaStream_t s);
void k_inv_avg4(PrepParams G, const float* a, int plane, float* out, cudaStream_t s);
void k_avg2(PrepParams G, const float* a, int axis, float* out, cudaStream_t s);
void k_avg4(PrepParams G, const float* a, int plane, float* out, cudaStream_t s);
void k_harmonic(PrepParams G, const float* invmu, int mode, float* out, cudaStream_t s);
void k_inv_clamped(PrepParams G, const float* mu, float* out, cudaStream_t s);
void k_one_plus(PrepParams G, const float* tau, float L, float* out, cudaStream_t s);
void k_scale(PrepParams G, const float* a, float sc, float* out, cudaStream_t s);
struct ViscoEmCoef {
    float DT, eps0, sumInv;   // sumInv = (sum_l 1/tau_l) / L
    int L;
    float cdScale[kMaxL];     // 1/(1 + DT/(2 tau_l)) / (L tau_l^2)
};
void k_visco_em(PrepParams G, const float* eps, const float* sig, const float* te, const float* ts, const ViscoEmCoef& c,
                float* ca, float* cb, float* const* cd, cudaStream_t s);
void k_cacb(PrepParams G, const float* eps, const float* sig, float DT, float* ca, float* cb, cudaStream_t s);

// host-side builders (tables.cpp)
struct OpHost {
    int n = 1, E = 0, full = 0;
    std::vector<float> tab;       // slots x kTabW (offset -kMaxHalf..kMaxHalf)
    float w[kTabW] = {};
};
OpHost build_op(int n, int order, OpKind kind, int stencilMode, int edgeReduce, float DH, float DT);
struct CpmlHost {
    std::vector<float> a_full, b_full, a_half, b_half;
    int ns = 0;
    int lo = 1;
};
CpmlHost build_cpml(int n, int width, bool dropTop, float NPower, float fc, float vmax, float DT, float DH);
std::vector<float> build_abs_coeff(int width, float dampingCoeff);
bool fd_coefficients(int order, std::vector<double>& c);

// error text for calls without a handle (wave_last_error(NULL))
void set_global_error(const std::string& msg);

// config parser (config.cpp)
int parse_config_file(const char* path, wave_config* cfg, std::string& err);

// wavelets (wavelets.cpp)
int make_wavelet(int shape, int nt, double dt, double fc, double amp, double tshift, float* out);

} // namespace wave
