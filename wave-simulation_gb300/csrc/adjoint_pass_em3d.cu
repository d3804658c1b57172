// adjoint_pass_em3d.cu — the per-pass adjoint kernels of the lossless 3-D
// EM equations, instantiated for every FD half-order (a
// translation unit of its own so that the build compiles the adjoint's
// kernels in parallel).
#include "adjoint.cuh"

namespace wave {
namespace {

template <int H>
void launch_h(int pass, const StepParams* Ps, const AdjShot* As, const BatchTile* W, const BatchSched& S, int grid, int vn,
              int pending, cudaStream_t s)
{
    const dim3 block(32, 8, 1);
    switch (pass) {
    case 13: adj::adj_pass<H, 13><<<grid, block, 0, s>>>(Ps, As, W, S, vn, pending); break;
    default: adj::adj_pass<H, 14><<<grid, block, 0, s>>>(Ps, As, W, S, vn, pending); break;
    }
}

} // namespace

void launch_adj_pass_em3d(int H, int pass, const StepParams* Ps, const AdjShot* As, const BatchTile* W, const BatchSched& S, int grid,
                          int vn, int pending, cudaStream_t s)
{
    switch (H) {
    case 1: launch_h<1>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    case 2: launch_h<2>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    case 3: launch_h<3>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    case 4: launch_h<4>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    case 5: launch_h<5>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    default: launch_h<6>(pass, Ps, As, W, S, grid, vn, pending, s); break;
    }
}

} // namespace wave
