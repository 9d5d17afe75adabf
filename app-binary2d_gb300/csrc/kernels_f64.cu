// kernels_f64.cu — FP64 stage kernels (the parity path).  Built with
// --fmad=false so that every FP64 operation rounds exactly as written.
#include "kernels.inc"

namespace b2d {

cudaError_t launch_stage_f64(int nf, const StageArgs& a, int grid, int tw, size_t smem, cudaStream_t s)
{
    if (nf == 3) return launch_one<3, double, 0>(a, grid, tw, smem, s);
    return launch_one<4, double, 0>(a, grid, tw, smem, s);
}

}  // namespace b2d
