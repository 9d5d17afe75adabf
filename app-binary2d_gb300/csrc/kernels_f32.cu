// kernels_f32.cu — FP32-stencil stage kernels over FP64 state (store 0) or
// compensated FP32 state (store 1).
#include "kernels.inc"

namespace b2d {

cudaError_t launch_stage_f32(int nf, int store, const StageArgs& a, int grid, int tw, size_t smem, cudaStream_t s)
{
    if (nf == 3) {
        if (store == 0) return launch_one<3, float, 0>(a, grid, tw, smem, s);
        return launch_one<3, float, 1>(a, grid, tw, smem, s);
    }
    if (store == 0) return launch_one<4, float, 0>(a, grid, tw, smem, s);
    return launch_one<4, float, 1>(a, grid, tw, smem, s);
}

}  // namespace b2d
