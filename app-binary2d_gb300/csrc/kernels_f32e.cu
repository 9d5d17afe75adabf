// kernels_f32e.cu — the paired-column Euler kernel (stage3e.cuh) over the
// compensated FP32 state, for tiles 64, 128, 256 or 512 columns wide; its own
// translation unit, compiled with kernels_f32.cu's fast-FP32 flags, so that
// the two build in parallel.
#include "kernels.inc"
#include "stage3e.cuh"

namespace b2d {

template <bool SINGLE, int TWMAX>
static cudaError_t launch_euler_impl(const StageArgs& a, int grid, int tw, cudaStream_t s)
{
    auto k = stage3e_kernel<SINGLE, TWMAX>;
    const size_t smem = s3e_smem_bytes(tw);
    cudaError_t e = opt_in_smem((const void*)k, smem);
    if (e != cudaSuccess) return e;
    k<<<grid, tw / 2 + 32, smem, s>>>(a);
    return cudaGetLastError();
}

static void (*euler_kernel(int nruns, int tw))(StageArgs)
{
    if (tw <= 128) return nruns == 1 ? stage3e_kernel<true, 128> : stage3e_kernel<false, 128>;
    if (tw == 256) return nruns == 1 ? stage3e_kernel<true, 256> : stage3e_kernel<false, 256>;
    return nruns == 1 ? stage3e_kernel<true, 512> : stage3e_kernel<false, 512>;
}

bool euler_paired_width(int tw) { return tw == 64 || tw == 128 || tw == 256 || tw == 512; }

int euler_paired_ctas_per_sm(int nruns, int tw)
{
    int n = 0;
    const size_t smem = s3e_smem_bytes(tw);
    void (*k)(StageArgs) = euler_kernel(nruns, tw);
    if (opt_in_smem((const void*)k, smem) != cudaSuccess) return 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, tw / 2 + 32, smem);
    return e == cudaSuccess ? n : 0;
}

cudaError_t launch_euler_paired(const StageArgs& a, int grid, int tw, cudaStream_t s)
{
    if (tw <= 128) return a.nruns == 1 ? launch_euler_impl<true, 128>(a, grid, tw, s)
                                       : launch_euler_impl<false, 128>(a, grid, tw, s);
    if (tw == 256) return a.nruns == 1 ? launch_euler_impl<true, 256>(a, grid, tw, s)
                                       : launch_euler_impl<false, 256>(a, grid, tw, s);
    return a.nruns == 1 ? launch_euler_impl<true, 512>(a, grid, tw, s) : launch_euler_impl<false, 512>(a, grid, tw, s);
}

}  // namespace b2d
