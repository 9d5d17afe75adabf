// kernels_f32.cu — FP32-stencil stage kernels over FP64 state (store 0) or
// compensated FP32 state (store 1).  Compensated tiles 64, 128, 256 or 512
// columns wide run the paired-column kernels: stage3.cuh (isothermal) and
// stage3e.cuh (Euler, kernels_f32e.cu); other tiles
// whose width is a multiple of 32 (at most 128) run the TMA-staged kernel of
// stage2.cuh; narrower tiles (blocks of fewer than 32 zones) run the generic
// kernel of stage.cuh.  The first two take row chunks across block rows.
#include "kernels.inc"
#include "stage3.cuh"

namespace b2d {

// the paired Euler kernel (kernels_f32e.cu)
bool euler_paired_width(int tw);
int euler_paired_ctas_per_sm(int nruns, int tw);
cudaError_t launch_euler_paired(const StageArgs& a, int grid, int tw, cudaStream_t s);

template <int NF, int STORE, bool SINGLE>
static cudaError_t launch_two_impl(const StageArgs& a, int grid, int tw, cudaStream_t s)
{
    auto k = stage2_kernel<NF, STORE, SINGLE>;
    size_t smem = s2_smem_bytes(NF, STORE, tw);
    // opt in for every size: the kernel's static shared memory counts toward
    // the 48 KB that needs no opt-in
    cudaError_t e = opt_in_smem((const void*)k, smem);
    if (e != cudaSuccess) return e;
    k<<<grid, tw + 32, smem, s>>>(a);
    return cudaGetLastError();
}

template <int NF, int STORE>
static cudaError_t launch_two(const StageArgs& a, int grid, int tw, cudaStream_t s)
{
    if (a.nruns == 1) return launch_two_impl<NF, STORE, true>(a, grid, tw, s);
    return launch_two_impl<NF, STORE, false>(a, grid, tw, s);
}

template <bool SINGLE, int TWMAX>
static cudaError_t launch_three_impl(const StageArgs& a, int grid, int tw, cudaStream_t s)
{
    auto k = stage3_kernel<SINGLE, TWMAX>;
    size_t smem = s3_smem_bytes(tw);
    cudaError_t e = opt_in_smem((const void*)k, smem);
    if (e != cudaSuccess) return e;
    k<<<grid, tw / 2 + 32 * s3_aux_warps(TWMAX), smem, s>>>(a);
    return cudaGetLastError();
}

template <int NF, int STORE>
static int two_ctas_per_sm(int nruns, int tw)
{
    int n = 0;
    const size_t smem = s2_smem_bytes(NF, STORE, tw);
    cudaError_t e = nruns == 1
        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stage2_kernel<NF, STORE, true>, tw + 32, smem)
        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, stage2_kernel<NF, STORE, false>, tw + 32, smem);
    return e == cudaSuccess ? n : 0;
}

// Resident CTAs per SM of the FP32 stage kernel that launch_stage_f32 runs for
// a tile width (the autotuner sizes row chunks to whole waves with it); 0 for
// the generic kernel, which takes no row chunks.
int stage_ctas_per_sm(int nf, int store, int nruns, int tw)
{
    int n = 0;
    if (nf == 4 && store == 1 && euler_paired_width(tw)) return euler_paired_ctas_per_sm(nruns, tw);
    if (nf == 3 && store == 1 && (tw == 64 || tw == 128 || tw == 256 || tw == 512)) {
        const size_t smem = s3_smem_bytes(tw);
        void (*k)(StageArgs);
        if (tw <= 128) k = nruns == 1 ? stage3_kernel<true, 128> : stage3_kernel<false, 128>;
        else if (tw == 256) k = nruns == 1 ? stage3_kernel<true, 256> : stage3_kernel<false, 256>;
        else k = nruns == 1 ? stage3_kernel<true, 512> : stage3_kernel<false, 512>;
        // the opt-in above 48 KB of dynamic shared memory, as at launch
        if (opt_in_smem((const void*)k, smem) != cudaSuccess) return 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, tw / 2 + 32 * s3_aux_warps(tw <= 128 ? 128 : tw), smem);
        return e == cudaSuccess ? n : 0;
    }
    if (tw % 32 == 0 && tw <= 128) {
        if (nf == 3) return store == 0 ? two_ctas_per_sm<3, 0>(nruns, tw) : two_ctas_per_sm<3, 1>(nruns, tw);
        return store == 0 ? two_ctas_per_sm<4, 0>(nruns, tw) : two_ctas_per_sm<4, 1>(nruns, tw);
    }
    return 0;
}

cudaError_t launch_stage_f32(int nf, int store, const StageArgs& a, int grid, int tw, size_t smem, cudaStream_t s)
{
    if (nf == 4 && store == 1 && euler_paired_width(tw)) return launch_euler_paired(a, grid, tw, s);
    if (nf == 3 && store == 1 && (tw == 64 || tw == 128))
        return a.nruns == 1 ? launch_three_impl<true, 128>(a, grid, tw, s)
                            : launch_three_impl<false, 128>(a, grid, tw, s);
    if (nf == 3 && store == 1 && tw == 256)
        return a.nruns == 1 ? launch_three_impl<true, 256>(a, grid, tw, s)
                            : launch_three_impl<false, 256>(a, grid, tw, s);
    if (nf == 3 && store == 1 && tw == 512)
        return a.nruns == 1 ? launch_three_impl<true, 512>(a, grid, tw, s)
                            : launch_three_impl<false, 512>(a, grid, tw, s);
    if (tw % 32 == 0 && tw <= 128) {
        if (nf == 3) return store == 0 ? launch_two<3, 0>(a, grid, tw, s) : launch_two<3, 1>(a, grid, tw, s);
        return store == 0 ? launch_two<4, 0>(a, grid, tw, s) : launch_two<4, 1>(a, grid, tw, s);
    }
    if (nf == 3) {
        if (store == 0) return launch_one<3, float, 0>(a, grid, tw, smem, s);
        return launch_one<3, float, 1>(a, grid, tw, smem, s);
    }
    if (store == 0) return launch_one<4, float, 0>(a, grid, tw, smem, s);
    return launch_one<4, float, 1>(a, grid, tw, smem, s);
}

}  // namespace b2d
