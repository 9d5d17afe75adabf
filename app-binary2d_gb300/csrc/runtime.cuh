// runtime.cuh — device-side descriptors shared by the kernels and the C ABI.
#pragma once

#include "../../include/b2d.h"
#include "physics.cuh"

namespace b2d {

constexpr int NSLOTS = 4;  // state slots: the advance input is kept intact until success

struct df32w { float hi, lo; };

// One run of a batch as the kernels see it.
struct RunDev {
    int N, bs, nb, nblocks;
    int tiles_i, tiles_j, ntiles, tile_base;
    int tiles_per_block, chunk0; // partial slots per block: the most ledger pieces a block receives;
                                 // the first row chunk the launch covers (a slab's; 0 for the whole run)
    int slab_lo, slab_hi;        // row slab: block rows [slab_lo, slab_hi) of the run are this context's
                                 // (slab_hi = 0: the whole run); the stage kernel's tiles, the max
                                 // speed and the orbital-element ledger cover only the slab
    int chunks, pad_;            // row chunks per column strip of the whole run (C of chunk_start);
                                 // tiles_i of them, from chunk0, are launched
    const double* xc;        // [N] cell centres by global index (block formula, mesh.rs:49-54)
    const double* xv;        // [nb][bs+1] block vertices (mesh.rs:42-47)
    const float* xcf;
    const float* xvf;
    const float* xvgf;       // [N+1] row faces by global index, FP32 (a block's first vertex at its lower boundary)
    void* slot[NSLOTS];      // conserved state per slot (STORE layout)
    const void* bg;          // BlockData::initial_conserved (STORE layout)
    double* ledger[NSLOTS];  // [nblocks][7][nf] per slot
    double* time;            // [NSLOTS]
    long long* iter;         // [NSLOTS]
    double* partial;         // [nblocks][tiles_per_block][7 nf] ledger pieces of the tiles over each block
    unsigned* counter;       // [nblocks]
    double* dt;              // [1]
    double* stage_time;      // [max_stages]
    double* orbit;           // [max_stages][10]: m, x, y, vx, vy of body 1 then body 2
    unsigned long long* amax;
    double binary_q, binary_e;
    double* elements[NSLOTS];    // [nblocks][7][4] orbital-element change per slot (nullptr: not tracked)
    double* stage_ds;            // [max_stages][nblocks][7 nf] block sums ds·dx·dy of each stage (nullptr: none)
    double* stage_de;            // [max_stages][nblocks][4][4] element change of the gas items of each stage
    double el0[4];               // unperturbed elements (a, M, q, e), physics.rs:411-417
    long long ntracers;          // massless tracer particles of this run (0: none)
    double* tracers[NSLOTS];     // [ntracers][2] positions (x, y) per state slot
    DevParams p;     // FP64 kernels
    DevParamsF pf;   // FP32 kernels
};

struct StageArgs {
    const RunDev* runs;
    int nruns;
    int th;
    int in_slot, base_slot, out_slot;
    int stage;
    int amax_flag;
    double bf;               // weight of the RK base state (br of godunov-core)
    b2d::df32w w1f, bff;     // 1 - bf and bf as double-float
    DevParamsF pf1;          // FP32 parameters of a single-run context, read as kernel arguments
    unsigned long long* err_key;  // failure key, ~0 when no zone failed
    unsigned* timeout_flag;       // set when a bounded wait gave up
};

// Row chunks of a column strip.  A run's N rows split into C chunks; chunk c
// covers rows [c N / C, (c + 1) N / C).  With C = N / th the chunks are the
// block-aligned tiles of height th; with C = ceil(N / rows) for rows <= bs a
// chunk crosses at most one block boundary.  C <= N and N^2 <= 2^31 (the
// mesh limit of validate, api.cu) keep c N and (r + 1) C below 2^32, so
// 32-bit unsigned arithmetic is exact (a 64-bit division costs the stage
// kernel about a thousand instructions).
__host__ __device__ inline int chunk_start(int c, int N, int C) { return (int)((unsigned)c * (unsigned)N / (unsigned)C); }
__host__ __device__ inline int chunk_of_row(int r, int N, int C)
{
    return (int)((((unsigned)r + 1u) * (unsigned)C - 1u) / (unsigned)N);
}
// chunks that cover rows of block row b (bs rows from b bs)
__host__ __device__ inline int chunks_in_block_row(int b, int bs, int N, int C)
{
    return chunk_of_row((b + 1) * bs - 1, N, C) - chunk_of_row(b * bs, N, C) + 1;
}

template <class R> __host__ __device__ inline const DevParamsT<R>& params_of(const RunDev& rd);
template <> __host__ __device__ inline const DevParamsT<double>& params_of<double>(const RunDev& rd) { return rd.p; }
template <> __host__ __device__ inline const DevParamsT<float>& params_of<float>(const RunDev& rd) { return rd.pf; }

}  // namespace b2d
