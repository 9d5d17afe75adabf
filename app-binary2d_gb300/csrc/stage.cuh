// stage.cuh — the fused RK-stage kernel.
//
// One launch performs one call of try_advance_rk (src/scheme.rs:88-173) for
// every run of a context: cons→prim (phase A), PLM slopes and HLLE + viscous
// fluxes (phase B), flux divergence + sources + RK average (phase C), the
// per-block source ledger (scheme.rs:288-313) and, on the last stage of an
// advance, the max signal speed used for the next dt (state.rs:121-133).
//
// Work decomposition.  A CTA owns a tile of TH rows (i, x) × TW columns
// (j, y, contiguous in memory) nested inside one mesh block, with one thread
// per column.  It marches down its rows: each iteration loads one new row of
// the stage input (plus the 2-zone guard halo), converts it to primitives,
// computes slopes and cell records two rows behind, face fluxes four rows
// behind and updates the row five rows behind, so every zone's primitive,
// slope and flux is computed once per tile (plus the halo) and only rows in
// flight live in shared memory.  Ring buffers rotate so that one
// __syncthreads per row orders all producer/consumer pairs.
#pragma once

#include "physics.cuh"
#include "runtime.cuh"
#include "tma.cuh"

namespace b2d {

// ----------------------------------------------------------------------------
// Double-float arithmetic for the compensated FP32 state (Knuth TwoSum,
// Dekker Fast2Sum and an FMA-based two-product).
struct df32 { float hi, lo; };

__device__ __forceinline__ df32 fast_two_sum(float a, float b)
{
    float s = a + b;
    float e = b - (s - a);
    return {s, e};
}

__device__ __forceinline__ df32 two_sum(float a, float b)
{
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}

__device__ __forceinline__ df32 df_add_f(df32 a, float b)
{
    df32 s = two_sum(a.hi, b);
    return fast_two_sum(s.hi, s.lo + a.lo);
}

__device__ __forceinline__ df32 df_add(df32 a, df32 b)
{
    df32 s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}

__device__ __forceinline__ df32 df_mul(df32 a, df32 b)
{
    float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    return fast_two_sum(p, e);
}

// ----------------------------------------------------------------------------
// State access.  STORE 0: FP64 planes [nf][N][N].  STORE 1: FP32 hi and lo
// planes [nf][2][N][N] (value = hi + lo).
template <int STORE> struct State;

template <> struct State<0> {
    using Full = double;
    template <class R> __device__ static __forceinline__ R load_r(const void* b, size_t nn, size_t idx, int f)
    {
        return (R)__ldg((const double*)b + f * nn + idx);
    }
    __device__ static __forceinline__ Full load_full(const void* b, size_t nn, size_t idx, int f)
    {
        return __ldg((const double*)b + f * nn + idx);
    }
    __device__ static __forceinline__ void store(void* b, size_t nn, size_t idx, int f, Full v)
    {
        ((double*)b)[f * nn + idx] = v;
    }
    __device__ static __forceinline__ double to_double(Full v) { return v; }
};

template <> struct State<1> {
    using Full = df32;
    template <class R> __device__ static __forceinline__ R load_r(const void* b, size_t nn, size_t idx, int f)
    {
        return (R)__ldg((const float*)b + (2 * f) * nn + idx);
    }
    __device__ static __forceinline__ Full load_full(const void* b, size_t nn, size_t idx, int f)
    {
        const float* p = (const float*)b;
        return {__ldg(p + (2 * f) * nn + idx), __ldg(p + (2 * f + 1) * nn + idx)};
    }
    __device__ static __forceinline__ void store(void* b, size_t nn, size_t idx, int f, Full v)
    {
        float* p = (float*)b;
        p[(2 * f) * nn + idx] = v.hi;
        p[(2 * f + 1) * nn + idx] = v.lo;
    }
    __device__ static __forceinline__ double to_double(Full v) { return (double)v.hi + (double)v.lo; }
};

__device__ __forceinline__ int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }

// Failure key of a zone: the reference surfaces the error of the first
// block, in mesh.block_indexes() order, whose 3x3 neighbour join fails
// (scheme.rs:126, 161-165); within that block the first failing neighbour
// in neighbour order (mesh.rs:101-110), within that neighbour the first
// failing zone in row-major order (scheme.rs:190-197).  The smallest key
// over all failing zones of the earliest failing stage is that error:
//   stage:10 | run:8 | block:16 | neighbour order:4 | zone:24 | code:2
__device__ __forceinline__ unsigned long long error_key(int stage, int run, const RunDev& rd, int gi, int gj, int code)
{
    const int nb = rd.nb, bs = rd.bs;
    const int ni = gi / bs, nj = gj / bs;
    const unsigned long long zone = (unsigned long long)((gi % bs) * bs + (gj % bs));
    unsigned long long best = ~0ull;
    for (int di = -1; di <= 1; ++di)
        for (int dj = -1; dj <= 1; ++dj) {
            int bi = (ni - di + nb) % nb, bj = (nj - dj + nb) % nb;   // n = b + (di, dj)
            unsigned long long k = ((unsigned long long)stage << 54) | ((unsigned long long)run << 46) |
                                   ((unsigned long long)(bi * nb + bj) << 30) |
                                   ((unsigned long long)((di + 1) * 3 + (dj + 1)) << 26) | (zone << 2) |
                                   (unsigned long long)code;
            best = k < best ? k : best;
        }
    return best;
}

// ----------------------------------------------------------------------------
template <int NF, class R, int STORE>
__global__ void __launch_bounds__(256) stage_kernel(StageArgs a)
{
    using L = CellLayout<NF>;
    using S = State<STORE>;
    using Full = typename S::Full;
    constexpr int CW = L::WIDTH;
    constexpr int NL = NITEMS * NF;

    const int TW = blockDim.x;
    const int TH = a.th;
    const int t = threadIdx.x;

    // --- locate run and tile -------------------------------------------------
    int ri = 0;
    const int g = blockIdx.x;
    while (ri + 1 < a.nruns && g >= a.runs[ri + 1].tile_base) ++ri;
    const RunDev& rd = a.runs[ri];
    if (g - rd.tile_base >= rd.ntiles) return;

    __shared__ DevParamsT<R> P;
    __shared__ Binary<R> B;
    __shared__ double orbd[10];
    __shared__ int failed;
    // an earlier stage failed: the advance is abandoned (the caller keeps its state)
    if (t == 0) failed = (*(volatile unsigned long long*)a.err_key != ~0ull);
    __syncthreads();
    if (failed) return;
    if (t == 0) P = params_of<R>(rd);
    if (t < 10) orbd[t] = rd.orbit[a.stage * 10 + t];
    __syncthreads();
    if (t == 0) {
        B.p1 = {(R)orbd[0], (R)orbd[1], (R)orbd[2], (R)orbd[3], (R)orbd[4]};
        B.p2 = {(R)orbd[5], (R)orbd[6], (R)orbd[7], (R)orbd[8], (R)orbd[9]};
    }

    const int N = rd.N, bs = rd.bs;
    const size_t nn = (size_t)N * N;
    const int lt = g - rd.tile_base;
    const int tj = lt % rd.tiles_j;
    const int ti = lt / rd.tiles_j + (rd.slab_hi > 0 ? rd.slab_lo * (bs / TH) : 0);   // tile rows of the slab
    const int i0 = ti * TH, j0 = tj * TW;
    const int bi = i0 / bs, bj = j0 / bs, li0 = i0 % bs, lj0 = j0 % bs;
    const int block = bi * rd.nb + bj;
    const int tib = (li0 / TH) * (bs / TW) + lj0 / TW;

    const void* uin = rd.slot[a.in_slot];
    const void* ubase = a.base_slot >= 0 ? rd.slot[a.base_slot] : nullptr;
    void* uout = rd.slot[a.out_slot];
    const void* ubg = rd.bg;
    const double dtd = *rd.dt;
    const double timed = rd.stage_time[a.stage];
    const R dt = (R)dtd;
    const R time = (R)timed;

    const R* xc = (const R*)(is_f64<R>() ? (const void*)rd.xc : (const void*)rd.xcf);
    const R* xv = (const R*)(is_f64<R>() ? (const void*)rd.xv : (const void*)rd.xvf);

    extern __shared__ __align__(128) unsigned char smem_raw[];   // one declaration for every stage kernel
    R* sP = (R*)smem_raw;                  // [4][TW+4][NF]   primitives
    R* sC = sP + 4 * (TW + 4) * NF;        // [3][TW+2][CW]   cell records
    R* sF = sC + 3 * (TW + 2) * CW;        // [2][TW+1][NF]   y-face fluxes
    poison_dynamic_smem(smem_raw);
    __syncthreads();

    const R theta = R(P.plm), pdt = R(P.pdt);

    R fx_prev[NF], fx_cur[NF];
    R led[NL];
#pragma unroll
    for (int k = 0; k < NL; ++k) led[k] = R(0);
    R amax = R(0);

    for (int k = 0; k < TH + 6; ++k) {
        const int rn = k - 2;

        // Phase 1: row rn of the stage input → primitives (try_block_primitive).
        if (rn <= TH + 1) {
            const int gi = wrap(i0 + rn, N);
            R* row = sP + ((rn + 8) & 3) * (TW + 4) * NF;
            for (int c = t - 2; c < TW + 2; c += TW) {
                const int gj = wrap(j0 + c, N);
                const size_t idx = (size_t)gi * N + gj;
                R u[NF], p[NF];
#pragma unroll
                for (int f = 0; f < NF; ++f) u[f] = S::template load_r<R>(uin, nn, idx, f);
                R bad = R(0);
                (void)bad;
                int e = try_to_primitive<NF, R>(P, u, p, bad);
                if (e && rn >= 0 && rn < TH && c >= 0 && c < TW)
                    atomicMin(a.err_key, error_key(a.stage, ri, rd, gi, gj, e));
#pragma unroll
                for (int f = 0; f < NF; ++f) row[(c + 2) * NF + f] = p[f];
            }
        }

        // Phase 2: slopes and cell records of row rg = rn - 2 (scheme.rs:216-254).
        const int rg = rn - 2;
        if (rg >= -1 && rg <= TH) {
            const R* P0 = sP + ((rg - 1 + 8) & 3) * (TW + 4) * NF;
            const R* P1 = sP + ((rg + 8) & 3) * (TW + 4) * NF;
            const R* P2 = sP + ((rg + 1 + 8) & 3) * (TW + 4) * NF;
            R* rec_row = sC + ((rg + 9) % 3) * (TW + 2) * CW;
            for (int c = t - 1; c < TW + 1; c += TW) {
                const R* a0 = P0 + (c + 2) * NF;
                const R* m = P1 + (c + 2) * NF;
                const R* q0 = P2 + (c + 2) * NF;
                const R* l = P1 + (c + 1) * NF;
                const R* r = P1 + (c + 3) * NF;
                R* rec = rec_row + (c + 1) * CW;
                const R thx = (a0[0] < pdt || m[0] < pdt || q0[0] < pdt) ? R(0) : theta;
                const R thy = (l[0] < pdt || m[0] < pdt || r[0] < pdt) ? R(0) : theta;
                R tmp[CW];
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    tmp[L::PC + f] = m[f];
                    tmp[L::GX + f] = plm_gradient(thx, a0[f], m[f], q0[f]);
                    tmp[L::GY + f] = plm_gradient(thy, l[f], m[f], r[f]);
                }
                cell_shear<NF, R>(P, tmp);
#pragma unroll
                for (int w = 0; w < CW; ++w) rec[w] = tmp[w];
            }
        }

        // Phase 3: x-face flux between rows rq and rq+1 (own column, registers)
        // and the y-face fluxes of row rn - 3 (scheme.rs:257-268).
        const int rq = rn - 4;
        if (rq >= -1 && rq <= TH - 1) {
            const R* l = sC + ((rq + 9) % 3) * (TW + 2) * CW + (t + 1) * CW;
            const R* r = sC + ((rq + 10) % 3) * (TW + 2) * CW + (t + 1) * CW;
            const R x = xv[bi * (bs + 1) + li0 + rq + 1];
            const R y = xc[j0 + t];
            intercell_flux<NF, R>(P, B, l, r, x, y, 0, fx_cur);
        }
        const int ry = rn - 3;
        if (ry >= 0 && ry <= TH - 1) {
            const R* rec_row = sC + ((ry + 9) % 3) * (TW + 2) * CW;
            R* frow = sF + ((ry + 8) & 1) * (TW + 1) * NF;
            const R x = xc[i0 + ry];
            for (int c = t; c < TW + 1; c += TW) {
                const R y = xv[bj * (bs + 1) + lj0 + c];
                R F[NF];
                intercell_flux<NF, R>(P, B, rec_row + c * CW, rec_row + (c + 1) * CW, x, y, 1, F);
#pragma unroll
                for (int f = 0; f < NF; ++f) frow[c * NF + f] = F[f];
            }
        }

        // Phase 4: update row ru = rn - 4 (compute_block_updated_solution,
        // scheme.rs:290-305, then the RK weighted average, state.rs:183-199).
        const int ru = rn - 4;
        if (ru >= 0 && ru <= TH - 1) {
            const R* frow = sF + ((ru + 8) & 1) * (TW + 1) * NF;
            const int gi = i0 + ru, gj = j0 + t;
            const size_t idx = (size_t)gi * N + gj;
            const R x = xc[gi], y = xc[gj];
            R uc[NF], u0[NF], it[NL];
            Full ucf[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                ucf[f] = S::load_full(uin, nn, idx, f);
                uc[f] = S::template load_r<R>(uin, nn, idx, f);
                u0[f] = S::template load_r<R>(ubg, nn, idx, f);
            }
            source_terms<NF, R>(P, B, uc, u0, x, y, time, dt, it);
            Full out[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                R tot = it[SINK1 * NF + f] + it[SINK2 * NF + f] + it[GRAV1 * NF + f] + it[GRAV2 * NF + f] +
                        it[BUFFER * NF + f] + it[COOLING * NF + f] + it[FAKE_MASS * NF + f];
                if constexpr (std::is_same<R, double>::value) {
                    double du = ((fx_cur[f] - fx_prev[f]) / P.dx + (frow[(t + 1) * NF + f] - frow[t * NF + f]) / P.dx) *
                                -dtd;
                    out[f] = ucf[f] + du + tot;
                } else {
                    const float idx_ = (float)P.inv_dx;
                    float du = ((fx_cur[f] - fx_prev[f]) + (frow[(t + 1) * NF + f] - frow[t * NF + f])) * idx_ * -dt;
                    float inc = du + tot;
                    if constexpr (STORE == 0) out[f] = ucf[f] + (double)inc;
                    else out[f] = df_add_f(ucf[f], inc);
                }
            }
            if (ubase) {
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    Full b0 = S::load_full(ubase, nn, idx, f);
                    if constexpr (STORE == 0) {
                        out[f] = out[f] * (-a.bf + 1.0) + b0 * a.bf;
                    } else {
                        if (a.bf == 0.5) {
                            df32 s = df_add(out[f], b0);
                            out[f] = {s.hi * 0.5f, s.lo * 0.5f};
                        } else {
                            out[f] = df_add(df_mul(out[f], df32{a.w1f.hi, a.w1f.lo}), df_mul(b0, df32{a.bff.hi, a.bff.lo}));
                        }
                    }
                }
            }
#pragma unroll
            for (int f = 0; f < NF; ++f) S::store(uout, nn, idx, f, out[f]);
#pragma unroll
            for (int k2 = 0; k2 < NL; ++k2) led[k2] = led[k2] + it[k2];
            if (a.amax_flag) {
                R uo[NF];
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    if constexpr (STORE == 0) uo[f] = (R)out[f];
                    else uo[f] = (R)out[f].hi;
                }
                R s = max_signal_speed<NF, R>(P, uo);
                amax = rmax(s, amax);  // NaN speeds are ignored, as f64::max does
            }
        }
#pragma unroll
        for (int f = 0; f < NF; ++f) fx_prev[f] = fx_cur[f];
        __syncthreads();
    }

    // --- per-tile ledger and max speed -----------------------------------------
    double* red = (double*)smem_raw;  // [TW] scratch, reused after the loop
    const double area = rd.p.dx * rd.p.dx;
    for (int k = 0; k < NL; ++k) {
        red[t] = (double)led[k];
        __syncthreads();
        for (int s = 1; s < TW; s <<= 1) {
            if ((t & (2 * s - 1)) == 0 && t + s < TW) red[t] += red[t + s];
            __syncthreads();
        }
        if (t == 0) rd.partial[((size_t)block * rd.tiles_per_block + tib) * NL + k] = red[0];
        __syncthreads();
    }
    if (a.amax_flag) {
        red[t] = (double)amax;
        __syncthreads();
        for (int s = 1; s < TW; s <<= 1) {
            if ((t & (2 * s - 1)) == 0 && t + s < TW) red[t] = fmax(red[t], red[t + s]);
            __syncthreads();
        }
        if (t == 0 && red[0] > 0.0) atomicMax(rd.amax, (unsigned long long)__double_as_longlong(red[0]));
    }

    // Last tile of a block to finish folds the tile partials into the block's
    // ledger: integrated_source_terms + ds·dx·dy (scheme.rs:307-313), averaged
    // like the conserved state (state.rs:196).
    __shared__ int is_last;
    if (t == 0) {
        __threadfence();
        unsigned prev = atomicAdd(rd.counter + block, 1u);
        is_last = (prev == (unsigned)rd.tiles_per_block - 1);
    }
    __syncthreads();
    if (is_last) {
        __threadfence();
        const double* lin = rd.ledger[a.in_slot] + (size_t)block * NL;
        const double* lbase = a.base_slot >= 0 ? rd.ledger[a.base_slot] + (size_t)block * NL : nullptr;
        double* lout = rd.ledger[a.out_slot] + (size_t)block * NL;
        for (int k = t; k < NL; k += TW) {
            double s = 0.0;
            for (int q = 0; q < rd.tiles_per_block; ++q) s += __ldcg(rd.partial + ((size_t)block * rd.tiles_per_block + q) * NL + k);
            double v = __ldcg(lin + k) + s * area;
            if (lbase) v = v * (-a.bf + 1.0) + __ldcg(lbase + k) * a.bf;
            lout[k] = v;
            // the block's ds·dx·dy of this stage, for the orbital-element ledger
            if (rd.stage_ds) rd.stage_ds[((size_t)a.stage * rd.nblocks + block) * NL + k] = s * area;
        }
        if (t == 0) rd.counter[block] = 0u;
    }
}

}  // namespace b2d
