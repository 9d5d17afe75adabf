// stage3.cuh — the isothermal, compensated-FP32 RK-stage kernel with two
// columns per thread and packed FP32x2 arithmetic.
//
// Same stage as stage2.cuh (try_advance_rk, src/scheme.rs:88-173, plus the RK
// average of state.rs:183-199) and the same TMA row staging and row pipeline;
// what changes is the thread mapping:
//
//  * Column pairs.  Interior thread t owns columns 2t and 2t+1 of the tile.
//    Every per-column quantity is a float2 {column 2t, column 2t+1} and the
//    arithmetic runs as Blackwell's packed FADD2 / FMUL2 / FFMA2, so one
//    instruction advances two zones.  The two x-faces below the pair, the two
//    y-faces on the pair's left (2t and 2t+1) and the pair's two updates are
//    each one packed evaluation.  Min/max, compares, selects and the special
//    function unit stay per column.
//  * Per-row costs (loop control, ring-slot and address arithmetic, waits,
//    the barrier, the warp reduction of the source ledger) are shared by two
//    zones.
//  * Exchange.  A pair needs its left neighbour's column for the y-slopes and
//    the face at 2t, and its right neighbour's first y-flux; both go through
//    float4 planes in shared memory as in stage2.
//  * Halo.  An extra warp owns the guard pairs (-2, -1) and (TW, TW+1) on lanes
//    0 and 1 (lane 1 also computes the y-faces at TW and TW+1, of which TW is
//    the tile's right face); the TMA producer is its lane 4 on 64- and
//    128-column tiles and lane 0 of a second extra warp on wider ones.  The halo lanes'
//    outer columns (-2 and TW+1) need stencil points outside the staged halo;
//    they read clamped in-bounds values and their results are never used.
//  * Row chunks.  A tile is a column strip's row chunk (chunk_start,
//    runtime.cuh).  Chunks may cross one block boundary, so that the number of
//    CTAs can be a whole number of waves (a CTA's time is set by its row chain,
//    not by how many CTAs share its SM).  The source ledger of a crossing
//    tile's rows in its first block row is reduced into a second shared bank
//    when the last of them is updated (one warp-uniform branch in the row
//    loop); after the loop warp 0 writes the main piece and the halo warp the
//    first, at once; a block's pieces are folded by its last piece, in piece
//    order.
#pragma once

#include "stage2.cuh"

namespace b2d {

// ---------------------------------------------------------------------------
// Packed FP32x2 arithmetic (sm_100+ FADD2 / FMUL2 / FFMA2, round to nearest).
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b as b * (-1) + a: one rounding, the same value as a subtraction
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

// Knuth TwoSum / Dekker Fast2Sum on pairs (the compensated state update).
struct df2 { float2 hi, lo; };

__device__ __forceinline__ df2 fast_two_sum2(float2 a, float2 b)
{
    const float2 s = add2(a, b);
    return {s, sub2(b, sub2(s, a))};
}

__device__ __forceinline__ df2 two_sum2(float2 a, float2 b)
{
    const float2 s = add2(a, b);
    const float2 bb = sub2(s, a);
    return {s, add2(sub2(a, sub2(s, bb)), sub2(b, bb))};
}

__device__ __forceinline__ df2 df_add_f2(df2 a, float2 b)
{
    const df2 s = two_sum2(a.hi, b);
    return fast_two_sum2(s.hi, add2(s.lo, a.lo));
}

__device__ __forceinline__ df2 df_add2(df2 a, df2 b)
{
    const df2 s = two_sum2(a.hi, b.hi);
    return fast_two_sum2(s.hi, add2(s.lo, add2(a.lo, b.lo)));
}

__device__ __forceinline__ df2 df_mul2(df2 a, df32 b)
{
    const float2 bh = f2(b.hi), bl = f2(b.lo);
    const float2 p = mul2(a.hi, bh);
    float2 e = fma2(a.hi, bh, mul2(p, f2(-1.0f)));
    e = fma2(a.hi, bl, fma2(a.lo, bh, e));
    return fast_two_sum2(p, e);
}

// Generalised minmod of each lane (see plm_gradient, physics.cuh).
__device__ __forceinline__ float2 plm_gradient2(float2 th, float2 a, float2 b, float2 c)
{
    const float2 x = mul2(th, sub2(b, a));
    const float2 y = mul2(f2(0.5f), sub2(c, a));
    const float2 z = mul2(th, sub2(c, b));
    const float2 lo = make_float2(fmaxf(fminf(fminf(x.x, y.x), z.x), 0.0f), fmaxf(fminf(fminf(x.y, y.y), z.y), 0.0f));
    const float2 hi = make_float2(fminf(fmaxf(fmaxf(x.x, y.x), z.x), 0.0f), fminf(fmaxf(fmaxf(x.y, y.y), z.y), 0.0f));
    return add2(lo, hi);
}

// Isothermal face sound speed of two faces (iso_face_cs2, stage2.cuh).
__device__ __forceinline__ float2 iso_face_cs2_2(const DevParamsF& P, const Binary<float>& B, float dx1sq,
                                                 float dx2sq, float2 cy1, float2 cy2)
{
    const float2 t1 = add2(f2(dx1sq), cy1), t2 = add2(f2(dx2sq), cy2);
    const float2 r1 = make_float2(rsqrtf(t1.x), rsqrtf(t1.y)), r2 = make_float2(rsqrtf(t2.x), rsqrtf(t2.y));
    return mul2(fma2(f2(B.p1.m), r1, mul2(f2(B.p2.m), r2)), f2(P.inv_mach2));
}

// Two isothermal faces normal to AXIS (intercell_flux, physics.rs:584-607, with
// hydro-iso2d's HLLE and the factored viscous stress of face_flux in
// stage2.cuh).  pcl/gl/tnl/ttl describe the left cells of the two faces,
// pcr/gr/tnr/ttr the right cells; (fx, fy) are the faces' positions.
template <int AXIS>
__device__ __forceinline__ void face_flux2(const DevParamsF& P, const Binary<float>& B, const float2* pcl,
                                           const float2* gl, float2 tnl, float2 ttl, const float2* pcr,
                                           const float2* gr, float2 tnr, float2 ttr, float2 fx, float2 fy,
                                           float2 cs2, float2* F)
{
    float2 pl[3], pr[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        pl[k] = fma2(gl[k], f2(0.5f), pcl[k]);
        pr[k] = fma2(gr[k], f2(-0.5f), pcr[k]);
    }
    // conserved and physical fluxes of the reconstructed states
    const float2 ul1 = mul2(pl[0], pl[1]), ul2 = mul2(pl[0], pl[2]);
    const float2 ur1 = mul2(pr[0], pr[1]), ur2 = mul2(pr[0], pr[2]);
    const float2 pgl = mul2(pl[0], cs2), pgr = mul2(pr[0], cs2);
    const float2 vl = AXIS == 0 ? pl[1] : pl[2];
    const float2 vr = AXIS == 0 ? pr[1] : pr[2];
    const float2 fl0 = mul2(pl[0], vl), fr0 = mul2(pr[0], vr);
    const float2 fl1 = AXIS == 0 ? fma2(ul1, vl, pgl) : mul2(ul1, vl);
    const float2 fr1 = AXIS == 0 ? fma2(ur1, vr, pgr) : mul2(ur1, vr);
    const float2 fl2 = AXIS == 1 ? fma2(ul2, vl, pgl) : mul2(ul2, vl);
    const float2 fr2 = AXIS == 1 ? fma2(ur2, vr, pgr) : mul2(ur2, vr);
    // outer wave speeds
    const float2 cs = make_float2(sqrtf(cs2.x), sqrtf(cs2.y));
    const float2 alm = sub2(vl, cs), alp = add2(vl, cs), arm = sub2(vr, cs), arp = add2(vr, cs);
    const float2 ap = make_float2(fmaxf(0.0f, fmaxf(alp.x, arp.x)), fmaxf(0.0f, fmaxf(alp.y, arp.y)));
    const float2 am = make_float2(fminf(0.0f, fminf(alm.x, arm.x)), fminf(0.0f, fminf(alm.y, arm.y)));
    const float2 d = sub2(ap, am);
    const float2 inv = make_float2(__fdividef(1.0f, d.x), __fdividef(1.0f, d.y));
    const float2 nam = mul2(am, f2(-1.0f));
    const float2 apam = mul2(ap, am);
    // F = (fl ap - fr am - (ul - ur) ap am) / (ap - am)
    F[0] = mul2(fma2(sub2(pr[0], pl[0]), apam, fma2(fr0, nam, mul2(fl0, ap))), inv);
    F[1] = mul2(fma2(sub2(ur1, ul1), apam, fma2(fr1, nam, mul2(fl1, ap))), inv);
    F[2] = mul2(fma2(sub2(ur2, ul2), apam, fma2(fr2, nam, mul2(fl2, ap))), inv);
    // viscous stress
    float2 k = f2(0.5f);
    if (P.visc != 0)
        k = make_float2(0.5f * alpha_face_factor<3>(P, B, fx.x, fy.x, cs2.x),
                        0.5f * alpha_face_factor<3>(P, B, fx.y, fy.y, cs2.y));
    const float2 tn = mul2(k, add2(tnl, tnr));
    const float2 tt = mul2(k, add2(ttl, ttr));
    F[1] = sub2(F[1], AXIS == 0 ? tn : tt);
    F[2] = sub2(F[2], AXIS == 0 ? tt : tn);
}

// One row of prefetch is enough here: a CTA spends microseconds per row, far
// more than a bulk copy takes (measured: depth 2 is 1 % slower).
constexpr int S3_DEPTH = 1;
constexpr int S3_SLOTS = S3_DEPTH + 4;   // stencil ring: a row is read again 3 rows after it lands
constexpr int S3_USLOTS = S3_DEPTH + 1;  // update ring

__host__ __device__ inline int s3_smem_bytes(int tw)
{
    int slots = S3_SLOTS * s2_slot_bytes(3, 1, tw) + S3_USLOTS * s2_uslot_bytes(3, 1, tw);
    int exch = 16 * (2 * (tw + 4) + 3 * 2 * (tw + 4) + 2 * (tw + 2));
    return slots + exch + 8 * (S3_SLOTS + S3_USLOTS);
}

// Warps beside the interior ones: the halo warp, and for 256- and 512-column
// tiles a warp of its own for the TMA producer (lane 0), so that the bulk-copy
// issue of a row does not add to the halo warp's time on its sub-partition
// (measured on the 2048^2 disk: 0.1320 against 0.1347 ms per stage at
// 512-column tiles).  Launch: TW / 2 + 32 * s3_aux_warps threads.
__host__ __device__ constexpr int s3_aux_warps(int twmax) { return twmax >= 256 ? 2 : 1; }
// The launch bound's thread count: the CTA's threads, except that the
// 512-column CTA (10 warps, 3 on some sub-partition) is declared as 384
// threads, which caps a thread at 168 registers as three warps on one
// sub-partition require.
__host__ __device__ constexpr int s3_launch_bound(int twmax)
{
    return twmax == 512 ? 384 : twmax / 2 + 32 * s3_aux_warps(twmax);
}

// TWMAX: the widest tile of the instantiation.  128: tiles of 64 or 128
// columns, 4 CTAs per SM; 256: 256-column tiles over two 128-column blocks
// (or one 256-column block), 4 interior warps to each halo warp, 2 CTAs per
// SM; 512: 512-column tiles over up to four blocks, 8 interior warps to each
// halo warp, 1 CTA per SM.
template <bool SINGLE, int TWMAX>
__global__ void __launch_bounds__(s3_launch_bound(TWMAX), TWMAX == 128 ? 4 : (TWMAX == 256 ? 2 : 1)) stage3_kernel(StageArgs a)
{
    constexpr int NF = 3;
    constexpr int H = 4;                     // staged halo columns per side: 16 bytes of FP32
    constexpr int NL = NITEMS * NF;

    const int TP = blockDim.x - 32 * s3_aux_warps(TWMAX);   // interior threads (column pairs)
    const int TW = 2 * TP;
    const int t = threadIdx.x;
    const int SW = TW + 2 * H;

    int ri = 0;
    const int g = blockIdx.x;
    while (ri + 1 < a.nruns && g >= a.runs[ri + 1].tile_base) ++ri;
    const RunDev& rd = a.runs[ri];
    if (g - rd.tile_base >= rd.ntiles) return;

    __shared__ DevParamsF Psh;
    const DevParamsF& P = params_for<SINGLE>(a, Psh);
    __shared__ Binary<float> B;
    __shared__ double orbd[10];
    __shared__ int failed, timeout;
    if (t == 0) {
        failed = (*(volatile unsigned long long*)a.err_key != ~0ull);
        timeout = 0;
    }
    __syncthreads();
    if (failed) return;
    if (!SINGLE && t == 0) Psh = rd.pf;
    if (t < 10) orbd[t] = rd.orbit[a.stage * 10 + t];
    __syncthreads();
    if (t == 0) {
        B.p1 = {(float)orbd[0], (float)orbd[1], (float)orbd[2], (float)orbd[3], (float)orbd[4]};
        B.p2 = {(float)orbd[5], (float)orbd[6], (float)orbd[7], (float)orbd[8], (float)orbd[9]};
    }

    const int N = rd.N, bs = rd.bs;
    const size_t nn = (size_t)N * N;
    const int lt = g - rd.tile_base;
    const int tj = lt % rd.tiles_j, ti = rd.chunk0 + lt / rd.tiles_j;
    // rows [i0, i0 + TH) of the column strip from j0: row chunk ti of C.  A chunk
    // of at most bs rows lies in one block row, or in two from its row rb; the
    // ledger piece of the last block row is the tile's main piece
    const int C = rd.chunks;
    const int i0 = chunk_start(ti, N, C), TH = chunk_start(ti + 1, N, C) - i0, j0 = tj * TW;
    const int bj = j0 / bs, lj0 = j0 % bs;
    const int rb = min(bs - i0 % bs, TH);
    const int bl = (i0 + TH - 1) / bs;
    const int block = bl * rd.nb + bj;
    const int tib = (ti - chunk_of_row(bl * bs, N, C)) * max(bs / TW, 1) + lj0 / TW;
    const bool has_base = a.base_slot >= 0;

    const float* uin = (const float*)rd.slot[a.in_slot];
    const float* ubase = has_base ? (const float*)rd.slot[a.base_slot] : nullptr;
    float* uout = (float*)rd.slot[a.out_slot];
    const float* ubg = (const float*)rd.bg;
    const float dt = (float)*rd.dt;
    const float time = (float)rd.stage_time[a.stage];
    const float* xc = rd.xcf;

    // ---- shared memory carve-up ------------------------------------------------
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int SLOT = s2_slot_bytes(NF, 1, TW);
    const int USLOT = s2_uslot_bytes(NF, 1, TW);
    unsigned char* slots = smem_raw;                          // stencil ring
    unsigned char* uslots = slots + S3_SLOTS * SLOT;          // update ring
    // float4 planes of two rows each.  Row slot c + 2 holds column c (face c for
    // sF), the even slots in the first half of the row and the odd ones in the
    // second: a pair's two records sit in the two halves, so a warp's accesses
    // are 16 bytes apart (no bank conflicts; adjacent float4s would be 2-way).
    float4* sP = (float4*)(uslots + S3_USLOTS * USLOT);       // [2][TW+4] primitives
    // cell records, column c at c+2: R0 = pc, gy0 | R1 = gy1, gy2, tyy, txy | R2 = gx, txx
    float4* sR0 = sP + 2 * (TW + 4);                          // [2][TW+4]
    float4* sR1 = sR0 + 2 * (TW + 4);
    float4* sR2 = sR1 + 2 * (TW + 4);
    float4* sF = sR2 + 2 * (TW + 4);                          // [2][TW+2] y-face fluxes
    uint64_t* bars = (uint64_t*)(sF + 2 * (TW + 2));          // [S3_SLOTS] stencil ring
    uint64_t* ubars = bars + S3_SLOTS;                        // [S3_USLOTS] update ring

    // ---- roles -----------------------------------------------------------------
    const bool interior = t < TP;
    const int hl = t - TP;                                    // lane in the halo warp (32: the producer warp)
    const bool active = interior || (hl >= 0 && hl < 2);
    const int c0 = interior ? 2 * t : (hl == 0 ? -2 : TW);   // first column of this thread's pair
    const bool producer = s3_aux_warps(TWMAX) == 2 ? hl == 32 : hl == 4;
    const int p = c0 >> 1;                                   // the pair's slot in a half row (-1 for the -2 pair)
    const int HR = TW / 2 + 2, HF = TW / 2 + 1;              // odd halves of the record and flux rows

    auto plane = [&](const float* base, int f, int part) -> const float* { return base + (size_t)(2 * f + part) * nn; };
    auto copy_row = [&](unsigned char* dst, const float* row, int w_halo, uint64_t* bar) {
        if (w_halo == 0) {
            bulk_load(dst, row + j0, TW * sizeof(float), bar);
        } else if (j0 >= H && j0 + TW + H <= N) {
            bulk_load(dst, row + j0 - H, SW * sizeof(float), bar);
        } else {
            bulk_load(dst, row + (j0 - H + N) % N, H * sizeof(float), bar);
            bulk_load(dst + H * sizeof(float), row + j0, TW * sizeof(float), bar);
            bulk_load(dst + (H + TW) * sizeof(float), row + (j0 + TW) % N, H * sizeof(float), bar);
        }
    };
    auto issue = [&](int r) {
        const int rr = r + 2;
        unsigned char* sb = slots + (rr % S3_SLOTS) * SLOT;
        uint64_t* bar = bars + rr % S3_SLOTS;
        const int gi = wrap(i0 + r, N);
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, NF * SW * sizeof(float));
        const size_t roff = (size_t)gi * N;
        for (int f = 0; f < NF; ++f) copy_row(sb + f * SW * sizeof(float), plane(uin, f, 0) + roff, 1, bar);
    };
    auto issue_update = [&](int r) {
        unsigned char* q = uslots + (r % S3_USLOTS) * USLOT;
        uint64_t* bar = ubars + r % S3_USLOTS;
        const size_t roff = (size_t)(i0 + r) * N;
        const uint32_t bytes = (2 + (has_base ? 2 : 0)) * NF * TW * sizeof(float);
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, bytes);
        for (int f = 0; f < NF; ++f, q += TW * sizeof(float)) copy_row(q, plane(uin, f, 1) + roff, 0, bar);
        for (int f = 0; f < NF; ++f, q += TW * sizeof(float)) copy_row(q, plane(ubg, f, 0) + roff, 0, bar);
        if (has_base) {
            for (int f = 0; f < NF; ++f, q += TW * sizeof(float)) copy_row(q, plane(ubase, f, 0) + roff, 0, bar);
            for (int f = 0; f < NF; ++f, q += TW * sizeof(float)) copy_row(q, plane(ubase, f, 1) + roff, 0, bar);
        }
    };

    poison_dynamic_smem(smem_raw);
    if (producer) {
        for (int s = 0; s < S3_SLOTS + S3_USLOTS; ++s) mbar_init(bars + s, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (producer)
        for (int r = -2; r < -2 + S3_DEPTH; ++r) issue(r);

    const float theta = P.plm, pdt = P.pdt, inv_dx = P.inv_dx;
    const bool half_avg = a.bf == 0.5;
    const df32 w1{a.w1f.hi, a.w1f.lo}, wb{a.bff.hi, a.bff.lo};
    const bool want_amax = a.amax_flag != 0;
    // positions: zone centres (y) of the pair, y of the pair's left faces
    const float2 yc2 = interior ? make_float2(xc[j0 + c0], xc[j0 + c0 + 1]) : f2(0.0f);
    const float2 yv2 = (interior || hl == 1) ? make_float2(rd.xvgf[j0 + c0], rd.xvgf[j0 + min(c0 + 1, TW)]) : f2(0.0f);
    const float* xv_row = rd.xvgf + i0;
    const float* xc_row = xc + i0;
    // dy^2 + s^2 of a pair of y positions to each body (recomputed where used:
    // registers are the scarcer resource here)
    auto col_part = [&](float2 y, float by) {
        const float2 d = sub2(y, f2(by));
        return fma2(d, d, f2(P.soft2));
    };

    float2 Pm1[NF], P0[NF];           // primitives of rows rg-1, rg (own pair)
    float2 fxA[NF], fxB[NF];          // x fluxes at faces ru-1/2, ru+1/2
    float2 xg[NF], xtn = f2(0.0f), xtt = f2(0.0f);   // row rg's x slopes and stresses, for this row's x faces
    constexpr int NLIVE = live_items<NF>();
    static_assert(group_size<NF, 0>() + group_size<NF, 1>() + group_size<NF, 2>() == NLIVE, "ledger groups");
    // [warp][item slot] of the main piece and of a crossing tile's first piece;
    // group 0 of the first piece per thread
    constexpr int NWI = TWMAX / 64 < 4 ? 4 : TWMAX / 64;   // bank rows: interior warps
    __shared__ float sLed[NWI][32], sLedA[NWI][32], sAccA[7][TWMAX / 2];
    const int lane = t & 31, warp = t >> 5;
    for (int i = t; i < NWI * 32; i += blockDim.x) sLed[i >> 5][i & 31] = sLedA[i >> 5][i & 31] = 0.0f;
    const int slot0 = group_writer_slot<NF, 0>(lane);
    float acc0[7] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};   // ledger group 0 of this pair, summed over rows
    const int slot1 = group_writer_slot<NF, 1>(lane);
    const int slot2 = group_writer_slot<NF, 2>(lane);
    const bool fake_on = P.fake_rate != 0.0f;
    float amax = 0.0f;
#pragma unroll
    for (int f = 0; f < NF; ++f) { Pm1[f] = P0[f] = fxA[f] = fxB[f] = xg[f] = f2(0.0f); }

    // row positions of the faces and updates, loaded one iteration ahead: x of
    // row rq's zone centres (y faces), of row ru's (update), of face rq + 1/2
    auto xc_at = [&](int r) { return xc_row[min(max(r, 0), TH - 1)]; };
    auto xv_at = [&](int r) { return xv_row[min(max(r, 0), TH)]; };
    float xq = xc_at(-4), xu = xc_at(-5), xvq = xv_at(-3);

    for (int k = 0; k < TH + 5; ++k) {
        const int rn = k - 2;
        const float xq_next = xc_at(k - 3), xvq_next = xv_at(k - 2);
        if (producer) {
            if (rn + S3_DEPTH <= TH + 1) issue(rn + S3_DEPTH);
            const int ur = rn - 3 + S3_DEPTH;
            if (ur >= 0 && ur <= TH - 1) issue_update(ur);
        }

        // the update ring's row rn - 3, waited for before the row's work so that
        // the update below runs without a wait inside it
        if (interior && rn >= 3 && rn - 3 <= TH - 1 &&
            !mbar_wait_bounded(ubars + (rn - 3) % S3_USLOTS, ((rn - 3) / S3_USLOTS) & 1))
            timeout = 1;

        // ---- phase 1: row rn -> primitives (try_block_primitive, scheme.rs:185-199) --
        float2 pn[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) pn[f] = f2(0.0f);
        if (rn <= TH + 1 && active) {
            const int rr = rn + 2;
            if (!mbar_wait_bounded(bars + rr % S3_SLOTS, (rr / S3_SLOTS) & 1)) timeout = 1;
            const float* sb = (const float*)(slots + (rr % S3_SLOTS) * SLOT);
            float ua[NF], ub[NF], pa[NF], pb[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const float2 u2 = *(const float2*)(sb + f * SW + c0 + H);
                ua[f] = u2.x;
                ub[f] = u2.y;
            }
            float bad = 0.0f;
            const int ea = try_to_primitive<NF, float>(P, ua, pa, bad);
            const int eb = try_to_primitive<NF, float>(P, ub, pb, bad);
            if ((ea || eb) && interior && rn >= 0 && rn < TH) {
                const int gi = i0 + rn;
                if (ea) atomicMin(a.err_key, error_key(a.stage, ri, rd, gi, j0 + c0, ea));
                if (eb) atomicMin(a.err_key, error_key(a.stage, ri, rd, gi, j0 + c0 + 1, eb));
            }
#pragma unroll
            for (int f = 0; f < NF; ++f) pn[f] = make_float2(pa[f], pb[f]);
            float4* row = sP + (rn & 1) * (TW + 4) + p + 1;
            row[0] = make_float4(pa[0], pa[1], pa[2], 0.0f);
            row[HR] = make_float4(pb[0], pb[1], pb[2], 0.0f);
        }

        // ---- phase 2: slopes and cell records of row rg = rn - 1 (scheme.rs:216-254) ---
        const int rg = rn - 1;
        if (rg >= -1 && rg <= TH && active) {
            const float4* prow = sP + (rg & 1) * (TW + 4);
            const float4 l4 = prow[HR + p];                    // column c0 - 1 (in the row, unused, for the -2 pair)
            const float4 r4 = prow[p + 2];                     // column c0 + 2 (in the row, unused, for the TW pair)
            float lv[3] = {l4.x, l4.y, l4.z}, rv[3] = {r4.x, r4.y, r4.z};
            // the two stencil points outside the staged columns: NaN in a
            // read-set check build (tma.cuh), whose states must not change
            if (hl == 0)
                for (int f = 0; f < 3; ++f) lv[f] = poison_or(lv[f]);
            if (hl == 1)
                for (int f = 0; f < 3; ++f) rv[f] = poison_or(rv[f]);
            const float2 thx = make_float2((Pm1[0].x < pdt || P0[0].x < pdt || pn[0].x < pdt) ? 0.0f : theta,
                                           (Pm1[0].y < pdt || P0[0].y < pdt || pn[0].y < pdt) ? 0.0f : theta);
            const float2 thy = make_float2((lv[0] < pdt || P0[0].x < pdt || P0[0].y < pdt) ? 0.0f : theta,
                                           (P0[0].x < pdt || P0[0].y < pdt || rv[0] < pdt) ? 0.0f : theta);
            float2 gx[NF], gy[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                gx[f] = plm_gradient2(thx, Pm1[f], P0[f], pn[f]);
                gy[f] = plm_gradient2(thy, make_float2(lv[f], P0[f].x), P0[f], make_float2(P0[f].y, rv[f]));
            }
            // factored stress_field terms (physics.rs:322-340; face_flux, stage2.cuh)
            const float2 da = mul2(gx[1], f2(inv_dx)), db = mul2(gy[2], f2(inv_dx));
            const float2 lb = mul2(f2(P.lambda), add2(da, db));
            const float2 cv = P.visc == 0 ? mul2(f2(P.nu), P0[0]) : P0[0];
            const float2 txx = mul2(cv, fma2(f2(4.0f / 3.0f), da, fma2(f2(-2.0f / 3.0f), db, lb)));
            const float2 tyy = mul2(cv, fma2(f2(4.0f / 3.0f), db, fma2(f2(-2.0f / 3.0f), da, lb)));
            const float2 txy = mul2(cv, mul2(add2(gx[2], gy[1]), f2(inv_dx)));
            // cell records of both columns
            const int o = (rg & 1) * (TW + 4) + p + 1;
            sR0[o] = make_float4(P0[0].x, P0[1].x, P0[2].x, gy[0].x);
            sR1[o] = make_float4(gy[1].x, gy[2].x, tyy.x, txy.x);
            sR2[o] = make_float4(gx[0].x, gx[1].x, gx[2].x, txx.x);
            sR0[o + HR] = make_float4(P0[0].y, P0[1].y, P0[2].y, gy[0].y);
            sR1[o + HR] = make_float4(gy[1].y, gy[2].y, tyy.y, txy.y);
            sR2[o + HR] = make_float4(gx[0].y, gx[1].y, gx[2].y, txx.y);
#ifdef B2D_POISON
            // the records of the outer guard columns -2 and TW + 1, which no face reads
            const float4 nan4 = make_float4(poison_or(0.0f), poison_or(0.0f), poison_or(0.0f), poison_or(0.0f));
            if (hl == 0) sR0[o] = sR1[o] = sR2[o] = nan4;
            if (hl == 1) sR0[o + HR] = sR1[o + HR] = sR2[o + HR] = nan4;
#endif
#pragma unroll
            for (int f = 0; f < NF; ++f) xg[f] = gx[f];
            xtn = txx;
            xtt = txy;
        }
        if (rn <= TH + 1) {
#pragma unroll
            for (int f = 0; f < NF; ++f) { Pm1[f] = P0[f]; P0[f] = pn[f]; }
        }

        // ---- phases 3 and 4 -------------------------------------------------------------
        const int rq = rn - 2;
        const int ru = rn - 3;
        const bool fy_ok = rq >= 0 && rq <= TH - 1;
        const bool fx_ok = rq >= -1 && rq <= TH - 1;
        const bool up_ok = ru >= 0 && ru <= TH - 1;
        // y fluxes of row rq at faces c0 and c0 + 1 (cells c0-1 | c0 and c0 | c0+1)
        auto y_flux = [&]() {
            const int ob = (rq & 1) * (TW + 4) + p;           // records of columns c0 - 1, c0, c0 + 1
            const float4 a0 = sR0[ob + HR], a1 = sR1[ob + HR];
            const float4 b0 = sR0[ob + 1], b1 = sR1[ob + 1];
            const float4 d0 = sR0[ob + HR + 1], d1 = sR1[ob + HR + 1];
            const float2 pcl[3] = {make_float2(a0.x, b0.x), make_float2(a0.y, b0.y), make_float2(a0.z, b0.z)};
            const float2 gl[3] = {make_float2(a0.w, b0.w), make_float2(a1.x, b1.x), make_float2(a1.y, b1.y)};
            const float2 pcr[3] = {make_float2(b0.x, d0.x), make_float2(b0.y, d0.y), make_float2(b0.z, d0.z)};
            const float2 gr[3] = {make_float2(b0.w, d0.w), make_float2(b1.x, d1.x), make_float2(b1.y, d1.y)};
            const float x = xq;
            const float d1x = x - B.p1.x, d2x = x - B.p2.x;
            const float2 cs2 = iso_face_cs2_2(P, B, d1x * d1x, d2x * d2x, col_part(yv2, B.p1.y), col_part(yv2, B.p2.y));
            float2 F[NF];
            face_flux2<1>(P, B, pcl, gl, make_float2(a1.z, b1.z), make_float2(a1.w, b1.w), pcr, gr,
                          make_float2(b1.z, d1.z), make_float2(b1.w, d1.w), f2(x), yv2, cs2, F);
            if (fy_ok) {
                float4* fo = sF + (rq & 1) * (TW + 2) + p;
                fo[0] = make_float4(F[0].x, F[1].x, F[2].x, 0.0f);
                fo[HF] = make_float4(F[0].y, F[1].y, F[2].y, 0.0f);
#ifdef B2D_POISON
                if (hl == 1) fo[HF] = make_float4(poison_or(0.0f), poison_or(0.0f), poison_or(0.0f), 0.0f);  // face TW + 1
#endif
            }
        };
        float2 fxn[NF];
        // The y fluxes, the update and the x fluxes of an interior pair in one
        // block without a wait (the update ring's row is waited for before
        // phase 1), so that the compiler can interleave their independent
        // chains; the halo lane of the tile's right face computes its y fluxes
        // apart (measured on the 2048^2 disk: 0.1273 ms per stage against
        // 0.1321 with one call site for both and the wait inside the update).
        if (interior && rn >= 1) {
            y_flux();

            // update of row ru
            {
                const int rc = min(max(ru, 0), TH - 1);
                const float* sb = (const float*)(slots + ((rc + 2) % S3_SLOTS) * SLOT);
                const float4* frow = sF + (ru & 1) * (TW + 2) + p;   // faces c0, c0 + 1, c0 + 2
                const float4 fa = frow[0], fb = frow[HF], fc = frow[1];
                const float2 fyl[3] = {make_float2(fa.x, fb.x), make_float2(fa.y, fb.y), make_float2(fa.z, fb.z)};
                const float2 fyr[3] = {make_float2(fb.x, fc.x), make_float2(fb.y, fc.y), make_float2(fb.z, fc.z)};
                const float x = xu;
                const float* q = (const float*)(uslots + (rc % S3_USLOTS) * USLOT);
                float2 uc[NF], ulo[NF], u0[NF];
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    uc[f] = *(const float2*)(sb + f * SW + c0 + H);
                    ulo[f] = *(const float2*)(q + f * TW + c0);
                    u0[f] = *(const float2*)(q + (NF + f) * TW + c0);
                }
                // sources of the pair (Physics::source_terms, physics.rs:423-457;
                // Isothermal::source_terms, physics.rs:528-582): gravity and the
                // buffer packed; sinks (a warp with a zone inside a sink radius)
                // and fake mass (a non-zero rate) per column
                float2 tot[NF];
                float led0[8], led1[8], led2[4];
                bool sinks_any;
                {
                    const float dx1 = x - B.p1.x, dx2 = x - B.p2.x;
                    const float2 dy1 = sub2(yc2, f2(B.p1.y)), dy2 = sub2(yc2, f2(B.p2.y));
                    // Plummer accelerations (kepler-two-body, restated): -m d / (d^2 + s^2)^(3/2)
                    const float2 t1 = fma2(dy1, dy1, f2(fmaf(dx1, dx1, P.soft2)));
                    const float2 t2 = fma2(dy2, dy2, f2(fmaf(dx2, dx2, P.soft2)));
                    const float2 r1 = make_float2(rsqrtf(t1.x), rsqrtf(t1.y));
                    const float2 r2 = make_float2(rsqrtf(t2.x), rsqrtf(t2.y));
                    const float2 sdt = mul2(uc[0], f2(dt));
                    const float2 q1 = mul2(mul2(sdt, f2(-B.p1.m)), mul2(r1, mul2(r1, r1)));
                    const float2 q2 = mul2(mul2(sdt, f2(-B.p2.m)), mul2(r2, mul2(r2, r2)));
                    const float2 g1x = mul2(q1, f2(dx1)), g1y = mul2(q1, dy1);
                    const float2 g2x = mul2(q2, f2(dx2)), g2y = mul2(q2, dy2);
                    // buffer: 0.5 rate (1 + tanh((r - R) / scale)) Omega_outer, 1 + tanh(y) = 2 / (1 + exp(-2y))
                    const float2 rr2 = fma2(yc2, yc2, f2(x * x));
                    const float2 yb = mul2(sub2(make_float2(sqrtf(rr2.x), sqrtf(rr2.y)), f2(P.domain_radius)),
                                           f2(-2.0f * P.inv_buffer_scale));
                    const float2 den = add2(f2(1.0f), make_float2(__expf(yb.x), __expf(yb.y)));
                    const float2 kb = mul2(f2(-2.0f * dt * P.half_rate_omega),
                                           make_float2(__fdividef(1.0f, den.x), __fdividef(1.0f, den.y)));
                    float2 bu[NF];
#pragma unroll
                    for (int f = 0; f < NF; ++f) bu[f] = mul2(sub2(uc[f], u0[f]), kb);
                    tot[0] = bu[0];
                    tot[1] = add2(add2(g1x, g2x), bu[1]);
                    tot[2] = add2(add2(g1y, g2y), bu[2]);
                    // ledger group 0 in item order: grav1 (x, y), grav2 (x, y), buffer (3 fields)
                    led0[0] = g1x.x + g1x.y; led0[1] = g1y.x + g1y.y;
                    led0[2] = g2x.x + g2x.y; led0[3] = g2y.x + g2y.y;
                    led0[4] = bu[0].x + bu[0].y; led0[5] = bu[1].x + bu[1].y; led0[6] = bu[2].x + bu[2].y;
                    led0[7] = 0.0f;
#pragma unroll
                    for (int m = 0; m < 8; ++m) led1[m] = 0.0f;
#pragma unroll
                    for (int m = 0; m < 4; ++m) led2[m] = 0.0f;
                    // sinks: only where a zone of the warp lies inside a sink radius
                    const float2 s1 = fma2(dy1, dy1, f2(dx1 * dx1)), s2 = fma2(dy2, dy2, f2(dx2 * dx2));
                    const bool near = s1.x < P.sink_r2 || s1.y < P.sink_r2 || s2.x < P.sink_r2 || s2.y < P.sink_r2;
                    sinks_any = __any_sync(0xffffffffu, near);
                    if (sinks_any) {
                        float it[NL];
#pragma unroll
                        for (int side = 0; side < 2; ++side) {
                            const float us[NF] = {side ? uc[0].y : uc[0].x, side ? uc[1].y : uc[1].x,
                                                  side ? uc[2].y : uc[2].x};
                            const float u0s[NF] = {side ? u0[0].y : u0[0].x, side ? u0[1].y : u0[1].x,
                                                   side ? u0[2].y : u0[2].x};
                            source_terms<NF, float, false>(P, B, us, u0s, x, side ? yc2.y : yc2.x, time, dt, it);
#pragma unroll
                            for (int f = 0; f < NF; ++f) {
                                const float sk = it[SINK1 * NF + f] + it[SINK2 * NF + f];
                                if (side) tot[f].y += sk;
                                else tot[f].x += sk;
                                led1[f] += it[SINK1 * NF + f];
                                led1[NF + f] += it[SINK2 * NF + f];
                            }
                        }
                    }
                    // fake mass: u0 rate dt unless Sigma < Sigma_0 threshold
                    if (fake_on) {
                        const bool offa = uc[0].x < u0[0].x * P.fake_thr, offb = uc[0].y < u0[0].y * P.fake_thr;
#pragma unroll
                        for (int f = 0; f < NF; ++f) {
                            const float2 fk = mul2(mul2(u0[f], f2(P.fake_rate)), f2(dt));
                            const float fa = offa ? 0.0f : fk.x, fb = offb ? 0.0f : fk.y;
                            tot[f] = add2(tot[f], make_float2(fa, fb));
                            led2[f] = fa + fb;
                        }
                    }
                }
                // flux divergence and the compensated RK update (scheme.rs:290-305; state.rs:183-199)
                const size_t idx = (size_t)(i0 + rc) * N + (j0 + c0);
                float2 uo[NF];
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    const float2 du = mul2(add2(sub2(fxB[f], fxA[f]), sub2(fyr[f], fyl[f])), f2(-inv_dx * dt));
                    const float2 inc = add2(du, tot[f]);
                    df2 o = df_add_f2(df2{uc[f], ulo[f]}, inc);
                    if (has_base) {
                        const df2 b0{*(const float2*)(q + (2 * NF + f) * TW + c0),
                                     *(const float2*)(q + (3 * NF + f) * TW + c0)};
                        if (half_avg) {
                            const df2 sm = df_add2(o, b0);
                            o = {mul2(sm.hi, f2(0.5f)), mul2(sm.lo, f2(0.5f))};
                        } else {
                            const df2 x1 = df_mul2(o, w1), x2 = df_mul2(b0, wb);
                            o = df_add2(x1, x2);
                        }
                    }
                    if (up_ok) {
                        *(float2*)(uout + (size_t)(2 * f) * nn + idx) = o.hi;
                        *(float2*)(uout + (size_t)(2 * f + 1) * nn + idx) = o.lo;
                    }
                    uo[f] = o.hi;
                }
                if (up_ok) {   // the same row for the whole warp
                    // group 0 (non-zero everywhere): the pair's running sums over the tile's rows
#pragma unroll
                    for (int m = 0; m < 7; ++m) acc0[m] += led0[m];
                    if (sinks_any) {
                        float v1[8];
#pragma unroll
                        for (int m = 0; m < 8; ++m) v1[m] = led1[m];
                        const float s1 = warp_sum_items<8>(v1, lane);
                        if (slot1 >= 0) sLed[warp][slot1] += s1;
                    }
                    if (fake_on) {
                        float v2[4];
#pragma unroll
                        for (int m = 0; m < 4; ++m) v2[m] = led2[m];
                        const float s2 = warp_sum_items<4>(v2, lane);
                        if (slot2 >= 0) sLed[warp][slot2] += s2;
                    }
                    if (ru == rb - 1 && rb < TH) {   // the first piece's last row: set its sums aside
                        __syncwarp();
                        sLedA[warp][lane] = sLed[warp][lane];
                        sLed[warp][lane] = 0.0f;
#pragma unroll
                        for (int m = 0; m < 7; ++m) { sAccA[m][t] = acc0[m]; acc0[m] = 0.0f; }
                    }
                }
                if (want_amax && up_ok) {
                    const float ua[NF] = {uo[0].x, uo[1].x, uo[2].x}, ub[NF] = {uo[0].y, uo[1].y, uo[2].y};
                    amax = fmaxf(fmaxf(max_signal_speed<NF, float>(P, ua), max_signal_speed<NF, float>(P, ub)), amax);
                }
            }

            // x fluxes of faces rq + 1/2 below the pair: row rq's records from shared
            // memory, row rq + 1 = rg's from this iteration's registers (primitives
            // in Pm1 after the rotation)
            {
                const int oa = (rq & 1) * (TW + 4) + p + 1;
                const float4 a0 = sR0[oa], a1 = sR1[oa], a2 = sR2[oa];
                const float4 e0 = sR0[oa + HR], e1 = sR1[oa + HR], e2 = sR2[oa + HR];
                const float2 pcl[3] = {make_float2(a0.x, e0.x), make_float2(a0.y, e0.y), make_float2(a0.z, e0.z)};
                const float2 gl[3] = {make_float2(a2.x, e2.x), make_float2(a2.y, e2.y), make_float2(a2.z, e2.z)};
                const float x = xvq;
                const float d1x = x - B.p1.x, d2x = x - B.p2.x;
                const float2 cs2 =
                    iso_face_cs2_2(P, B, d1x * d1x, d2x * d2x, col_part(yc2, B.p1.y), col_part(yc2, B.p2.y));
                face_flux2<0>(P, B, pcl, gl, make_float2(a2.w, e2.w), make_float2(a1.w, e1.w), Pm1, xg, xtn, xtt,
                              f2(x), yc2, cs2, fxn);
            }
        } else if (hl == 1 && fy_ok) {
            y_flux();
        }
        if (fx_ok) {
#pragma unroll
            for (int f = 0; f < NF; ++f) { fxA[f] = fxB[f]; fxB[f] = fxn[f]; }
        }
        xu = xq;
        xq = xq_next;
        xvq = xvq_next;
        __syncthreads();
    }

    // ---- max speed of the tile (deterministic tree over the CTA; the ring is idle) --
    double* red = (double*)smem_raw;
    const int NT = blockDim.x;
    if (a.amax_flag) {
        red[t] = (double)amax;
        __syncthreads();
        for (int s = 1; s < NT; s <<= 1) {
            if ((t & (2 * s - 1)) == 0 && t + s < NT) red[t] = fmax(red[t], red[t + s]);
            __syncthreads();
        }
        if (t == 0 && red[0] > 0.0) atomicMax(rd.amax, (unsigned long long)__double_as_longlong(red[0]));
    }
    if (t == 0 && timeout) atomicOr(a.timeout_flag, 1u);

    // ---- ledger pieces, one per block under the tile: its block row(s) times its
    // block column(s), each flushed by its own warp --------------------------------
    if (interior) {   // whole warps: group 0's column sums of the main piece's rows, one warp reduction
        float v0[8];
#pragma unroll
        for (int m = 0; m < 7; ++m) v0[m] = acc0[m];
        v0[7] = 0.0f;
        const float s0 = warp_sum_items<8>(v0, lane);
        if (slot0 >= 0) sLed[warp][slot0] += s0;
    }
    __syncthreads();
    const int brow = block / rd.nb, bcol = block - brow * rd.nb;
    const int ncol = max(TW / rd.bs, 1), wpc = TP / 32 / ncol;   // block columns; interior warps over each
    const int lslot = tib % max(rd.bs / TW, 1);
    const int npiece = (rb < TH ? 2 : 1) * ncol;                 // the main block row's pieces, then the first's
    for (int k = warp; k < npiece; k += blockDim.x / 32) {
        const int c = k % ncol;
        if (k < ncol)
            flush_piece<NF>(rd, brow, bcol + c, lslot, TW, sLed + c * wpc, wpc, nullptr, 0, a.in_slot, a.base_slot,
                            a.out_slot, a.stage, a.bf);
        else
            flush_piece<NF>(rd, brow - 1, bcol + c, lslot, TW, sLedA + c * wpc, wpc,
                            &sAccA[0][c * wpc * 32], TWMAX / 2, a.in_slot, a.base_slot,
                            a.out_slot, a.stage, a.bf);
    }
}

}  // namespace b2d
