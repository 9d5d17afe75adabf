// stage2.cuh — the FP32-stencil RK-stage kernel with TMA row staging.
//
// Same stage as stage.cuh (try_advance_rk, src/scheme.rs:88-173, plus the RK
// average of state.rs:183-199), reorganised for throughput:
//
//  * Row staging by TMA.  One producer lane issues 1-D bulk copies
//    (cp.async.bulk) of whole tile rows — the stage input with its 2-zone
//    guard halo (wrapped periodically, mesh.rs:101-110), the background and
//    the RK base — into a ring of shared-memory slots, DEPTH rows ahead of
//    use.  Each slot completes on its own mbarrier; every wait is bounded.
//  * Column ownership.  Thread t < TW owns column t of the tile and keeps
//    that column's vertical history (primitives, cell records, x-fluxes) in
//    registers.  A fifth "halo" warp owns the four guard columns.  Shared
//    memory only carries the horizontal exchange (primitives for the y slope,
//    cell records for the y face, y fluxes for the right face), in float4
//    planes that are free of bank conflicts.
//  * Pipeline per marching row rn: load/convert row rn, slopes and cell
//    records of row rn-1, fluxes of row rn-2, update of row rn-3; one
//    __syncthreads per row.
#pragma once

#include "stage.cuh"
#include "tma.cuh"

namespace b2d {

constexpr int S2_DEPTH = 2;              // rows staged ahead of use
constexpr int S2_SLOTS = S2_DEPTH + 4;   // stencil ring: a row is read again 3 rows after it lands
constexpr int S2_USLOTS = S2_DEPTH + 1;  // update ring: a row is read once, at its update

// Bytes of one stencil slot: the stage input's stencil words of one tile row
// with its halo (hi plane of the compensated store, or the FP64 state).
__host__ __device__ inline int s2_slot_bytes(int nf, int store, int tw)
{
    return store == 1 ? 4 * nf * (tw + 8) : 8 * nf * (tw + 4);
}

// Bytes of one update slot: what the update of a row reads besides the stencil
// words (compensated: lo | bg hi | base hi | base lo; FP64: bg | base).
__host__ __device__ inline int s2_uslot_bytes(int nf, int store, int tw)
{
    return store == 1 ? 4 * 4 * nf * tw : 8 * 2 * nf * tw;
}

__host__ __device__ inline int s2_smem_bytes(int nf, int store, int tw)
{
    int slots = S2_SLOTS * s2_slot_bytes(nf, store, tw) + S2_USLOTS * s2_uslot_bytes(nf, store, tw);
    int exch = 16 * (2 * (tw + 4) + 3 * 2 * (tw + 2) + 2 * (tw + 1));
    return slots + exch + 8 * (S2_SLOTS + S2_USLOTS);
}

// Viscous stress, factored.  The face stress of stress_field (physics.rs:
// 322-349) with the `nu` closure of scheme.rs:230-247 is
//   tau_nn = (rho_l nu_l (s_nn,l + lambda bulk_l) + rho_r nu_r (s_nn,r + lambda bulk_r)) / 2
// (and tau_t alike with s_xy and no bulk term).  nu_l = nu_r = nu for a
// constant viscosity; for the alpha model nu_side = K(face) * cs2 with
// K = alpha / Omega_2(face) / sqrt(gamma - 1), cs2 taken at the face from the
// potential (isothermal, so nu_l = nu_r again) or from the cell's own
// pressure (Euler).  Each cell therefore carries T_nn = c rho (s_nn + lambda
// bulk) and T_xy = c rho s_xy with c = nu (constant), 1 (isothermal alpha) or
// gamma p / rho (Euler alpha), and a face needs tau = K (T_l + T_r) / 2 with
// K = 1 for the constant model: the stress algebra runs once per cell instead
// of twice per face, and the alpha factor once per face instead of once per
// side.  (This reassociates the FP32 stress; the FP64 kernels keep the
// reference's order.)
template <int NF>
__device__ __forceinline__ float cell_visc_scale(const DevParamsF& P, const float* pc)
{
    if (P.visc == 0) return P.nu * pc[0];
    if constexpr (NF == 3) return pc[0];
    else return P.gamma * pc[3];
}

// K of the alpha model at a face (the cs2 of an isothermal face included).
template <int NF>
__device__ __forceinline__ float alpha_face_factor(const DevParamsF& P, const Binary<float>& b, float x, float y,
                                                   float cs2_face)
{
    float dx1 = x - b.p1.x, dy1 = y - b.p1.y, dx2 = x - b.p2.x, dy2 = y - b.p2.y;
    float a1 = sqrtf(dx1 * dx1 + dy1 * dy1) + P.eps_dx;
    float a2 = sqrtf(dx2 * dx2 + dy2 * dy2) + P.eps_dx;
    float w2 = __fdividef(b.p1.m, a1 * a1 * a1) + __fdividef(b.p2.m, a2 * a2 * a2);
    float k = P.nu * rsqrtf(w2) * P.inv_sqrt_gm;
    if constexpr (NF == 3) k *= cs2_face;
    return k;
}

// Isothermal face sound speed cs2 = -phi / M^2 (physics.rs:584-607) with the
// Plummer potential phi = -sum_k m_k / sqrt(dx_k^2 + dy_k^2 + s^2): the x part
// of each distance is shared by a tile row and the y part (with s^2) by a
// column, so a face adds the two and takes one reciprocal root per body.
__device__ __forceinline__ float iso_face_cs2(const DevParamsF& P, const Binary<float>& B, float dx1sq, float dx2sq,
                                              float cy1, float cy2)
{
    return (B.p1.m * rsqrtf(dx1sq + cy1) + B.p2.m * rsqrtf(dx2sq + cy2)) * P.inv_mach2;
}

// intercell_flux (physics.rs:584-607 iso, 776-803 euler) from the two cells'
// primitive (pc), slope along the face normal (g) and factored stresses (tn:
// normal-normal, tt: off-diagonal); cs2 is the isothermal face sound speed
// (unused for Euler).
template <int NF, int AXIS>
__device__ __forceinline__ void face_flux(const DevParamsF& P, const Binary<float>& B, const float* pcl,
                                          const float* gl, float tnl, float ttl, const float* pcr,
                                          const float* gr, float tnr, float ttr, float x, float y, float cs2,
                                          float* F)
{
    float pl[NF], pr[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        pl[k] = pcl[k] + 0.5f * gl[k];
        pr[k] = pcr[k] - 0.5f * gr[k];
    }
    const float k = P.visc == 0 ? 0.5f : 0.5f * alpha_face_factor<NF>(P, B, x, y, cs2);
    const float tn = k * (tnl + tnr);
    const float tt = k * (ttl + ttr);
    const float tau_x = AXIS == 0 ? tn : tt;
    const float tau_y = AXIS == 0 ? tt : tn;
    hlle<NF, float>(P, pl, pr, AXIS, cs2, F);
    F[1] -= tau_x;
    F[2] -= tau_y;
    if constexpr (NF == 4) F[3] -= tau_x * 0.5f * (pcl[1] + pcr[1]) + tau_y * 0.5f * (pcl[2] + pcr[2]);
}

// Source ledger items that can be non-zero (grav mass, isothermal cooling and
// Euler fake mass are identically zero).
template <int NF> __device__ __forceinline__ constexpr bool item_live(int k)
{
    const int item = k / NF, f = k % NF;
    if ((item == GRAV1 || item == GRAV2) && f == 0) return false;
    if (NF == 3 && item == COOLING) return false;
    if (NF == 4 && item == FAKE_MASS) return false;
    return true;
}

template <int NF> __host__ __device__ constexpr int live_items()
{
    int n = 0;
    for (int k = 0; k < NITEMS * NF; ++k) {
        const int item = k / NF, f = k % NF;
        bool dead = ((item == GRAV1 || item == GRAV2) && f == 0) || (NF == 3 && item == COOLING) ||
                    (NF == 4 && item == FAKE_MASS);
        n += dead ? 0 : 1;
    }
    return n;
}

// Reduction groups of the live items: 0 = gravity, buffer and cooling (non-zero
// almost everywhere), 1 = the two sinks (zero outside the sink radii), 2 =
// fake mass (zero unless a fake-mass rate is set).  A warp reduces group 1
// only when one of its zones lies inside a sink, and group 2 only for a
// non-zero rate: the sums are the same, since the skipped terms are zeros.
template <int NF> __host__ __device__ constexpr int item_group(int k)
{
    const int item = k / NF;
    return (item == SINK1 || item == SINK2) ? 1 : (item == FAKE_MASS ? 2 : 0);
}

template <int NF, int G> __host__ __device__ constexpr int group_size()
{
    int n = 0;
    for (int k = 0; k < NITEMS * NF; ++k) {
        const int item = k / NF, f = k % NF;
        bool dead = ((item == GRAV1 || item == GRAV2) && f == 0) || (NF == 3 && item == COOLING) ||
                    (NF == 4 && item == FAKE_MASS);
        n += (!dead && item_group<NF>(k) == G) ? 1 : 0;
    }
    return n;
}

template <int N> __host__ __device__ constexpr int pow2_at_least()
{
    int p = 1;
    while (p < N) p <<= 1;
    return p;
}

// Sum K values (K a power of two, K <= 32) over the 32 lanes of a warp by
// recursive halving: after the call lane l holds the warp total of value
// item_of_lane(l, K); 2K - 1 shuffles in all.
template <int K> __device__ __forceinline__ float warp_sum_items(float (&v)[K], int lane)
{
#pragma unroll
    for (int half = K / 2, off = 16; half >= 1; half >>= 1, off >>= 1) {
        const bool upper = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const float send = upper ? v[i] : v[i + half];
            const float keep = upper ? v[i + half] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    float s = v[0];
    for (int off = 16 / K; off >= 1; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    return s;
}

// Which value of warp_sum_items lane l ends up holding.
template <int K> __device__ __forceinline__ int item_of_lane(int lane)
{
    int item = 0;
    for (int half = K / 2, off = 16; half >= 1; half >>= 1, off >>= 1)
        if (lane & off) item += half;
    return item;
}

// The per-warp ledger slot (index among the live items) that `lane` adds its
// warp_sum_items result of group G to, or -1.
template <int NF, int G> __device__ __forceinline__ int group_writer_slot(int lane)
{
    constexpr int NG = group_size<NF, G>();
    constexpr int KG = pow2_at_least<NG>();
    if (NG == 0 || (lane & (32 / KG - 1)) != 0) return -1;
    const int m = item_of_lane<KG>(lane);
    if (m >= NG) return -1;
    int live = 0, member = 0;
    for (int k = 0; k < NITEMS * NF; ++k) {
        if (!item_live<NF>(k)) continue;
        if (item_group<NF>(k) == G) {
            if (member == m) return live;
            ++member;
        }
        ++live;
    }
    return -1;
}

// Warp-sum the live items of group G of this zone's `it` and add them to the
// warp's ledger slots.
template <int NF, int G>
__device__ __forceinline__ void reduce_group(const float* it, int lane, int slot, float* led)
{
    constexpr int NG = group_size<NF, G>();
    constexpr int KG = pow2_at_least<NG>();
    float v[KG];
    int j = 0;
#pragma unroll
    for (int k = 0; k < NITEMS * NF; ++k)
        if (item_live<NF>(k) && item_group<NF>(k) == G) v[j++] = it[k];
#pragma unroll
    for (int k = NG; k < KG; ++k) v[k] = 0.0f;
    const float s = warp_sum_items<KG>(v, lane);
    if (slot >= 0) led[slot] += s;
}

template <bool SINGLE>
__device__ __forceinline__ const DevParamsF& params_for(const StageArgs& a, const DevParamsF& shared_copy)
{
    if constexpr (SINGLE) return a.pf1;
    else return shared_copy;
}

// One ledger piece of a tile (its columns in block (brow, bj)), by one warp
// after the row loop (stage2 and stage3 kernels): sums over the bank rows of
// the nw interior warps over those columns, the piece's slot in the block's partials, and the fold of
// the block's pieces (in piece order) by the block's last piece.  acc (a
// crossing tile's first piece) holds group 0 per thread of those warps, to be
// reduced here first.  Out of line, so that it does not weigh on the row
// loop's register allocation; no CTA barrier, so that warps can flush
// several pieces at once.
template <int NF>
__device__ __noinline__ void flush_piece(const RunDev& rd, int brow, int bj, int lslot, int TW, float (*bank)[32],
                                         int nw, const float* acc, int acc_stride, int in_slot, int base_slot,
                                         int out_slot, int stage, double bf)
{
    constexpr int NL = NITEMS * NF;
    const int lane = threadIdx.x & 31;
    if (acc) {
        float v0[8];
#pragma unroll
        for (int m = 0; m < 7; ++m) {
            v0[m] = 0.0f;
            for (int w = 0; w < nw; ++w) v0[m] += acc[m * acc_stride + lane + 32 * w];
        }
        v0[7] = 0.0f;
        const float s0 = warp_sum_items<8>(v0, lane);
        const int slot0 = group_writer_slot<NF, 0>(lane);
        if (slot0 >= 0) bank[0][slot0] += s0;
        __syncwarp();
    }
    const int bs = rd.bs, nc = rd.chunks, per_row = max(bs / TW, 1);
    const int ti = rd.chunk0 + ((int)blockIdx.x - rd.tile_base) / rd.tiles_j;
    const int block = brow * rd.nb + bj;
    const int piece = (ti - chunk_of_row(brow * bs, rd.N, nc)) * per_row + lslot;
    const int pieces = chunks_in_block_row(brow, bs, rd.N, nc) * per_row;
    if (lane < NL) {
        int j = 0;
        bool live = false;
        for (int k2 = 0; k2 < NL; ++k2) {
            if (k2 == lane) { live = item_live<NF>(k2); break; }
            if (item_live<NF>(k2)) ++j;
        }
        double s = 0.0;
        if (live)
            for (int w = 0; w < nw; ++w) s += (double)bank[w][j];
        rd.partial[((size_t)block * rd.tiles_per_block + piece) * NL + lane] = s;
        __threadfence();   // visible before the counter below counts this piece
    }
    __syncwarp();
    unsigned last = 0;
    if (lane == 0) last = atomicAdd(rd.counter + block, 1u) == (unsigned)pieces - 1;
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return;
    __threadfence();
    if (lane < NL) {
        const double area = (double)rd.p.dx * rd.p.dx;
        double s = 0.0;
        for (int q = 0; q < pieces; ++q)
            s += __ldcg(rd.partial + ((size_t)block * rd.tiles_per_block + q) * NL + lane);
        double v = __ldcg(rd.ledger[in_slot] + (size_t)block * NL + lane) + s * area;
        if (base_slot >= 0) v = v * (-bf + 1.0) + __ldcg(rd.ledger[base_slot] + (size_t)block * NL + lane) * bf;
        rd.ledger[out_slot][(size_t)block * NL + lane] = v;
        // the block's ds·dx·dy of this stage, for the orbital-element ledger
        if (rd.stage_ds) rd.stage_ds[((size_t)stage * rd.nblocks + block) * NL + lane] = s * area;
    }
    if (lane == 0) rd.counter[block] = 0u;
}

template <int NF, int STORE, bool SINGLE>
__global__ void __launch_bounds__(160, (NF == 3 && STORE == 1) ? 4 : 3) stage2_kernel(StageArgs a)
{
    using E = typename std::conditional<STORE == 1, float, double>::type;
    constexpr int H = STORE == 1 ? 4 : 2;     // staged halo columns per side: 16 bytes
    constexpr int RQ = (2 * NF + 2 + 3) / 4;  // float4 planes of a y-face record
    constexpr int NL = NITEMS * NF;

    const int TW = blockDim.x - 32;
    const int t = threadIdx.x;
    const int SW = TW + 2 * H;

    int ri = 0;
    const int g = blockIdx.x;
    while (ri + 1 < a.nruns && g >= a.runs[ri + 1].tile_base) ++ri;
    const RunDev& rd = a.runs[ri];
    if (g - rd.tile_base >= rd.ntiles) return;

    // Physics parameters: a single-run launch reads them from the kernel
    // arguments (constant-bank operands, no load instruction); a batched
    // launch stages its run's parameters in shared memory.
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
    // rows [i0, i0 + TH): row chunk ti of C (chunk_start, runtime.cuh); a chunk
    // of at most bs rows lies in one block row, or in two from its row rb, and
    // its ledger piece in the last of them is the tile's main piece
    const int C = rd.chunks;
    const int i0 = chunk_start(ti, N, C), TH = chunk_start(ti + 1, N, C) - i0, j0 = tj * TW;
    const int bj = j0 / bs, lj0 = j0 % bs;
    const int rb = min(bs - i0 % bs, TH);
    const int bl = (i0 + TH - 1) / bs;
    const int block = bl * rd.nb + bj;
    const int tib = (ti - chunk_of_row(bl * bs, N, C)) * (bs / TW) + lj0 / TW;
    const bool has_base = a.base_slot >= 0;

    const E* uin = (const E*)rd.slot[a.in_slot];
    const E* ubase = has_base ? (const E*)rd.slot[a.base_slot] : nullptr;
    E* uout = (E*)rd.slot[a.out_slot];
    const E* ubg = (const E*)rd.bg;
    const float dt = (float)*rd.dt;
    const float time = (float)rd.stage_time[a.stage];
    const float* xc = rd.xcf;
    const float* xv = rd.xvf;

    // ---- shared memory carve-up ------------------------------------------------
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int SLOT = s2_slot_bytes(NF, STORE, TW);
    const int USLOT = s2_uslot_bytes(NF, STORE, TW);
    unsigned char* slots = smem_raw;                          // stencil ring
    unsigned char* uslots = slots + S2_SLOTS * SLOT;          // update ring
    float4* sP = (float4*)(uslots + S2_USLOTS * USLOT);       // [2][TW+4]  primitives of a row
    float4* sR0 = sP + 2 * (TW + 4);                          // [2][TW+2]  cell record, 3 float4 planes
    float4* sR1 = sR0 + 2 * (TW + 2);
    float4* sR2 = sR1 + 2 * (TW + 2);
    float4* sF = sR2 + 2 * (TW + 2);                          // [2][TW+1]  y-face fluxes
    uint64_t* bars = (uint64_t*)(sF + 2 * (TW + 1));          // [S2_SLOTS] stencil ring
    uint64_t* ubars = bars + S2_SLOTS;                        // [S2_USLOTS] update ring

    // ---- roles -----------------------------------------------------------------
    const bool interior = t < TW;
    const int hl = t - TW;                                    // lane in the halo warp
    const bool active = interior || (hl >= 0 && hl < 4);
    const int c = interior ? t : (hl < 2 ? hl - 2 : TW + hl - 2);
    const bool has_rec = active && c >= -1 && c <= TW;
    const bool has_fy = active && c >= 0 && c <= TW;
    const bool producer = (hl == 4);

    // stencil plane of field f in the stage input (hi plane for the compensated store)
    auto plane = [&](const E* base, int f, int part) -> const E* {
        return STORE == 1 ? base + (size_t)(2 * f + part) * nn : base + (size_t)f * nn;
    };

    // ---- producer: stage tile row r into its slot -----------------------------------
    auto copy_row = [&](unsigned char* dst, const E* row, int w_halo, uint64_t* bar) {
        if (w_halo == 0) {
            bulk_load(dst, row + j0, TW * sizeof(E), bar);
        } else if (j0 >= H && j0 + TW + H <= N) {
            bulk_load(dst, row + j0 - H, SW * sizeof(E), bar);
        } else {
            bulk_load(dst, row + (j0 - H + N) % N, H * sizeof(E), bar);
            bulk_load(dst + H * sizeof(E), row + j0, TW * sizeof(E), bar);
            bulk_load(dst + (H + TW) * sizeof(E), row + (j0 + TW) % N, H * sizeof(E), bar);
        }
    };
    // stencil words of tile row r (r in [-2, TH+1]) into the stencil ring
    auto issue = [&](int r) {
        const int rr = r + 2;
        unsigned char* sb = slots + (rr % S2_SLOTS) * SLOT;
        uint64_t* bar = bars + rr % S2_SLOTS;
        const int gi = wrap(i0 + r, N);
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, NF * SW * sizeof(E));
        const size_t roff = (size_t)gi * N;
        for (int f = 0; f < NF; ++f) copy_row(sb + f * SW * sizeof(E), plane(uin, f, 0) + roff, 1, bar);
    };
    // the rest of what the update of tile row r (r in [0, TH)) reads, into the update ring
    auto issue_update = [&](int r) {
        unsigned char* q = uslots + (r % S2_USLOTS) * USLOT;
        uint64_t* bar = ubars + r % S2_USLOTS;
        const size_t roff = (size_t)(i0 + r) * N;
        uint32_t bytes;
        if (STORE == 1) bytes = (2 + (has_base ? 2 : 0)) * NF * TW * sizeof(E);
        else bytes = (1 + (has_base ? 1 : 0)) * NF * TW * sizeof(E);
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, bytes);
        {
            if (STORE == 1) {
                for (int f = 0; f < NF; ++f, q += TW * sizeof(E)) copy_row(q, plane(uin, f, 1) + roff, 0, bar);
                for (int f = 0; f < NF; ++f, q += TW * sizeof(E)) copy_row(q, plane(ubg, f, 0) + roff, 0, bar);
                if (has_base) {
                    for (int f = 0; f < NF; ++f, q += TW * sizeof(E)) copy_row(q, plane(ubase, f, 0) + roff, 0, bar);
                    for (int f = 0; f < NF; ++f, q += TW * sizeof(E)) copy_row(q, plane(ubase, f, 1) + roff, 0, bar);
                }
            } else {
                for (int f = 0; f < NF; ++f, q += TW * sizeof(E)) copy_row(q, plane(ubg, f, 0) + roff, 0, bar);
                if (has_base)
                    for (int f = 0; f < NF; ++f, q += TW * sizeof(E)) copy_row(q, plane(ubase, f, 0) + roff, 0, bar);
            }
        }
    };

    poison_dynamic_smem(smem_raw);
    if (producer) {
        for (int s = 0; s < S2_SLOTS + S2_USLOTS; ++s) mbar_init(bars + s, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (producer)
        for (int r = -2; r < -2 + S2_DEPTH; ++r) issue(r);

    const float theta = P.plm, pdt = P.pdt, inv_dx = P.inv_dx;
    const bool half_avg = a.bf == 0.5;                  // RK2: (u + u0) / 2
    const df32 w1{a.w1f.hi, a.w1f.lo}, wb{a.bff.hi, a.bff.lo};
    const double bf = a.bf, w1d = -a.bf + 1.0;
    const bool want_amax = a.amax_flag != 0;
    // positions of this thread's column: zone centre y and left y-face
    const float yc_own = interior ? xc[j0 + c] : 0.0f;
    const float yv_own = has_fy ? xv[bj * (bs + 1) + lj0 + c] : 0.0f;
    const float* xv_row = rd.xvgf + i0;                // x of face (i0 + r) - 1/2 is xv_row[r]
    const float* xc_row = xc + i0;
    // column parts (dy^2 + s^2) of the body distances of this column's faces
    float cyv1 = 0.0f, cyv2 = 0.0f, cyc1 = 0.0f, cyc2 = 0.0f;
    if constexpr (NF == 3) {
        const float dv1 = yv_own - B.p1.y, dv2 = yv_own - B.p2.y, dc1 = yc_own - B.p1.y, dc2 = yc_own - B.p2.y;
        cyv1 = dv1 * dv1 + P.soft2;
        cyv2 = dv2 * dv2 + P.soft2;
        cyc1 = dc1 * dc1 + P.soft2;
        cyc2 = dc2 * dc2 + P.soft2;
    }

    float Pm1[NF], P0[NF];               // primitives of rows rg-1, rg (own column)
    float rxa[2 * NF + 2], rxb[2 * NF + 2];  // x-face records of rows rq, rq+1: pc, gx, txx, txy
    float fxA[NF], fxB[NF];              // x fluxes at faces ru-1/2, ru+1/2
    // source ledger: per-warp accumulators of the live items, one lane each
    constexpr int NLIVE = live_items<NF>();
    static_assert(group_size<NF, 0>() + group_size<NF, 1>() + group_size<NF, 2>() == NLIVE, "ledger groups");
    __shared__ float sLed[4][32], sLedA[4][32];   // [warp][item slot]: main piece, a crossing tile's first piece
    const int lane = t & 31, warp = t >> 5;
    if (t < 128) sLed[t >> 5][t & 31] = sLedA[t >> 5][t & 31] = 0.0f;
    const int slot0 = group_writer_slot<NF, 0>(lane);
    const int slot1 = group_writer_slot<NF, 1>(lane);
    const int slot2 = group_writer_slot<NF, 2>(lane);
    const bool fake_on = group_size<NF, 2>() > 0 && P.fake_rate != 0.0f;
    float amax = 0.0f;
#pragma unroll
    for (int f = 0; f < NF; ++f) { Pm1[f] = P0[f] = fxA[f] = fxB[f] = 0.0f; }
#pragma unroll
    for (int w = 0; w < 2 * NF + 2; ++w) rxa[w] = rxb[w] = 0.0f;

    for (int k = 0; k < TH + 5; ++k) {
        const int rn = k - 2;
        if (producer) {
            if (rn + S2_DEPTH <= TH + 1) issue(rn + S2_DEPTH);
            const int ur = rn - 3 + S2_DEPTH;                // update row needed S2_DEPTH rows from now
            if (ur >= 0 && ur <= TH - 1) issue_update(ur);
        }

        // ---- phase 1: row rn -> primitives (try_block_primitive, scheme.rs:185-199) --
        float pn[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) pn[f] = 0.0f;
        if (rn <= TH + 1 && active) {
            const int rr = rn + 2;
            uint64_t* bar = bars + rr % S2_SLOTS;
            if (!mbar_wait_bounded(bar, (rr / S2_SLOTS) & 1)) timeout = 1;
            const E* sb = (const E*)(slots + (rr % S2_SLOTS) * SLOT);
            float u[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) u[f] = (float)sb[f * SW + c + H];
            float bad = 0.0f;
            int e = try_to_primitive<NF, float>(P, u, pn, bad);
            if (e && interior && rn >= 0 && rn < TH) {
                const int gi = i0 + rn;
                atomicMin(a.err_key, error_key(a.stage, ri, rd, gi, j0 + c, e));
            }
            sP[(rn & 1) * (TW + 4) + c + 2] = make_float4(pn[0], pn[1], pn[2], NF == 4 ? pn[NF - 1] : 0.0f);
        }

        // ---- phase 2: slopes and cell record of row rg = rn - 1 (scheme.rs:216-254) ---
        const int rg = rn - 1;
        if (rg >= -1 && rg <= TH && has_rec) {
            const float4 l4 = sP[(rg & 1) * (TW + 4) + c + 1];
            const float4 r4 = sP[(rg & 1) * (TW + 4) + c + 3];
            const float lv[4] = {l4.x, l4.y, l4.z, l4.w}, rv[4] = {r4.x, r4.y, r4.z, r4.w};
            const float thx = (Pm1[0] < pdt || P0[0] < pdt || pn[0] < pdt) ? 0.0f : theta;
            const float thy = (lv[0] < pdt || P0[0] < pdt || rv[0] < pdt) ? 0.0f : theta;
            float gx[NF], gy[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                gx[f] = plm_gradient(thx, Pm1[f], P0[f], pn[f]);
                gy[f] = plm_gradient(thy, lv[f], P0[f], rv[f]);
            }
            // stress_field terms (physics.rs:322-340), factored per cell (see face_flux)
            const float da = gx[1] * inv_dx, db = gy[2] * inv_dx;
            const float lb = P.lambda * (da + db);
            const float cv = cell_visc_scale<NF>(P, P0);
            const float txx = cv * ((4.0f / 3.0f) * da - (2.0f / 3.0f) * db + lb);
            const float tyy = cv * ((4.0f / 3.0f) * db - (2.0f / 3.0f) * da + lb);
            const float txy = cv * ((gx[2] + gy[1]) * inv_dx);
            // y-face record for the right neighbour: pc | gy | tyy, txy
            float yr[4 * RQ];
#pragma unroll
            for (int f = 0; f < NF; ++f) { yr[f] = P0[f]; yr[NF + f] = gy[f]; }
            yr[2 * NF] = tyy;
            yr[2 * NF + 1] = txy;
#pragma unroll
            for (int w = 2 * NF + 2; w < 4 * RQ; ++w) yr[w] = 0.0f;
            const int o = (rg & 1) * (TW + 2) + c + 1;
            sR0[o] = make_float4(yr[0], yr[1], yr[2], yr[3]);
            sR1[o] = make_float4(yr[4], yr[5], yr[6], yr[7]);
            if constexpr (RQ == 3) sR2[o] = make_float4(yr[8], yr[9], yr[10], yr[11]);
            // x-face record kept in registers
#pragma unroll
            for (int w = 0; w < 2 * NF + 2; ++w) rxa[w] = rxb[w];
#pragma unroll
            for (int f = 0; f < NF; ++f) { rxb[f] = P0[f]; rxb[NF + f] = gx[f]; }
            rxb[2 * NF] = txx;
            rxb[2 * NF + 1] = txy;
        }
        if (rn <= TH + 1) {
#pragma unroll
            for (int f = 0; f < NF; ++f) { Pm1[f] = P0[f]; P0[f] = pn[f]; }
        }

        // ---- phases 3 and 4 -------------------------------------------------------------
        // y flux of row rq = rn - 2 (this column's left face), update of row ru = rn - 3 and
        // x flux of face rq + 1/2 (scheme.rs:257-268, 290-305; state.rs:183-199).  Interior
        // threads run all three every iteration as one straight-line block (row indices
        // clamped, side effects masked) so the compiler can interleave the independent
        // dependency chains; the halo lane of column TW runs the y flux only.
        const int rq = rn - 2;
        const int ru = rn - 3;
        const bool fy_ok = rq >= 0 && rq <= TH - 1;
        const bool fx_ok = rq >= -1 && rq <= TH - 1;
        const bool up_ok = ru >= 0 && ru <= TH - 1;
        auto y_flux = [&]() {
            const int ol = (rq & 1) * (TW + 2) + c, orr = ol + 1;
            const float4 v0 = sR0[ol], v1 = sR1[ol], v2 = RQ == 3 ? sR2[ol] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 w0 = sR0[orr], w1v = sR1[orr], w2 = RQ == 3 ? sR2[orr] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float L[12] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w, v2.x, v2.y, v2.z, v2.w};
            const float Rr[12] = {w0.x, w0.y, w0.z, w0.w, w1v.x, w1v.y, w1v.z, w1v.w, w2.x, w2.y, w2.z, w2.w};
            const float x = xc_row[min(max(rq, 0), TH - 1)];
            float cs2 = 0.0f;
            if constexpr (NF == 3) {
                const float d1 = x - B.p1.x, d2 = x - B.p2.x;
                cs2 = iso_face_cs2(P, B, d1 * d1, d2 * d2, cyv1, cyv2);
            }
            float F[NF];
            face_flux<NF, 1>(P, B, L, L + NF, L[2 * NF], L[2 * NF + 1], Rr, Rr + NF, Rr[2 * NF], Rr[2 * NF + 1], x,
                             yv_own, cs2, F);
            if (fy_ok) sF[(rq & 1) * (TW + 1) + c] = make_float4(F[0], F[1], F[2], NF == 4 ? F[NF - 1] : 0.0f);
        };
        float fxn[NF];
        if (interior && rn >= 1) {   // before rn = 1 no face or update row is valid
            y_flux();

            // update of row ru
            {
                const int rc = min(max(ru, 0), TH - 1);
                const E* sb = (const E*)(slots + ((rc + 2) % S2_SLOTS) * SLOT);
                const float4 fl4 = sF[(ru & 1) * (TW + 1) + c], fr4 = sF[(ru & 1) * (TW + 1) + c + 1];
                const float fyl[4] = {fl4.x, fl4.y, fl4.z, fl4.w}, fyr[4] = {fr4.x, fr4.y, fr4.z, fr4.w};
                const float x = xc_row[rc];
                float uc[NF], u0[NF];
                if (up_ok && !mbar_wait_bounded(ubars + rc % S2_USLOTS, (rc / S2_USLOTS) & 1)) timeout = 1;
                const E* q = (const E*)(uslots + (rc % S2_USLOTS) * USLOT);
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    uc[f] = (float)sb[f * SW + c + H];
                    u0[f] = STORE == 1 ? (float)q[(NF + f) * TW + c] : (float)q[f * TW + c];
                }
                float it[NL];
                const bool sinks_on = source_terms<NF, float, true>(P, B, uc, u0, x, yc_own, time, dt, it);
                // the items' total, leaving out the ones that are zero for the whole warp
                float tot[NF];
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    tot[f] = it[GRAV1 * NF + f] + it[GRAV2 * NF + f] + it[BUFFER * NF + f];
                    if constexpr (NF == 4) tot[f] += it[COOLING * NF + f];
                }
                if (sinks_on) {
#pragma unroll
                    for (int f = 0; f < NF; ++f) tot[f] += it[SINK1 * NF + f] + it[SINK2 * NF + f];
                }
                if (NF == 3 && fake_on) {
#pragma unroll
                    for (int f = 0; f < NF; ++f) tot[f] += it[FAKE_MASS * NF + f];
                }
                const size_t idx = (size_t)(i0 + rc) * N + (j0 + c);
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    float du = ((fxB[f] - fxA[f]) + (fyr[f] - fyl[f])) * inv_dx * -dt;
                    float inc = du + tot[f];
                    if constexpr (STORE == 1) {
                        df32 o = df_add_f(df32{(float)sb[f * SW + c + H], (float)q[f * TW + c]}, inc);
                        if (has_base) {
                            df32 b0{(float)q[(2 * NF + f) * TW + c], (float)q[(3 * NF + f) * TW + c]};
                            if (half_avg) {
                                df32 sm = df_add(o, b0);
                                o = {sm.hi * 0.5f, sm.lo * 0.5f};
                            } else {
                                o = df_add(df_mul(o, w1), df_mul(b0, wb));
                            }
                        }
                        if (up_ok) {
                            ((float*)uout)[(size_t)(2 * f) * nn + idx] = o.hi;
                            ((float*)uout)[(size_t)(2 * f + 1) * nn + idx] = o.lo;
                        }
                        uc[f] = o.hi;
                    } else {
                        double o = (double)sb[f * SW + c + H] + (double)inc;
                        if (has_base) o = o * w1d + (double)q[(NF + f) * TW + c] * bf;
                        if (up_ok) ((double*)uout)[(size_t)f * nn + idx] = o;
                        uc[f] = (float)o;
                    }
                }
                if (up_ok) {   // the same row for the whole warp
                    reduce_group<NF, 0>(it, lane, slot0, sLed[warp]);
                    if (sinks_on) reduce_group<NF, 1>(it, lane, slot1, sLed[warp]);
                    if (fake_on) reduce_group<NF, 2>(it, lane, slot2, sLed[warp]);
                    if (ru == rb - 1 && rb < TH) {   // the first piece's last row: set its sums aside
                        __syncwarp();
                        sLedA[warp][lane] = sLed[warp][lane];
                        sLed[warp][lane] = 0.0f;
                    }
                }
                if (want_amax && up_ok) amax = fmaxf(max_signal_speed<NF, float>(P, uc), amax);
            }

            // x flux of face rq + 1/2
            {
                const float x = xv_row[min(max(rq + 1, 0), TH)];
                float cs2 = 0.0f;
                if constexpr (NF == 3) {
                    const float d1 = x - B.p1.x, d2 = x - B.p2.x;
                    cs2 = iso_face_cs2(P, B, d1 * d1, d2 * d2, cyc1, cyc2);
                }
                face_flux<NF, 0>(P, B, rxa, rxa + NF, rxa[2 * NF], rxa[2 * NF + 1], rxb, rxb + NF, rxb[2 * NF],
                                 rxb[2 * NF + 1], x, yc_own, cs2, fxn);
            }
        } else if (hl == 2 && fy_ok) {
            y_flux();
        }
        if (fx_ok) {
#pragma unroll
            for (int f = 0; f < NF; ++f) { fxA[f] = fxB[f]; fxB[f] = fxn[f]; }
        }
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

    // ---- ledger pieces: the main piece by warp 0, a crossing tile's first piece (the
    // block row above) by warp 1, at once ----------------------------------------
    __syncthreads();
    const int brow = block / rd.nb, lslot = tib % (rd.bs / TW);
    if (warp == 0)
        flush_piece<NF>(rd, brow, block - brow * rd.nb, lslot, TW, sLed, TW / 32, nullptr, 0, a.in_slot, a.base_slot,
                        a.out_slot, a.stage, a.bf);
    else if (warp == 1 && rb < TH)
        flush_piece<NF>(rd, brow - 1, block - brow * rd.nb, lslot, TW, sLedA, TW / 32, nullptr, 0, a.in_slot,
                        a.base_slot, a.out_slot, a.stage, a.bf);
}

}  // namespace b2d
