// stage3e.cuh — the Euler, compensated-FP32 RK-stage kernel with two columns
// per thread and packed FP32x2 arithmetic.
//
// The stage of stage2.cuh's Euler instantiation (try_advance_rk,
// src/scheme.rs:88-173; Euler::try_to_primitive physics.rs:631-660,
// intercell_flux 776-803, source_terms 683-774; the RK average of
// state.rs:183-199) on the thread mapping of stage3.cuh: column pairs in
// float2 registers, the TMA row ring, the halo warp (lanes 0 and 1 own the
// guard pairs, lane 4 the producer), row chunks that cross at most one block boundary, and
// tiles across block columns.  What the fourth field changes:
//
//  * Cell records take four float4 planes: pc | gy | gx | (tyy, txy, txx).
//    A y face reads planes 0, 1 and 3 of its two cells, an x face planes 0, 2
//    and 3 of the row above it (the row below is in registers).
//  * Each side of a face has its own sound speed sqrt(gamma p / rho).
//  * The viscous stress works on the energy flux with the face-average of
//    the two cell-centre velocities; the alpha model's nu of a cell is
//    K(face) gamma p (cell_visc_scale, stage2.cuh).
//  * Sources: gravity and its work, the buffer and the cooling of the
//    specific internal energy (beta or T^4 law, Mach ceiling) packed; the
//    cooling item carries rho de in the energy field only (see
//    source_terms, physics.cuh); sinks per column, in warps with a zone
//    inside a sink radius.
//  * The ledger's group 0 (gravity, buffer, cooling: 14 live items, 11 of
//    them non-zero in FP32) is summed per thread over the tile's rows and
//    over the warp once per ledger piece (at a crossing tile's first-piece
//    row and after the loop).
#pragma once

#include "stage3.cuh"

namespace b2d {

__host__ __device__ inline int s3e_smem_bytes(int tw)
{
    int slots = S3_SLOTS * s2_slot_bytes(4, 1, tw) + S3_USLOTS * s2_uslot_bytes(4, 1, tw);
    int exch = 16 * (2 * (tw + 4) + 4 * 2 * (tw + 4) + 2 * (tw + 2));
    return slots + exch + 8 * (S3_SLOTS + S3_USLOTS);
}

__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(__fdividef(1.0f, a.x), __fdividef(1.0f, a.y)); }
__device__ __forceinline__ float2 sqrt2(float2 a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }

// The floors and checks of Euler::try_to_primitive (physics.rs:631-660) on one
// zone's primitives: 0, 1 (negative density) or 2 (non-positive pressure).
__device__ __forceinline__ int euler_floors(const DevParamsF& P, float* p)
{
    if (P.has_density_floor && p[0] < P.density_floor) {
        p[0] = P.density_floor;
        p[1] = 0.0f;
        p[2] = 0.0f;
        p[3] = P.density_floor_pow_gamma;
    }
    if (p[0] < 0.0f) return 1;
    if (P.has_pressure_floor && p[3] < P.pressure_floor) p[3] = P.pressure_floor;
    if (p[3] <= 0.0f) return 2;
    return 0;
}

// Three-input FP32 minimum and maximum (PTX min/max with three sources, sm_100+).
__device__ __forceinline__ float min3f(float a, float b, float c)
{
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Generalised minmod of each lane (plm_gradient, physics.cuh) as the median of
// min(x, y, z), max(x, y, z) and 0: the minimum when all three are positive,
// the maximum when all are negative, else 0 — min(max(lo, 0), hi) for lo <= hi.
__device__ __forceinline__ float2 plm_gradient2m(float2 th, float2 a, float2 b, float2 c)
{
    const float2 x = mul2(th, sub2(b, a));
    const float2 y = mul2(f2(0.5f), sub2(c, a));
    const float2 z = mul2(th, sub2(c, b));
    return make_float2(fminf(fmaxf(min3f(x.x, y.x, z.x), 0.0f), max3f(x.x, y.x, z.x)),
                       fminf(fmaxf(min3f(x.y, y.y, z.y), 0.0f), max3f(x.y, y.y, z.y)));
}

// e^x - 1 of two small arguments (|x| <= 0.35): the Taylor series
// x (1 + x/2 + x^2/6 + ... + x^7/8!) in Horner form; the first omitted term,
// x^9/9!, is below 6e-10 |x| there.
__device__ __forceinline__ float2 expm1_small2(float2 x)
{
    float2 p = f2(1.0f / 40320.0f);
    p = fma2(p, x, f2(1.0f / 5040.0f));
    p = fma2(p, x, f2(1.0f / 720.0f));
    p = fma2(p, x, f2(1.0f / 120.0f));
    p = fma2(p, x, f2(1.0f / 24.0f));
    p = fma2(p, x, f2(1.0f / 6.0f));
    p = fma2(p, x, f2(0.5f));
    p = fma2(p, x, f2(1.0f));
    return mul2(p, x);
}

// Scalar FP32 pieces of the paired kernel written with explicit roundings
// (fmaf, __fmul_rn, __fadd_rn: no contraction left to the compiler), so that
// every instantiation of the kernel (tile widths 128, 256, 512) rounds them
// alike and the states stay independent of the tiling.

// Euler cons -> prim without floors (physics.rs:696): rho, vx, vy, p.
__device__ __forceinline__ void euler_prim_exact(const DevParamsF& P, const float* u, float* p)
{
    const float ir = __fdividef(1.0f, u[0]);
    p[0] = u[0];
    p[1] = __fmul_rn(u[1], ir);
    p[2] = __fmul_rn(u[2], ir);
    const float v2 = fmaf(p[1], p[1], __fmul_rn(p[2], p[2]));
    p[3] = __fmul_rn(fmaf(__fmul_rn(-0.5f, u[0]), v2, u[3]), P.gm1);
}

// Euler::max_signal_speed (physics.rs:679-681): max(|vx|, |vy|) + sqrt(gamma p / rho).
__device__ __forceinline__ float euler_max_speed_exact(const DevParamsF& P, const float* u)
{
    float p[4];
    euler_prim_exact(P, u, p);
    const float cs = sqrtf(__fmul_rn(__fmul_rn(P.gamma, p[3]), __fdividef(1.0f, p[0])));
    return __fadd_rn(fmaxf(fabsf(p[1]), fabsf(p[2])), cs);
}

// Physics::sink_kernel (physics.rs:388-397): rate (1 - r^2 / s^2)^2 inside the sink radius s.
__device__ __forceinline__ float sink_rate_exact(const DevParamsF& P, float dx, float dy)
{
    const float r2 = fmaf(dx, dx, __fmul_rn(dy, dy));
    if (r2 < P.sink_r2) {
        const float t = fmaf(-r2, P.inv_sink_r2, 1.0f);
        return __fmul_rn(P.sink_rate, __fmul_rn(t, t));
    }
    return 0.0f;
}

// The torque-free sink velocity: the gas velocity relative to the body,
// projected on the radial direction, plus the body's velocity (physics.rs:743-756).
__device__ __forceinline__ void torque_free_exact(const DevParamsF& P, const PointMass<float>& b, float x, float y,
                                                  float vx, float vy, float& vxc, float& vyc)
{
    const float vxb = P.one_body ? 0.0f : b.vx, vyb = P.one_body ? 0.0f : b.vy;
    const float ddx = x - b.x, ddy = y - b.y;
    const float r = sqrtf(fmaf(ddx, ddx, __fmul_rn(ddy, ddy)));
    const float rx = __fdividef(ddx, r), ry = __fdividef(ddy, r);
    const float dvdotr = fmaf(vx - vxb, rx, __fmul_rn(vy - vyb, ry));
    vxc = fmaf(dvdotr, rx, vxb);
    vyc = fmaf(dvdotr, ry, vyb);
}

// The sink items of one Euler zone (the sink part of Euler::source_terms,
// physics.rs:683-774): -rate u dt (impartial sinks) or -rate dt times the
// torque-free state (rho, rho v_sink, rho e + rho v_sink^2 / 2).
__device__ __forceinline__ void euler_sink_items(const DevParamsF& P, const Binary<float>& B, const float* u, float x,
                                                 float y, float dt, float* s1, float* s2)
{
    const float sr1 = __fmul_rn(sink_rate_exact(P, x - B.p1.x, y - B.p1.y), -dt);
    const float sr2 = __fmul_rn(sink_rate_exact(P, x - B.p2.x, y - B.p2.y), -dt);
    if (P.sink_model == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            s1[k] = __fmul_rn(u[k], sr1);
            s2[k] = __fmul_rn(u[k], sr2);
        }
    } else {
        float p[4];
        euler_prim_exact(P, u, p);
        const float e0 = __fmul_rn(__fdividef(p[3], p[0]), P.inv_gm1);
        float v1x, v1y, v2x, v2y;
        torque_free_exact(P, B.p1, x, y, p[1], p[2], v1x, v1y);
        torque_free_exact(P, B.p2, x, y, p[1], p[2], v2x, v2y);
        const float sd = p[0], hs = __fmul_rn(0.5f, sd);
        const float a1[4] = {sd, __fmul_rn(sd, v1x), __fmul_rn(sd, v1y),
                             fmaf(sd, e0, __fmul_rn(hs, fmaf(v1x, v1x, __fmul_rn(v1y, v1y))))};
        const float a2[4] = {sd, __fmul_rn(sd, v2x), __fmul_rn(sd, v2y),
                             fmaf(sd, e0, __fmul_rn(hs, fmaf(v2x, v2x, __fmul_rn(v2y, v2y))))};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            s1[k] = __fmul_rn(a1[k], sr1);
            s2[k] = __fmul_rn(a2[k], sr2);
        }
    }
}

// 0.5 K of the alpha model at two faces (x, fy.x) and (x, fy.y)
// (alpha_face_factor, stage2.cuh, without the isothermal cs2):
// K = alpha / sqrt(gamma - 1) / sqrt(sum m / a^3) with a the distance to each
// body.  1 / a^3 is taken as rsqrt(a^2)^3: the reference's a = |d| + 1e-12 dx
// (scheme.rs:244) differs from |d| below FP32 resolution unless |d| is
// under about 1e-7 dx, and at |d| = 0 both give K = 0 (1 / 0 = inf, rsqrt(inf) = 0).
__device__ __forceinline__ float2 alpha_half_k2(const DevParamsF& P, const Binary<float>& B, float x, float2 fy)
{
    const float dx1 = x - B.p1.x, dx2 = x - B.p2.x;
    const float2 dy1 = sub2(fy, f2(B.p1.y)), dy2 = sub2(fy, f2(B.p2.y));
    const float2 d1 = fma2(dy1, dy1, f2(dx1 * dx1)), d2 = fma2(dy2, dy2, f2(dx2 * dx2));
    const float2 q1 = make_float2(rsqrtf(d1.x), rsqrtf(d1.y)), q2 = make_float2(rsqrtf(d2.x), rsqrtf(d2.y));
    const float2 w2 = fma2(f2(B.p1.m), mul2(q1, mul2(q1, q1)), mul2(f2(B.p2.m), mul2(q2, mul2(q2, q2))));
    return mul2(f2(0.5f * P.nu * P.inv_sqrt_gm), make_float2(rsqrtf(w2.x), rsqrtf(w2.y)));
}

// Two Euler faces normal to AXIS (intercell_flux, physics.rs:776-803, with
// hydro-euler's HLLE and the factored stress of face_flux in stage2.cuh).
// pcl/gl/tnl/ttl: the faces' left cells (primitives, slopes along the
// normal, factored stresses), pcr/gr/tnr/ttr the right cells; (fx, fy.x)
// and (fx, fy.y) the faces' positions.
template <int AXIS>
__device__ __forceinline__ void euler_face_flux2(const DevParamsF& P, const Binary<float>& B, const float2* pcl,
                                                 const float2* gl, float2 tnl, float2 ttl, const float2* pcr,
                                                 const float2* gr, float2 tnr, float2 ttr, float fx, float2 fy,
                                                 float2* F)
{
    float2 pl[4], pr[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        pl[k] = fma2(gl[k], f2(0.5f), pcl[k]);
        pr[k] = fma2(gr[k], f2(-0.5f), pcr[k]);
    }
    // conserved states: rho v and the total energy rho v^2 / 2 + p / (gamma - 1)
    const float2 ul1 = mul2(pl[0], pl[1]), ul2 = mul2(pl[0], pl[2]);
    const float2 ur1 = mul2(pr[0], pr[1]), ur2 = mul2(pr[0], pr[2]);
    const float2 ul3 = fma2(mul2(f2(0.5f), pl[0]), fma2(pl[1], pl[1], mul2(pl[2], pl[2])), mul2(pl[3], f2(P.inv_gm1)));
    const float2 ur3 = fma2(mul2(f2(0.5f), pr[0]), fma2(pr[1], pr[1], mul2(pr[2], pr[2])), mul2(pr[3], f2(P.inv_gm1)));
    // sound speeds sqrt(gamma p / rho) of the two sides
    const float2 csl = sqrt2(mul2(mul2(f2(P.gamma), pl[3]), rcp2(pl[0])));
    const float2 csr = sqrt2(mul2(mul2(f2(P.gamma), pr[3]), rcp2(pr[0])));
    const float2 vl = AXIS == 0 ? pl[1] : pl[2];
    const float2 vr = AXIS == 0 ? pr[1] : pr[2];
    // physical fluxes
    const float2 fl0 = mul2(pl[0], vl), fr0 = mul2(pr[0], vr);
    const float2 fl1 = AXIS == 0 ? fma2(ul1, vl, pl[3]) : mul2(ul1, vl);
    const float2 fr1 = AXIS == 0 ? fma2(ur1, vr, pr[3]) : mul2(ur1, vr);
    const float2 fl2 = AXIS == 1 ? fma2(ul2, vl, pl[3]) : mul2(ul2, vl);
    const float2 fr2 = AXIS == 1 ? fma2(ur2, vr, pr[3]) : mul2(ur2, vr);
    const float2 fl3 = mul2(add2(ul3, pl[3]), vl), fr3 = mul2(add2(ur3, pr[3]), vr);
    // outer wave speeds
    const float2 alm = sub2(vl, csl), alp = add2(vl, csl), arm = sub2(vr, csr), arp = add2(vr, csr);
    const float2 ap = make_float2(fmaxf(0.0f, fmaxf(alp.x, arp.x)), fmaxf(0.0f, fmaxf(alp.y, arp.y)));
    const float2 am = make_float2(fminf(0.0f, fminf(alm.x, arm.x)), fminf(0.0f, fminf(alm.y, arm.y)));
    const float2 inv = rcp2(sub2(ap, am));
    const float2 nam = mul2(am, f2(-1.0f));
    const float2 apam = mul2(ap, am);
    // F = (fl ap - fr am - (ul - ur) ap am) / (ap - am)
    F[0] = mul2(fma2(sub2(pr[0], pl[0]), apam, fma2(fr0, nam, mul2(fl0, ap))), inv);
    F[1] = mul2(fma2(sub2(ur1, ul1), apam, fma2(fr1, nam, mul2(fl1, ap))), inv);
    F[2] = mul2(fma2(sub2(ur2, ul2), apam, fma2(fr2, nam, mul2(fl2, ap))), inv);
    F[3] = mul2(fma2(sub2(ur3, ul3), apam, fma2(fr3, nam, mul2(fl3, ap))), inv);
    // viscous stress and its work with the face-average cell-centre velocity
    const float2 k = P.visc != 0 ? alpha_half_k2(P, B, fx, fy) : f2(0.5f);
    const float2 tn = mul2(k, add2(tnl, tnr));
    const float2 tt = mul2(k, add2(ttl, ttr));
    const float2 taux = AXIS == 0 ? tn : tt, tauy = AXIS == 0 ? tt : tn;
    F[1] = sub2(F[1], taux);
    F[2] = sub2(F[2], tauy);
    const float2 vxa = mul2(f2(0.5f), add2(pcl[1], pcr[1])), vya = mul2(f2(0.5f), add2(pcl[2], pcr[2]));
    F[3] = sub2(F[3], fma2(taux, vxa, mul2(tauy, vya)));
}

template <bool SINGLE, int TWMAX>
__global__ void __launch_bounds__(TWMAX / 2 + 32, TWMAX == 128 ? 4 : (TWMAX == 256 ? 2 : 1))
stage3e_kernel(StageArgs a)
{
    constexpr int NF = 4;
    constexpr int H = 4;                     // staged halo columns per side: 16 bytes of FP32

    const int TP = blockDim.x - 32;          // interior threads (column pairs)
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
    // rows [i0, i0 + TH) of the column strip from j0: row chunk ti of C (as in stage3.cuh)
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
    // float4 planes of two rows each; column c at slot c + 2, the even columns
    // in the first half of the row and the odd ones in the second (stage3.cuh)
    float4* sP = (float4*)(uslots + S3_USLOTS * USLOT);       // [2][TW+4] primitives
    // cell records: R0 = pc | R1 = gy | R2 = gx | R3 = tyy, txy, txx
    float4* sR0 = sP + 2 * (TW + 4);
    float4* sR1 = sR0 + 2 * (TW + 4);
    float4* sR2 = sR1 + 2 * (TW + 4);
    float4* sR3 = sR2 + 2 * (TW + 4);
    float4* sF = sR3 + 2 * (TW + 4);                          // [2][TW+2] y-face fluxes
    uint64_t* bars = (uint64_t*)(sF + 2 * (TW + 2));          // [S3_SLOTS] stencil ring
    uint64_t* ubars = bars + S3_SLOTS;                        // [S3_USLOTS] update ring

    // ---- roles -----------------------------------------------------------------
    const bool interior = t < TP;
    const int hl = t - TP;                                    // lane in the halo warp
    const bool active = interior || (hl >= 0 && hl < 2);
    const int c0 = interior ? 2 * t : (hl == 0 ? -2 : TW);   // first column of this thread's pair
    const bool producer = (hl == 4);
    const int p = c0 >> 1;                                   // the pair's slot in a half row (-1 for the -2 pair)
    const int HR = TW / 2 + 2, HF = TW / 2 + 1;              // odd halves of the record and flux rows

    auto plane = [&](const float* base, int f, int part) -> const float* { return base + (size_t)(2 * f + part) * nn; };
    auto copy_row = [&](unsigned char* dst, const float* row, int w_halo, uint64_t* bar) {
        if (w_halo == 0) {
            bulk_load(dst, row + j0, TW * sizeof(float), bar);
        } else if (j0 >= H && j0 + TW + H <= N) {
            bulk_load(dst, row + j0 - H, SW * sizeof(float), bar);
        } else if (j0 == 0 && TW + H <= N) {   // the mesh's left edge: the left halo wraps to the row's end
            bulk_load(dst, row + N - H, H * sizeof(float), bar);
            bulk_load(dst + H * sizeof(float), row, (TW + H) * sizeof(float), bar);
        } else if (j0 >= H) {                  // the right edge (j0 + TW = N): the right halo wraps to column 0
            bulk_load(dst, row + j0 - H, (TW + H) * sizeof(float), bar);
            bulk_load(dst + (TW + H) * sizeof(float), row, H * sizeof(float), bar);
        } else {                               // one strip spans the row: both halos wrap
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
    // the T^4 law's slow-start factor exp(-2 pi / (t + dt)) of this stage (physics.rs:683-774)
    const float slow = P.cooling_slow_start ? __expf(-6.283185307f / (time + dt)) : 1.0f;
    // positions: zone centres (y) of the pair, y of the pair's left faces
    const float2 yc2 = interior ? make_float2(xc[j0 + c0], xc[j0 + c0 + 1]) : f2(0.0f);
    const float2 yv2 = (interior || hl == 1) ? make_float2(rd.xvgf[j0 + c0], rd.xvgf[j0 + min(c0 + 1, TW)]) : f2(0.0f);
    const float* xv_row = rd.xvgf + i0;
    const float* xc_row = xc + i0;

    float2 Pm1[NF], P0[NF];           // primitives of rows rg-1, rg (own pair)
    float2 fxA[NF], fxB[NF];          // x fluxes at faces ru-1/2, ru+1/2
    float2 xg[NF], xtn = f2(0.0f), xtt = f2(0.0f);   // row rg's x slopes and stresses, for this row's x faces
    constexpr int NLIVE = live_items<NF>();
    static_assert(group_size<NF, 0>() + group_size<NF, 1>() + group_size<NF, 2>() == NLIVE, "ledger groups");
    static_assert(group_size<NF, 0>() == 14 && group_size<NF, 1>() == 8 && group_size<NF, 2>() == 0, "Euler groups");
    constexpr int NWI = TWMAX / 64 < 4 ? 4 : TWMAX / 64;   // bank rows: interior warps
    __shared__ float sLed[NWI][32], sLedA[NWI][32];          // [warp][item slot]: main piece, a crossing tile's first
    const int lane = t & 31, warp = t >> 5;
    for (int i = t; i < NWI * 32; i += blockDim.x) sLed[i >> 5][i & 31] = sLedA[i >> 5][i & 31] = 0.0f;
    const int slot0 = group_writer_slot<NF, 0>(lane);
    const int slot1 = group_writer_slot<NF, 1>(lane);
    // group 0 of this pair summed over rows: grav1 (x, y, e), grav2 (x, y, e),
    // buffer (4 fields), cooling (energy; its mass and momentum are zero)
    float acc0[11];
#pragma unroll
    for (int m = 0; m < 11; ++m) acc0[m] = 0.0f;
    // the warp's total of acc0 into a bank row, in item order, and a fresh start
    auto flush_acc = [&](float* bank) {
        float v[16];
#pragma unroll
        for (int m = 0; m < 10; ++m) v[m] = acc0[m];
        v[10] = v[11] = v[12] = 0.0f;
        v[13] = acc0[10];
        v[14] = v[15] = 0.0f;
        const float s0 = warp_sum_items<16>(v, lane);
        if (slot0 >= 0) bank[slot0] += s0;
#pragma unroll
        for (int m = 0; m < 11; ++m) acc0[m] = 0.0f;
    };
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

        // ---- phase 1: row rn -> primitives (try_block_primitive, scheme.rs:185-199) --
        float2 pn[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) pn[f] = f2(0.0f);
        if (rn <= TH + 1 && active) {
            const int rr = rn + 2;
            if (!mbar_wait_bounded(bars + rr % S3_SLOTS, (rr / S3_SLOTS) & 1)) timeout = 1;
            const float* sb = (const float*)(slots + (rr % S3_SLOTS) * SLOT);
            float2 u[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) u[f] = *(const float2*)(sb + f * SW + c0 + H);
            // the conversion packed, the floors and checks per zone
            const float2 ir = rcp2(u[0]);
            const float2 vx = mul2(u[1], ir), vy = mul2(u[2], ir);
            const float2 ps = mul2(sub2(u[3], mul2(mul2(f2(0.5f), u[0]), fma2(vx, vx, mul2(vy, vy)))), f2(P.gm1));
            float pa[NF] = {u[0].x, vx.x, vy.x, ps.x}, pb[NF] = {u[0].y, vx.y, vy.y, ps.y};
            const int ea = euler_floors(P, pa);
            const int eb = euler_floors(P, pb);
            if ((ea || eb) && interior && rn >= 0 && rn < TH) {
                const int gi = i0 + rn;
                if (ea) atomicMin(a.err_key, error_key(a.stage, ri, rd, gi, j0 + c0, ea));
                if (eb) atomicMin(a.err_key, error_key(a.stage, ri, rd, gi, j0 + c0 + 1, eb));
            }
#pragma unroll
            for (int f = 0; f < NF; ++f) pn[f] = make_float2(pa[f], pb[f]);
            float4* row = sP + (rn & 1) * (TW + 4) + p + 1;
            row[0] = make_float4(pa[0], pa[1], pa[2], pa[3]);
            row[HR] = make_float4(pb[0], pb[1], pb[2], pb[3]);
        }

        // ---- phase 2: slopes and cell records of row rg = rn - 1 (scheme.rs:216-254) ---
        const int rg = rn - 1;
        if (rg >= -1 && rg <= TH && active) {
            const float4* prow = sP + (rg & 1) * (TW + 4);
            const float4 l4 = prow[HR + p];                    // column c0 - 1 (in the row, unused, for the -2 pair)
            const float4 r4 = prow[p + 2];                     // column c0 + 2 (in the row, unused, for the TW pair)
            float lv[4] = {l4.x, l4.y, l4.z, l4.w}, rv[4] = {r4.x, r4.y, r4.z, r4.w};
            // the two stencil points outside the staged columns: NaN in a
            // read-set check build (tma.cuh), whose states must not change
            if (hl == 0)
                for (int f = 0; f < 4; ++f) lv[f] = poison_or(lv[f]);
            if (hl == 1)
                for (int f = 0; f < 4; ++f) rv[f] = poison_or(rv[f]);
            const float2 thx = make_float2((Pm1[0].x < pdt || P0[0].x < pdt || pn[0].x < pdt) ? 0.0f : theta,
                                           (Pm1[0].y < pdt || P0[0].y < pdt || pn[0].y < pdt) ? 0.0f : theta);
            const float2 thy = make_float2((lv[0] < pdt || P0[0].x < pdt || P0[0].y < pdt) ? 0.0f : theta,
                                           (P0[0].x < pdt || P0[0].y < pdt || rv[0] < pdt) ? 0.0f : theta);
            float2 gx[NF], gy[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                gx[f] = plm_gradient2m(thx, Pm1[f], P0[f], pn[f]);
                gy[f] = plm_gradient2m(thy, make_float2(lv[f], P0[f].x), P0[f], make_float2(P0[f].y, rv[f]));
            }
            // factored stress_field terms (physics.rs:322-340; face_flux, stage2.cuh)
            const float2 da = mul2(gx[1], f2(inv_dx)), db = mul2(gy[2], f2(inv_dx));
            const float2 lb = mul2(f2(P.lambda), add2(da, db));
            const float2 cv = P.visc == 0 ? mul2(f2(P.nu), P0[0]) : mul2(f2(P.gamma), P0[3]);
            const float2 txx = mul2(cv, fma2(f2(4.0f / 3.0f), da, fma2(f2(-2.0f / 3.0f), db, lb)));
            const float2 tyy = mul2(cv, fma2(f2(4.0f / 3.0f), db, fma2(f2(-2.0f / 3.0f), da, lb)));
            const float2 txy = mul2(cv, mul2(add2(gx[2], gy[1]), f2(inv_dx)));
            // cell records of both columns
            const int o = (rg & 1) * (TW + 4) + p + 1;
            sR0[o] = make_float4(P0[0].x, P0[1].x, P0[2].x, P0[3].x);
            sR1[o] = make_float4(gy[0].x, gy[1].x, gy[2].x, gy[3].x);
            sR2[o] = make_float4(gx[0].x, gx[1].x, gx[2].x, gx[3].x);
            sR3[o] = make_float4(tyy.x, txy.x, txx.x, 0.0f);
            sR0[o + HR] = make_float4(P0[0].y, P0[1].y, P0[2].y, P0[3].y);
            sR1[o + HR] = make_float4(gy[0].y, gy[1].y, gy[2].y, gy[3].y);
            sR2[o + HR] = make_float4(gx[0].y, gx[1].y, gx[2].y, gx[3].y);
            sR3[o + HR] = make_float4(tyy.y, txy.y, txx.y, 0.0f);
#ifdef B2D_POISON
            // the records of the outer guard columns -2 and TW + 1, which no face reads
            const float4 nan4 = make_float4(poison_or(0.0f), poison_or(0.0f), poison_or(0.0f), poison_or(0.0f));
            if (hl == 0) sR0[o] = sR1[o] = sR2[o] = sR3[o] = nan4;
            if (hl == 1) sR0[o + HR] = sR1[o + HR] = sR2[o + HR] = sR3[o + HR] = nan4;
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
            const float4 a0 = sR0[ob + HR], a1 = sR1[ob + HR], a3 = sR3[ob + HR];
            const float4 b0 = sR0[ob + 1], b1 = sR1[ob + 1], b3 = sR3[ob + 1];
            const float4 d0 = sR0[ob + HR + 1], d1 = sR1[ob + HR + 1], d3 = sR3[ob + HR + 1];
            const float2 pcl[4] = {make_float2(a0.x, b0.x), make_float2(a0.y, b0.y), make_float2(a0.z, b0.z),
                                   make_float2(a0.w, b0.w)};
            const float2 gl[4] = {make_float2(a1.x, b1.x), make_float2(a1.y, b1.y), make_float2(a1.z, b1.z),
                                  make_float2(a1.w, b1.w)};
            const float2 pcr[4] = {make_float2(b0.x, d0.x), make_float2(b0.y, d0.y), make_float2(b0.z, d0.z),
                                   make_float2(b0.w, d0.w)};
            const float2 gr[4] = {make_float2(b1.x, d1.x), make_float2(b1.y, d1.y), make_float2(b1.z, d1.z),
                                  make_float2(b1.w, d1.w)};
            const float x = xq;
            float2 F[NF];
            euler_face_flux2<1>(P, B, pcl, gl, make_float2(a3.x, b3.x), make_float2(a3.y, b3.y), pcr, gr,
                                make_float2(b3.x, d3.x), make_float2(b3.y, d3.y), x, yv2, F);
            if (fy_ok) {
                float4* fo = sF + (rq & 1) * (TW + 2) + p;
                fo[0] = make_float4(F[0].x, F[1].x, F[2].x, F[3].x);
                fo[HF] = make_float4(F[0].y, F[1].y, F[2].y, F[3].y);
#ifdef B2D_POISON
                if (hl == 1) fo[HF] = make_float4(poison_or(0.0f), poison_or(0.0f), poison_or(0.0f), poison_or(0.0f));
#endif
            }
        };
        float2 fxn[NF];
        if ((interior && rn >= 1) || (hl == 1 && fy_ok)) y_flux();
        if (interior && rn >= 1) {

            // update of row ru
            {
                const int rc = min(max(ru, 0), TH - 1);
                const float* sb = (const float*)(slots + ((rc + 2) % S3_SLOTS) * SLOT);
                const float4* frow = sF + (ru & 1) * (TW + 2) + p;   // faces c0, c0 + 1, c0 + 2
                const float4 fa = frow[0], fb = frow[HF], fc = frow[1];
                const float2 fyl[4] = {make_float2(fa.x, fb.x), make_float2(fa.y, fb.y), make_float2(fa.z, fb.z),
                                       make_float2(fa.w, fb.w)};
                const float2 fyr[4] = {make_float2(fb.x, fc.x), make_float2(fb.y, fc.y), make_float2(fb.z, fc.z),
                                       make_float2(fb.w, fc.w)};
                const float x = xu;
                if (up_ok && !mbar_wait_bounded(ubars + rc % S3_USLOTS, (rc / S3_USLOTS) & 1)) timeout = 1;
                const float* q = (const float*)(uslots + (rc % S3_USLOTS) * USLOT);
                float2 uc[NF], u0[NF];
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    uc[f] = *(const float2*)(sb + f * SW + c0 + H);
                    u0[f] = *(const float2*)(q + (NF + f) * TW + c0);
                }
                // sources of the pair (Physics::source_terms, physics.rs:423-457;
                // Euler::source_terms, physics.rs:683-774)
                float2 tot[NF];
                float v0[11];                 // ledger group 0 of the pair (acc0's order)
                bool sinks_any;
                float led1[8];
                {
                    const float dx1 = x - B.p1.x, dx2 = x - B.p2.x;
                    const float2 dy1 = sub2(yc2, f2(B.p1.y)), dy2 = sub2(yc2, f2(B.p2.y));
                    // Plummer accelerations: -m d / (d^2 + s^2)^(3/2)
                    const float2 t1 = fma2(dy1, dy1, f2(fmaf(dx1, dx1, P.soft2)));
                    const float2 t2 = fma2(dy2, dy2, f2(fmaf(dx2, dx2, P.soft2)));
                    const float2 r1 = make_float2(rsqrtf(t1.x), rsqrtf(t1.y));
                    const float2 r2 = make_float2(rsqrtf(t2.x), rsqrtf(t2.y));
                    const float2 r13 = mul2(r1, mul2(r1, r1)), r23 = mul2(r2, mul2(r2, r2));
                    // primitive velocities and specific internal energy (no floors, physics.rs:696)
                    const float2 ir = rcp2(uc[0]);
                    const float2 vx = mul2(uc[1], ir), vy = mul2(uc[2], ir);
                    const float2 v2 = fma2(vx, vx, mul2(vy, vy));
                    const float2 e0 = mul2(sub2(uc[3], mul2(mul2(f2(0.5f), uc[0]), v2)), ir);
                    // gravity and its work
                    const float2 sdt = mul2(uc[0], f2(dt));
                    const float2 q1 = mul2(mul2(sdt, f2(-B.p1.m)), r13);
                    const float2 q2 = mul2(mul2(sdt, f2(-B.p2.m)), r23);
                    const float2 g1x = mul2(q1, f2(dx1)), g1y = mul2(q1, dy1);
                    const float2 g2x = mul2(q2, f2(dx2)), g2y = mul2(q2, dy2);
                    const float2 g1e = fma2(g1x, vx, mul2(g1y, vy)), g2e = fma2(g2x, vx, mul2(g2y, vy));
                    // buffer: 0.5 rate (1 + tanh((r - R) / scale)) Omega_outer, 1 + tanh(y) = 2 / (1 + exp(-2y))
                    const float2 rr2 = fma2(yc2, yc2, f2(x * x));
                    const float2 yb = mul2(sub2(sqrt2(rr2), f2(P.domain_radius)), f2(-2.0f * P.inv_buffer_scale));
                    const float2 den = add2(f2(1.0f), make_float2(__expf(yb.x), __expf(yb.y)));
                    const float2 kb = mul2(f2(-2.0f * dt * P.half_rate_omega), rcp2(den));
                    float2 bu[NF];
#pragma unroll
                    for (int f = 0; f < NF; ++f) bu[f] = mul2(sub2(uc[f], u0[f]), kb);
                    // cooling of the specific internal energy, de = e_cooled - e0 formed
                    // directly (expm1 / log1p; see source_terms, physics.cuh)
                    float2 dec;
                    if (P.cooling_kind == 1) {
                        // beta-cooling: e -> e exp(-Omega dt / beta), Omega^2 = sum m / (d^2 + s^2)^(3/2)
                        const float2 om = sqrt2(fma2(f2(B.p1.m), r13, mul2(f2(B.p2.m), r23)));
                        const float2 c = mul2(om, f2(-dt * P.inv_cool_beta));
                        if (__any_sync(0xffffffffu, fabsf(c.x) > 0.35f || fabsf(c.y) > 0.35f))
                            dec = mul2(e0, make_float2(expm1f(c.x), expm1f(c.y)));
                        else
                            dec = mul2(e0, expm1_small2(c));
                    } else {
                        // T^4 law: e -> e (1 + 3 a e^3 dt)^(-1/3), a = coefficient / rho^n x slow start
                        float d2[2];
#pragma unroll
                        for (int s = 0; s < 2; ++s) {
                            const float rho = s ? uc[0].y : uc[0].x, e = s ? e0.y : e0.x;
                            float rho_n = 1.0f;
                            for (int m = 0; m < P.density_index; ++m) rho_n *= rho;
                            const float ac = __fdividef(P.cool_coef, rho_n) * slow;
                            d2[s] = e * expm1f(log1pf(3.0f * ac * (e * e * e) * dt) * (-1.0f / 3.0f));
                        }
                        dec = make_float2(d2[0], d2[1]);
                    }
                    if (P.has_mach_ceiling) {
                        // e >= 2 e_kinetic / (gamma (gamma - 1) M^2)
                        const float2 ek = mul2(f2(0.5f * P.k_mach_ceiling), v2);
                        const float eca = e0.x + dec.x, ecb = e0.y + dec.y;
                        const float ma = fmaxf(eca, ek.x), mb = fmaxf(ecb, ek.y);
                        if (ma != eca) dec.x = ma - e0.x;
                        if (mb != ecb) dec.y = mb - e0.y;
                    }
                    const float2 cool = mul2(uc[0], dec);
                    tot[0] = bu[0];
                    tot[1] = add2(add2(g1x, g2x), bu[1]);
                    tot[2] = add2(add2(g1y, g2y), bu[2]);
                    tot[3] = add2(add2(add2(g1e, g2e), bu[3]), cool);
                    v0[0] = g1x.x + g1x.y; v0[1] = g1y.x + g1y.y; v0[2] = g1e.x + g1e.y;
                    v0[3] = g2x.x + g2x.y; v0[4] = g2y.x + g2y.y; v0[5] = g2e.x + g2e.y;
#pragma unroll
                    for (int f = 0; f < NF; ++f) v0[6 + f] = bu[f].x + bu[f].y;
                    v0[10] = cool.x + cool.y;
#pragma unroll
                    for (int m = 0; m < 8; ++m) led1[m] = 0.0f;
                    // sinks: only where a zone of the warp lies inside a sink radius
                    const float2 s1 = fma2(dy1, dy1, f2(dx1 * dx1)), s2 = fma2(dy2, dy2, f2(dx2 * dx2));
                    const bool near = s1.x < P.sink_r2 || s1.y < P.sink_r2 || s2.x < P.sink_r2 || s2.y < P.sink_r2;
                    sinks_any = __any_sync(0xffffffffu, near);
                    if (sinks_any) {
#pragma unroll 1
                        for (int side = 0; side < 2; ++side) {
                            const float us[NF] = {side ? uc[0].y : uc[0].x, side ? uc[1].y : uc[1].x,
                                                  side ? uc[2].y : uc[2].x, side ? uc[3].y : uc[3].x};
                            float sk1[NF], sk2[NF];
                            euler_sink_items(P, B, us, x, side ? yc2.y : yc2.x, dt, sk1, sk2);
#pragma unroll
                            for (int f = 0; f < NF; ++f) {
                                const float sk = sk1[f] + sk2[f];
                                if (side) tot[f].y += sk;
                                else tot[f].x += sk;
                                led1[f] += sk1[f];
                                led1[NF + f] += sk2[f];
                            }
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
                    const float2 ulo = *(const float2*)(q + f * TW + c0);
                    df2 o = df_add_f2(df2{uc[f], ulo}, inc);
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
#pragma unroll
                    for (int m = 0; m < 11; ++m) acc0[m] += v0[m];
                    if (sinks_any) {
                        const float s1 = warp_sum_items<8>(led1, lane);
                        if (slot1 >= 0) sLed[warp][slot1] += s1;
                    }
                    if (ru == rb - 1 && rb < TH) {   // the first piece's last row: set its sums aside
                        __syncwarp();
                        sLedA[warp][lane] = sLed[warp][lane];
                        sLed[warp][lane] = 0.0f;
                        __syncwarp();
                        flush_acc(sLedA[warp]);
                    }
                }
                if (want_amax && up_ok) {
                    const float ua[NF] = {uo[0].x, uo[1].x, uo[2].x, uo[3].x};
                    const float ub[NF] = {uo[0].y, uo[1].y, uo[2].y, uo[3].y};
                    amax = fmaxf(fmaxf(euler_max_speed_exact(P, ua), euler_max_speed_exact(P, ub)), amax);
                }
            }

            // x fluxes of faces rq + 1/2 below the pair: row rq's records from shared
            // memory, row rq + 1 = rg's from this iteration's registers (primitives
            // in Pm1 after the rotation)
            {
                const int oa = (rq & 1) * (TW + 4) + p + 1;
                const float4 a0 = sR0[oa], a2 = sR2[oa], a3 = sR3[oa];
                const float4 e0 = sR0[oa + HR], e2 = sR2[oa + HR], e3 = sR3[oa + HR];
                const float2 pcl[4] = {make_float2(a0.x, e0.x), make_float2(a0.y, e0.y), make_float2(a0.z, e0.z),
                                       make_float2(a0.w, e0.w)};
                const float2 gl[4] = {make_float2(a2.x, e2.x), make_float2(a2.y, e2.y), make_float2(a2.z, e2.z),
                                      make_float2(a2.w, e2.w)};
                const float x = xvq;
                euler_face_flux2<0>(P, B, pcl, gl, make_float2(a3.z, e3.z), make_float2(a3.y, e3.y), Pm1, xg, xtn,
                                    xtt, x, yc2, fxn);
            }
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

    // ---- ledger pieces, one per block under the tile, each flushed by its own warp --
    if (interior) flush_acc(sLed[warp]);   // whole warps: the main piece's group 0
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
            flush_piece<NF>(rd, brow - 1, bcol + c, lslot, TW, sLedA + c * wpc, wpc, nullptr, 0, a.in_slot,
                            a.base_slot, a.out_slot, a.stage, a.bf);
    }
}

}  // namespace b2d
