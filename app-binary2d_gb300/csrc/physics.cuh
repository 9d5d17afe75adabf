// physics.cuh — per-zone and per-face physics of binary2d's finite-volume
// step, as device functions templated on the stencil arithmetic R.
//
// R = double: the parity path.  Every expression is evaluated in the order
// of the reference's Rust source (this translation unit is compiled with
// --fmad=false), so the FP64 kernel reproduces the CPU restatement bit for
// bit apart from the last-ulp differences of tanh / sin / cos / pow / exp.
// R = float: the mixed-precision path.  Same formulas, reassociated for
// throughput (reciprocals, rsqrt, fused multiply-add), intrinsics for
// division and square roots.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>

namespace b2d {

enum { SINK1 = 0, SINK2, GRAV1, GRAV2, BUFFER, COOLING, FAKE_MASS, NITEMS };

// Physics parameters in device form, built on the host from b2d_config.
// DevParamsT<double> serves the FP64 kernels, DevParamsT<float> the FP32
// kernels (no double arithmetic or conversion in their inner loops).
template <class T> struct DevParamsT {
    int hydro;            // 0 iso, 1 euler
    int visc;             // 0 constant nu, 1 alpha
    int sink_model;       // 0 impartial, 1 torque-free
    int one_body;
    int has_mach_ceiling, has_density_floor, has_pressure_floor, density_index;
    int cooling_kind, cooling_slow_start, has_dt_min, pad_;
    T dx, inv_dx;
    T cfl, dt_min;
    T plm, pdt;                       // θ and the PLM density trigger (0 if unset)
    T nu;                             // ν or α
    T lambda;                         // lambda_multiplier
    T mach2, inv_mach2;               // mach_number² (iso)
    T gamma, gm1, inv_gm1;            // γ, γ - 1 (euler; iso γ = 1)
    T sqrt_gm, inv_sqrt_gm;           // sqrt(γ) for α viscosity
    T soft2;                          // softening_length²
    T sink_r2, inv_sink_r2, sink_rate;
    T domain_radius, buffer_scale, inv_buffer_scale, half_buffer_rate, omega_outer, half_rate_omega;
    T fake_thr, fake_rate;
    T density_floor, pressure_floor, density_floor_pow_gamma;
    T mach_ceiling2;                  // mach_ceiling²
    T k_mach_ceiling;                 // 2 / (γ (γ - 1) mach_ceiling²)
    T cool_coef, cool_beta, inv_cool_beta;
    T eps_dx;                         // 1e-12 · dx (α viscosity)
};
using DevParams = DevParamsT<double>;
using DevParamsF = DevParamsT<float>;

template <class R> struct PointMass { R m, x, y, vx, vy; };
template <class R> struct Binary { PointMass<R> p1, p2; };

template <class R> __device__ __forceinline__ bool is_f64() { return std::is_same<R, double>::value; }

// a / b: IEEE division in FP64, fast reciprocal division in FP32.
template <class R> __device__ __forceinline__ R dvd(R a, R b)
{
    if constexpr (std::is_same<R, double>::value) return a / b;
    else return __fdividef(a, b);
}

template <class R> __device__ __forceinline__ R rmax(R a, R b) { return fmax(a, b); }
template <> __device__ __forceinline__ float rmax<float>(float a, float b) { return fmaxf(a, b); }
template <class R> __device__ __forceinline__ R rmin(R a, R b) { return fmin(a, b); }
template <> __device__ __forceinline__ float rmin<float>(float a, float b) { return fminf(a, b); }
template <class R> __device__ __forceinline__ R rabs(R a) { return fabs(a); }
template <> __device__ __forceinline__ float rabs<float>(float a) { return fabsf(a); }
template <class R> __device__ __forceinline__ R rsqrt_(R a) { return sqrt(a); }
template <> __device__ __forceinline__ float rsqrt_<float>(float a) { return sqrtf(a); }

// ---------------------------------------------------------------------------
// godunov-core piecewise_linear::plm_gradient (restated): generalised minmod
// of θ(b - a), (c - a)/2, θ(c - b) — the smallest magnitude when all three
// share a sign, else zero.  Written as max(min(x, y, z), 0) + min(max(x, y, z), 0):
// with all three positive the first term is the minimum and the second 0,
// with all negative the first is 0 and the second the maximum (the value of
// smallest magnitude), with mixed signs (or a zero) both are 0.  min and max
// round nothing, so this is the same value as the sign-test form, in four
// min/max and one add instead of six compares and two selects.
template <class R> __device__ __forceinline__ R plm_gradient(R th, R a, R b, R c)
{
    R x = th * (b - a);
    R y = R(0.5) * (c - a);
    R z = th * (c - b);
    return rmax(rmin(rmin(x, y), z), R(0)) + rmin(rmax(rmax(x, y), z), R(0));
}

// ---------------------------------------------------------------------------
// Plummer potential and acceleration of a point mass (kepler-two-body,
// restated; acceleration form of tools/indep_res_analysis.py:182-194).
template <class R> __device__ __forceinline__ R point_potential(const PointMass<R>& p, R x, R y, R s2)
{
    R dx = x - p.x, dy = y - p.y;
    R r2 = dx * dx + dy * dy;
    if constexpr (std::is_same<R, double>::value) return -p.m / sqrt(r2 + s2);
    else return -p.m * rsqrtf(r2 + s2);
}

template <class R>
__device__ __forceinline__ void point_acceleration(const PointMass<R>& p, R x, R y, R s2, R& ax, R& ay)
{
    R dx = x - p.x, dy = y - p.y;
    R t2 = dx * dx + dy * dy + s2;
    if constexpr (std::is_same<R, double>::value) {
        double d3 = t2 * sqrt(t2);
        ax = -p.m * dx / d3;
        ay = -p.m * dy / d3;
    } else {
        float r = rsqrtf(t2);
        float k = -p.m * (r * r * r);
        ax = k * dx;
        ay = k * dy;
    }
}

template <class R> __device__ __forceinline__ R binary_potential(const Binary<R>& b, R x, R y, R s2)
{
    return point_potential(b.p1, x, y, s2) + point_potential(b.p2, x, y, s2);
}

// ---------------------------------------------------------------------------
// Conserved <-> primitive (hydro-iso2d / hydro-euler, restated).
template <int NF, class R> __device__ __forceinline__ void prim_to_cons(const DevParamsT<R>& P, const R* p, R* u)
{
    u[0] = p[0];
    u[1] = p[0] * p[1];
    u[2] = p[0] * p[2];
    if constexpr (NF == 4) {
        if constexpr (std::is_same<R, double>::value)
            u[3] = 0.5 * p[0] * (p[1] * p[1] + p[2] * p[2]) + p[3] / P.gm1;
        else
            u[3] = 0.5f * p[0] * (p[1] * p[1] + p[2] * p[2]) + p[3] * P.inv_gm1;
    }
}

template <int NF, class R> __device__ __forceinline__ void cons_to_prim_raw(const DevParamsT<R>& P, const R* u, R* p)
{
    p[0] = u[0];
    if constexpr (std::is_same<R, double>::value) {
        p[1] = u[1] / u[0];
        p[2] = u[2] / u[0];
        if constexpr (NF == 4) p[3] = (u[3] - 0.5 * u[0] * (p[1] * p[1] + p[2] * p[2])) * P.gm1;
    } else {
        float ir = __fdividef(1.0f, u[0]);
        p[1] = u[1] * ir;
        p[2] = u[2] * ir;
        if constexpr (NF == 4) p[3] = (u[3] - 0.5f * u[0] * (p[1] * p[1] + p[2] * p[2])) * P.gm1;
    }
}

// Hydrodynamics::try_to_primitive (physics.rs:489-503 iso, 631-660 euler).
// Returns 0, 1 (negative density) or 2 (negative pressure).
template <int NF, class R>
__device__ __forceinline__ int try_to_primitive(const DevParamsT<R>& P, const R* u_in, R* p, R& bad)
{
    if constexpr (NF == 3) {
        R u[3] = {u_in[0], u_in[1], u_in[2]};
        if (P.has_density_floor && u[0] < R(P.density_floor)) {
            u[1] = R(0);
            u[2] = R(0);
            u[0] = R(P.density_floor);
        }
        cons_to_prim_raw<3, R>(P, u, p);
        if (u[0] < R(0)) { bad = u[0]; return 1; }
        return 0;
    } else {
        cons_to_prim_raw<4, R>(P, u_in, p);
        if (P.has_density_floor && p[0] < R(P.density_floor)) {
            p[0] = R(P.density_floor);
            p[1] = R(0);
            p[2] = R(0);
            p[3] = R(P.density_floor_pow_gamma);
        }
        if (p[0] < R(0)) { bad = p[0]; return 1; }
        if (P.has_pressure_floor && p[3] < R(P.pressure_floor)) p[3] = R(P.pressure_floor);
        if (!(p[3] > R(0))) { if (p[3] <= R(0)) { bad = p[3]; return 2; } }
        return 0;
    }
}

// Hydrodynamics::max_signal_speed (physics.rs:521-526 iso; 679-681 euler).
template <int NF, class R> __device__ __forceinline__ R max_signal_speed(const DevParamsT<R>& P, const R* u)
{
    R p[NF];
    cons_to_prim_raw<NF, R>(P, u, p);
    R v = rmax(rabs(p[1]), rabs(p[2]));
    if constexpr (NF == 4) {
        R cs = rsqrt_(R(P.gamma) * p[3] / p[0]);
        return v + cs;
    }
    return v;
}

// ---------------------------------------------------------------------------
// HLLE (hydro-iso2d / hydro-euler riemann_hlle, restated).
template <int NF, class R>
__device__ __forceinline__ void physical_flux(const R* p, const R* u, int axis, R pg, R* f)
{
    R vn = axis == 0 ? p[1] : p[2];
    f[0] = u[0] * vn;
    f[1] = u[1] * vn + (axis == 0 ? pg : R(0));
    f[2] = u[2] * vn + (axis == 1 ? pg : R(0));
    if constexpr (NF == 4) f[3] = (u[3] + pg) * vn;
}

template <int NF, class R>
__device__ __forceinline__ void hlle(const DevParamsT<R>& P, const R* pl, const R* pr, int axis, R cs2, R* F)
{
    R ul[NF], ur[NF], fl[NF], fr[NF];
    prim_to_cons<NF, R>(P, pl, ul);
    prim_to_cons<NF, R>(P, pr, ur);
    R csl, csr, pgl, pgr;
    if constexpr (NF == 3) {
        csl = rsqrt_(cs2);
        csr = csl;
        pgl = pl[0] * cs2;
        pgr = pr[0] * cs2;
    } else {
        csl = rsqrt_(R(P.gamma) * pl[3] / pl[0]);
        csr = rsqrt_(R(P.gamma) * pr[3] / pr[0]);
        pgl = pl[3];
        pgr = pr[3];
    }
    physical_flux<NF, R>(pl, ul, axis, pgl, fl);
    physical_flux<NF, R>(pr, ur, axis, pgr, fr);
    R vl = axis == 0 ? pl[1] : pl[2];
    R vr = axis == 0 ? pr[1] : pr[2];
    R alm = vl - csl, alp = vl + csl;
    R arm = vr - csr, arp = vr + csr;
    R ap = rmax(R(0), rmax(alp, arp));
    R am = rmin(R(0), rmin(alm, arm));
    if constexpr (std::is_same<R, double>::value) {
#pragma unroll
        for (int k = 0; k < NF; ++k) F[k] = (fl[k] * ap - fr[k] * am - (ul[k] - ur[k]) * ap * am) / (ap - am);
    } else {
        float inv = __fdividef(1.0f, ap - am);
        float apam = ap * am;
#pragma unroll
        for (int k = 0; k < NF; ++k) F[k] = (fl[k] * ap - fr[k] * am - (ul[k] - ur[k]) * apam) * inv;
    }
}

// ---------------------------------------------------------------------------
// Cell record: what a face flux needs from one cell (CellData, physics.rs:77-82,
// plus the velocity-gradient combinations of stress_field, physics.rs:322-340).
template <int NF> struct CellLayout {
    static constexpr int PC = 0, GX = NF, GY = 2 * NF, SXX = 3 * NF, SXY = 3 * NF + 1, SYY = 3 * NF + 2,
                         BULK = 3 * NF + 3, WIDTH = 3 * NF + 4;
};

// Velocity-gradient terms of stress_field, evaluated once per cell.
template <int NF, class R> __device__ __forceinline__ void cell_shear(const DevParamsT<R>& P, R* rec)
{
    using L = CellLayout<NF>;
    const R gxvx = rec[L::GX + 1], gxvy = rec[L::GX + 2], gyvx = rec[L::GY + 1], gyvy = rec[L::GY + 2];
    if constexpr (std::is_same<R, double>::value) {
        const double dx = P.dx, dy = P.dx;
        rec[L::SXX] = 4.0 / 3.0 * gxvx / dx - 2.0 / 3.0 * gyvy / dy;
        rec[L::SXY] = 1.0 / 1.0 * gxvy / dx + 1.0 / 1.0 * gyvx / dy;
        rec[L::SYY] = -2.0 / 3.0 * gxvx / dx + 4.0 / 3.0 * gyvy / dy;
        rec[L::BULK] = gxvx / dx + gyvy / dy;
    } else {
        const float id = P.inv_dx;
        const float a = gxvx * id, b = gyvy * id;
        rec[L::SXX] = (4.0f / 3.0f) * a - (2.0f / 3.0f) * b;
        rec[L::SXY] = (gxvy + gyvx) * id;
        rec[L::SYY] = (4.0f / 3.0f) * b - (2.0f / 3.0f) * a;
        rec[L::BULK] = a + b;
    }
}

// CellData::stress_field(nu, lambda, ...) for (row, col) = (axis, X|Y).
template <int NF, class R>
__device__ __forceinline__ R stress(const R* rec, R nu, R lam_nu, int row, int col)
{
    using L = CellLayout<NF>;
    R shear, bulk;
    if (row == 0 && col == 0) { shear = rec[L::SXX]; bulk = rec[L::BULK]; }
    else if (row == 1 && col == 1) { shear = rec[L::SYY]; bulk = rec[L::BULK]; }
    else { shear = rec[L::SXY]; bulk = R(0); }
    return rec[L::PC] * (nu * shear + lam_nu * bulk);
}

// The `nu` closure of compute_block_fluxes (scheme.rs:230-247).
template <int NF, class R>
__device__ __forceinline__ R face_nu(const DevParamsT<R>& P, const Binary<R>& b, R x, R y, const R* rec)
{
    if (P.visc == 0) return R(P.nu);
    using L = CellLayout<NF>;
    R dx1 = x - b.p1.x, dy1 = y - b.p1.y, dx2 = x - b.p2.x, dy2 = y - b.p2.y;
    R r1 = rsqrt_(dx1 * dx1 + dy1 * dy1);
    R r2 = rsqrt_(dx2 * dx2 + dy2 * dy2);
    R cs2;
    if constexpr (NF == 3) {
        R gpot = binary_potential(b, x, y, R(P.soft2));
        if constexpr (std::is_same<R, double>::value) cs2 = -gpot / P.mach2;
        else cs2 = -gpot * P.inv_mach2;
    } else {
        cs2 = dvd(P.gamma * rec[L::PC + 3], rec[L::PC]);
    }
    R eps = P.eps_dx;
    R a1 = r1 + eps, a2 = r2 + eps;
    R twofreq = rsqrt_(b.p1.m / (a1 * a1 * a1) + b.p2.m / (a2 * a2 * a2));
    if constexpr (std::is_same<R, double>::value) return P.nu * cs2 / twofreq / P.sqrt_gm;
    else return dvd(P.nu * cs2, twofreq) * P.inv_sqrt_gm;
}

// Hydrodynamics::intercell_flux (physics.rs:584-607 iso, 776-803 euler) for
// cells l, r across a face at (x, y) normal to `axis`.
template <int NF, class R>
__device__ __forceinline__ void intercell_flux(const DevParamsT<R>& P, const Binary<R>& b, const R* l, const R* r, R x,
                                               R y, int axis, R* F)
{
    using L = CellLayout<NF>;
    const int G = axis == 0 ? L::GX : L::GY;
    R pl[NF], pr[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        pl[k] = l[L::PC + k] + l[G + k] * R(0.5);
        pr[k] = r[L::PC + k] - r[G + k] * R(0.5);
    }
    R lnu = face_nu<NF, R>(P, b, x, y, l);
    R rnu = face_nu<NF, R>(P, b, x, y, r);
    R lam = R(P.lambda);
    R tau_x = R(0.5) * (stress<NF, R>(l, lnu, lam * lnu, axis, 0) + stress<NF, R>(r, rnu, lam * rnu, axis, 0));
    R tau_y = R(0.5) * (stress<NF, R>(l, lnu, lam * lnu, axis, 1) + stress<NF, R>(r, rnu, lam * rnu, axis, 1));
    R cs2 = R(0);
    if constexpr (NF == 3) {
        R phi = binary_potential(b, x, y, R(P.soft2));
        if constexpr (std::is_same<R, double>::value) cs2 = -phi / P.mach2;
        else cs2 = -phi * P.inv_mach2;
    }
    hlle<NF, R>(P, pl, pr, axis, cs2, F);
    F[0] = F[0] + R(0);
    F[1] = F[1] + -tau_x;
    F[2] = F[2] + -tau_y;
    if constexpr (NF == 4) {
        R vx = R(0.5) * (l[L::PC + 1] + r[L::PC + 1]);
        R vy = R(0.5) * (l[L::PC + 2] + r[L::PC + 2]);
        F[3] = F[3] + -(tau_x * vx + tau_y * vy);
    }
}

// ---------------------------------------------------------------------------
// Source terms.  Physics::sink_kernel (physics.rs:388-397), Physics::source_terms
// (physics.rs:423-457), Isothermal::source_terms (physics.rs:528-582),
// Euler::source_terms (physics.rs:683-774).
template <class R> __device__ __forceinline__ R sink_kernel(const DevParamsT<R>& P, R dx, R dy)
{
    R r2 = dx * dx + dy * dy;
    R s2 = R(P.sink_r2);
    if (r2 < s2) {
        R t;
        if constexpr (std::is_same<R, double>::value) t = 1.0 - r2 / s2;
        else t = 1.0f - r2 * P.inv_sink_r2;
        return R(P.sink_rate) * (t * t);
    }
    return R(0);
}

template <class R>
__device__ __forceinline__ void torque_free_velocity(const DevParamsT<R>& P, const PointMass<R>& b, R x, R y, R vx, R vy,
                                                     R& vxc, R& vyc)
{
    R vxb = P.one_body ? R(0) : b.vx;
    R vyb = P.one_body ? R(0) : b.vy;
    R r = rsqrt_((x - b.x) * (x - b.x) + (y - b.y) * (y - b.y));
    R rx = dvd(x - b.x, r), ry = dvd(y - b.y, r);
    R dvdotr = (vx - vxb) * rx + (vy - vyb) * ry;
    vxc = dvdotr * rx + vxb;
    vyc = dvdotr * ry + vyb;
}

// Buffer rate 0.5·rate·(1 + tanh((r - R)/scale))·Ω_outer (physics.rs:443-446).
template <class R> __device__ __forceinline__ R buffer_rate(const DevParamsT<R>& P, R x, R y)
{
    if constexpr (std::is_same<R, double>::value) {
        double r = sqrt(x * x + y * y);
        double yb = (r - P.domain_radius) / P.buffer_scale;
        return P.half_buffer_rate * (1.0 + tanh(yb)) * P.omega_outer;
    } else {
        // 1 + tanh(y) = 2 / (1 + exp(-2y))
        float r = sqrtf(x * x + y * y);
        float yb = (r - P.domain_radius) * P.inv_buffer_scale;
        float e = __expf(-2.0f * yb);
        return P.half_rate_omega * __fdividef(2.0f, 1.0f + e);
    }
}

// SPARSE (called by all 32 lanes of a warp together): the sink terms are
// evaluated only when a zone of the warp lies inside a sink radius, and fake
// mass only for a non-zero rate; otherwise those items are the zeros the full
// formulas give.  Returns whether the sink items were evaluated.
template <int NF, class R, bool SPARSE = false>
__device__ __forceinline__ bool source_terms(const DevParamsT<R>& P, const Binary<R>& b, const R* u, const R* u0, R x, R y,
                                             R t, R dt, R* it /* [NITEMS][NF] */)
{
    const R s2 = R(P.soft2);
    R ax1, ay1, ax2, ay2;
    point_acceleration(b.p1, x, y, s2, ax1, ay1);
    point_acceleration(b.p2, x, y, s2, ax2, ay2);
    const R sigma = u[0];
    const R fx1 = sigma * ax1, fy1 = sigma * ay1, fx2 = sigma * ax2, fy2 = sigma * ay2;
    bool sinks_on = true;
    if constexpr (SPARSE) {
        const R d1x = x - b.p1.x, d1y = y - b.p1.y, d2x = x - b.p2.x, d2y = y - b.p2.y;
        const bool near = (d1x * d1x + d1y * d1y < R(P.sink_r2)) || (d2x * d2x + d2y * d2y < R(P.sink_r2));
        sinks_on = __any_sync(0xffffffffu, near);
    }
    R sr1 = R(0), sr2 = R(0);
    if (sinks_on) {
        sr1 = sink_kernel(P, x - b.p1.x, y - b.p1.y);
        sr2 = sink_kernel(P, x - b.p2.x, y - b.p2.y);
    }
    const R br = buffer_rate(P, x, y);
    const R kb = -dt * br;

    if constexpr (NF == 3) {
        R fake[3];
        if ((SPARSE && P.fake_rate == R(0)) || u[0] < u0[0] * R(P.fake_thr)) {
            fake[0] = fake[1] = fake[2] = R(0);
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) fake[k] = u0[k] * R(P.fake_rate) * dt;
        }
        R s1[3] = {R(0), R(0), R(0)}, s2v[3] = {R(0), R(0), R(0)};
        if (!sinks_on) {
        } else if (P.sink_model == 0) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                s1[k] = u[k] * -sr1;
                s2v[k] = u[k] * -sr2;
            }
        } else {
            R p[3];
            cons_to_prim_raw<3, R>(P, u, p);
            R v1x, v1y, v2x, v2y;
            torque_free_velocity(P, b.p1, x, y, p[1], p[2], v1x, v1y);
            torque_free_velocity(P, b.p2, x, y, p[1], p[2], v2x, v2y);
            R sd = p[0];
            R a1[3] = {sd, sd * v1x, sd * v1y}, a2[3] = {sd, sd * v2x, sd * v2y};
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                s1[k] = a1[k] * -sr1;
                s2v[k] = a2[k] * -sr2;
            }
        }
        R g1[3] = {R(0), fx1, fy1}, g2[3] = {R(0), fx2, fy2};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            it[GRAV1 * 3 + k] = g1[k] * dt;
            it[GRAV2 * 3 + k] = g2[k] * dt;
            it[SINK1 * 3 + k] = s1[k] * dt;
            it[SINK2 * 3 + k] = s2v[k] * dt;
            it[BUFFER * 3 + k] = (u[k] - u0[k]) * kb;
            it[COOLING * 3 + k] = R(0);
            it[FAKE_MASS * 3 + k] = fake[k];
        }
    } else {
        R p0[4];
        cons_to_prim_raw<4, R>(P, u, p0);
        const R vx = p0[1], vy = p0[2];
        const R g = R(P.gamma);
        R e0;
        if constexpr (std::is_same<R, double>::value) e0 = p0[3] / p0[0] / P.gm1;
        else e0 = dvd(p0[3], p0[0]) * P.inv_gm1;
        R ec;
        // FP32: the cooled minus the initial specific energy, formed directly
        // (e0 (exp(-c) - 1), e0 ((1 + x)^(-1/3) - 1) through expm1 and log1p):
        // as a difference of two near-equal energies it loses ~1e-7 / (c or x)
        // of its value, 1e-3 for changes of 1e-4 per stage.  The cooling item's
        // mass and momentum are zero in FP32: uc - u there is only the rounding
        // of a prim -> cons round trip (1e-16 of rho v in FP64, 1e-7 in FP32,
        // more than a weak cooling's energy term)
        R dec = R(0);
        if (P.cooling_kind == 1) {
            // β-cooling (not in the reference): e → e·exp(-Ω dt / β)
            R d1x = x - b.p1.x, d1y = y - b.p1.y, d2x = x - b.p2.x, d2y = y - b.p2.y;
            R t1 = d1x * d1x + d1y * d1y + s2, t2 = d2x * d2x + d2y * d2y + s2;
            R om;
            if constexpr (std::is_same<R, double>::value)
                om = sqrt(b.p1.m / (t1 * sqrt(t1)) + b.p2.m / (t2 * sqrt(t2)));
            else {
                float q1 = rsqrtf(t1), q2 = rsqrtf(t2);
                om = sqrtf(b.p1.m * q1 * q1 * q1 + b.p2.m * q2 * q2 * q2);
            }
            if constexpr (std::is_same<R, double>::value) ec = e0 * exp(-om * dt / P.cool_beta);
            else {
                dec = e0 * expm1f(-om * dt * P.inv_cool_beta);
                ec = e0 + dec;
            }
        } else {
            R f = R(1);
            if (P.cooling_slow_start) {
                if constexpr (std::is_same<R, double>::value) f = exp(-(2.0 * 3.14159265358979323846) / (t + dt));
                else f = __expf(-6.283185307f / (t + dt));
            }
            R rho_n = R(1);
            for (int k = 0; k < P.density_index; ++k) rho_n *= p0[0];
            R a = dvd(R(P.cool_coef), rho_n) * f;
            if constexpr (std::is_same<R, double>::value) ec = e0 * pow(1.0 + 3.0 * a * (e0 * e0 * e0) * dt, -1.0 / 3.0);
            else {
                dec = e0 * expm1f(log1pf(3.0f * a * (e0 * e0 * e0) * dt) * (-1.0f / 3.0f));
                ec = e0 + dec;
            }
        }
        if (P.has_mach_ceiling) {
            R ek = R(0.5) * (p0[1] * p0[1] + p0[2] * p0[2]);
            if constexpr (std::is_same<R, double>::value) ec = fmax(ec, 2.0 * ek / g / P.gm1 / P.mach_ceiling2);
            else {
                const R ecm = fmaxf(ec, ek * P.k_mach_ceiling);
                if (ecm != ec) {   // the ceiling binds (or ec was not a number)
                    dec = ecm - e0;
                    ec = ecm;
                }
            }
        }
        R pc[4] = {p0[0], p0[1], p0[2], p0[0] * ec * R(P.gm1)};
        R uc[4];
        prim_to_cons<4, R>(P, pc, uc);
        R s1[4] = {R(0), R(0), R(0), R(0)}, s2v[4] = {R(0), R(0), R(0), R(0)};
        if (!sinks_on) {
        } else if (P.sink_model == 0) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                s1[k] = u[k] * -sr1;
                s2v[k] = u[k] * -sr2;
            }
        } else {
            R v1x, v1y, v2x, v2y;
            torque_free_velocity(P, b.p1, x, y, vx, vy, v1x, v1y);
            torque_free_velocity(P, b.p2, x, y, vx, vy, v2x, v2y);
            R v1sq = v1x * v1x + v1y * v1y, v2sq = v2x * v2x + v2y * v2y;
            R sd = p0[0];
            R a1[4] = {sd, sd * v1x, sd * v1y, sd * e0 + R(0.5) * sd * v1sq};
            R a2[4] = {sd, sd * v2x, sd * v2y, sd * e0 + R(0.5) * sd * v2sq};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                s1[k] = a1[k] * -sr1;
                s2v[k] = a2[k] * -sr2;
            }
        }
        R g1[4] = {R(0), fx1, fy1, fx1 * vx + fy1 * vy};
        R g2[4] = {R(0), fx2, fy2, fx2 * vx + fy2 * vy};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            it[GRAV1 * 4 + k] = g1[k] * dt;
            it[GRAV2 * 4 + k] = g2[k] * dt;
            it[SINK1 * 4 + k] = s1[k] * dt;
            it[SINK2 * 4 + k] = s2v[k] * dt;
            it[BUFFER * 4 + k] = (u[k] - u0[k]) * kb;
            if constexpr (std::is_same<R, double>::value) it[COOLING * 4 + k] = uc[k] - u[k];
            else it[COOLING * 4 + k] = k == 3 ? p0[0] * dec : R(0);
            it[FAKE_MASS * 4 + k] = R(0);
        }
    }
    return sinks_on;
}

}  // namespace b2d
