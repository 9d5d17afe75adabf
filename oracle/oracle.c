/*
 * oracle.c — CPU FP64 restatement of binary2d's explicit finite-volume RK
 * step on the block mesh (clemson-cal/app-binary2d 0.2.1).
 *
 * TEST INFRASTRUCTURE ONLY: the correctness oracle for the CUDA path and the
 * timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU legs load it.  PARITY UNPINNED: the reference cannot be compiled here
 * and ships no golden vectors (see oracle.h for the un-vendored
 * dependencies whose published methods are restated below).
 *
 * Compile with -ffp-contract=off: every floating-point operation below is
 * evaluated in the order written, which is the order of the reference's Rust
 * expressions (left-associative, no fused multiply-add).
 *
 * Threading follows the reference's tokio design (src/scheme.rs:108-158):
 * three phases per RK stage (primitive, fluxes, update), one task per block
 * per phase, drawn by a pool of worker threads.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

#define NITEMS 7
enum { SINK1 = 0, SINK2, GRAV1, GRAV2, BUFFER, COOLING, FAKE_MASS };

#define ORBITAL_PERIOD (2.0 * 3.14159265358979323846) /* physics.rs:21 */

typedef struct orbit { oracle_point_mass p1, p2; } orbit;

static int nfields(const oracle_config* c) { return c->hydro_kind == 1 ? 4 : 3; }

/* ======================================================================== */
/* Mesh geometry, src/mesh.rs                                                */

/* Mesh::block_length, mesh.rs:27-29 */
static double block_length(const oracle_config* c)
{
    return 2.0 * c->domain_radius / (double)c->num_blocks;
}

/* Mesh::cell_spacing, mesh.rs:86-88 */
static double cell_spacing(const oracle_config* c)
{
    return block_length(c) / (double)c->block_size;
}

/* Mesh::block_vertices, mesh.rs:42-47: ndarray linspace(start, start + L,
 * bs + 1), i.e. start + step·k with step = (end - start) / bs. */
void oracle_block_vertices(const oracle_config* c, int32_t b, double* xv)
{
    double start = -c->domain_radius + (double)b * block_length(c); /* mesh.rs:31-36 */
    double end = start + block_length(c);
    double step = (end - start) / (double)c->block_size;
    for (int k = 0; k <= c->block_size; ++k)
        xv[k] = start + step * (double)k;
}

/* Mesh::cell_centers, mesh.rs:49-54: adjacent means of the vertices. */
void oracle_cell_centers(const oracle_config* c, int32_t b, double* xc)
{
    double xv[c->block_size + 1];
    oracle_block_vertices(c, b, xv);
    for (int k = 0; k < c->block_size; ++k)
        xc[k] = (xv[k] + xv[k + 1]) * 0.5;
}

/* ======================================================================== */
/* Two-body orbit (kepler-two-body, un-vendored; restated).                  */
/*                                                                           */
/* OrbitalElements(a, M, q, e) (physics.rs:411-417): semi-major axis a, total */
/* mass M, mass ratio q, eccentricity e, G = 1.  Periapsis on +x at t = 0,    */
/* counter-clockwise motion.  Mean anomaly n·t with n = sqrt(M / a^3);        */
/* Kepler's equation E - e sin E = n t solved by Newton's method from E = n t.*/
/* Body 1 has mass M/(1+q) and body 2 M q/(1+q); each sits on the opposite    */
/* side of the centre of mass at distances proportional to the other's mass. */
static void orbital_state_from_time(const oracle_config* c, double t, orbit* o)
{
    double a, M, q, e;
    if (c->one_body) { a = 1e-12; M = 1.0; q = 1.0; e = 0.0; }  /* physics.rs:412-413 */
    else { a = 1.0; M = 1.0; q = c->binary_mass_ratio; e = c->binary_eccentricity; }

    double n = sqrt(M / (a * a * a));
    double mean = n * t;
    double E = mean;
    for (int k = 0; k < 64; ++k) {
        double f = E - e * sin(E) - mean;
        if (fabs(f) < 1e-15) break;
        E = E - f / (1.0 - e * cos(E));
    }
    double cE = cos(E), sE = sin(E);
    double b = sqrt(1.0 - e * e);
    double x = a * (cE - e);
    double y = a * b * sE;
    double edot = n / (1.0 - e * cE);
    double vx = -a * sE * edot;
    double vy = a * b * cE * edot;
    double m1 = M / (1.0 + q);
    double m2 = M * q / (1.0 + q);
    double f1 = m2 / M, f2 = m1 / M;
    o->p1.m = m1; o->p1.x = -x * f1; o->p1.y = -y * f1; o->p1.vx = -vx * f1; o->p1.vy = -vy * f1;
    o->p2.m = m2; o->p2.x = x * f2; o->p2.y = y * f2; o->p2.vx = vx * f2; o->p2.vy = vy * f2;
}

void oracle_orbital_state(const oracle_config* c, double t, oracle_point_mass* p1,
                          oracle_point_mass* p2)
{
    orbit o;
    orbital_state_from_time(c, t, &o);
    *p1 = o.p1;
    *p2 = o.p2;
}

/* Plummer potential and acceleration of one point mass, softening s
 * (restated; acceleration form of tools/indep_res_analysis.py:182-194). */
static double point_potential(const oracle_point_mass* p, double x, double y, double s)
{
    double dx = x - p->x, dy = y - p->y;
    double r2 = dx * dx + dy * dy;
    return -p->m / sqrt(r2 + s * s);
}

static void point_acceleration(const oracle_point_mass* p, double x, double y, double s,
                               double* ax, double* ay)
{
    double dx = x - p->x, dy = y - p->y;
    double t2 = dx * dx + dy * dy + s * s;
    double d3 = t2 * sqrt(t2);
    *ax = -p->m * dx / d3;
    *ay = -p->m * dy / d3;
}

/* Physics::softening_length, physics.rs:399-405 */
static double softening_length(const oracle_config* c)
{
    return c->has_softening_length ? c->softening_length : c->sink_radius;
}

/* OrbitalState::gravitational_potential at a face, scheme.rs:214-215 */
static double binary_potential(const orbit* o, double x, double y, double s)
{
    return point_potential(&o->p1, x, y, s) + point_potential(&o->p2, x, y, s);
}

/* ======================================================================== */
/* Conserved <-> primitive (hydro-iso2d / hydro-euler, restated)             */

static void prim_to_cons(const oracle_config* c, const double* p, double* u)
{
    u[0] = p[0];
    u[1] = p[0] * p[1];
    u[2] = p[0] * p[2];
    if (c->hydro_kind == 1) {
        double g = c->gamma_law_index;
        u[3] = 0.5 * p[0] * (p[1] * p[1] + p[2] * p[2]) + p[3] / (g - 1.0);
    }
}

static void cons_to_prim_raw(const oracle_config* c, const double* u, double* p)
{
    p[0] = u[0];
    p[1] = u[1] / u[0];
    p[2] = u[2] / u[0];
    if (c->hydro_kind == 1) {
        double g = c->gamma_law_index;
        p[3] = (u[3] - 0.5 * u[0] * (p[1] * p[1] + p[2] * p[2])) * (g - 1.0);
    }
}

void oracle_prim_to_cons(const oracle_config* c, const double* p, double* u)
{
    prim_to_cons(c, p, u);
}

/* Hydrodynamics::try_to_primitive: Isothermal physics.rs:489-503, Euler
 * physics.rs:631-660.  Returns 0 or an error code; *bad is the offending value. */
static int try_to_primitive(const oracle_config* c, const double* u_in, double* p, double* bad)
{
    if (c->hydro_kind == 0) {
        double u[3] = {u_in[0], u_in[1], u_in[2]};
        if (c->has_density_floor && u[0] < c->density_floor) {
            u[1] = 0.0;
            u[2] = 0.0;
            u[0] = c->density_floor;
        }
        if (u[0] < 0.0) { *bad = u[0]; return ORACLE_NEG_DENSITY; }
        cons_to_prim_raw(c, u, p);
        return 0;
    }
    cons_to_prim_raw(c, u_in, p);
    if (c->has_density_floor && p[0] < c->density_floor) {
        p[0] = c->density_floor;
        p[1] = 0.0;
        p[2] = 0.0;
        p[3] = pow(c->density_floor, c->gamma_law_index);
    }
    if (p[0] < 0.0) { *bad = p[0]; return ORACLE_NEG_DENSITY; }
    if (c->has_pressure_floor && p[3] < c->pressure_floor) p[3] = c->pressure_floor;
    if (p[3] <= 0.0) { *bad = p[3]; return ORACLE_NEG_PRESSURE; }
    return 0;
}

int oracle_cons_to_prim(const oracle_config* c, const double* u, double* p)
{
    double bad;
    return try_to_primitive(c, u, p, &bad);
}

/* Hydrodynamics::max_signal_speed: Isothermal physics.rs:521-526
 * (max(|vx|,|vy|), no sound speed); Euler physics.rs:679-681 (hydro-euler's
 * primitive max_signal_speed, restated as max(|vx|,|vy|) + c_s). */
static double zone_max_signal_speed(const oracle_config* c, const double* u)
{
    double p[4];
    cons_to_prim_raw(c, u, p);
    double v = fmax(fabs(p[1]), fabs(p[2]));
    if (c->hydro_kind == 1) {
        double cs = sqrt(c->gamma_law_index * p[3] / p[0]);
        return v + cs;
    }
    return v;
}

/* ======================================================================== */
/* PLM gradient (godunov-core piecewise_linear::plm_gradient3/4, restated): */
/* generalised minmod of θ(b - a), (c - a)/2, θ(c - b), component-wise.       */
double oracle_plm_gradient(double theta, double a, double b, double c)
{
    double x = theta * (b - a);
    double y = 0.5 * (c - a);
    double z = theta * (c - b);
    if (x > 0.0 && y > 0.0 && z > 0.0) return fmin(x, fmin(y, z));
    if (x < 0.0 && y < 0.0 && z < 0.0) return fmax(x, fmax(y, z));
    return 0.0;
}

/* ======================================================================== */
/* Physical flux and HLLE (hydro-iso2d / hydro-euler riemann_hlle, restated):*/
/* F = (F_L a+ - F_R a- - (U_L - U_R) a+ a-) / (a+ - a-),                     */
/* a+ = max(0, vL + cL, vR + cR), a- = min(0, vL - cL, vR - cR).              */
static void physical_flux(const oracle_config* c, const double* p, const double* u, int axis,
                          double cs2, double* f)
{
    double vn = p[1 + axis];
    double pg = c->hydro_kind == 0 ? p[0] * cs2 : p[3];
    f[0] = u[0] * vn;
    f[1] = u[1] * vn + (axis == 0 ? pg : 0.0);
    f[2] = u[2] * vn + (axis == 1 ? pg : 0.0);
    if (c->hydro_kind == 1) f[3] = (u[3] + pg) * vn;
}

void oracle_physical_flux(const oracle_config* c, const double* p, int32_t axis, double cs2,
                          double* f)
{
    double u[4];
    prim_to_cons(c, p, u);
    physical_flux(c, p, u, axis, cs2, f);
}

static void hlle(const oracle_config* c, const double* pl, const double* pr, int axis,
                 double cs2, double* F)
{
    int nf = nfields(c);
    double ul[4], ur[4], fl[4], fr[4];
    prim_to_cons(c, pl, ul);
    prim_to_cons(c, pr, ur);
    physical_flux(c, pl, ul, axis, cs2, fl);
    physical_flux(c, pr, ur, axis, cs2, fr);
    double csl, csr;
    if (c->hydro_kind == 0) {
        csl = sqrt(cs2);
        csr = csl;
    } else {
        csl = sqrt(c->gamma_law_index * pl[3] / pl[0]);
        csr = sqrt(c->gamma_law_index * pr[3] / pr[0]);
    }
    double vl = pl[1 + axis], vr = pr[1 + axis];
    double alm = vl - csl, alp = vl + csl;
    double arm = vr - csr, arp = vr + csr;
    double ap = fmax(0.0, fmax(alp, arp));
    double am = fmin(0.0, fmin(alm, arm));
    for (int k = 0; k < nf; ++k)
        F[k] = (fl[k] * ap - fr[k] * am - (ul[k] - ur[k]) * ap * am) / (ap - am);
}

void oracle_hlle(const oracle_config* c, const double* pl, const double* pr, int32_t axis,
                 double cs2, double* flux)
{
    hlle(c, pl, pr, axis, cs2, flux);
}

/* ======================================================================== */
/* Viscous stress, CellData::stress_field (physics.rs:322-340).              */
typedef struct cell_data { const double *pc, *gx, *gy; } cell_data;

static double stress_field(const cell_data* d, double nu, double lambda, double dx, double dy,
                           int row, int col)
{
    double shear, bulk;
    if (row == 0 && col == 0) {
        shear = 4.0 / 3.0 * d->gx[1] / dx - 2.0 / 3.0 * d->gy[2] / dy;
        bulk = d->gx[1] / dx + d->gy[2] / dy;
    } else if (row == 1 && col == 1) {
        shear = -2.0 / 3.0 * d->gx[1] / dx + 4.0 / 3.0 * d->gy[2] / dy;
        bulk = d->gx[1] / dx + d->gy[2] / dy;
    } else {
        shear = 1.0 / 1.0 * d->gx[2] / dx + 1.0 / 1.0 * d->gy[1] / dy;
        bulk = 0.0;
    }
    return d->pc[0] * (nu * shear + lambda * bulk);
}

/* Hydrodynamics::intercell_flux: Isothermal physics.rs:584-607, Euler
 * physics.rs:776-803. */
static void intercell_flux(const oracle_config* c, const cell_data* l, const cell_data* r,
                           double lnu, double rnu, double dx, double dy, double phi, int axis,
                           double* F)
{
    int nf = nfields(c);
    const double* gl = axis == 0 ? l->gx : l->gy;
    const double* gr = axis == 0 ? r->gx : r->gy;
    double pl[4], pr[4];
    for (int k = 0; k < nf; ++k) {
        pl[k] = l->pc[k] + gl[k] * 0.5;
        pr[k] = r->pc[k] - gr[k] * 0.5;
    }
    double lam = c->lambda_multiplier;
    double tau_x = 0.5 * (stress_field(l, lnu, lam * lnu, dx, dy, axis, 0) +
                          stress_field(r, rnu, lam * rnu, dx, dy, axis, 0));
    double tau_y = 0.5 * (stress_field(l, lnu, lam * lnu, dx, dy, axis, 1) +
                          stress_field(r, rnu, lam * rnu, dx, dy, axis, 1));
    double cs2 = 0.0;
    if (c->hydro_kind == 0) cs2 = -phi / (c->mach_number * c->mach_number);
    hlle(c, pl, pr, axis, cs2, F);
    F[0] = F[0] + 0.0;
    F[1] = F[1] + -tau_x;
    F[2] = F[2] + -tau_y;
    if (c->hydro_kind == 1) {
        double vx = 0.5 * (l->pc[1] + r->pc[1]);
        double vy = 0.5 * (l->pc[2] + r->pc[2]);
        F[3] = F[3] + -(tau_x * vx + tau_y * vy);
    }
}

/* Face viscosity, the `nu` closure of scheme.rs:230-247. */
static double face_nu(const oracle_config* c, const orbit* o, double x, double y,
                      const cell_data* d, double dx)
{
    if (c->viscosity_kind == 0) return c->viscosity;
    double alpha = c->viscosity;
    double x1 = o->p1.x, y1 = o->p1.y, x2 = o->p2.x, y2 = o->p2.y;
    double r1 = sqrt((x - x1) * (x - x1) + (y - y1) * (y - y1));
    double r2 = sqrt((x - x2) * (x - x2) + (y - y2) * (y - y2));
    double m1 = o->p1.m, m2 = o->p2.m;
    double gm = c->hydro_kind == 1 ? c->gamma_law_index : 1.0;
    double cs2;
    if (c->hydro_kind == 0) {
        double gpot = binary_potential(o, x, y, softening_length(c));
        cs2 = -gpot / (c->mach_number * c->mach_number);  /* physics.rs:859-861 */
    } else {
        cs2 = gm * d->pc[3] / d->pc[0];                    /* physics.rs:868-870 */
    }
    double a1 = r1 + 1e-12 * dx, a2 = r2 + 1e-12 * dx;
    double twofreq = sqrt(m1 / (a1 * a1 * a1) + m2 / (a2 * a2 * a2));
    return alpha * cs2 / twofreq / sqrt(gm);
}

/* ======================================================================== */
/* Source terms.  Physics::sink_kernel physics.rs:388-397, Physics::source_terms */
/* physics.rs:423-457, Isothermal::source_terms physics.rs:528-582,           */
/* Euler::source_terms physics.rs:683-774.                                    */
static double sink_kernel(const oracle_config* c, double dx, double dy)
{
    double r2 = dx * dx + dy * dy;
    double s2 = c->sink_radius * c->sink_radius;
    if (r2 < s2) {
        double t = 1.0 - r2 / s2;
        return c->sink_rate * (t * t);
    }
    return 0.0;
}

typedef struct source_terms_t {
    double fx1, fy1, fx2, fy2, sink_rate1, sink_rate2, buffer_rate;
} source_terms_t;

static source_terms_t physics_source_terms(const oracle_config* c, const orbit* o, double x,
                                           double y, double sigma)
{
    source_terms_t st;
    double s = softening_length(c);
    double ax1, ay1, ax2, ay2;
    point_acceleration(&o->p1, x, y, s, &ax1, &ay1);
    point_acceleration(&o->p2, x, y, s, &ax2, &ay2);
    st.fx1 = sigma * ax1;
    st.fy1 = sigma * ay1;
    st.fx2 = sigma * ax2;
    st.fy2 = sigma * ay2;
    st.sink_rate1 = sink_kernel(c, x - o->p1.x, y - o->p1.y);
    st.sink_rate2 = sink_kernel(c, x - o->p2.x, y - o->p2.y);
    double R = c->domain_radius;
    double r = sqrt(x * x + y * y);
    double yb = (r - R) / c->buffer_scale;
    double omega_outer = sqrt((o->p1.m + o->p2.m) / (R * R * R));
    st.buffer_rate = 0.5 * c->buffer_rate * (1.0 + tanh(yb)) * omega_outer;
    return st;
}

/* Torque-free sink velocity (physics.rs:551-570 / 741-762), Dittmann & Ryan
 * (2021) eq. 12: keep the gas velocity component along the body-gas line,
 * replace the rest by the body's velocity. */
static void torque_free_velocity(const oracle_config* c, const oracle_point_mass* b, double x,
                                 double y, double vx, double vy, double* vxc, double* vyc)
{
    double vxb = c->one_body ? 0.0 : b->vx;
    double vyb = c->one_body ? 0.0 : b->vy;
    double r = sqrt((x - b->x) * (x - b->x) + (y - b->y) * (y - b->y));
    double rx = (x - b->x) / r, ry = (y - b->y) / r;
    double dvdotr = (vx - vxb) * rx + (vy - vyb) * ry;
    *vxc = dvdotr * rx + vxb;
    *vyc = dvdotr * ry + vyb;
}

/* Ω used by β-cooling (new option, not in the reference): softened
 * two-body orbital frequency sqrt(Σ_k m_k / (r_k² + s²)^{3/2}). */
static double beta_cooling_omega(const oracle_config* c, const orbit* o, double x, double y)
{
    double s = softening_length(c);
    double d1x = x - o->p1.x, d1y = y - o->p1.y, d2x = x - o->p2.x, d2y = y - o->p2.y;
    double t1 = d1x * d1x + d1y * d1y + s * s;
    double t2 = d2x * d2x + d2y * d2y + s * s;
    return sqrt(o->p1.m / (t1 * sqrt(t1)) + o->p2.m / (t2 * sqrt(t2)));
}

static void source_terms(const oracle_config* c, const double* u, const double* u0, double x,
                         double y, double t, double dt, const orbit* o, double* it /*[7][nf]*/)
{
    int nf = nfields(c);
    if (c->hydro_kind == 0) {
        /* Isothermal::source_terms, physics.rs:528-582 */
        double fake[3];
        if (u[0] < u0[0] * c->fake_mass_threshold) {
            fake[0] = fake[1] = fake[2] = 0.0;
        } else {
            for (int k = 0; k < 3; ++k) fake[k] = u0[k] * c->fake_mass_rate * dt;
        }
        source_terms_t st = physics_source_terms(c, o, x, y, u[0]);
        double s1[3], s2[3];
        if (c->sink_model == 0) {
            for (int k = 0; k < 3; ++k) {
                s1[k] = u[k] * -st.sink_rate1;
                s2[k] = u[k] * -st.sink_rate2;
            }
        } else {
            double p[3];
            cons_to_prim_raw(c, u, p);
            double v1x, v1y, v2x, v2y;
            torque_free_velocity(c, &o->p1, x, y, p[1], p[2], &v1x, &v1y);
            torque_free_velocity(c, &o->p2, x, y, p[1], p[2], &v2x, &v2y);
            double sd = p[0];
            double a1[3] = {sd, sd * v1x, sd * v1y}, a2[3] = {sd, sd * v2x, sd * v2y};
            for (int k = 0; k < 3; ++k) {
                s1[k] = a1[k] * -st.sink_rate1;
                s2[k] = a2[k] * -st.sink_rate2;
            }
        }
        double g1[3] = {0.0, st.fx1, st.fy1}, g2[3] = {0.0, st.fx2, st.fy2};
        double kb = -dt * st.buffer_rate;
        for (int k = 0; k < 3; ++k) {
            it[GRAV1 * nf + k] = g1[k] * dt;
            it[GRAV2 * nf + k] = g2[k] * dt;
            it[SINK1 * nf + k] = s1[k] * dt;
            it[SINK2 * nf + k] = s2[k] * dt;
            it[BUFFER * nf + k] = (u[k] - u0[k]) * kb;
            it[COOLING * nf + k] = 0.0;
            it[FAKE_MASS * nf + k] = fake[k];
        }
        return;
    }

    /* Euler::source_terms, physics.rs:683-774 (u = stage state, u0 = background) */
    double g = c->gamma_law_index;
    source_terms_t st = physics_source_terms(c, o, x, y, u[0]);
    double p0[4] = {0.0, 0.0, 0.0, 0.0};
    cons_to_prim_raw(c, u, p0);
    double vx = p0[1], vy = p0[2];
    double e0 = p0[3] / p0[0] / (g - 1.0);
    double ec;
    if (c->cooling_kind == 1) {
        double omega = beta_cooling_omega(c, o, x, y);
        ec = e0 * exp(-omega * dt / c->cooling_beta);
    } else {
        double f = c->cooling_slow_start ? exp(-ORBITAL_PERIOD / (t + dt)) : 1.0;
        double rho_n = 1.0;
        for (int k = 0; k < c->density_index; ++k) rho_n *= p0[0];
        double a = c->cooling_coefficient / rho_n * f;
        ec = e0 * pow(1.0 + 3.0 * a * (e0 * e0 * e0) * dt, -1.0 / 3.0);
    }
    if (c->has_mach_ceiling) {
        double ek = 0.5 * (p0[1] * p0[1] + p0[2] * p0[2]);
        double mc = c->mach_ceiling;
        ec = fmax(ec, 2.0 * ek / g / (g - 1.0) / (mc * mc));
    }
    double pc[4] = {p0[0], p0[1], p0[2], p0[0] * ec * (g - 1.0)};
    double uc[4];
    prim_to_cons(c, pc, uc);

    double s1[4], s2[4];
    if (c->sink_model == 0) {
        for (int k = 0; k < 4; ++k) {
            s1[k] = u[k] * -st.sink_rate1;
            s2[k] = u[k] * -st.sink_rate2;
        }
    } else {
        double v1x, v1y, v2x, v2y;
        torque_free_velocity(c, &o->p1, x, y, vx, vy, &v1x, &v1y);
        torque_free_velocity(c, &o->p2, x, y, vx, vy, &v2x, &v2y);
        double v1sq = v1x * v1x + v1y * v1y, v2sq = v2x * v2x + v2y * v2y;
        double sd = p0[0];
        double a1[4] = {sd, sd * v1x, sd * v1y, sd * e0 + 0.5 * sd * v1sq};
        double a2[4] = {sd, sd * v2x, sd * v2y, sd * e0 + 0.5 * sd * v2sq};
        for (int k = 0; k < 4; ++k) {
            s1[k] = a1[k] * -st.sink_rate1;
            s2[k] = a2[k] * -st.sink_rate2;
        }
    }
    double g1[4] = {0.0, st.fx1, st.fy1, st.fx1 * vx + st.fy1 * vy};
    double g2[4] = {0.0, st.fx2, st.fy2, st.fx2 * vx + st.fy2 * vy};
    double kb = -dt * st.buffer_rate;
    for (int k = 0; k < 4; ++k) {
        it[GRAV1 * nf + k] = g1[k] * dt;
        it[GRAV2 * nf + k] = g2[k] * dt;
        it[SINK1 * nf + k] = s1[k] * dt;
        it[SINK2 * nf + k] = s2[k] * dt;
        it[BUFFER * nf + k] = (u[k] - u0[k]) * kb;
        it[COOLING * nf + k] = uc[k] - u[k];
        it[FAKE_MASS * nf + k] = 0.0;
    }
}

void oracle_source_terms(const oracle_config* c, const double* u, const double* u0, double x,
                         double y, double t, double dt, double* items)
{
    orbit o;
    orbital_state_from_time(c, t, &o);
    source_terms(c, u, u0, x, y, t, dt, &o, items);
}

/* ======================================================================== */
/* Worker pool: one task per block per phase (scheme.rs:108-158).            */

typedef struct pool pool;
typedef void (*task_fn)(pool* pl, int worker, int task);

struct pool {
    int nthreads;
    pthread_barrier_t barrier;
    atomic_int next;
    int ntasks;
    task_fn fn;
    int quit;
    void* arg;
};

typedef struct worker_arg { pool* pl; int id; } worker_arg;

static void run_tasks(pool* pl, int id)
{
    for (;;) {
        int t = atomic_fetch_add(&pl->next, 1);
        if (t >= pl->ntasks) break;
        pl->fn(pl, id, t);
    }
}

static void* worker_main(void* p)
{
    worker_arg* wa = (worker_arg*)p;
    pool* pl = wa->pl;
    for (;;) {
        pthread_barrier_wait(&pl->barrier);
        if (pl->quit) break;
        run_tasks(pl, wa->id);
        pthread_barrier_wait(&pl->barrier);
    }
    return NULL;
}

static void pool_run(pool* pl, int ntasks, task_fn fn)
{
    pl->ntasks = ntasks;
    pl->fn = fn;
    atomic_store(&pl->next, 0);
    if (pl->nthreads > 1) pthread_barrier_wait(&pl->barrier);
    run_tasks(pl, 0);
    if (pl->nthreads > 1) pthread_barrier_wait(&pl->barrier);
}

/* ======================================================================== */
/* One RK stage: try_advance_rk (scheme.rs:88-173).                          */

typedef struct stage_ctx {
    const oracle_config* c;
    int nf, nb, bs;
    double dx, time, dt;
    orbit o;
    const double* cons_in;  /* stage input */
    const double* bg;       /* BlockData::initial_conserved */
    const double* led_in;
    double* cons_out;
    double* led_out;
    double* prim;           /* phase A output, block layout */
    int* perr;              /* per block error code */
    double* pbad;           /* per block offending value */
    int* pzone;             /* per block first failing zone */
    double** scratch;       /* per worker */
    double* fxs;            /* per block x fluxes (bs+1)*bs*nf */
    double* fys;            /* per block y fluxes bs*(bs+1)*nf */
    double* xc;             /* [nb][bs] cell centres */
    double* xv;             /* [nb][bs+1] vertices */
    const double* el_in;    /* orbital_elements_change of the stage input, [nb][nb][7][4] */
    double* el_out;         /* ... of the stage output (NULL: not tracked) */
    int* unbound;           /* per block: its perturbed orbit is unbound */
} stage_ctx;

/* Phase A: try_block_primitive, scheme.rs:185-199 */
static void task_primitive(pool* pl, int w, int b)
{
    (void)w;
    stage_ctx* s = (stage_ctx*)pl->arg;
    int nf = s->nf, n = s->bs * s->bs;
    const double* u = s->cons_in + (size_t)b * n * nf;
    double* p = s->prim + (size_t)b * n * nf;
    s->perr[b] = 0;
    for (int z = 0; z < n; ++z) {
        double bad = 0.0;
        int e = try_to_primitive(s->c, u + z * nf, p + z * nf, &bad);
        if (e && !s->perr[b]) {
            s->perr[b] = e;
            s->pbad[b] = bad;
            s->pzone[b] = z;
        }
    }
}

/* Phase B: halo extension (ndarray_ops::extend_from_neighbor_arrays_2d with
 * 2 guard zones, scheme.rs:126-127; periodic neighbours mesh.rs:101-110) and
 * compute_block_fluxes (scheme.rs:201-271). */
static void task_fluxes(pool* pl, int w, int b)
{
    stage_ctx* s = (stage_ctx*)pl->arg;
    const oracle_config* c = s->c;
    int nf = s->nf, bs = s->bs, nb = s->nb, n = bs * bs;
    int bi = b / nb, bj = b % nb;
    int E = bs + 4;
    double* pe = s->scratch[w];
    double* gx = pe + (size_t)E * E * nf;          /* (bs+2) x (bs+4) */
    double* gy = gx + (size_t)(bs + 2) * E * nf;   /* (bs+4) x (bs+2) */

    for (int i = 0; i < E; ++i) {
        int gi = bi * bs + i - 2;
        int nbi = ((gi + nb * bs) / bs) % nb;
        int li = (gi + nb * bs) % bs;
        for (int j = 0; j < E; ++j) {
            int gj = bj * bs + j - 2;
            int nbj = ((gj + nb * bs) / bs) % nb;
            int lj = (gj + nb * bs) % bs;
            const double* src = s->prim + ((size_t)(nbi * nb + nbj) * n + li * bs + lj) * nf;
            memcpy(pe + ((size_t)i * E + j) * nf, src, nf * sizeof(double));
        }
    }

    double pdt = c->has_plm_density_trigger ? c->plm_density_trigger : 0.0;
    /* gx = map_stencil3(pe, Axis(0), ...), scheme.rs:224 */
    for (int i = 0; i < bs + 2; ++i) {
        for (int j = 0; j < E; ++j) {
            const double* a = pe + ((size_t)i * E + j) * nf;
            const double* m = a + (size_t)E * nf;
            const double* q = m + (size_t)E * nf;
            double th = (a[0] < pdt || m[0] < pdt || q[0] < pdt) ? 0.0 : c->plm;
            double* g = gx + ((size_t)i * E + j) * nf;
            for (int k = 0; k < nf; ++k) g[k] = oracle_plm_gradient(th, a[k], m[k], q[k]);
        }
    }
    /* gy = map_stencil3(pe, Axis(1), ...), scheme.rs:225 */
    for (int i = 0; i < E; ++i) {
        for (int j = 0; j < bs + 2; ++j) {
            const double* a = pe + ((size_t)i * E + j) * nf;
            const double* m = a + nf;
            const double* q = m + nf;
            double th = (a[0] < pdt || m[0] < pdt || q[0] < pdt) ? 0.0 : c->plm;
            double* g = gy + ((size_t)i * (bs + 2) + j) * nf;
            for (int k = 0; k < nf; ++k) g[k] = oracle_plm_gradient(th, a[k], m[k], q[k]);
        }
    }

    /* cell_data over the (bs+2)^2 cells with local index -1..bs, scheme.rs:250-254:
     * pc = pe[1..-1, 1..-1], gx[.., 1..-1], gy[1..-1, ..] */
#define CD(ci, cj) ((cell_data){pe + ((size_t)((ci) + 2) * E + (cj) + 2) * nf, \
                                gx + ((size_t)((ci) + 1) * E + (cj) + 2) * nf, \
                                gy + ((size_t)((ci) + 2) * (bs + 2) + (cj) + 1) * nf})
    double dx = s->dx, dy = s->dx;
    double soft = softening_length(c);
    const double* xc = s->xc;
    const double* xv = s->xv;
    double* fx = s->fxs + (size_t)b * (bs + 1) * bs * nf;
    double* fy = s->fys + (size_t)b * bs * (bs + 1) * nf;

    /* fx, scheme.rs:257-261: faces at vertices xv[i] (i = 0..bs) x centres yc[j] */
    for (int i = 0; i <= bs; ++i) {
        for (int j = 0; j < bs; ++j) {
            cell_data l = CD(i - 1, j), r = CD(i, j);
            double x = xv[bi * (bs + 1) + i], y = xc[bj * bs + j];
            double lnu = face_nu(c, &s->o, x, y, &l, dx);
            double rnu = face_nu(c, &s->o, x, y, &r, dx);
            double phi = binary_potential(&s->o, x, y, soft);
            intercell_flux(c, &l, &r, lnu, rnu, dx, dy, phi, 0, fx + ((size_t)i * bs + j) * nf);
        }
    }
    /* fy, scheme.rs:264-268: faces at centres xc[i] x vertices yv[j] */
    for (int i = 0; i < bs; ++i) {
        for (int j = 0; j <= bs; ++j) {
            cell_data l = CD(i, j - 1), r = CD(i, j);
            double x = xc[bi * bs + i], y = xv[bj * (bs + 1) + j];
            double lnu = face_nu(c, &s->o, x, y, &l, dx);
            double rnu = face_nu(c, &s->o, x, y, &r, dx);
            double phi = binary_potential(&s->o, x, y, soft);
            intercell_flux(c, &l, &r, lnu, rnu, dx, dy, phi, 1,
                           fy + ((size_t)i * (bs + 1) + j) * nf);
        }
    }
#undef CD
}

/* OrbitalElements::perturb (kepler-two-body, un-vendored; restated from
 * two-body mechanics).  At the orbital state `o`, body 1 gains mass dm1 and
 * momentum (dpx1, dpy1) and body 2 gains dm2 and (dpx2, dpy2), each at a
 * fixed position; the new elements follow from the relative orbit:
 * M' = m1' + m2', q' = m2' / m1', E = |v|^2 / 2 - M' / |r|, a' = -M' / (2E),
 * h = r x v, e' = sqrt(1 + 2 E h^2 / M'^2).  Returns 0 for E >= 0
 * (UnboundOrbitalState, physics.rs:34-35), else writes (a', M', q', e') - el. */
static int perturb(const orbit* o, const double* el, double dm1, double dm2, double dpx1, double dpx2,
                   double dpy1, double dpy2, double* de)
{
    double m1 = o->p1.m + dm1, m2 = o->p2.m + dm2;
    double u1x = (o->p1.m * o->p1.vx + dpx1) / m1, u1y = (o->p1.m * o->p1.vy + dpy1) / m1;
    double u2x = (o->p2.m * o->p2.vx + dpx2) / m2, u2y = (o->p2.m * o->p2.vy + dpy2) / m2;
    double M = m1 + m2;
    double rx = o->p2.x - o->p1.x, ry = o->p2.y - o->p1.y;
    double vx = u2x - u1x, vy = u2y - u1y;
    double r = sqrt(rx * rx + ry * ry);
    double E = 0.5 * (vx * vx + vy * vy) - M / r;
    if (!(E < 0.0)) return 0;
    double h = rx * vy - ry * vx;
    double e2 = 1.0 + 2.0 * E * h * h / (M * M);
    de[0] = -M / (2.0 * E) - el[0];
    de[1] = M - el[1];
    de[2] = m2 / m1 - el[2];
    de[3] = (e2 > 0.0 ? sqrt(e2) : 0.0) - el[3];
    return 1;
}

/* Physics::orbital_elements (physics.rs:411-417): (a, M, q, e). */
static void unperturbed_elements(const oracle_config* c, double* el)
{
    if (c->one_body) { el[0] = 1e-12; el[1] = 1.0; el[2] = 1.0; el[3] = 0.0; }
    else { el[0] = 1.0; el[1] = 1.0; el[2] = c->binary_mass_ratio; el[3] = c->binary_eccentricity; }
}

/* ItemizedChange::perturbation, state.rs:258-281: the sink and gravity items
 * of the gas are taken from the bodies (negated), buffer, cooling and fake
 * mass leave the orbit alone.  ds holds the block's sums times dx dy. */
static int block_perturbation(const oracle_config* c, const orbit* o, const double* ds, int nf, double* de)
{
    double el[4];
    unperturbed_elements(c, el);
    for (int k = 0; k < NITEMS * 4; ++k) de[k] = 0.0;
    const double* s1 = ds + SINK1 * nf;
    const double* s2 = ds + SINK2 * nf;
    const double* g1 = ds + GRAV1 * nf;
    const double* g2 = ds + GRAV2 * nf;
    int ok = 1;
    ok &= perturb(o, el, -s1[0], 0.0, -s1[1], 0.0, -s1[2], 0.0, de + SINK1 * 4);
    ok &= perturb(o, el, 0.0, -s2[0], 0.0, -s2[1], 0.0, -s2[2], de + SINK2 * 4);
    ok &= perturb(o, el, -g1[0], 0.0, -g1[1], 0.0, -g1[2], 0.0, de + GRAV1 * 4);
    ok &= perturb(o, el, 0.0, -g2[0], 0.0, -g2[1], 0.0, -g2[2], de + GRAV2 * 4);
    return ok;
}

/* Phase C: compute_block_updated_solution, scheme.rs:273-317 */
static void task_update(pool* pl, int w, int b)
{
    (void)w;
    stage_ctx* s = (stage_ctx*)pl->arg;
    const oracle_config* c = s->c;
    int nf = s->nf, bs = s->bs, nb = s->nb, n = bs * bs;
    int bi = b / nb, bj = b % nb;
    double dx = s->dx, dy = s->dx, dt = s->dt;
    const double* fx = s->fxs + (size_t)b * (bs + 1) * bs * nf;
    const double* fy = s->fys + (size_t)b * bs * (bs + 1) * nf;
    const double* uin = s->cons_in + (size_t)b * n * nf;
    const double* ubg = s->bg + (size_t)b * n * nf;
    double* uout = s->cons_out + (size_t)b * n * nf;
    double ds[NITEMS * 4];
    double it[NITEMS * 4];
    for (int k = 0; k < NITEMS * nf; ++k) ds[k] = 0.0;

    for (int i = 0; i < bs; ++i) {
        for (int j = 0; j < bs; ++j) {
            const double* fxl = fx + ((size_t)i * bs + j) * nf;
            const double* fxr = fx + ((size_t)(i + 1) * bs + j) * nf;
            const double* fyl = fy + ((size_t)i * (bs + 1) + j) * nf;
            const double* fyr = fyl + nf;
            const double* uc = uin + ((size_t)i * bs + j) * nf;
            const double* u0 = ubg + ((size_t)i * bs + j) * nf;
            double x = s->xc[bi * bs + i], y = s->xc[bj * bs + j];
            source_terms(c, uc, u0, x, y, s->time, dt, &s->o, it);
            double* out = uout + ((size_t)i * bs + j) * nf;
            for (int k = 0; k < nf; ++k) {
                double du = ((fxr[k] - fxl[k]) / dx + (fyr[k] - fyl[k]) / dy) * -dt;
                double tot = it[SINK1 * nf + k] + it[SINK2 * nf + k] + it[GRAV1 * nf + k] +
                             it[GRAV2 * nf + k] + it[BUFFER * nf + k] + it[COOLING * nf + k] +
                             it[FAKE_MASS * nf + k];
                out[k] = uc[k] + du + tot;
            }
            for (int k = 0; k < NITEMS * nf; ++k) ds[k] = ds[k] + it[k];
        }
    }
    double area = dx * dy;
    for (int k = 0; k < NITEMS * nf; ++k) ds[k] = ds[k] * area;
    if (s->led_out) {
        for (int k = 0; k < NITEMS * nf; ++k)
            s->led_out[(size_t)b * NITEMS * nf + k] = s->led_in[(size_t)b * NITEMS * nf + k] + ds[k];
    }
    /* de = ds.perturbation(time, physics.orbital_elements()), scheme.rs:307-314 */
    if (s->el_out) {
        double de[NITEMS * 4];
        s->unbound[b] = !block_perturbation(c, &s->o, ds, nf, de);
        for (int k = 0; k < NITEMS * 4; ++k)
            s->el_out[(size_t)b * NITEMS * 4 + k] = s->el_in[(size_t)b * NITEMS * 4 + k] + de[k];
    }
}

/* ======================================================================== */
/* advance (scheme.rs:323-349) with the RK schemes of godunov-core           */
/* (restated: Shu–Osher SSP forms) and the weighted averages of              */
/* state.rs:183-252.                                                         */

typedef struct rk_state {
    double* cons;
    double* led;
    double* tr;       /* tracer positions [n][2] */
    double* el;       /* orbital_elements_change [nb][nb][7][4] */
    double time;
    int64_t iteration;
} rk_state;

/* Massless tracers (no reference code: its README names them).  dx/dt =
 * v(x) with v the stage input's gas velocity, bilinear between the four
 * surrounding cell centres of the uniform mesh; the stage's weighted average
 * with the base position is taken on the same periodic image; positions wrap
 * into [-R, R). */
static void tracer_velocity(const stage_ctx* s, const double* cons, int i, int j, double* vx, double* vy)
{
    int bs = s->bs, nb = s->nb, nf = s->nf;
    const double* u = cons + ((((size_t)(i / bs) * nb + j / bs) * bs + i % bs) * bs + j % bs) * nf;
    *vx = u[1] / u[0];
    *vy = u[2] / u[0];
}

static void advance_tracers(const stage_ctx* s, const double* cons_in, const double* tin, const double* tbase,
                            double bf, double* tout, int64_t n)
{
    const double R = s->c->domain_radius, dx = s->dx, dt = s->dt, L = 2.0 * R;
    const int N = s->nb * s->bs;
    for (int64_t k = 0; k < n; ++k) {
        double x = tin[2 * k], y = tin[2 * k + 1];
        double gx = (x + R) / dx - 0.5, gy = (y + R) / dx - 0.5;
        double fi = floor(gx), fj = floor(gy);
        double ax = gx - fi, ay = gy - fj;
        int i0 = (int)fi, j0 = (int)fj;
        i0 = ((i0 % N) + N) % N;
        j0 = ((j0 % N) + N) % N;
        int i1 = i0 + 1 == N ? 0 : i0 + 1, j1 = j0 + 1 == N ? 0 : j0 + 1;
        double v00x, v00y, v10x, v10y, v01x, v01y, v11x, v11y;
        tracer_velocity(s, cons_in, i0, j0, &v00x, &v00y);
        tracer_velocity(s, cons_in, i1, j0, &v10x, &v10y);
        tracer_velocity(s, cons_in, i0, j1, &v01x, &v01y);
        tracer_velocity(s, cons_in, i1, j1, &v11x, &v11y);
        double w00 = (1.0 - ax) * (1.0 - ay), w10 = ax * (1.0 - ay), w01 = (1.0 - ax) * ay, w11 = ax * ay;
        double vx = w00 * v00x + w10 * v10x + w01 * v01x + w11 * v11x;
        double vy = w00 * v00y + w10 * v10y + w01 * v01y + w11 * v11y;
        double xo = x + dt * vx, yo = y + dt * vy;
        if (tbase) {
            double xb = tbase[2 * k], yb = tbase[2 * k + 1];
            if (xo - xb > R) xo -= L;
            else if (xo - xb < -R) xo += L;
            if (yo - yb > R) yo -= L;
            else if (yo - yb < -R) yo += L;
            xo = xo * (-bf + 1.0) + xb * bf;
            yo = yo * (-bf + 1.0) + yb * bf;
        }
        if (xo >= R) xo -= L;
        if (xo < -R) xo += L;
        if (yo >= R) yo -= L;
        if (yo < -R) yo += L;
        tout[2 * k] = xo;
        tout[2 * k + 1] = yo;
    }
}

static void weighted_average(rk_state* s1, double bf, const rk_state* s0, size_t ncons,
                             size_t nled, size_t nel)
{
    double w1 = -bf + 1.0;
    for (size_t k = 0; k < ncons; ++k) s1->cons[k] = s1->cons[k] * w1 + s0->cons[k] * bf;
    for (size_t k = 0; k < nled; ++k) s1->led[k] = s1->led[k] * w1 + s0->led[k] * bf;
    for (size_t k = 0; k < nel; ++k) s1->el[k] = s1->el[k] * w1 + s0->el[k] * bf;
    s1->time = s1->time * w1 + s0->time * bf;
}

typedef struct advance_ctx {
    stage_ctx st;
    pool* pl;
    int failed;
    oracle_error err;
    int64_t ntracers;
} advance_ctx;

/* One call of try_advance_rk: state `in` -> `out` at time in->time.  Tracers
 * are advanced here too; `base`/`bf` give the weighted average that follows
 * the stage (NULL: none). */
static int stage(advance_ctx* a, const rk_state* in, rk_state* out, const rk_state* base, double bf)
{
    stage_ctx* s = &a->st;
    s->time = in->time;
    orbital_state_from_time(s->c, in->time, &s->o);
    s->cons_in = in->cons;
    s->led_in = in->led;
    s->cons_out = out->cons;
    s->led_out = out->led;
    s->el_in = in->el;
    s->el_out = out->el;
    a->pl->arg = s;
    int nblocks = s->nb * s->nb;
    pool_run(a->pl, nblocks, task_primitive);

    /* Error surfaced in block order through the 3x3 neighbour joins
     * (scheme.rs:126, 161-165). */
    for (int b = 0; b < nblocks; ++b) {
        int bi = b / s->nb, bj = b % s->nb;
        for (int di = -1; di <= 1; ++di) {
            for (int dj = -1; dj <= 1; ++dj) {
                int ni = (bi + s->nb + di) % s->nb, nj = (bj + s->nb + dj) % s->nb;
                int nbk = ni * s->nb + nj;
                if (s->perr[nbk]) {
                    int z = s->pzone[nbk];
                    oracle_error* e = &a->err;
                    memset(e, 0, sizeof *e);
                    e->code = s->perr[nbk];
                    e->block_i = ni;
                    e->block_j = nj;
                    e->zone_i = z / s->bs;
                    e->zone_j = z % s->bs;
                    e->value = s->pbad[nbk];
                    e->x = s->xc[ni * s->bs + e->zone_i];
                    e->y = s->xc[nj * s->bs + e->zone_j];
                    e->time = in->time;
                    e->binary[0] = s->o.p1.x;
                    e->binary[1] = s->o.p1.y;
                    e->binary[2] = s->o.p2.x;
                    e->binary[3] = s->o.p2.y;
                    return e->code;
                }
            }
        }
    }
    pool_run(a->pl, nblocks, task_fluxes);
    pool_run(a->pl, nblocks, task_update);
    /* An unbound orbit fails the stage after every block's primitives were
     * converted: HydroErrorType::OrbitalEvolutionError at position (0, 0)
     * with the binary's state (scheme.rs:308-309), first block in order. */
    for (int b = 0; b < nblocks && s->el_out; ++b) {
        if (s->unbound[b]) {
            oracle_error* e = &a->err;
            memset(e, 0, sizeof *e);
            e->code = ORACLE_UNBOUND_ORBIT;
            e->block_i = b / s->nb;
            e->block_j = b % s->nb;
            e->time = in->time;
            e->binary[0] = s->o.p1.x;
            e->binary[1] = s->o.p1.y;
            e->binary[2] = s->o.p2.x;
            e->binary[3] = s->o.p2.y;
            return e->code;
        }
    }
    if (a->ntracers > 0)
        advance_tracers(s, in->cons, in->tr, base ? base->tr : NULL, bf, out->tr, a->ntracers);
    out->time = in->time + s->dt;
    out->iteration = in->iteration + 1;
    return 0;
}

double oracle_max_signal_speed(const oracle_config* c, const double* cons)
{
    int nf = nfields(c);
    size_t nz = (size_t)c->num_blocks * c->num_blocks * c->block_size * c->block_size;
    double a = 0.0;
    for (size_t z = 0; z < nz; ++z) a = fmax(zone_max_signal_speed(c, cons + z * nf), a);
    return a;
}

/* State::max_signal_speed (state.rs:121-133) over the blocks of block rows
 * [row_lo, row_hi) of a whole-mesh array: a row slab's share of the global
 * maximum, which the slabs' owners reduce with max. */
double oracle_max_signal_speed_rows(const oracle_config* c, const double* cons, int32_t row_lo, int32_t row_hi)
{
    int nf = nfields(c), nb = c->num_blocks, bs = c->block_size;
    size_t per_row = (size_t)nb * bs * bs;
    double a = 0.0;
    for (size_t z = (size_t)row_lo * per_row; z < (size_t)row_hi * per_row; ++z)
        a = fmax(zone_max_signal_speed(c, cons + z * nf), a);
    return a;
}

int oracle_advance(const oracle_config* c, double* cons, double* ledger, const double* background,
                   double* time, int64_t* iteration, int32_t fold, double* dt_out,
                   int32_t nthreads, oracle_error* err, double* tracers, int64_t ntracers,
                   double* elements)
{
    int nf = nfields(c), nb = c->num_blocks, bs = c->block_size;
    int nblocks = nb * nb;
    size_t ncons = (size_t)nblocks * bs * bs * nf;
    size_t nled = (size_t)nblocks * NITEMS * nf;
    size_t nel = elements ? (size_t)nblocks * NITEMS * 4 : 0;
    if (nthreads < 1) nthreads = 1;

    /* dt, scheme.rs:336-340 */
    double dx = cell_spacing(c);
    double dt = c->cfl * dx / oracle_max_signal_speed(c, cons);
    if (c->has_dt_min) dt = fmax(dt, c->dt_min);
    if (dt_out) *dt_out = dt;

    advance_ctx a;
    memset(&a, 0, sizeof a);
    stage_ctx* s = &a.st;
    s->c = c;
    s->nf = nf;
    s->nb = nb;
    s->bs = bs;
    s->dx = dx;
    s->dt = dt;
    s->bg = background;
    s->xc = malloc(sizeof(double) * nb * bs);
    s->xv = malloc(sizeof(double) * nb * (bs + 1));
    for (int b = 0; b < nb; ++b) {
        oracle_cell_centers(c, b, s->xc + b * bs);
        oracle_block_vertices(c, b, s->xv + b * (bs + 1));
    }
    s->prim = malloc(sizeof(double) * ncons);
    s->perr = calloc(nblocks, sizeof(int));
    s->pbad = calloc(nblocks, sizeof(double));
    s->pzone = calloc(nblocks, sizeof(int));
    s->unbound = calloc(nblocks, sizeof(int));
    s->fxs = malloc(sizeof(double) * (size_t)nblocks * (bs + 1) * bs * nf);
    s->fys = malloc(sizeof(double) * (size_t)nblocks * (bs + 1) * bs * nf);
    size_t E = bs + 4;
    size_t scratch = (E * E + 2 * (bs + 2) * E) * nf;
    s->scratch = malloc(sizeof(double*) * nthreads);
    for (int t = 0; t < nthreads; ++t) s->scratch[t] = malloc(sizeof(double) * scratch);

    /* five state slots: s0 (input), s1, s2, s3 and a spare */
    rk_state st[4];
    a.ntracers = tracers ? ntracers : 0;
    for (int k = 0; k < 4; ++k) {
        st[k].cons = malloc(sizeof(double) * ncons);
        st[k].led = calloc(nled, sizeof(double));
        st[k].tr = a.ntracers > 0 ? malloc(sizeof(double) * 2 * (size_t)a.ntracers) : NULL;
        st[k].el = nel ? malloc(sizeof(double) * nel) : NULL;
    }
    if (nel) memcpy(st[0].el, elements, sizeof(double) * nel);
    if (a.ntracers > 0) memcpy(st[0].tr, tracers, sizeof(double) * 2 * (size_t)a.ntracers);
    memcpy(st[0].cons, cons, sizeof(double) * ncons);
    if (ledger) memcpy(st[0].led, ledger, sizeof(double) * nled);
    st[0].time = *time;
    st[0].iteration = *iteration;

    pool pl;
    memset(&pl, 0, sizeof pl);
    pl.nthreads = nthreads;
    pthread_t* th = NULL;
    worker_arg* wa = NULL;
    if (nthreads > 1) {
        pthread_barrier_init(&pl.barrier, NULL, nthreads);
        th = malloc(sizeof(pthread_t) * nthreads);
        wa = malloc(sizeof(worker_arg) * nthreads);
        for (int t = 1; t < nthreads; ++t) {
            wa[t].pl = &pl;
            wa[t].id = t;
            pthread_create(&th[t], NULL, worker_main, &wa[t]);
        }
    }
    a.pl = &pl;

    int rc = 0;
    for (int f = 0; f < fold && !rc; ++f) {
        rk_state* s0 = &st[0];
        if (c->rk_order == 1) {
            rc = stage(&a, s0, &st[1], NULL, 0.0);
            if (!rc) { rk_state t = st[0]; st[0] = st[1]; st[1] = t; }
        } else if (c->rk_order == 2) {
            rc = stage(&a, s0, &st[1], NULL, 0.0);
            if (!rc) rc = stage(&a, &st[1], &st[2], s0, 0.5);
            if (!rc) {
                weighted_average(&st[2], 0.5, s0, ncons, nled, nel);      /* br = 1/2 */
                st[2].iteration = (st[2].iteration + s0->iteration) / 2;
                rk_state t = st[0]; st[0] = st[2]; st[2] = t;
            }
        } else {
            rc = stage(&a, s0, &st[1], NULL, 0.0);
            if (!rc) rc = stage(&a, &st[1], &st[2], s0, 3.0 / 4.0);
            if (!rc) {
                weighted_average(&st[2], 3.0 / 4.0, s0, ncons, nled, nel); /* br = 3/4 */
                rc = stage(&a, &st[2], &st[3], s0, 1.0 / 3.0);
            }
            if (!rc) {
                weighted_average(&st[3], 1.0 / 3.0, s0, ncons, nled, nel); /* br = 1/3 */
                st[3].iteration = s0->iteration + 1;
                rk_state t = st[0]; st[0] = st[3]; st[3] = t;
            }
        }
    }

    if (nthreads > 1) {
        pl.quit = 1;
        pthread_barrier_wait(&pl.barrier);
        for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
        pthread_barrier_destroy(&pl.barrier);
        free(th);
        free(wa);
    }

    if (!rc) {
        memcpy(cons, st[0].cons, sizeof(double) * ncons);
        if (ledger) memcpy(ledger, st[0].led, sizeof(double) * nled);
        *time = st[0].time;
        *iteration = st[0].iteration;
        if (a.ntracers > 0) memcpy(tracers, st[0].tr, sizeof(double) * 2 * (size_t)a.ntracers);
        if (nel) memcpy(elements, st[0].el, sizeof(double) * nel);
    } else if (err) {
        *err = a.err;
    }

    for (int k = 0; k < 4; ++k) { free(st[k].cons); free(st[k].led); free(st[k].tr); free(st[k].el); }
    for (int t = 0; t < nthreads; ++t) free(s->scratch[t]);
    free(s->scratch);
    free(s->xc); free(s->xv); free(s->prim); free(s->perr); free(s->pbad); free(s->pzone); free(s->unbound);
    free(s->fxs); free(s->fys);
    return rc;
}

/* One RK stage (try_advance_rk, scheme.rs:88-173) of the blocks in block
 * rows [row_lo, row_hi) only: the unit of work of a split of the mesh into
 * row slabs, one per rank (no counterpart in the reference, which advances
 * every block in one process).  The arrays are whole-mesh, block layout; of
 * cons_in the stage reads the slab and its halo rows, the 2 zone rows on
 * either side that the halo extension takes from the neighbouring block rows
 * (extend_from_neighbor_arrays_2d with 2 guard zones, scheme.rs:126-127;
 * periodic neighbours, mesh.rs:101-110), so a rank that holds its slab and
 * the neighbours' edge rows computes its blocks exactly as a whole-mesh
 * stage does.  (The primitives of the neighbouring block rows are converted
 * whole, but only their halo rows are read, and a failure is reported for
 * the slab's own blocks: a neighbour's failure is its owner's to report.)
 * With base_cons the weighted average out = out (1 - bf) + base bf follows,
 * for the state and the ledger (state.rs:183-199).  Single-threaded; the
 * orbital-element change is not tracked.  Returns 0 or the error code of the
 * slab's first failing block in block order. */
int oracle_stage_rows(const oracle_config* c, const double* cons_in, double* cons_out, const double* base_cons,
                      double bf, const double* background, const double* led_in, double* led_out,
                      const double* led_base, double time, double dt, int32_t row_lo, int32_t row_hi,
                      oracle_error* err)
{
    int nf = nfields(c), nb = c->num_blocks, bs = c->block_size;
    int nblocks = nb * nb, n = bs * bs;
    if (row_lo < 0 || row_hi > nb || row_lo >= row_hi) return -1;
    size_t ncons = (size_t)nblocks * n * nf;
    advance_ctx a;
    memset(&a, 0, sizeof a);
    stage_ctx* s = &a.st;
    s->c = c;
    s->nf = nf;
    s->nb = nb;
    s->bs = bs;
    s->dx = cell_spacing(c);
    s->dt = dt;
    s->time = time;
    s->bg = background;
    orbital_state_from_time(c, time, &s->o);
    s->cons_in = cons_in;
    s->cons_out = cons_out;
    s->led_in = led_in;
    s->led_out = led_out;
    s->xc = malloc(sizeof(double) * nb * bs);
    s->xv = malloc(sizeof(double) * nb * (bs + 1));
    for (int b = 0; b < nb; ++b) {
        oracle_cell_centers(c, b, s->xc + b * bs);
        oracle_block_vertices(c, b, s->xv + b * (bs + 1));
    }
    s->prim = malloc(sizeof(double) * ncons);
    s->perr = calloc(nblocks, sizeof(int));
    s->pbad = calloc(nblocks, sizeof(double));
    s->pzone = calloc(nblocks, sizeof(int));
    s->unbound = calloc(nblocks, sizeof(int));
    s->fxs = malloc(sizeof(double) * (size_t)nblocks * (bs + 1) * bs * nf);
    s->fys = malloc(sizeof(double) * (size_t)nblocks * (bs + 1) * bs * nf);
    size_t E = bs + 4;
    double* scratch = malloc(sizeof(double) * (E * E + 2 * (bs + 2) * E) * nf);
    s->scratch = &scratch;
    pool pl;
    memset(&pl, 0, sizeof pl);
    pl.nthreads = 1;
    pl.arg = s;

    /* phase A over the slab and the block rows on either side (for the halo) */
    for (int bi = row_lo - 1; bi <= row_hi; ++bi) {
        int ri = (bi % nb + nb) % nb;
        for (int bj = 0; bj < nb; ++bj) task_primitive(&pl, 0, ri * nb + bj);
    }
    int rc = 0;
    for (int b = row_lo * nb; b < row_hi * nb && !rc; ++b) {
        if (s->perr[b]) {
            oracle_error* e = &a.err;
            memset(e, 0, sizeof *e);
            e->code = s->perr[b];
            e->block_i = b / nb;
            e->block_j = b % nb;
            e->zone_i = s->pzone[b] / bs;
            e->zone_j = s->pzone[b] % bs;
            e->value = s->pbad[b];
            e->x = s->xc[e->block_i * bs + e->zone_i];
            e->y = s->xc[e->block_j * bs + e->zone_j];
            e->time = time;
            e->binary[0] = s->o.p1.x;
            e->binary[1] = s->o.p1.y;
            e->binary[2] = s->o.p2.x;
            e->binary[3] = s->o.p2.y;
            rc = e->code;
        }
    }
    if (!rc) {
        for (int b = row_lo * nb; b < row_hi * nb; ++b) task_fluxes(&pl, 0, b);
        for (int b = row_lo * nb; b < row_hi * nb; ++b) task_update(&pl, 0, b);
        if (base_cons) {
            double w1 = -bf + 1.0;
            size_t z0 = (size_t)row_lo * nb * n * nf, z1 = (size_t)row_hi * nb * n * nf;
            for (size_t k = z0; k < z1; ++k) cons_out[k] = cons_out[k] * w1 + base_cons[k] * bf;
            if (led_out && led_base) {
                size_t l0 = (size_t)row_lo * nb * NITEMS * nf, l1 = (size_t)row_hi * nb * NITEMS * nf;
                for (size_t k = l0; k < l1; ++k) led_out[k] = led_out[k] * w1 + led_base[k] * bf;
            }
        }
    } else if (err) {
        *err = a.err;
    }
    free(scratch);
    free(s->xc); free(s->xv); free(s->prim); free(s->perr); free(s->pbad); free(s->pzone); free(s->unbound);
    free(s->fxs); free(s->fys);
    return rc;
}

/* ======================================================================== */
/* Initial state: BlockState::from_model (state.rs:74-86) for InfiniteDisk   */
/* (disks.rs:137-157), plus the synthetic cavity and seeded noise (new).     */

/* SplitMix64 finaliser (Steele, Lea & Flood 2014; Vigna's public-domain
 * constants) used as a counter-based hash. */
static uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double zone_uniform(uint64_t seed, int run, int gi, int gj)
{
    uint64_t h = mix64(mix64(mix64(seed) ^ (uint64_t)(uint32_t)run) ^
                       (((uint64_t)(uint32_t)gi << 32) | (uint64_t)(uint32_t)gj));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

/* InitialModel::primitive_at (disks.rs): InfiniteDisk 137-157,
 * InfiniteAlphaDisk 172-193, FiniteDisk 20-115, ResidualTest 208-228. */
static void model_primitive(const oracle_config* c, const oracle_disk_model* m, double x, double y, double* p)
{
    double gm = c->hydro_kind == 1 ? c->gamma_law_index : 1.0;
    double r = sqrt(x * x + y * y);
    double mach = c->hydro_kind == 0 ? c->mach_number : m->mach_number;
    double sd, vx, vy, pg;
    if (m->kind == 1) {
        sd = m->surface_density * pow(r, -3.0 / 5.0);
        double vp = pow(r, -0.5);
        vx = vp * (-y / r);
        vy = vp * (x / r);
        double ma = mach * pow(r, -1.0 / 20.0);
        double cs = vp / ma;
        pg = cs * cs * sd / gm;
    } else if (m->kind == 2) {
        double r0 = m->disk_radius, dr = m->disk_width, md = m->disk_mass, rs = m->disk_softening;
        double pi = 3.14159265358979323846;
        double q0 = r0 / dr;
        double total = pi * dr * dr * (exp(-(q0 * q0)) + sqrt(pi) * r0 / dr * (1.0 + erf(r0 / dr)));
        double sigma0 = md / total;
        double vp = pow(r, -0.5);
        vx = vp * (-y / r);
        vy = vp * (x / r);
        double z = (r - r0) / dr;
        sd = sigma0 * exp(-(z * z));
        double kep2 = 1.0 * 1.0 * r * r / pow(r * r + rs * rs, 1.5);
        double cs2 = kep2 / (mach * mach);
        pg = sd * cs2 / gm;
    } else if (m->kind == 3) {
        double phi = atan2(x, y);
        double r1 = sqrt((x - 1.0) * (x - 1.0) + (y - 1.0) * (y - 1.0));
        double r2 = sqrt((x + 1.0) * (x + 1.0) + (y + 1.0) * (y + 1.0));
        sd = 1.0 + exp(-(r1 * r1));
        pg = 1.0 + exp(-(r2 * r2));
        double damp = exp(-5.0 / r - r * r / 3.0);
        double vp = pow(r, -0.5) * damp;
        double vr = sin(phi - 3.14159 / 4.0) * damp;
        vx = vp * (-y / r) + vr * (x / r);
        vy = vp * (x / r) + vr * (y / r);
    } else {
        sd = m->surface_density;
        double vp = pow(r, -0.5);
        vx = vp * (-y / r);
        vy = vp * (x / r);
        double cs = vp / mach;
        pg = cs * cs * sd / gm;
    }
    p[0] = sd;
    p[1] = vx;
    p[2] = vy;
    p[3] = pg;
}

int oracle_initial_state(const oracle_config* c, const oracle_disk_model* m, double* cons)
{
    int nf = nfields(c), nb = c->num_blocks, bs = c->block_size;
    double* xc = malloc(sizeof(double) * nb * bs);
    for (int b = 0; b < nb; ++b) oracle_cell_centers(c, b, xc + b * bs);
    for (int bi = 0; bi < nb; ++bi)
        for (int bj = 0; bj < nb; ++bj)
            for (int i = 0; i < bs; ++i)
                for (int j = 0; j < bs; ++j) {
                    double x = xc[bi * bs + i], y = xc[bj * bs + j];
                    double r = sqrt(x * x + y * y);
                    double p[4];
                    model_primitive(c, m, x, y, p);
                    if (r < m->core_radius) {
                        /* synthetic solid-body core: v and c_s scaled by (r / r_core)^(3/2) */
                        double s = pow(r / m->core_radius, 1.5);
                        p[1] = p[1] * s;
                        p[2] = p[2] * s;
                        p[3] = p[3] * (s * s);
                    }
                    if (m->edge_width > 0.0) {
                        /* synthetic: at rest at the domain edge */
                        double w = m->edge_width;
                        double f = 0.5 * (1.0 - tanh((r - (c->domain_radius - w)) / (0.3 * w)));
                        p[1] = p[1] * f;
                        p[2] = p[2] * f;
                    }
                    if (m->cavity_radius > 0.0) {
                        double f = fmax(m->cavity_floor, exp(-pow(m->cavity_radius / r, 12.0)));
                        p[0] = p[0] * f;
                        p[3] = p[3] * f;
                    }
                    if (m->noise != 0.0) {
                        double u = zone_uniform(m->seed, m->run, bi * bs + i, bj * bs + j);
                        double f = 1.0 + m->noise * (2.0 * u - 1.0);
                        p[0] = p[0] * f;
                        p[3] = p[3] * f;
                    }
                    size_t z = (((size_t)(bi * nb + bj) * bs + i) * bs + j) * nf;
                    prim_to_cons(c, p, cons + z);
                }
    free(xc);
    return 0;
}
