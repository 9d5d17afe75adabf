/*
 * oracle.h — CPU FP64 restatement of binary2d's explicit finite-volume step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the
 * CUDA path and the timed CPU baseline; nothing in the product links it.
 *
 * PARITY UNPINNED.  The reference (clemson-cal/app-binary2d 0.2.1) is Rust
 * and cannot be built here (no cargo/rustc), it ships no tests, golden vectors
 * or fixtures, and its per-zone arithmetic lives in five un-vendored git
 * dependencies (Cargo.lock:201-305):
 *     godunov-core     @ d8dd524ad7bb0e0a83f976a1a3cca335e3432b07  (PLM, RK)
 *     hydro-iso2d      @ eb18a386dabd7fda0dbfd2eb940fcbb393a58fe5  (iso HLLE)
 *     hydro-euler      @ fc929f9b00da8bb8546fa10c0ef59f909791428f  (Euler HLLE)
 *     kepler-two-body  @ 2d8a0f5374052ab7f4f60c5bbbc37c4e5283b4a4  (Kepler)
 *     ndarray-ops      @ 725bc21610a040bd305ea32c9cd4700469edbdb7  (stencils)
 * Those functions are restated here from their published methods
 * (generalised-minmod PLM, HLLE with outer-wave estimates, Shu–Osher SSP
 * Runge–Kutta, Newton solution of Kepler's equation); the code in src/ of the
 * reference is restated line by line with file:line citations in oracle.c.
 *
 * The config struct below has exactly the layout of b2d_config in the
 * product's C ABI, so one ctypes description serves both libraries.
 */
#ifndef B2D_ORACLE_H
#define B2D_ORACLE_H

#include <stdint.h>

typedef struct oracle_config {
    int32_t num_blocks;
    int32_t block_size;
    double  domain_radius;
    int32_t hydro_kind;
    int32_t density_index;
    double  mach_number;
    double  gamma_law_index;
    double  cooling_coefficient;
    double  pressure_floor;
    double  density_floor;
    int32_t has_pressure_floor;
    int32_t has_density_floor;
    int32_t cooling_slow_start;
    int32_t cooling_kind;
    double  cooling_beta;
    double  buffer_rate;
    double  buffer_scale;
    double  binary_eccentricity;
    double  binary_mass_ratio;
    double  lambda_multiplier;
    double  viscosity;
    int32_t viscosity_kind;
    int32_t sink_model;
    double  cfl;
    double  plm;
    double  plm_density_trigger;
    double  fake_mass_threshold;
    double  fake_mass_rate;
    double  mach_ceiling;
    double  sink_radius;
    double  sink_rate;
    double  softening_length;
    double  dt_min;
    int32_t has_plm_density_trigger;
    int32_t one_body;
    int32_t rk_order;
    int32_t has_mach_ceiling;
    int32_t has_softening_length;
    int32_t has_dt_min;
} oracle_config;

typedef struct oracle_error {
    int32_t code;
    int32_t run;
    int32_t block_i, block_j, zone_i, zone_j;
    double  value;
    double  x, y;
    double  time;
    double  binary[4];
} oracle_error;

typedef struct oracle_disk_model {
    double   surface_density;
    double   mach_number;
    double   cavity_radius;
    double   cavity_floor;
    double   noise;
    uint64_t seed;
    int32_t  run;
    int32_t  kind;   /* 0 infinite, 1 infinite alpha, 2 finite, 3 residual test */
    double   disk_mass;
    double   disk_width;
    double   disk_radius;
    double   disk_softening;
    double   core_radius;
    double   edge_width;
} oracle_disk_model;

/* m, x, y, vx, vy of each body */
typedef struct oracle_point_mass { double m, x, y, vx, vy; } oracle_point_mass;

#define ORACLE_OK 0
#define ORACLE_NEG_DENSITY 1
#define ORACLE_NEG_PRESSURE 2
#define ORACLE_UNBOUND_ORBIT 3

/* scheme::advance: fold RK steps with one dt; cons [nb][nb][bs][bs][nf],
 * ledger [nb][nb][7][nf] (may be NULL), background like cons, elements the
 * orbital_elements_change [nb][nb][7][4] of (a, M, q, e) (may be NULL). */
int oracle_advance(const oracle_config* cfg, double* cons, double* ledger,
                   const double* background, double* time, int64_t* iteration,
                   int32_t fold, double* dt_out, int32_t nthreads,
                   oracle_error* err, double* tracers /* [n][2] or NULL */,
                   int64_t ntracers, double* elements /* or NULL */);

double oracle_max_signal_speed(const oracle_config* cfg, const double* cons);

/* The maximum signal speed over block rows [row_lo, row_hi). */
double oracle_max_signal_speed_rows(const oracle_config* cfg, const double* cons, int32_t row_lo,
                                    int32_t row_hi);

/* One RK stage of the blocks in block rows [row_lo, row_hi) of whole-mesh
 * arrays (a row slab of a split mesh): reads the slab and its 2-zone halo
 * rows of cons_in; base_cons (or NULL) with weight bf gives the RK average. */
int oracle_stage_rows(const oracle_config* cfg, const double* cons_in, double* cons_out,
                      const double* base_cons, double bf, const double* background,
                      const double* led_in, double* led_out, const double* led_base,
                      double time, double dt, int32_t row_lo, int32_t row_hi,
                      oracle_error* err);

int oracle_initial_state(const oracle_config* cfg, const oracle_disk_model* m,
                         double* cons);

void oracle_orbital_state(const oracle_config* cfg, double t,
                          oracle_point_mass* p1, oracle_point_mass* p2);

/* Pointwise pieces, exposed for identity tests. */
double oracle_plm_gradient(double theta, double a, double b, double c);
void oracle_hlle(const oracle_config* cfg, const double* pl, const double* pr,
                 int32_t axis, double cs2, double* flux);
void oracle_physical_flux(const oracle_config* cfg, const double* p,
                          int32_t axis, double cs2, double* flux);
void oracle_prim_to_cons(const oracle_config* cfg, const double* p, double* u);
int oracle_cons_to_prim(const oracle_config* cfg, const double* u, double* p);
void oracle_source_terms(const oracle_config* cfg, const double* u,
                         const double* u0, double x, double y, double t,
                         double dt, double* items /* [7][nf] */);
void oracle_cell_centers(const oracle_config* cfg, int32_t block, double* xc);
void oracle_block_vertices(const oracle_config* cfg, int32_t block, double* xv);

#endif
