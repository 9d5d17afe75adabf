// host_ic.cpp — host-side mesh geometry and initial conditions.
//
// Compiled with -ffp-contract=off so the tables and initial states are the
// same on every host architecture.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <thread>
#include <vector>

#include "../../include/b2d.h"

namespace b2d {

// Mesh::block_vertices (src/mesh.rs:42-47): ndarray linspace from the block
// start to start + block_length with block_size + 1 points.
void host_block_vertices(const b2d_config* c, int b, double* xv)
{
    double L = 2.0 * c->domain_radius / (double)c->num_blocks;  // mesh.rs:27-29
    double start = -c->domain_radius + (double)b * L;              // mesh.rs:31-36
    double end = start + L;
    double step = (end - start) / (double)c->block_size;
    for (int k = 0; k <= c->block_size; ++k) xv[k] = start + step * (double)k;
}

// Mesh::cell_centers (src/mesh.rs:49-54): adjacent means of the vertices.
void host_cell_centers(const b2d_config* c, int b, double* xc)
{
    std::vector<double> xv(c->block_size + 1);
    host_block_vertices(c, b, xv.data());
    for (int k = 0; k < c->block_size; ++k) xc[k] = (xv[k] + xv[k + 1]) * 0.5;
}

// Counter-based uniform deviate keyed by (seed, run, global zone index):
// SplitMix64 finaliser (Steele, Lea & Flood 2014).
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

// InitialModel::primitive_at of the reference's models (src/disks.rs):
// (Σ, vx, vy, p) at (x, y) before the synthetic cavity and noise.
static void model_primitive(const b2d_config* c, const b2d_disk_model* m, double x, double y, double* p)
{
    const double gm = c->hydro_kind == B2D_EULER ? c->gamma_law_index : 1.0;
    const double r = std::sqrt(x * x + y * y);
    // hydro.global_mach_number().or(model.mach_number): isothermal uses its own
    const double mach = c->hydro_kind == B2D_ISOTHERMAL ? c->mach_number : m->mach_number;
    double sd, vx, vy, pg;
    if (m->kind == B2D_MODEL_INFINITE_ALPHA_DISK) {                  // disks.rs:172-193
        sd = m->surface_density * std::pow(r, -3.0 / 5.0);
        double vp = std::pow(r, -0.5);
        vx = vp * (-y / r);
        vy = vp * (x / r);
        double ma = mach * std::pow(r, -1.0 / 20.0);
        double cs = vp / ma;
        pg = cs * cs * sd / gm;
    } else if (m->kind == B2D_MODEL_FINITE_DISK) {                   // disks.rs:20-115
        const double r0 = m->disk_radius, dr = m->disk_width, md = m->disk_mass, rs = m->disk_softening;
        const double pi = 3.14159265358979323846;
        const double q0 = r0 / dr;
        const double total = pi * dr * dr * (std::exp(-(q0 * q0)) + std::sqrt(pi) * r0 / dr * (1.0 + std::erf(r0 / dr)));
        const double sigma0 = md / total;
        double vp = std::pow(r, -0.5);
        vx = vp * (-y / r);
        vy = vp * (x / r);
        double z = (r - r0) / dr;
        sd = sigma0 * std::exp(-(z * z));
        double kep2 = 1.0 * 1.0 * r * r / std::pow(r * r + rs * rs, 1.5);
        double cs2 = kep2 / (mach * mach);
        pg = sd * cs2 / gm;
    } else if (m->kind == B2D_MODEL_RESIDUAL_TEST) {                 // disks.rs:208-228
        double phi = std::atan2(x, y);
        double r1 = std::sqrt((x - 1.0) * (x - 1.0) + (y - 1.0) * (y - 1.0));
        double r2 = std::sqrt((x + 1.0) * (x + 1.0) + (y + 1.0) * (y + 1.0));
        sd = 1.0 + std::exp(-(r1 * r1));
        pg = 1.0 + std::exp(-(r2 * r2));
        double damp = std::exp(-5.0 / r - r * r / 3.0);
        double vp = std::pow(r, -0.5) * damp;
        double vr = std::sin(phi - 3.14159 / 4.0) * damp;
        vx = vp * (-y / r) + vr * (x / r);
        vy = vp * (x / r) + vr * (y / r);
    } else {                                                          // disks.rs:137-157
        sd = m->surface_density;
        double vp = std::pow(r, -0.5);
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

}  // namespace b2d

// BlockState::from_model (src/state.rs:74-86): the model's primitive at each
// cell centre, then the synthetic cavity and noise described in b2d.h, then
// to_conserved.
extern "C" b2d_status b2d_initial_state(const b2d_config* c, const b2d_disk_model* m, double* cons)
{
    if (!c || !m || !cons) return B2D_ERR_INVALID;
    const int nf = c->hydro_kind == B2D_EULER ? 4 : 3;
    const int nb = c->num_blocks, bs = c->block_size;
    std::vector<double> xc((size_t)nb * bs);
    for (int b = 0; b < nb; ++b) b2d::host_cell_centers(c, b, xc.data() + (size_t)b * bs);
    const double gm = c->hydro_kind == B2D_EULER ? c->gamma_law_index : 1.0;
    const double mach = c->hydro_kind == B2D_ISOTHERMAL ? c->mach_number : m->mach_number;

    auto fill_rows = [&](int bi0, int bi1) {
        for (int bi = bi0; bi < bi1; ++bi)
            for (int bj = 0; bj < nb; ++bj)
                for (int i = 0; i < bs; ++i)
                    for (int j = 0; j < bs; ++j) {
                        double x = xc[(size_t)bi * bs + i], y = xc[(size_t)bj * bs + j];
                        double r = std::sqrt(x * x + y * y);
                        double p[4];
                        b2d::model_primitive(c, m, x, y, p);
                        double sd = p[0], vx = p[1], vy = p[2], pg = p[3];
                        if (r < m->core_radius) {
                            // solid-body core: v and c_s scaled by (r / r_core)^(3/2)
                            double s = std::pow(r / m->core_radius, 1.5);
                            vx = vx * s;
                            vy = vy * s;
                            pg = pg * (s * s);
                        }
                        if (m->edge_width > 0.0) {
                            // synthetic: at rest at the domain edge
                            const double w = m->edge_width;
                            const double f = 0.5 * (1.0 - std::tanh((r - (c->domain_radius - w)) / (0.3 * w)));
                            vx = vx * f;
                            vy = vy * f;
                        }
                        if (m->cavity_radius > 0.0) {
                            double f = std::fmax(m->cavity_floor, std::exp(-std::pow(m->cavity_radius / r, 12.0)));
                            sd = sd * f;
                            pg = pg * f;
                        }
                        if (m->noise != 0.0) {
                            double u = b2d::zone_uniform(m->seed, m->run, bi * bs + i, bj * bs + j);
                            double f = 1.0 + m->noise * (2.0 * u - 1.0);
                            sd = sd * f;
                            pg = pg * f;
                        }
                        double* u = cons + ((((size_t)bi * nb + bj) * bs + i) * bs + j) * nf;
                        u[0] = sd;
                        u[1] = sd * vx;
                        u[2] = sd * vy;
                        if (nf == 4) u[3] = 0.5 * sd * (vx * vx + vy * vy) + pg / (gm - 1.0);
                    }
    };
    unsigned nt = std::thread::hardware_concurrency();
    if (nt == 0) nt = 1;
    nt = std::min<unsigned>(nt, (unsigned)nb);
    std::vector<std::thread> th;
    for (unsigned k = 0; k < nt; ++k) {
        int a = (int)((size_t)nb * k / nt), b = (int)((size_t)nb * (k + 1) / nt);
        th.emplace_back(fill_rows, a, b);
    }
    for (auto& t : th) t.join();
    return B2D_OK;
}
