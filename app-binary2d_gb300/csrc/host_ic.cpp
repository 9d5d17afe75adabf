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

}  // namespace b2d

// BlockState::from_model (src/state.rs:74-86) with InfiniteDiskModel::primitive_at
// (src/disks.rs:137-157): Σ constant, Keplerian v_φ = r^-1/2, c_s = v_φ / Mach,
// p = c_s² Σ / γ; then the synthetic cavity and noise described in b2d.h.
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
                        double sd = m->surface_density;
                        if (m->cavity_radius > 0.0)
                            sd = sd * std::fmax(m->cavity_floor, std::exp(-std::pow(m->cavity_radius / r, 12.0)));
                        if (m->noise != 0.0) {
                            double u = b2d::zone_uniform(m->seed, m->run, bi * bs + i, bj * bs + j);
                            sd = sd * (1.0 + m->noise * (2.0 * u - 1.0));
                        }
                        double vp = std::pow(r, -0.5);
                        double vx = vp * (-y / r);
                        double vy = vp * (x / r);
                        double cs = vp / mach;
                        double pg = cs * cs * sd / gm;
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
