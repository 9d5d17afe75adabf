// api.cu — the C ABI of include/b2d.h: contexts, state transfer, and the
// advance driver (the role of scheme::advance, src/scheme.rs:323-349).
//
// Built with --fmad=false: the Kepler solve and the time bookkeeping of the
// prologue kernel round exactly like the FP64 CPU restatement.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "elements.cuh"
#include "runtime.cuh"

namespace b2d {
cudaError_t launch_stage_f64(int nf, const StageArgs& a, int grid, int tw, size_t smem, cudaStream_t s);
cudaError_t launch_stage_f32(int nf, int store, const StageArgs& a, int grid, int tw, size_t smem, cudaStream_t s);
int stage_ctas_per_sm(int nf, int store, int nruns, int tw);
void host_block_vertices(const b2d_config* c, int b, double* xv);
void host_cell_centers(const b2d_config* c, int b, double* xc);
}  // namespace b2d

using namespace b2d;

static thread_local std::string g_last_error;

static b2d_status fail(b2d_status s, const std::string& msg)
{
    g_last_error = msg;
    return s;
}

#define CUDA_TRY(expr)                                                                              \
    do {                                                                                            \
        cudaError_t e_ = (expr);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(B2D_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));          \
    } while (0)

extern "C" const char* b2d_last_error(void) { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// Device kernels of the runtime.

// Two-body orbit at time t: OrbitalElements::orbital_state_from_time
// (kepler-two-body, restated; called at physics.rs:419-421).  Elements
// (a, M, q, e) = (1, 1, q, e), or (1e-12, 1, 1, 0) for one_body
// (physics.rs:411-417).  Periapsis on +x at t = 0; Newton iteration on
// Kepler's equation E - e sin E = n t from E = n t.
__device__ void kepler_orbit(const RunDev& rd, double t, double* o)
{
    double a, M, q, e;
    if (rd.p.one_body) { a = 1e-12; M = 1.0; q = 1.0; e = 0.0; }
    else { a = 1.0; M = 1.0; q = rd.binary_q; e = rd.binary_e; }
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
    o[0] = m1; o[1] = -x * f1; o[2] = -y * f1; o[3] = -vx * f1; o[4] = -vy * f1;
    o[5] = m2; o[6] = x * f2; o[7] = y * f2; o[8] = vx * f2; o[9] = vy * f2;
}

// Start of an advance, one CTA per run: dt = cfl·dx / max signal speed
// (floored by dt_min, scheme.rs:336-340), the stage times of all `fold` RK
// steps (try_advance_rk stamps t + dt, scheme.rs:168-170; weighted_average
// averages time, state.rs:213-214), and the binary at each stage time.
__global__ void prologue_kernel(const RunDev* runs, int fold, int rk, int start, int final_slot,
                                const unsigned long long* err_key, long long* adv_count)
{
    const RunDev& rd = runs[blockIdx.x];
    const int stages = rk;
    __shared__ int failed;
    // a failure is pending: this advance and every later one are abandoned
    if (threadIdx.x == 0) failed = (*(volatile const unsigned long long*)err_key != ~0ull);
    __syncthreads();
    if (failed) return;
    if (threadIdx.x == 0 && blockIdx.x == 0) *adv_count += 1;
    if (threadIdx.x == 0) {
        double amax = __longlong_as_double((long long)*rd.amax);
        double dt = rd.p.cfl * rd.p.dx / amax;
        if (rd.p.has_dt_min) dt = fmax(dt, rd.p.dt_min);
        *rd.dt = dt;
        *rd.amax = 0ull;
        double t = rd.time[start];
        int s = 0;
        for (int f = 0; f < fold; ++f) {
            const double t0 = t;
            if (rk == 1) {
                rd.stage_time[s++] = t0;
                t = t0 + dt;
            } else if (rk == 2) {
                rd.stage_time[s++] = t0;
                double t1 = t0 + dt;
                rd.stage_time[s++] = t1;
                double t2 = t1 + dt;
                t = t2 * (-0.5 + 1.) + t0 * 0.5;
            } else {
                rd.stage_time[s++] = t0;
                double t1 = t0 + dt;
                rd.stage_time[s++] = t1;
                double t2 = t1 + dt;
                double t2a = t2 * (-0.75 + 1.) + t0 * 0.75;
                rd.stage_time[s++] = t2a;
                double t3 = t2a + dt;
                const double bf = 1.0 / 3.0;
                t = t3 * (-bf + 1.) + t0 * bf;
            }
        }
        rd.time[final_slot] = t;
        rd.iter[final_slot] = rd.iter[start] + fold;
    }
    __syncthreads();
    for (int s = threadIdx.x; s < fold * stages; s += blockDim.x) kepler_orbit(rd, rd.stage_time[s], rd.orbit + 10 * s);
}

// State::max_signal_speed (state.rs:121-133) of one run's slot, in the
// precision the stage kernels use for it at the end of an advance: FP64 for
// the FP64 path, FP32 of the stored (high) words for the FP32 paths (FP64
// divisions and roots on a whole mesh are slow on this GPU).
template <int NF, int STORE, class R>
__global__ void max_speed_kernel(const RunDev* runs, int run, int slot)
{
    const RunDev& rd = runs[run];
    const size_t nn = (size_t)rd.N * rd.N;
    // a row slab's zones only (its block rows are contiguous in the planes)
    const size_t z0 = rd.slab_hi > 0 ? (size_t)rd.slab_lo * rd.bs * rd.N : 0;
    const size_t z1 = rd.slab_hi > 0 ? (size_t)rd.slab_hi * rd.bs * rd.N : nn;
    R a = R(0);
    for (size_t z = z0 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; z < z1; z += (size_t)gridDim.x * blockDim.x) {
        R u[NF];
        for (int f = 0; f < NF; ++f) {
            if (STORE == 0) u[f] = (R)((const double*)rd.slot[slot])[f * nn + z];
            else u[f] = (R)((const float*)rd.slot[slot])[(2 * f) * nn + z];
        }
        a = rmax(max_signal_speed<NF, R>(params_of<R>(rd), u), a);
    }
    __shared__ double red[256];
    red[threadIdx.x] = a;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0 && red[0] > 0.0) atomicMax(rd.amax, (unsigned long long)__double_as_longlong(red[0]));
}

// Block layout [nb][nb][bs][bs][nf] (host) <-> field planes (device).  A CTA
// takes LAYOUT_ZONES consecutive zones of the host layout: the host side
// (which may be a page-locked host buffer read or written in place over the
// CPU-GPU link) moves as one contiguous, coalesced sweep through shared
// memory, and each field plane is written (read) by one thread per zone, 32
// consecutive words per warp.
constexpr int LAYOUT_ZONES = 256;

// Plane index of host-layout zone q (block-major: block, row, column).  A
// run has at most 2^31 zones (validate), so 32-bit unsigned divisions do: a
// 64-bit division costs about 150 instructions.
__device__ __forceinline__ size_t plane_index(unsigned q, unsigned N, unsigned bs, unsigned nb)
{
    const unsigned r = q / bs, lj = q - r * bs;
    const unsigned b = r / bs, li = r - b * bs;
    const unsigned bi = b / nb, bj = b - bi * nb;
    return (size_t)(bi * bs + li) * N + bj * bs + lj;
}

__global__ void __launch_bounds__(LAYOUT_ZONES) scatter_kernel(const double* src, void* dst, int N, int bs, int nb,
                                                               int nf, int store)
{
    __shared__ double buf[LAYOUT_ZONES * 4];
    const size_t nn = (size_t)N * N;
    const int t = threadIdx.x;
    for (size_t q0 = (size_t)blockIdx.x * LAYOUT_ZONES; q0 < nn; q0 += (size_t)gridDim.x * LAYOUT_ZONES) {
        const int nz = (int)min((size_t)LAYOUT_ZONES, nn - q0);
        for (int e = t; e < nz * nf; e += LAYOUT_ZONES) buf[e] = src[q0 * nf + e];
        __syncthreads();
        if (t < nz) {
            const size_t z = plane_index((unsigned)(q0 + t), N, bs, nb);
            for (int f = 0; f < nf; ++f) {
                const double v = buf[t * nf + f];
                if (store == 0) {
                    ((double*)dst)[f * nn + z] = v;
                } else {
                    const float hi = (float)v;
                    const float lo = (float)(v - (double)hi);
                    ((float*)dst)[(2 * f) * nn + z] = hi;
                    ((float*)dst)[(2 * f + 1) * nn + z] = lo;
                }
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(LAYOUT_ZONES) gather_kernel(const void* src, double* dst, int N, int bs, int nb,
                                                              int nf, int store)
{
    __shared__ double buf[LAYOUT_ZONES * 4];
    const size_t nn = (size_t)N * N;
    const int t = threadIdx.x;
    for (size_t q0 = (size_t)blockIdx.x * LAYOUT_ZONES; q0 < nn; q0 += (size_t)gridDim.x * LAYOUT_ZONES) {
        const int nz = (int)min((size_t)LAYOUT_ZONES, nn - q0);
        if (t < nz) {
            const size_t z = plane_index((unsigned)(q0 + t), N, bs, nb);
            for (int f = 0; f < nf; ++f) {
                double v;
                if (store == 0) v = ((const double*)src)[f * nn + z];
                else v = (double)((const float*)src)[(2 * f) * nn + z] + (double)((const float*)src)[(2 * f + 1) * nn + z];
                buf[t * nf + f] = v;
            }
        }
        __syncthreads();
        for (int e = t; e < nz * nf; e += LAYOUT_ZONES) dst[q0 * nf + e] = buf[e];
        __syncthreads();
    }
}

// Launch shape of the layout kernels for one run: LAYOUT_ZONES threads, at
// most 4096 CTAs striding over the run's zones.
static unsigned layout_blocks(int N)
{
    const size_t nn = (size_t)N * N;
    return (unsigned)std::min<size_t>((nn + LAYOUT_ZONES - 1) / LAYOUT_ZONES, 4096);
}

// ---------------------------------------------------------------------------
// Host-side context.

namespace {

struct RunHost {
    b2d_config cfg;
    int N, bs, nb, nblocks;
    size_t state_bytes;
    void* slot[NSLOTS] = {};
    void* bg = nullptr;
    double* ledger[NSLOTS] = {};
    double* elements[NSLOTS] = {};
    double* partial = nullptr;
    unsigned* counter = nullptr;
    double *xc = nullptr, *xv = nullptr;
    float *xcf = nullptr, *xvf = nullptr, *xvgf = nullptr;
    double* stage_time = nullptr;
    double* orbit = nullptr;
    double* stage_ds = nullptr;
    double* stage_de = nullptr;
    std::vector<double> hxc;
};

// Host mirror of the per-context control block in device memory.
struct Control {
    b2d_error err;
    int pad_[2];
};

struct StagePlan {
    int in, base, out;
    double bf;
};

}  // namespace

struct b2d_ctx {
    int nruns = 0, nf = 3, precision = 0, hydro = 0, rk = 2;
    int tw = 64, th = 64;
    int strip_rows = 0;   // > 0: the paired FP32 kernel covers column strips in row chunks of at most this many rows
    // a slab advance in progress (b2d_slab_begin .. b2d_slab_end)
    std::vector<StagePlan> slab_plan;
    int slab_fold = 0, slab_start = -1, slab_final = -1, slab_next = -1;
    int cur = 0;
    std::vector<RunHost> runs;
    std::vector<RunDev> rdev_h;
    RunDev* rdev = nullptr;
    // control arrays (device)
    double* d_dt = nullptr;           // [nruns]
    double* d_time = nullptr;         // [nruns][NSLOTS]
    long long* d_iter = nullptr;      // [nruns][NSLOTS]
    unsigned long long* d_amax = nullptr;  // [nruns]
    unsigned long long* d_err_key = nullptr;  // failure key (~0: none)
    unsigned* d_timeout = nullptr;            // a bounded wait gave up
    long long* d_adv_count = nullptr;       // advances begun without a pending failure
    long long adv_base = 0;
    std::vector<std::pair<int, std::vector<StagePlan>>> window;  // advances since the last check
    double* d_staging = nullptr;
    size_t staging_bytes = 0;
    // pipelined host transfers (b2d_upload_conserved_async / b2d_download_async):
    // copy streams, double-buffered device staging and their events
    cudaStream_t up_stream = nullptr, down_stream = nullptr;
    double* d_in[2] = {};
    double* d_out[2] = {};
    cudaEvent_t in_copied[2] = {}, in_used[2] = {}, out_ready[2] = {}, out_copied[2] = {};
    long long n_up = 0, n_down = 0;
    int max_stages = 0;
    cudaStream_t stream = nullptr;
    bool use_graphs = true;
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
    long long launches = 0;
    int total_tiles = 0;
    int pending_final = -1;
    // instrumentation
    bool instrument = false;
    std::vector<cudaEvent_t> ev;
    double stage_ms_total = 0.0;
    long long stage_count = 0;
};

static int rsize_of(int precision) { return precision == B2D_PREC_FP64 ? 8 : 4; }

static size_t stage_smem_bytes(int nf, int rsize, int tw)
{
    int cw = 3 * nf + 4;
    size_t elems = 4 * (size_t)(tw + 4) * nf + 3 * (size_t)(tw + 2) * cw + 2 * (size_t)(tw + 1) * nf;
    size_t bytes = elems * rsize;
    size_t red = (size_t)tw * 8;
    return std::max(bytes, red);
}

template <class T> static DevParamsT<T> make_params(const b2d_config& c)
{
    DevParamsT<T> p;
    memset(&p, 0, sizeof p);
    p.hydro = c.hydro_kind;
    p.visc = c.viscosity_kind;
    p.sink_model = c.sink_model;
    p.one_body = c.one_body;
    p.has_mach_ceiling = c.has_mach_ceiling;
    p.has_density_floor = c.has_density_floor;
    p.has_pressure_floor = c.has_pressure_floor;
    p.density_index = c.density_index;
    p.cooling_kind = c.cooling_kind;
    p.cooling_slow_start = c.cooling_slow_start;
    p.has_dt_min = c.has_dt_min;
    double block_length = 2.0 * c.domain_radius / (double)c.num_blocks;  // mesh.rs:27-29
    double dx = block_length / (double)c.block_size;                     // mesh.rs:86-88
    p.dx = (T)dx;
    p.inv_dx = (T)(1.0 / dx);
    p.cfl = (T)c.cfl;
    p.dt_min = (T)c.dt_min;
    p.plm = (T)c.plm;
    p.pdt = (T)(c.has_plm_density_trigger ? c.plm_density_trigger : 0.0);  // scheme.rs:216-220
    p.nu = (T)c.viscosity;
    p.lambda = (T)c.lambda_multiplier;
    p.mach2 = (T)(c.mach_number * c.mach_number);
    p.inv_mach2 = (T)(1.0 / (c.mach_number * c.mach_number));
    double gamma = c.hydro_kind == B2D_EULER ? c.gamma_law_index : 1.0;  // physics.rs:477-479
    p.gamma = (T)gamma;
    p.gm1 = (T)(gamma - 1.0);
    p.inv_gm1 = (T)(1.0 / (gamma - 1.0));
    p.sqrt_gm = (T)sqrt(gamma);
    p.inv_sqrt_gm = (T)(1.0 / sqrt(gamma));
    double s = c.has_softening_length ? c.softening_length : c.sink_radius;  // physics.rs:399-405
    p.soft2 = (T)(s * s);
    p.sink_r2 = (T)(c.sink_radius * c.sink_radius);
    p.inv_sink_r2 = (T)(1.0 / (c.sink_radius * c.sink_radius));
    p.sink_rate = (T)c.sink_rate;
    p.domain_radius = (T)c.domain_radius;
    p.buffer_scale = (T)c.buffer_scale;
    p.inv_buffer_scale = (T)(1.0 / c.buffer_scale);
    p.half_buffer_rate = (T)(0.5 * c.buffer_rate);
    double q = c.one_body ? 1.0 : c.binary_mass_ratio;
    double m1 = 1.0 / (1.0 + q), m2 = 1.0 * q / (1.0 + q);
    double R = c.domain_radius;
    double omega_outer = sqrt((m1 + m2) / (R * R * R));                  // physics.rs:445
    p.omega_outer = (T)omega_outer;
    p.half_rate_omega = (T)(0.5 * c.buffer_rate * omega_outer);
    p.fake_thr = (T)c.fake_mass_threshold;
    p.fake_rate = (T)c.fake_mass_rate;
    p.density_floor = (T)c.density_floor;
    p.pressure_floor = (T)c.pressure_floor;
    p.density_floor_pow_gamma = (T)(c.has_density_floor ? pow(c.density_floor, gamma) : 0.0);
    p.mach_ceiling2 = (T)(c.mach_ceiling * c.mach_ceiling);
    p.k_mach_ceiling = (T)(c.has_mach_ceiling ? 2.0 / (gamma * (gamma - 1.0) * c.mach_ceiling * c.mach_ceiling) : 0.0);
    p.cool_coef = (T)c.cooling_coefficient;
    p.cool_beta = (T)c.cooling_beta;
    p.inv_cool_beta = (T)(c.cooling_beta != 0.0 ? 1.0 / c.cooling_beta : 0.0);
    p.eps_dx = (T)(1e-12 * dx);
    return p;
}

static b2d_status validate(const b2d_config& c, int hydro, int rk)
{
    if (c.num_blocks < 1 || c.block_size < 1) return fail(B2D_ERR_INVALID, "num_blocks and block_size must be positive");
    if (c.hydro_kind != hydro) return fail(B2D_ERR_INVALID, "all runs of a context must share the hydro kind");
    if (c.rk_order != rk) return fail(B2D_ERR_INVALID, "all runs of a context must share rk_order");
    if (rk < 1 || rk > 3) return fail(B2D_ERR_INVALID, "rk_order must be 1, 2 or 3");
    long long N = (long long)c.num_blocks * c.block_size;
    if (N * N > (1ll << 31)) return fail(B2D_ERR_INVALID, "mesh too large (more than 2^31 zones per run)");
    if (!(c.domain_radius > 0)) return fail(B2D_ERR_INVALID, "domain_radius must be positive");
    if (c.num_blocks > 256 || c.block_size > 4096)
        return fail(B2D_ERR_INVALID, "num_blocks must be at most 256 and block_size at most 4096");
    return B2D_OK;
}

static int default_tile_w(int bs)
{
    for (int w : {128, 64, 32})
        if (bs % w == 0) return w;
    return bs;
}

static bool tile_ok(const b2d_ctx* ctx, int tw, int th)
{
    // the paired FP32 kernels' 128-, 256- and 512-column tiles may also span
    // whole blocks side by side (blocks of 64 columns or more)
    const bool span = ctx->precision == B2D_PREC_FP32_COMP && (tw == 128 || tw == 256 || tw == 512);
    if (tw < 1 || th < 1 || tw > (span ? 512 : 256)) return false;
    for (const RunHost& r : ctx->runs) {
        if (r.bs % th) return false;
        if (r.bs % tw && !(span && r.bs >= 64 && tw % r.bs == 0 && r.N % tw == 0)) return false;
    }
    if (tw % 32 != 0) {
        // a partial warp is allowed only when it is the whole block width
        for (const RunHost& r : ctx->runs)
            if (r.bs != tw) return false;
    }
    return true;
}

static void free_ctx(b2d_ctx* ctx)
{
    if (!ctx) return;
    for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
    for (RunHost& r : ctx->runs) {
        for (int s = 0; s < NSLOTS; ++s) { cudaFree(r.slot[s]); cudaFree(r.ledger[s]); cudaFree(r.elements[s]); }
        const size_t ri = &r - ctx->runs.data();
        if (ri < ctx->rdev_h.size())
            for (int s = 0; s < NSLOTS; ++s) cudaFree(ctx->rdev_h[ri].tracers[s]);
        cudaFree(r.bg); cudaFree(r.partial); cudaFree(r.counter);
        cudaFree(r.xc); cudaFree(r.xv); cudaFree(r.xcf); cudaFree(r.xvf); cudaFree(r.xvgf);
        cudaFree(r.stage_time); cudaFree(r.orbit); cudaFree(r.stage_ds); cudaFree(r.stage_de);
    }
    cudaFree(ctx->rdev); cudaFree(ctx->d_dt); cudaFree(ctx->d_time); cudaFree(ctx->d_iter);
    cudaFree(ctx->d_amax); cudaFree(ctx->d_err_key); cudaFree(ctx->d_adv_count); cudaFree(ctx->d_timeout); cudaFree(ctx->d_staging);
    for (cudaEvent_t e : ctx->ev) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->up_stream) cudaStreamDestroy(ctx->up_stream);
    if (ctx->down_stream) cudaStreamDestroy(ctx->down_stream);
    for (int b = 0; b < 2; ++b) {
        cudaFree(ctx->d_in[b]);
        cudaFree(ctx->d_out[b]);
        for (cudaEvent_t e : {ctx->in_copied[b], ctx->in_used[b], ctx->out_ready[b], ctx->out_copied[b]})
            if (e) cudaEventDestroy(e);
    }
    delete ctx;
}

// Rebuild the tile bookkeeping for the current tile shape and push the run
// descriptors to the device.
// The stage kernel the context launches takes row chunks: a paired-column
// kernel or the TMA-staged one (launch_stage_f32 makes the same choice), not
// the FP64 or the generic kernel.
static bool chunk_kernel(const b2d_ctx* ctx)
{
    if (ctx->precision == B2D_PREC_FP64) return false;
    if (ctx->precision == B2D_PREC_FP32_COMP &&
        (ctx->tw == 64 || ctx->tw == 128 || ctx->tw == 256 || ctx->tw == 512))
        return true;
    return ctx->tw % 32 == 0 && ctx->tw <= 128;
}

// Row chunks per column strip of a run: block-aligned tiles of height th, or,
// with strip rows set and a chunk-taking kernel launched, ceil(N / rows)
// chunks that may cross one block boundary each.
static int row_chunks(const b2d_ctx* ctx, const RunHost& r)
{
    if (ctx->strip_rows > 0 && chunk_kernel(ctx)) return (r.N + ctx->strip_rows - 1) / ctx->strip_rows;
    return r.N / ctx->th;
}

static b2d_status sync_rundev(b2d_ctx* ctx)
{
    int base = 0;
    for (int i = 0; i < ctx->nruns; ++i) {
        RunHost& r = ctx->runs[i];
        RunDev& d = ctx->rdev_h[i];
        // a slab launches the block-aligned chunks (tile height th) of its own block rows
        d.chunks = d.slab_hi > 0 ? r.N / ctx->th : row_chunks(ctx, r);
        d.chunk0 = d.slab_hi > 0 ? d.slab_lo * (r.bs / ctx->th) : 0;
        d.tiles_i = d.slab_hi > 0 ? (d.slab_hi - d.slab_lo) * (r.bs / ctx->th) : d.chunks;
        d.tiles_j = r.N / ctx->tw;
        d.ntiles = d.tiles_i * d.tiles_j;
        d.tile_base = base;
        // partial slots of the block with the most chunk pieces (every block:
        // bs / th for block-aligned tiles)
        int most = 0;
        if (d.slab_hi > 0) most = r.bs / ctx->th;   // a slab's tiles are block-aligned
        else
            for (int b = 0; b < r.nb; ++b) most = std::max(most, chunks_in_block_row(b, r.bs, r.N, d.chunks));
        d.tiles_per_block = most * std::max(r.bs / ctx->tw, 1);
        base += d.ntiles;
        CUDA_TRY(cudaFree(r.partial));
        r.partial = nullptr;
        CUDA_TRY(cudaMalloc(&r.partial, sizeof(double) * r.nblocks * d.tiles_per_block * NITEMS * ctx->nf));
        d.partial = r.partial;
    }
    ctx->total_tiles = base;
    CUDA_TRY(cudaMemcpy(ctx->rdev, ctx->rdev_h.data(), sizeof(RunDev) * ctx->nruns, cudaMemcpyHostToDevice));
    for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
    ctx->graphs.clear();
    return B2D_OK;
}

static b2d_status ensure_stage_capacity(b2d_ctx* ctx, int fold)
{
    int need = fold * ctx->rk;
    if (need <= ctx->max_stages) return B2D_OK;
    int cap = std::max(need, 64);
    for (int i = 0; i < ctx->nruns; ++i) {
        RunHost& r = ctx->runs[i];
        CUDA_TRY(cudaFree(r.stage_time));
        CUDA_TRY(cudaFree(r.orbit));
        CUDA_TRY(cudaFree(r.stage_ds));
        CUDA_TRY(cudaFree(r.stage_de));
        r.stage_time = nullptr;
        r.orbit = nullptr;
        r.stage_ds = nullptr;
        r.stage_de = nullptr;
        CUDA_TRY(cudaMalloc(&r.stage_time, sizeof(double) * cap));
        CUDA_TRY(cudaMalloc(&r.orbit, sizeof(double) * 10 * cap));
        CUDA_TRY(cudaMalloc(&r.stage_ds, sizeof(double) * cap * r.nblocks * NITEMS * ctx->nf));
        CUDA_TRY(cudaMalloc(&r.stage_de, sizeof(double) * cap * r.nblocks * 16));
        ctx->rdev_h[i].stage_time = r.stage_time;
        ctx->rdev_h[i].orbit = r.orbit;
        ctx->rdev_h[i].stage_ds = r.stage_ds;
        ctx->rdev_h[i].stage_de = r.stage_de;
    }
    ctx->max_stages = cap;
    CUDA_TRY(cudaMemcpy(ctx->rdev, ctx->rdev_h.data(), sizeof(RunDev) * ctx->nruns, cudaMemcpyHostToDevice));
    for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
    ctx->graphs.clear();
    return B2D_OK;
}

extern "C" b2d_ctx* b2d_create(const b2d_config* cfgs, int32_t nruns, int32_t precision, b2d_status* status)
{
    b2d_status st_dummy;
    if (!status) status = &st_dummy;
    if (!cfgs || nruns < 1 || nruns > 256) { *status = fail(B2D_ERR_INVALID, "need 1 to 256 runs"); return nullptr; }
    if (precision < 0 || precision > 2) { *status = fail(B2D_ERR_INVALID, "bad precision"); return nullptr; }
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev == 0) {
        *status = fail(B2D_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(ce));
        return nullptr;
    }
    b2d_ctx* ctx = new b2d_ctx;
    ctx->nruns = nruns;
    ctx->precision = precision;
    ctx->hydro = cfgs[0].hydro_kind;
    ctx->rk = cfgs[0].rk_order;
    ctx->nf = ctx->hydro == B2D_EULER ? 4 : 3;
    int min_bs = 1 << 30;
    for (int i = 0; i < nruns; ++i) {
        b2d_status v = validate(cfgs[i], ctx->hydro, ctx->rk);
        if (v != B2D_OK) { *status = v; free_ctx(ctx); return nullptr; }
        min_bs = std::min(min_bs, cfgs[i].block_size);
    }
#define CREATE_TRY(expr)                                                                         \
    do {                                                                                         \
        cudaError_t e_ = (expr);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            *status = fail(B2D_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));    \
            free_ctx(ctx);                                                                       \
            return nullptr;                                                                      \
        }                                                                                        \
    } while (0)
    CREATE_TRY(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    CREATE_TRY(cudaMalloc(&ctx->rdev, sizeof(RunDev) * nruns));
    CREATE_TRY(cudaMalloc(&ctx->d_dt, sizeof(double) * nruns));
    CREATE_TRY(cudaMalloc(&ctx->d_time, sizeof(double) * nruns * NSLOTS));
    CREATE_TRY(cudaMalloc(&ctx->d_iter, sizeof(long long) * nruns * NSLOTS));
    CREATE_TRY(cudaMalloc(&ctx->d_amax, sizeof(unsigned long long) * nruns));
    CREATE_TRY(cudaMalloc(&ctx->d_err_key, sizeof(unsigned long long)));
    CREATE_TRY(cudaMalloc(&ctx->d_adv_count, sizeof(long long)));
    CREATE_TRY(cudaMalloc(&ctx->d_timeout, sizeof(unsigned)));
    CREATE_TRY(cudaMemset(ctx->d_timeout, 0, sizeof(unsigned)));
    CREATE_TRY(cudaMemset(ctx->d_adv_count, 0, sizeof(long long)));
    CREATE_TRY(cudaMemset(ctx->d_time, 0, sizeof(double) * nruns * NSLOTS));
    CREATE_TRY(cudaMemset(ctx->d_iter, 0, sizeof(long long) * nruns * NSLOTS));
    CREATE_TRY(cudaMemset(ctx->d_amax, 0, sizeof(unsigned long long) * nruns));
    CREATE_TRY(cudaMemset(ctx->d_err_key, 0xff, sizeof(unsigned long long)));
    CREATE_TRY(cudaMemset(ctx->d_dt, 0, sizeof(double) * nruns));

    ctx->runs.resize(nruns);
    ctx->rdev_h.resize(nruns);
    const int store = precision == B2D_PREC_FP32_COMP ? 1 : 0;
    for (int i = 0; i < nruns; ++i) {
        RunHost& r = ctx->runs[i];
        RunDev& d = ctx->rdev_h[i];
        memset(&d, 0, sizeof d);
        r.cfg = cfgs[i];
        r.bs = cfgs[i].block_size;
        r.nb = cfgs[i].num_blocks;
        r.N = r.bs * r.nb;
        r.nblocks = r.nb * r.nb;
        size_t nn = (size_t)r.N * r.N;
        r.state_bytes = store == 1 ? nn * ctx->nf * 2 * sizeof(float) : nn * ctx->nf * sizeof(double);
        for (int s = 0; s < NSLOTS; ++s) {
            CREATE_TRY(cudaMalloc(&r.slot[s], r.state_bytes));
            CREATE_TRY(cudaMemset(r.slot[s], 0, r.state_bytes));
            CREATE_TRY(cudaMalloc(&r.ledger[s], sizeof(double) * r.nblocks * NITEMS * ctx->nf));
            CREATE_TRY(cudaMemset(r.ledger[s], 0, sizeof(double) * r.nblocks * NITEMS * ctx->nf));
            CREATE_TRY(cudaMalloc(&r.elements[s], sizeof(double) * r.nblocks * NITEMS * 4));
            CREATE_TRY(cudaMemset(r.elements[s], 0, sizeof(double) * r.nblocks * NITEMS * 4));
        }
        CREATE_TRY(cudaMalloc(&r.bg, r.state_bytes));
        CREATE_TRY(cudaMemset(r.bg, 0, r.state_bytes));
        CREATE_TRY(cudaMalloc(&r.counter, sizeof(unsigned) * r.nblocks));
        CREATE_TRY(cudaMemset(r.counter, 0, sizeof(unsigned) * r.nblocks));
        // geometry tables
        std::vector<double> xc(r.N), xv((size_t)r.nb * (r.bs + 1));
        for (int b = 0; b < r.nb; ++b) {
            host_cell_centers(&cfgs[i], b, xc.data() + (size_t)b * r.bs);
            host_block_vertices(&cfgs[i], b, xv.data() + (size_t)b * (r.bs + 1));
        }
        std::vector<float> xcf(xc.begin(), xc.end()), xvf(xv.begin(), xv.end());
        // row faces by global index: face k of block k / bs, the last block's top face last
        std::vector<float> xvgf((size_t)r.N + 1);
        for (int k = 0; k < r.N; ++k) xvgf[k] = xvf[(size_t)(k / r.bs) * (r.bs + 1) + k % r.bs];
        xvgf[r.N] = xvf[(size_t)(r.nb - 1) * (r.bs + 1) + r.bs];
        r.hxc = xc;
        CREATE_TRY(cudaMalloc(&r.xc, sizeof(double) * xc.size()));
        CREATE_TRY(cudaMalloc(&r.xv, sizeof(double) * xv.size()));
        CREATE_TRY(cudaMalloc(&r.xcf, sizeof(float) * xc.size()));
        CREATE_TRY(cudaMalloc(&r.xvf, sizeof(float) * xv.size()));
        CREATE_TRY(cudaMalloc(&r.xvgf, sizeof(float) * xvgf.size()));
        CREATE_TRY(cudaMemcpy(r.xc, xc.data(), sizeof(double) * xc.size(), cudaMemcpyHostToDevice));
        CREATE_TRY(cudaMemcpy(r.xv, xv.data(), sizeof(double) * xv.size(), cudaMemcpyHostToDevice));
        CREATE_TRY(cudaMemcpy(r.xcf, xcf.data(), sizeof(float) * xc.size(), cudaMemcpyHostToDevice));
        CREATE_TRY(cudaMemcpy(r.xvf, xvf.data(), sizeof(float) * xv.size(), cudaMemcpyHostToDevice));
        CREATE_TRY(cudaMemcpy(r.xvgf, xvgf.data(), sizeof(float) * xvgf.size(), cudaMemcpyHostToDevice));

        d.N = r.N; d.bs = r.bs; d.nb = r.nb; d.nblocks = r.nblocks;
        d.xc = r.xc; d.xv = r.xv; d.xcf = r.xcf; d.xvf = r.xvf; d.xvgf = r.xvgf;
        for (int s = 0; s < NSLOTS; ++s) {
            d.slot[s] = r.slot[s];
            d.ledger[s] = r.ledger[s];
            d.elements[s] = r.elements[s];
        }
        // OrbitalElements of the run (physics.rs:411-417)
        if (cfgs[i].one_body) { d.el0[0] = 1e-12; d.el0[1] = 1.0; d.el0[2] = 1.0; d.el0[3] = 0.0; }
        else {
            d.el0[0] = 1.0;
            d.el0[1] = 1.0;
            d.el0[2] = cfgs[i].binary_mass_ratio;
            d.el0[3] = cfgs[i].binary_eccentricity;
        }
        d.bg = r.bg;
        d.time = ctx->d_time + (size_t)i * NSLOTS;
        d.iter = ctx->d_iter + (size_t)i * NSLOTS;
        d.counter = r.counter;
        d.dt = ctx->d_dt + i;
        d.amax = ctx->d_amax + i;
        d.binary_q = cfgs[i].binary_mass_ratio;
        d.binary_e = cfgs[i].binary_eccentricity;
        d.p = make_params<double>(cfgs[i]);
        d.pf = make_params<float>(cfgs[i]);
        ctx->staging_bytes = std::max(ctx->staging_bytes, nn * ctx->nf * sizeof(double));
    }
    CREATE_TRY(cudaMalloc(&ctx->d_staging, ctx->staging_bytes));
    ctx->tw = default_tile_w(min_bs);
    ctx->th = std::min(64, min_bs);
    while (!tile_ok(ctx, ctx->tw, ctx->th) && ctx->th > 1) ctx->th /= 2;
    if (!tile_ok(ctx, ctx->tw, ctx->th)) {
        *status = fail(B2D_ERR_INVALID, "runs of a context need a common tile shape (block sizes must share a divisor)");
        free_ctx(ctx);
        return nullptr;
    }
    if (sync_rundev(ctx) != B2D_OK) { *status = B2D_ERR_CUDA; free_ctx(ctx); return nullptr; }
    if (ensure_stage_capacity(ctx, 16) != B2D_OK) { *status = B2D_ERR_CUDA; free_ctx(ctx); return nullptr; }
    *status = B2D_OK;
    return ctx;
#undef CREATE_TRY
}

extern "C" void b2d_destroy(b2d_ctx* ctx)
{
    if (ctx) cudaStreamSynchronize(ctx->stream);
    free_ctx(ctx);
}

extern "C" int32_t b2d_num_fields(const b2d_ctx* ctx) { return ctx ? ctx->nf : 0; }

static int store_of(const b2d_ctx* ctx) { return ctx->precision == B2D_PREC_FP32_COMP ? 1 : 0; }

static b2d_status launch_max_speed(b2d_ctx* ctx, int run, int slot)
{
    CUDA_TRY(cudaMemsetAsync(ctx->d_amax + run, 0, sizeof(unsigned long long), ctx->stream));
    int grid = 4 * 152;
    const bool f64 = ctx->precision == B2D_PREC_FP64;
    if (ctx->nf == 3) {
        if (f64) max_speed_kernel<3, 0, double><<<grid, 256, 0, ctx->stream>>>(ctx->rdev, run, slot);
        else if (store_of(ctx) == 0) max_speed_kernel<3, 0, float><<<grid, 256, 0, ctx->stream>>>(ctx->rdev, run, slot);
        else max_speed_kernel<3, 1, float><<<grid, 256, 0, ctx->stream>>>(ctx->rdev, run, slot);
    } else {
        if (f64) max_speed_kernel<4, 0, double><<<grid, 256, 0, ctx->stream>>>(ctx->rdev, run, slot);
        else if (store_of(ctx) == 0) max_speed_kernel<4, 0, float><<<grid, 256, 0, ctx->stream>>>(ctx->rdev, run, slot);
        else max_speed_kernel<4, 1, float><<<grid, 256, 0, ctx->stream>>>(ctx->rdev, run, slot);
    }
    ctx->launches++;
    CUDA_TRY(cudaGetLastError());
    return B2D_OK;
}

extern "C" b2d_status b2d_upload_state(b2d_ctx* ctx, int32_t run, const double* cons, const double* background,
                                       const double* ledger, double time, int64_t iteration_num, int64_t iteration_den)
{
    if (!ctx || run < 0 || run >= ctx->nruns || !cons) return fail(B2D_ERR_INVALID, "bad arguments");
    if (iteration_den != 1) return fail(B2D_ERR_INVALID, "iteration must be an integer at step boundaries");
    RunHost& r = ctx->runs[run];
    size_t n = (size_t)r.N * r.N * ctx->nf;
    int store = store_of(ctx);
    CUDA_TRY(cudaMemcpyAsync(ctx->d_staging, cons, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    scatter_kernel<<<layout_blocks(r.N), LAYOUT_ZONES, 0, ctx->stream>>>(ctx->d_staging, r.slot[ctx->cur], r.N, r.bs, r.nb, ctx->nf, store);
    ctx->launches++;
    CUDA_TRY(cudaGetLastError());
    if (background) {
        CUDA_TRY(cudaMemcpyAsync(ctx->d_staging, background, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        scatter_kernel<<<layout_blocks(r.N), LAYOUT_ZONES, 0, ctx->stream>>>(ctx->d_staging, r.bg, r.N, r.bs, r.nb, ctx->nf, store);
        ctx->launches++;
        CUDA_TRY(cudaGetLastError());
    }
    size_t nled = (size_t)r.nblocks * NITEMS * ctx->nf;
    if (ledger) CUDA_TRY(cudaMemcpyAsync(r.ledger[ctx->cur], ledger, nled * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    else CUDA_TRY(cudaMemsetAsync(r.ledger[ctx->cur], 0, nled * sizeof(double), ctx->stream));
    CUDA_TRY(cudaMemsetAsync(r.elements[ctx->cur], 0, sizeof(double) * r.nblocks * NITEMS * 4, ctx->stream));
    long long it = iteration_num;
    CUDA_TRY(cudaMemcpyAsync(ctx->d_time + (size_t)run * NSLOTS + ctx->cur, &time, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(ctx->d_iter + (size_t)run * NSLOTS + ctx->cur, &it, sizeof(long long), cudaMemcpyHostToDevice, ctx->stream));
    b2d_status s = launch_max_speed(ctx, run, ctx->cur);
    if (s != B2D_OK) return s;
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return B2D_OK;
}

// Device address of a page-locked (cudaHostRegister / cudaMallocHost) host
// buffer that is 16-byte aligned, or nullptr.  The layout kernels read and
// write such buffers in place over the CPU-GPU link, so the copy and the
// layout change are one pass; other buffers go through the device staging
// buffer.
static void* mapped_host(const void* p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer || ((uintptr_t)at.devicePointer & 15u)) return nullptr;
    return at.devicePointer;
}

extern "C" b2d_status b2d_upload_conserved(b2d_ctx* ctx, int32_t run, const double* cons)
{
    if (!ctx || run < 0 || run >= ctx->nruns || !cons) return fail(B2D_ERR_INVALID, "bad arguments");
    RunHost& r = ctx->runs[run];
    size_t n = (size_t)r.N * r.N * ctx->nf;
    const double* src = (const double*)mapped_host(cons);
    if (!src) {
        CUDA_TRY(cudaMemcpyAsync(ctx->d_staging, cons, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
        src = ctx->d_staging;
    }
    scatter_kernel<<<layout_blocks(r.N), LAYOUT_ZONES, 0, ctx->stream>>>(src, r.slot[ctx->cur], r.N, r.bs, r.nb, ctx->nf, store_of(ctx));
    ctx->launches++;
    CUDA_TRY(cudaGetLastError());
    b2d_status s = launch_max_speed(ctx, run, ctx->cur);
    if (s != B2D_OK) return s;
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return B2D_OK;
}

// ---------------------------------------------------------------------------
// Pipelined host transfers.  Two copy streams move page-locked host buffers
// through double-buffered device staging while the context stream computes;
// the context stream only runs the layout kernels, so a step of a pipelined
// loop costs scatter + advance + gather on the device and the copies overlap
// the neighbouring steps' advances.

static b2d_status ensure_pipeline(b2d_ctx* ctx)
{
    if (ctx->up_stream) return B2D_OK;
    CUDA_TRY(cudaStreamCreateWithFlags(&ctx->up_stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&ctx->down_stream, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
        CUDA_TRY(cudaMalloc(&ctx->d_in[b], ctx->staging_bytes));
        CUDA_TRY(cudaMalloc(&ctx->d_out[b], ctx->staging_bytes));
        for (cudaEvent_t* e : {&ctx->in_copied[b], &ctx->in_used[b], &ctx->out_ready[b], &ctx->out_copied[b]})
            CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    return B2D_OK;
}

extern "C" b2d_status b2d_upload_conserved_async(b2d_ctx* ctx, int32_t run, const double* cons)
{
    if (!ctx || run < 0 || run >= ctx->nruns || !cons) return fail(B2D_ERR_INVALID, "bad arguments");
    b2d_status st = ensure_pipeline(ctx);
    if (st != B2D_OK) return st;
    RunHost& r = ctx->runs[run];
    const size_t n = (size_t)r.N * r.N * ctx->nf;
    const int b = (int)(ctx->n_up++ & 1);
    // the staging buffer is free once the scatter that last read it has run
    CUDA_TRY(cudaStreamWaitEvent(ctx->up_stream, ctx->in_used[b], 0));
    CUDA_TRY(cudaMemcpyAsync(ctx->d_in[b], cons, n * sizeof(double), cudaMemcpyHostToDevice, ctx->up_stream));
    CUDA_TRY(cudaEventRecord(ctx->in_copied[b], ctx->up_stream));
    CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ctx->in_copied[b], 0));
    scatter_kernel<<<layout_blocks(r.N), LAYOUT_ZONES, 0, ctx->stream>>>(ctx->d_in[b], r.slot[ctx->cur], r.N, r.bs, r.nb, ctx->nf,
                                                       store_of(ctx));
    ctx->launches++;
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaEventRecord(ctx->in_used[b], ctx->stream));
    return launch_max_speed(ctx, run, ctx->cur);
}

extern "C" b2d_status b2d_download_async(b2d_ctx* ctx, int32_t run, double* cons)
{
    if (!ctx || run < 0 || run >= ctx->nruns || !cons) return fail(B2D_ERR_INVALID, "bad arguments");
    b2d_status st = ensure_pipeline(ctx);
    if (st != B2D_OK) return st;
    RunHost& r = ctx->runs[run];
    const size_t n = (size_t)r.N * r.N * ctx->nf;
    const int b = (int)(ctx->n_down++ & 1);
    // the staging buffer is free once the copy that last read it has finished
    CUDA_TRY(cudaStreamWaitEvent(ctx->stream, ctx->out_copied[b], 0));
    gather_kernel<<<layout_blocks(r.N), LAYOUT_ZONES, 0, ctx->stream>>>(r.slot[ctx->cur], ctx->d_out[b], r.N, r.bs, r.nb, ctx->nf,
                                                      store_of(ctx));
    ctx->launches++;
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaEventRecord(ctx->out_ready[b], ctx->stream));
    CUDA_TRY(cudaStreamWaitEvent(ctx->down_stream, ctx->out_ready[b], 0));
    CUDA_TRY(cudaMemcpyAsync(cons, ctx->d_out[b], n * sizeof(double), cudaMemcpyDeviceToHost, ctx->down_stream));
    CUDA_TRY(cudaEventRecord(ctx->out_copied[b], ctx->down_stream));
    return B2D_OK;
}

extern "C" b2d_status b2d_transfers_wait(b2d_ctx* ctx, int32_t pending)
{
    if (!ctx || pending < 0 || pending > 1) return fail(B2D_ERR_INVALID, "bad arguments");
    if (!ctx->up_stream) return B2D_OK;
    if (pending == 0) {
        CUDA_TRY(cudaStreamSynchronize(ctx->up_stream));
        CUDA_TRY(cudaStreamSynchronize(ctx->down_stream));
        return B2D_OK;
    }
    // every download but the newest has landed (downloads complete in order)
    if (ctx->n_down >= 2) CUDA_TRY(cudaEventSynchronize(ctx->out_copied[(ctx->n_down - 2) & 1]));
    return B2D_OK;
}

extern "C" b2d_status b2d_download_state(b2d_ctx* ctx, int32_t run, double* cons, double* time, int64_t* iteration_num,
                                         int64_t* iteration_den)
{
    if (!ctx || run < 0 || run >= ctx->nruns) return fail(B2D_ERR_INVALID, "bad arguments");
    RunHost& r = ctx->runs[run];
    size_t n = (size_t)r.N * r.N * ctx->nf;
    if (cons) {
        double* dst = (double*)mapped_host(cons);
        gather_kernel<<<layout_blocks(r.N), LAYOUT_ZONES, 0, ctx->stream>>>(r.slot[ctx->cur], dst ? dst : ctx->d_staging, r.N, r.bs, r.nb,
                                                         ctx->nf, store_of(ctx));
        ctx->launches++;
        CUDA_TRY(cudaGetLastError());
        if (!dst) CUDA_TRY(cudaMemcpyAsync(cons, ctx->d_staging, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    }
    double t = 0;
    long long it = 0;
    CUDA_TRY(cudaMemcpyAsync(&t, ctx->d_time + (size_t)run * NSLOTS + ctx->cur, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(&it, ctx->d_iter + (size_t)run * NSLOTS + ctx->cur, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (time) *time = t;
    if (iteration_num) *iteration_num = it;
    if (iteration_den) *iteration_den = 1;
    return B2D_OK;
}

extern "C" b2d_status b2d_download_ledger(b2d_ctx* ctx, int32_t run, double* ledger)
{
    if (!ctx || run < 0 || run >= ctx->nruns || !ledger) return fail(B2D_ERR_INVALID, "bad arguments");
    RunHost& r = ctx->runs[run];
    size_t nled = (size_t)r.nblocks * NITEMS * ctx->nf;
    CUDA_TRY(cudaMemcpyAsync(ledger, r.ledger[ctx->cur], nled * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return B2D_OK;
}

extern "C" b2d_status b2d_max_signal_speed(b2d_ctx* ctx, int32_t run, double* out)
{
    if (!ctx || run < 0 || run >= ctx->nruns || !out) return fail(B2D_ERR_INVALID, "bad arguments");
    unsigned long long bits = 0;
    CUDA_TRY(cudaMemcpyAsync(&bits, ctx->d_amax + run, sizeof bits, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    double v;
    memcpy(&v, &bits, sizeof v);
    *out = v;
    return B2D_OK;
}

// ---------------------------------------------------------------------------
// The advance.

__host__ __device__ static int free_slot(int a, int b, int c)
{
    for (int s = 0; s < NSLOTS; ++s)
        if (s != a && s != b && s != c) return s;
    return -1;
}

// Slot schedule of `fold` RK steps from slot `start`, which is left intact.
static std::vector<StagePlan> plan_advance(int rk, int fold, int start, int* final_slot)
{
    std::vector<StagePlan> plan;
    int base = start;
    for (int f = 0; f < fold; ++f) {
        if (rk == 1) {
            int a = free_slot(start, base, -1);
            plan.push_back({base, -1, a, 0.0});
            base = a;
        } else if (rk == 2) {
            int a = free_slot(start, base, -1);
            plan.push_back({base, -1, a, 0.0});
            int b = free_slot(start, base, a);
            plan.push_back({a, base, b, 0.5});
            base = b;
        } else {
            int a = free_slot(start, base, -1);
            plan.push_back({base, -1, a, 0.0});
            int b = free_slot(start, base, a);
            plan.push_back({a, base, b, 0.75});
            int c = free_slot(start, base, b);
            plan.push_back({b, base, c, 1.0 / 3.0});
            base = c;
        }
    }
    *final_slot = base;
    return plan;
}

// ItemizedChange<OrbitalElements> of every block over one advance
// (compute_block_updated_solution, scheme.rs:307-314), after the stage
// kernels, which only record each block's stage sums ds·dx·dy: the serial
// FP64 perturbation stays out of their tails.  Two launches:
//  * elements_de_kernel — one thread per (stage, block, gas item sink1, sink2,
//    grav1, grav2): that item's perturbation (ItemizedChange::perturbation,
//    state.rs:258-281).  An unbound perturbed orbit fails its stage with
//    OrbitalEvolutionError, reported at position (0, 0) as in the reference.
//    The reference converts every block's primitives before it updates any
//    block, so within a stage a cons->prim failure anywhere wins: the key's
//    block field is saturated and the failing block's index rides in the
//    zone field; an earlier stage still wins through the stage field.
//  * elements_sum_kernel — one thread per (block, element component): the
//    stages in order, e_out = e_in + de averaged like the state
//    (state.rs:191-197), in the slot schedule of plan_advance.
__global__ void elements_de_kernel(const RunDev* runs, int nstages, unsigned long long* err_key)
{
    const int run = blockIdx.z;
    const RunDev& rd = runs[run];
    const int s = blockIdx.y;
    const int id = blockIdx.x * blockDim.x + threadIdx.x;   // block * 4 + item
    if (s >= nstages || id >= rd.nblocks * 4 || !rd.stage_ds || !rd.stage_de) return;
    const int block = id >> 2, item = id & 3;
    if (rd.slab_hi > 0 && (block / rd.nb < rd.slab_lo || block / rd.nb >= rd.slab_hi)) return;   // another slab's
    const int nf = rd.p.hydro == B2D_EULER ? 4 : 3;
    const double* ds = rd.stage_ds + ((size_t)s * rd.nblocks + block) * NITEMS * nf + item * nf;
    const double* orbit = rd.orbit + 10 * s;
    double* de = rd.stage_de + (((size_t)s * rd.nblocks + block) * 4 + item) * 4;
    // pert1 (body 1: sink1, grav1) and pert2 (body 2: sink2, grav2), state.rs:261-269
    const bool ok = (item == 0 || item == 2)
                        ? perturb_elements(orbit, rd.el0, -ds[0], 0.0, -ds[1], 0.0, -ds[2], 0.0, de)
                        : perturb_elements(orbit, rd.el0, 0.0, -ds[0], 0.0, -ds[1], 0.0, -ds[2], de);
    if (!ok) {
        de[0] = de[1] = de[2] = de[3] = 0.0;
        const unsigned long long key = ((unsigned long long)s << 54) | ((unsigned long long)run << 46) |
                                       (0xffffull << 30) | (0xfull << 26) | ((unsigned long long)block << 2) | 3ull;
        atomicMin(err_key, key);
    }
}

__global__ void elements_sum_kernel(const RunDev* runs, int fold, int rk, int start)
{
    const int run = blockIdx.y;
    const RunDev& rd = runs[run];
    const int id = blockIdx.x * blockDim.x + threadIdx.x;   // block * 28 + item * 4 + component
    if (id >= rd.nblocks * NITEMS * 4 || !rd.stage_de || !rd.elements[start]) return;
    const int block = id / (NITEMS * 4), k = id % (NITEMS * 4), item = k / 4;
    if (rd.slab_hi > 0 && (block / rd.nb < rd.slab_lo || block / rd.nb >= rd.slab_hi)) return;
    double e[NSLOTS];
    e[start] = rd.elements[start][id];
    int s = 0;
    auto stage = [&](int in, int base_slot, int out, double bf) {
        const double de = item < 4 ? rd.stage_de[((size_t)s * rd.nblocks + block) * 16 + k] : 0.0;
        double v = e[in] + de;
        if (base_slot >= 0) v = v * (-bf + 1.0) + e[base_slot] * bf;
        e[out] = v;
        ++s;
    };
    // the schedule of plan_advance
    int base = start;
    for (int f = 0; f < fold; ++f) {
        if (rk == 1) {
            const int a = free_slot(start, base, -1);
            stage(base, -1, a, 0.0);
            base = a;
        } else if (rk == 2) {
            const int a = free_slot(start, base, -1);
            stage(base, -1, a, 0.0);
            const int b = free_slot(start, base, a);
            stage(a, base, b, 0.5);
            base = b;
        } else {
            const int a = free_slot(start, base, -1);
            stage(base, -1, a, 0.0);
            const int b = free_slot(start, base, a);
            stage(a, base, b, 0.75);
            const int c = free_slot(start, base, b);
            stage(b, base, c, 1.0 / 3.0);
            base = c;
        }
    }
    rd.elements[base][id] = e[base];
}

static int max_blocks(const b2d_ctx* ctx)
{
    int m = 0;
    for (const RunHost& r : ctx->runs) m = std::max(m, r.nblocks);
    return m;
}

static df32w split_df(double v)
{
    float hi = (float)v;
    float lo = (float)(v - (double)hi);
    return {hi, lo};
}

static b2d_status launch_stage(b2d_ctx* ctx, const StagePlan& sp, int stage, int amax_flag)
{
    StageArgs a;
    a.runs = ctx->rdev;
    a.nruns = ctx->nruns;
    a.th = ctx->th;
    a.in_slot = sp.in;
    a.base_slot = sp.base;
    a.out_slot = sp.out;
    a.stage = stage;
    a.amax_flag = amax_flag;
    a.bf = sp.bf;
    a.w1f = split_df(-sp.bf + 1.0);
    a.bff = split_df(sp.bf);
    a.err_key = ctx->d_err_key;
    a.timeout_flag = ctx->d_timeout;
    a.pf1 = ctx->rdev_h[0].pf;
    size_t smem = stage_smem_bytes(ctx->nf, rsize_of(ctx->precision), ctx->tw);
    cudaError_t e;
    if (ctx->precision == B2D_PREC_FP64) e = launch_stage_f64(ctx->nf, a, ctx->total_tiles, ctx->tw, smem, ctx->stream);
    else e = launch_stage_f32(ctx->nf, store_of(ctx), a, ctx->total_tiles, ctx->tw, smem, ctx->stream);
    if (e != cudaSuccess) return fail(B2D_ERR_CUDA, std::string("stage kernel launch: ") + cudaGetErrorString(e));
    return B2D_OK;
}

// ---------------------------------------------------------------------------
// Massless tracer particles (no counterpart in the reference's code; its
// README names them).  dx/dt = v(x, t) with v the gas velocity of the stage
// input, bilinear between the four surrounding cell centres of the uniform
// mesh, advanced by the same RK stages and weighted averages as the state and
// wrapped into the periodic domain [-R, R)^2.  Positions are FP64.
// Gas velocity of one cell.  R = double is the FP64 parity arithmetic; the
// FP32 paths interpolate in FP32 (the FP64 divisions would dominate on this
// GPU) and keep the positions in FP64.
template <class R, int STORE>
__device__ __forceinline__ void tracer_cell_velocity(const RunDev& rd, int slot, int i, int j, R& vx, R& vy)
{
    const size_t nn = (size_t)rd.N * rd.N, idx = (size_t)i * rd.N + j;
    R u[3];
    for (int f = 0; f < 3; ++f) {
        if (STORE == 0) u[f] = (R)((const double*)rd.slot[slot])[f * nn + idx];
        else u[f] = (R)((const float*)rd.slot[slot])[(2 * f) * nn + idx];
    }
    if constexpr (std::is_same<R, double>::value) {
        vx = u[1] / u[0];
        vy = u[2] / u[0];
    } else {
        const float ir = __fdividef(1.0f, u[0]);
        vx = u[1] * ir;
        vy = u[2] * ir;
    }
}

template <class T, int STORE>
__global__ void tracer_kernel(const RunDev* runs, int run, int in_slot, int base_slot, int out_slot, double bf)
{
    const RunDev& rd = runs[run];
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= rd.ntracers) return;
    const double R = rd.p.domain_radius, dx = rd.p.dx, dt = *rd.dt;
    const int N = rd.N;
    const double x = rd.tracers[in_slot][2 * k], y = rd.tracers[in_slot][2 * k + 1];
    const double L = 2.0 * R;
    T ax, ay;
    int i0, j0;
    if constexpr (std::is_same<T, double>::value) {
        // the oracle's arithmetic
        const double gx = (x + R) / dx - 0.5, gy = (y + R) / dx - 0.5;
        const double fi = floor(gx), fj = floor(gy);
        ax = gx - fi;
        ay = gy - fj;
        i0 = (int)fi;
        j0 = (int)fj;
    } else {
        // FP64 is slow on this GPU: the cell from an FP32 estimate, the offset in
        // it exactly from FP64 (one fused step), then FP32 for the rest
        const double xr = x + R, yr = y + R;
        const float idx_f = (float)rd.p.inv_dx;
        i0 = (int)floorf((float)xr * idx_f - 0.5f);
        j0 = (int)floorf((float)yr * idx_f - 0.5f);
        ax = (float)fma(-((double)i0 + 0.5), dx, xr) * idx_f;
        ay = (float)fma(-((double)j0 + 0.5), dx, yr) * idx_f;
        // the FP32 estimate can be one cell off within its rounding of a boundary
        if (ax < 0.0f) { --i0; ax += 1.0f; } else if (ax >= 1.0f) { ++i0; ax -= 1.0f; }
        if (ay < 0.0f) { --j0; ay += 1.0f; } else if (ay >= 1.0f) { ++j0; ay -= 1.0f; }
    }
    // positions are kept in [-R, R), so the cell index is in [-1, N - 1]: one
    // conditional wrap, then a clamp that keeps any other input in bounds
    i0 = i0 < 0 ? i0 + N : i0;
    j0 = j0 < 0 ? j0 + N : j0;
    i0 = min(max(i0, 0), N - 1);
    j0 = min(max(j0, 0), N - 1);
    const int i1 = i0 + 1 == N ? 0 : i0 + 1, j1 = j0 + 1 == N ? 0 : j0 + 1;
    T v00x, v00y, v10x, v10y, v01x, v01y, v11x, v11y;
    tracer_cell_velocity<T, STORE>(rd, in_slot, i0, j0, v00x, v00y);
    tracer_cell_velocity<T, STORE>(rd, in_slot, i1, j0, v10x, v10y);
    tracer_cell_velocity<T, STORE>(rd, in_slot, i0, j1, v01x, v01y);
    tracer_cell_velocity<T, STORE>(rd, in_slot, i1, j1, v11x, v11y);
    const T one = T(1);
    const T w00 = (one - ax) * (one - ay), w10 = ax * (one - ay), w01 = (one - ax) * ay, w11 = ax * ay;
    const T vx = w00 * v00x + w10 * v10x + w01 * v01x + w11 * v11x;
    const T vy = w00 * v00y + w10 * v10y + w01 * v01y + w11 * v11y;
    double xo, yo;
    if constexpr (std::is_same<T, double>::value) {
        xo = x + dt * vx;
        yo = y + dt * vy;
        if (base_slot >= 0) {
            // average with the base position on the same periodic image
            const double xb = rd.tracers[base_slot][2 * k], yb = rd.tracers[base_slot][2 * k + 1];
            if (xo - xb > R) xo -= L;
            else if (xo - xb < -R) xo += L;
            if (yo - yb > R) yo -= L;
            else if (yo - yb < -R) yo += L;
            xo = xo * (-bf + 1.0) + xb * bf;
            yo = yo * (-bf + 1.0) + yb * bf;
        }
    } else {
        // the stage's displacement in FP32, accumulated in FP64
        const float dtf = (float)dt;
        xo = x + (double)(dtf * vx);
        yo = y + (double)(dtf * vy);
        if (base_slot >= 0) {
            // base + (new - base) (1 - bf), on the base's periodic image
            const double xb = rd.tracers[base_slot][2 * k], yb = rd.tracers[base_slot][2 * k + 1];
            double ddx = xo - xb, ddy = yo - yb;
            const float Rf = (float)R;
            if ((float)ddx > Rf) ddx -= L;
            else if ((float)ddx < -Rf) ddx += L;
            if ((float)ddy > Rf) ddy -= L;
            else if ((float)ddy < -Rf) ddy += L;
            const double w1 = -bf + 1.0;
            xo = fma(ddx, w1, xb);
            yo = fma(ddy, w1, yb);
        }
    }
    if (xo >= R) xo -= L;
    if (xo < -R) xo += L;
    if (yo >= R) yo -= L;
    if (yo < -R) yo += L;
    rd.tracers[out_slot][2 * k] = xo;
    rd.tracers[out_slot][2 * k + 1] = yo;
}

static b2d_status launch_tracers(b2d_ctx* ctx, const StagePlan& sp, bool count)
{
    for (int r = 0; r < ctx->nruns; ++r) {
        const long long n = ctx->rdev_h[r].ntracers;
        if (n <= 0) continue;
        const int threads = 256;
        const unsigned grid = (unsigned)((n + threads - 1) / threads);
        if (ctx->precision == B2D_PREC_FP64)
            tracer_kernel<double, 0><<<grid, threads, 0, ctx->stream>>>(ctx->rdev, r, sp.in, sp.base, sp.out, sp.bf);
        else if (ctx->precision == B2D_PREC_FP32_STATE64)
            tracer_kernel<float, 0><<<grid, threads, 0, ctx->stream>>>(ctx->rdev, r, sp.in, sp.base, sp.out, sp.bf);
        else
            tracer_kernel<float, 1><<<grid, threads, 0, ctx->stream>>>(ctx->rdev, r, sp.in, sp.base, sp.out, sp.bf);
        CUDA_TRY(cudaGetLastError());
        if (count) ctx->launches++;
    }
    return B2D_OK;
}

// The two per-advance orbital-element kernels (after the stage kernels).
static b2d_status launch_elements(b2d_ctx* ctx, int fold, int start, int nstages, bool count)
{
    const dim3 dg((unsigned)((max_blocks(ctx) * 4 + 127) / 128), (unsigned)nstages, (unsigned)ctx->nruns);
    elements_de_kernel<<<dg, 128, 0, ctx->stream>>>(ctx->rdev, nstages, ctx->d_err_key);
    CUDA_TRY(cudaGetLastError());
    const dim3 sg((unsigned)((max_blocks(ctx) * NITEMS * 4 + 127) / 128), (unsigned)ctx->nruns);
    elements_sum_kernel<<<sg, 128, 0, ctx->stream>>>(ctx->rdev, fold, ctx->rk, start);
    CUDA_TRY(cudaGetLastError());
    if (count) ctx->launches += 2;
    return B2D_OK;
}

static b2d_status enqueue_advance(b2d_ctx* ctx, int fold, int start, int* final_slot, bool count)
{
    std::vector<StagePlan> plan = plan_advance(ctx->rk, fold, start, final_slot);
    prologue_kernel<<<ctx->nruns, 32, 0, ctx->stream>>>(ctx->rdev, fold, ctx->rk, start, *final_slot, ctx->d_err_key,
                                                         ctx->d_adv_count);
    CUDA_TRY(cudaGetLastError());
    if (count) ctx->launches++;
    for (size_t s = 0; s < plan.size(); ++s) {
        bool timed = ctx->instrument;
        if (timed) {
            while (ctx->ev.size() < 2 * plan.size()) {
                cudaEvent_t e;
                CUDA_TRY(cudaEventCreate(&e));
                ctx->ev.push_back(e);
            }
            CUDA_TRY(cudaEventRecord(ctx->ev[2 * s], ctx->stream));
        }
        b2d_status st = launch_stage(ctx, plan[s], (int)s, s + 1 == plan.size());
        if (st != B2D_OK) return st;
        if (timed) CUDA_TRY(cudaEventRecord(ctx->ev[2 * s + 1], ctx->stream));
        if (count) ctx->launches++;
        st = launch_tracers(ctx, plan[s], count);
        if (st != B2D_OK) return st;
    }
    return launch_elements(ctx, fold, start, (int)plan.size(), count);
}

extern "C" b2d_status b2d_set_tracers(b2d_ctx* ctx, int32_t run, int64_t n, const double* xy)
{
    if (!ctx || run < 0 || run >= ctx->nruns || n < 0 || (n > 0 && !xy)) return fail(B2D_ERR_INVALID, "bad arguments");
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    RunDev& d = ctx->rdev_h[run];
    for (int s = 0; s < NSLOTS; ++s) {
        CUDA_TRY(cudaFree(d.tracers[s]));
        d.tracers[s] = nullptr;
    }
    d.ntracers = 0;
    if (n > 0) {
        for (int s = 0; s < NSLOTS; ++s) CUDA_TRY(cudaMalloc(&d.tracers[s], sizeof(double) * 2 * (size_t)n));
        CUDA_TRY(cudaMemcpy(d.tracers[ctx->cur], xy, sizeof(double) * 2 * (size_t)n, cudaMemcpyHostToDevice));
        d.ntracers = n;
    }
    CUDA_TRY(cudaMemcpy(ctx->rdev, ctx->rdev_h.data(), sizeof(RunDev) * ctx->nruns, cudaMemcpyHostToDevice));
    for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
    ctx->graphs.clear();
    return B2D_OK;
}

extern "C" b2d_status b2d_get_tracers(b2d_ctx* ctx, int32_t run, double* xy)
{
    if (!ctx || run < 0 || run >= ctx->nruns || !xy) return fail(B2D_ERR_INVALID, "bad arguments");
    const RunDev& d = ctx->rdev_h[run];
    if (d.ntracers > 0)
        CUDA_TRY(cudaMemcpyAsync(xy, d.tracers[ctx->cur], sizeof(double) * 2 * (size_t)d.ntracers,
                                 cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return B2D_OK;
}

static b2d_status run_advance(b2d_ctx* ctx, int fold, int* final_slot)
{
    if (fold * ctx->rk > 1023) return fail(B2D_ERR_INVALID, "fold x rk_order must be at most 1023");
    b2d_status st = ensure_stage_capacity(ctx, fold);
    if (st != B2D_OK) return st;
    const int start = ctx->cur;
    {
        int fs;
        ctx->window.emplace_back(start, plan_advance(ctx->rk, fold, start, &fs));
    }
    if (!ctx->use_graphs || ctx->instrument) {
        st = enqueue_advance(ctx, fold, start, final_slot, true);
        if (st != B2D_OK) return st;
        if (ctx->instrument) {
            CUDA_TRY(cudaStreamSynchronize(ctx->stream));
            for (int s = 0; s < fold * ctx->rk; ++s) {
                float ms = 0;
                CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev[2 * s], ctx->ev[2 * s + 1]));
                ctx->stage_ms_total += ms;
                ctx->stage_count++;
            }
        }
        return B2D_OK;
    }
    auto key = std::make_pair(fold, start);
    auto it = ctx->graphs.find(key);
    if (it == ctx->graphs.end()) {
        cudaGraph_t g;
        CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        st = enqueue_advance(ctx, fold, start, final_slot, false);
        cudaError_t ec = cudaStreamEndCapture(ctx->stream, &g);
        if (st != B2D_OK) return st;
        if (ec != cudaSuccess) return fail(B2D_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
        cudaGraphExec_t ge;
        CUDA_TRY(cudaGraphInstantiate(&ge, g, 0));
        cudaGraphDestroy(g);
        it = ctx->graphs.emplace(key, ge).first;
    } else {
        plan_advance(ctx->rk, fold, start, final_slot);
    }
    CUDA_TRY(cudaGraphLaunch(it->second, ctx->stream));
    ctx->launches += b2d_launches_per_advance(ctx, fold);
    return B2D_OK;
}

// Host restatement of try_to_primitive's failure value (physics.rs:489-503,
// 631-660) for the zone named by a failure key.
static double failure_value(const b2d_config& c, const double* u, int code)
{
    if (c.hydro_kind == B2D_ISOTHERMAL) return u[0];
    double g = c.gamma_law_index;
    double p[4] = {u[0], u[1] / u[0], u[2] / u[0], 0.0};
    p[3] = (u[3] - 0.5 * u[0] * (p[1] * p[1] + p[2] * p[2])) * (g - 1.0);
    if (c.has_density_floor && p[0] < c.density_floor) {
        p[0] = c.density_floor; p[1] = 0.0; p[2] = 0.0; p[3] = pow(c.density_floor, g);
    }
    if (code == 1) return p[0];
    if (c.has_pressure_floor && p[3] < c.pressure_floor) p[3] = c.pressure_floor;
    return p[3];
}

static b2d_status decode_failure(b2d_ctx* ctx, unsigned long long key, const std::vector<StagePlan>& plan,
                                 b2d_error* e)
{
    memset(e, 0, sizeof *e);
    const int stage = (int)(key >> 54);
    const int run = (int)((key >> 46) & 0xff);
    const int blk = (int)((key >> 30) & 0xffff);
    const int order = (int)((key >> 26) & 0xf);
    const int zone = (int)((key >> 2) & 0xffffff);
    e->code = (int)(key & 3);
    e->run = run;
    RunHost& r = ctx->runs[run];
    const int nb = r.nb, bs = r.bs;
    double orb[10];
    if (e->code == B2D_ERR_UNBOUND_ORBIT) {
        // OrbitalEvolutionError is reported at position (0, 0) (scheme.rs:308-309);
        // the failing block's index is carried in the zone field.
        e->block_i = zone / nb;
        e->block_j = zone % nb;
        CUDA_TRY(cudaMemcpy(&e->time, r.stage_time + stage, sizeof(double), cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(orb, r.orbit + 10 * stage, sizeof orb, cudaMemcpyDeviceToHost));
        e->binary[0] = orb[1]; e->binary[1] = orb[2]; e->binary[2] = orb[6]; e->binary[3] = orb[7];
        return B2D_OK;
    }
    const int bi = blk / nb, bj = blk % nb, di = order / 3 - 1, dj = order % 3 - 1;
    e->block_i = (bi + di + nb) % nb;
    e->block_j = (bj + dj + nb) % nb;
    e->zone_i = zone / bs;
    e->zone_j = zone % bs;
    const int gi = e->block_i * bs + e->zone_i, gj = e->block_j * bs + e->zone_j;
    e->x = r.hxc[gi];
    e->y = r.hxc[gj];
    const size_t nn = (size_t)r.N * r.N, idx = (size_t)gi * r.N + gj;
    const int slot = plan.at(stage).in;
    double u[4] = {0, 0, 0, 0};
    for (int f = 0; f < ctx->nf; ++f) {
        if (store_of(ctx) == 0) {
            CUDA_TRY(cudaMemcpy(&u[f], (const double*)r.slot[slot] + f * nn + idx, sizeof(double), cudaMemcpyDeviceToHost));
        } else {
            float hl[2];
            CUDA_TRY(cudaMemcpy(&hl[0], (const float*)r.slot[slot] + (2 * f) * nn + idx, sizeof(float), cudaMemcpyDeviceToHost));
            CUDA_TRY(cudaMemcpy(&hl[1], (const float*)r.slot[slot] + (2 * f + 1) * nn + idx, sizeof(float), cudaMemcpyDeviceToHost));
            u[f] = (double)hl[0] + (double)hl[1];
        }
    }
    e->value = failure_value(r.cfg, u, e->code);
    CUDA_TRY(cudaMemcpy(&e->time, r.stage_time + stage, sizeof(double), cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(orb, r.orbit + 10 * stage, sizeof orb, cudaMemcpyDeviceToHost));
    e->binary[0] = orb[1]; e->binary[1] = orb[2]; e->binary[2] = orb[6]; e->binary[3] = orb[7];
    return B2D_OK;
}

static b2d_status finish_advance(b2d_ctx* ctx, int final_slot, double* dt_out, b2d_error* err_out)
{
    unsigned long long key = ~0ull;
    long long count = 0;
    CUDA_TRY(cudaMemcpyAsync(&key, ctx->d_err_key, sizeof key, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaMemcpyAsync(&count, ctx->d_adv_count, sizeof count, cudaMemcpyDeviceToHost, ctx->stream));
    unsigned tmo = 0;
    CUDA_TRY(cudaMemcpyAsync(&tmo, ctx->d_timeout, sizeof tmo, cudaMemcpyDeviceToHost, ctx->stream));
    std::vector<double> dts(ctx->nruns);
    CUDA_TRY(cudaMemcpyAsync(dts.data(), ctx->d_dt, sizeof(double) * ctx->nruns, cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    auto window = std::move(ctx->window);
    ctx->window.clear();
    const long long base = ctx->adv_base;
    ctx->adv_base = count;
    if (dt_out) memcpy(dt_out, dts.data(), sizeof(double) * ctx->nruns);
    if (tmo) {
        CUDA_TRY(cudaMemsetAsync(ctx->d_timeout, 0, sizeof(unsigned), ctx->stream));
        CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        return fail(B2D_ERR_TIMEOUT, "a bounded wait on a staging barrier gave up; the step's results are invalid");
    }
    if (key != ~0ull) {
        // the failing advance is the last one whose prologue ran
        long long k = count - 1 - base;
        if (k < 0 || k >= (long long)window.size()) return fail(B2D_ERR_CUDA, "failure bookkeeping lost");
        const int start = window[k].first;
        b2d_error err;
        b2d_status s = decode_failure(ctx, key, window[k].second, &err);
        if (s != B2D_OK) return s;
        if (err_out) *err_out = err;
        CUDA_TRY(cudaMemsetAsync(ctx->d_err_key, 0xff, sizeof(unsigned long long), ctx->stream));
        ctx->cur = start;
        for (int r = 0; r < ctx->nruns; ++r) {
            s = launch_max_speed(ctx, r, start);
            if (s != B2D_OK) return s;
        }
        CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        return fail((b2d_status)err.code, "hydro error during advance");
    }
    if (final_slot >= 0) ctx->cur = final_slot;
    return B2D_OK;
}

extern "C" b2d_status b2d_advance(b2d_ctx* ctx, int32_t fold, double* dt_out, b2d_error* err_out)
{
    if (!ctx || fold < 1) return fail(B2D_ERR_INVALID, "bad arguments");
    int final_slot = -1;
    b2d_status st = run_advance(ctx, fold, &final_slot);
    if (st != B2D_OK) return st;
    return finish_advance(ctx, final_slot, dt_out, err_out);
}

extern "C" b2d_status b2d_advance_async(b2d_ctx* ctx, int32_t fold)
{
    if (!ctx || fold < 1) return fail(B2D_ERR_INVALID, "bad arguments");
    int final_slot = -1;
    b2d_status st = run_advance(ctx, fold, &final_slot);
    if (st != B2D_OK) return st;
    ctx->cur = final_slot;
    return B2D_OK;
}

extern "C" b2d_status b2d_synchronize(b2d_ctx* ctx, double* dt_out, b2d_error* err_out)
{
    if (!ctx) return fail(B2D_ERR_INVALID, "bad arguments");
    return finish_advance(ctx, -1, dt_out, err_out);
}

extern "C" b2d_status b2d_set_tile(b2d_ctx* ctx, int32_t tile_w, int32_t tile_h)
{
    if (!ctx) return fail(B2D_ERR_INVALID, "bad arguments");
    int tw = tile_w ? tile_w : ctx->tw, th = tile_h ? tile_h : ctx->th;
    if (!tile_ok(ctx, tw, th)) return fail(B2D_ERR_INVALID, "tile must divide the block size (width a multiple of 32, at most 256)");
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->tw = tw;
    ctx->th = th;
    return sync_rundev(ctx);
}

extern "C" b2d_status b2d_get_tile(const b2d_ctx* ctx, int32_t* tile_w, int32_t* tile_h)
{
    if (!ctx) return fail(B2D_ERR_INVALID, "bad arguments");
    if (tile_w) *tile_w = ctx->tw;
    if (tile_h) *tile_h = ctx->th;
    return B2D_OK;
}

extern "C" b2d_status b2d_set_strip_rows(b2d_ctx* ctx, int32_t rows)
{
    if (!ctx || rows < 0) return fail(B2D_ERR_INVALID, "bad arguments");
    if (rows > 0) {
        if (rows < 8) return fail(B2D_ERR_INVALID, "strip rows must be 0 or at least 8");
        for (const RunHost& r : ctx->runs)
            if (rows > r.bs) return fail(B2D_ERR_INVALID, "strip rows must not exceed the block size");
    }
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    ctx->strip_rows = rows;
    return sync_rundev(ctx);
}

extern "C" b2d_status b2d_get_strip_rows(const b2d_ctx* ctx, int32_t* rows)
{
    if (!ctx || !rows) return fail(B2D_ERR_INVALID, "bad arguments");
    *rows = ctx->strip_rows;
    return B2D_OK;
}

extern "C" b2d_status b2d_set_graphs(b2d_ctx* ctx, int32_t enable)
{
    if (!ctx) return fail(B2D_ERR_INVALID, "bad arguments");
    ctx->use_graphs = enable != 0;
    return B2D_OK;
}

extern "C" int64_t b2d_launch_count(const b2d_ctx* ctx) { return ctx ? ctx->launches : 0; }

extern "C" int64_t b2d_launches_per_advance(const b2d_ctx* ctx, int32_t fold)
{
    if (!ctx) return 0;
    int with_tracers = 0;
    for (const RunDev& d : ctx->rdev_h) with_tracers += d.ntracers > 0 ? 1 : 0;
    return 3 + (int64_t)fold * ctx->rk * (1 + with_tracers);
}

extern "C" b2d_status b2d_set_instrument(b2d_ctx* ctx, int32_t enable)
{
    if (!ctx) return fail(B2D_ERR_INVALID, "bad arguments");
    ctx->instrument = enable != 0;
    ctx->stage_ms_total = 0.0;
    ctx->stage_count = 0;
    return B2D_OK;
}

extern "C" b2d_status b2d_stage_stats(const b2d_ctx* ctx, int64_t* count, double* total_ms)
{
    if (!ctx) return fail(B2D_ERR_INVALID, "bad arguments");
    if (count) *count = ctx->stage_count;
    if (total_ms) *total_ms = ctx->stage_ms_total;
    return B2D_OK;
}

extern "C" b2d_status b2d_time_stages(b2d_ctx* ctx, int32_t fold, int32_t reps, double* ms_per_stage)
{
    if (!ctx || fold < 1 || reps < 1 || !ms_per_stage) return fail(B2D_ERR_INVALID, "bad arguments");
    bool was = ctx->instrument;
    b2d_set_instrument(ctx, 1);
    for (int r = 0; r < reps; ++r) {
        int fs;
        b2d_status st = run_advance(ctx, fold, &fs);
        if (st != B2D_OK) { ctx->instrument = was; return st; }
        ctx->cur = fs;
    }
    *ms_per_stage = ctx->stage_count ? ctx->stage_ms_total / ctx->stage_count : 0.0;
    ctx->instrument = was;
    return B2D_OK;
}

extern "C" b2d_status b2d_stream(const b2d_ctx* ctx, void** stream)
{
    if (!ctx || !stream) return fail(B2D_ERR_INVALID, "bad arguments");
    *stream = (void*)ctx->stream;
    return B2D_OK;
}

extern "C" b2d_status b2d_pin_host(void* ptr, uint64_t bytes)
{
    CUDA_TRY(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
    return B2D_OK;
}

extern "C" b2d_status b2d_unpin_host(void* ptr)
{
    CUDA_TRY(cudaHostUnregister(ptr));
    return B2D_OK;
}

extern "C" b2d_status b2d_set_device(int32_t device)
{
    CUDA_TRY(cudaSetDevice(device));
    return B2D_OK;
}

// ---------------------------------------------------------------------------
// Tile autotuner: time every tile shape that divides the block size with CUDA
// events on the context's stream, keep the fastest.  The advances run from
// the current slot, which the slot schedule never overwrites, so the state is
// unchanged afterwards (the max signal speed is recomputed).
static b2d_status time_tile(b2d_ctx* ctx, int fold, int reps, double* ms)
{
    ctx->instrument = true;
    ctx->stage_ms_total = 0.0;
    ctx->stage_count = 0;
    for (int r = 0; r < reps + 1; ++r) {
        int fs;
        std::vector<StagePlan> plan = plan_advance(ctx->rk, fold, ctx->cur, &fs);
        b2d_status st = enqueue_advance(ctx, fold, ctx->cur, &fs, true);
        if (st != B2D_OK) { ctx->instrument = false; return st; }
        CUDA_TRY(cudaStreamSynchronize(ctx->stream));
        if (r == 0) continue;  // warm-up
        for (size_t s = 0; s < plan.size(); ++s) {
            float m = 0;
            CUDA_TRY(cudaEventElapsedTime(&m, ctx->ev[2 * s], ctx->ev[2 * s + 1]));
            ctx->stage_ms_total += m;
            ctx->stage_count++;
        }
    }
    ctx->instrument = false;
    *ms = ctx->stage_ms_total / std::max<long long>(ctx->stage_count, 1);
    return B2D_OK;
}

// Strip rows for the chunk-taking kernel at the context's tile width: for the
// fewest whole waves of resident CTAs that chunks of at most a block's rows
// fill, and the next two, the shortest chunks that still fit in them.
static std::vector<int> strip_row_candidates(const b2d_ctx* ctx)
{
    std::vector<int> out;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return out;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return out;
    const int per_sm = stage_ctas_per_sm(ctx->nf, store_of(ctx), ctx->nruns, ctx->tw);
    if (sms <= 0 || per_sm <= 0) return out;
    const long long slots = (long long)sms * per_sm;
    int min_bs = 1 << 30;
    for (const RunHost& r : ctx->runs) min_bs = std::min(min_bs, r.bs);
    auto ctas = [&](int rows) {
        long long n = 0;
        for (const RunHost& r : ctx->runs) n += (long long)((r.N + rows - 1) / rows) * (r.N / ctx->tw);
        return n;
    };
    long long waves = (ctas(min_bs) + slots - 1) / slots;
    for (int c = 0; c < 3; ++c, ++waves) {
        int best = 0;
        for (int rows = min_bs; rows >= 8 && ctas(rows) <= waves * slots; --rows) best = rows;
        if (best && std::find(out.begin(), out.end(), best) == out.end()) out.push_back(best);
    }
    return out;
}

// A candidate replaces the fastest so far only when it is faster by more than
// timing noise, so that the choice is the same from run to run.
constexpr double AUTOTUNE_MARGIN = 0.99;

extern "C" b2d_status b2d_autotune(b2d_ctx* ctx, int32_t fold, int32_t reps, int32_t* tile_w, int32_t* tile_h,
                                   double* ms_per_stage)
{
    if (!ctx || fold < 1 || reps < 1) return fail(B2D_ERR_INVALID, "bad arguments");
    b2d_status st = ensure_stage_capacity(ctx, fold);
    if (st != B2D_OK) return st;
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    const int max_w = ctx->precision == B2D_PREC_FP64 || ctx->precision == B2D_PREC_FP32_COMP ? 256 : 128;
    int best_w = ctx->tw, best_h = ctx->th, best_rows = 0;
    double best = 1e300;
    ctx->strip_rows = 0;
    for (int w : {32, 64, 128, 256}) {
        if (w > max_w) continue;
        for (int h : {8, 16, 32, 64, 128}) {
            if (!tile_ok(ctx, w, h)) continue;
            ctx->tw = w;
            ctx->th = h;
            st = sync_rundev(ctx);
            if (st != B2D_OK) return st;
            double ms = 0;
            st = time_tile(ctx, fold, reps, &ms);
            if (st != B2D_OK) return st;
            if (ms < best * AUTOTUNE_MARGIN) { best = ms; best_w = w; best_h = h; }
        }
    }
    // row chunks of the FP32 kernels, at each tile width that takes them (the
    // widest first: the fewest halo warps)
    for (int w : {512, 256, 128, 64, 32}) {
        int h = 0;
        for (int hh : {64, 32, 16, 8})
            if (!h && tile_ok(ctx, w, hh)) h = hh;
        if (!h) continue;
        ctx->tw = w;
        ctx->th = h;
        if (!chunk_kernel(ctx)) continue;
        for (int rows : strip_row_candidates(ctx)) {
            ctx->strip_rows = rows;
            st = sync_rundev(ctx);
            if (st != B2D_OK) return st;
            double ms = 0;
            st = time_tile(ctx, fold, reps, &ms);
            if (st != B2D_OK) return st;
            if (ms < best * AUTOTUNE_MARGIN) { best = ms; best_w = w; best_h = h; best_rows = rows; }
        }
        ctx->strip_rows = 0;
    }
    // discard what the trial advances left behind
    long long count = 0;
    CUDA_TRY(cudaMemcpy(&count, ctx->d_adv_count, sizeof count, cudaMemcpyDeviceToHost));
    ctx->adv_base = count;
    ctx->window.clear();
    CUDA_TRY(cudaMemset(ctx->d_err_key, 0xff, sizeof(unsigned long long)));
    CUDA_TRY(cudaMemset(ctx->d_timeout, 0, sizeof(unsigned)));
    ctx->tw = best_w;
    ctx->th = best_h;
    ctx->strip_rows = best_rows;
    st = sync_rundev(ctx);
    if (st != B2D_OK) return st;
    for (int r = 0; r < ctx->nruns; ++r) {
        st = launch_max_speed(ctx, r, ctx->cur);
        if (st != B2D_OK) return st;
    }
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (tile_w) *tile_w = best_w;
    if (tile_h) *tile_h = best_h;
    if (ms_per_stage) *ms_per_stage = best;
    return B2D_OK;
}

// ---------------------------------------------------------------------------
// Row slabs: one run split across contexts (one per GPU or process), each of
// which advances the blocks of its own block rows.  No counterpart in the
// reference, which advances every block of a run in one process; its block
// dataflow joins each block with its 3x3 neighbours and extends a 2-zone
// halo (src/scheme.rs:119-133, periodic neighbours src/mesh.rs:101-110), so a
// slab needs the 2 zone rows on either side of it from the neighbouring slabs
// before every stage, the global maximum signal speed for dt once per
// advance, and its blocks' ledgers summed with the others' by the caller.

extern "C" b2d_status b2d_set_slab(b2d_ctx* ctx, int32_t run, int32_t block_row_lo, int32_t block_row_hi)
{
    if (!ctx || run < 0 || run >= ctx->nruns) return fail(B2D_ERR_INVALID, "bad arguments");
    RunDev& d = ctx->rdev_h[run];
    const bool whole = block_row_lo == 0 && block_row_hi == 0;
    if (!whole && (block_row_lo < 0 || block_row_hi > d.nb || block_row_lo >= block_row_hi))
        return fail(B2D_ERR_INVALID, "slab rows must satisfy 0 <= lo < hi <= num_blocks");
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    d.slab_lo = whole ? 0 : block_row_lo;
    d.slab_hi = whole ? 0 : block_row_hi;
    b2d_status st = sync_rundev(ctx);
    if (st != B2D_OK) return st;
    // the stored maximum signal speed becomes the slab's
    st = launch_max_speed(ctx, run, ctx->cur);
    if (st != B2D_OK) return st;
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return B2D_OK;
}

extern "C" b2d_status b2d_slab_begin(b2d_ctx* ctx, int32_t fold, const double* amax)
{
    if (!ctx || fold < 1 || !amax) return fail(B2D_ERR_INVALID, "bad arguments");
    if (ctx->slab_next >= 0) return fail(B2D_ERR_INVALID, "a slab advance is already in progress");
    if (fold * ctx->rk > 1023) return fail(B2D_ERR_INVALID, "fold x rk_order must be at most 1023");
    b2d_status st = ensure_stage_capacity(ctx, fold);
    if (st != B2D_OK) return st;
    // dt comes from the maximum signal speed over every slab of each run
    std::vector<unsigned long long> bits(ctx->nruns);
    memcpy(bits.data(), amax, sizeof(double) * ctx->nruns);
    CUDA_TRY(cudaMemcpyAsync(ctx->d_amax, bits.data(), sizeof(unsigned long long) * ctx->nruns, cudaMemcpyHostToDevice,
                             ctx->stream));
    const int start = ctx->cur;
    ctx->slab_plan = plan_advance(ctx->rk, fold, start, &ctx->slab_final);
    ctx->slab_fold = fold;
    ctx->slab_start = start;
    ctx->slab_next = 0;
    ctx->window.emplace_back(start, ctx->slab_plan);
    prologue_kernel<<<ctx->nruns, 32, 0, ctx->stream>>>(ctx->rdev, fold, ctx->rk, start, ctx->slab_final, ctx->d_err_key,
                                                         ctx->d_adv_count);
    CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));   // bits is host memory of this call
    return B2D_OK;
}

extern "C" b2d_status b2d_slab_stage(b2d_ctx* ctx)
{
    if (!ctx || ctx->slab_next < 0 || ctx->slab_next >= (int)ctx->slab_plan.size())
        return fail(B2D_ERR_INVALID, "no slab stage left to run");
    const int s = ctx->slab_next;
    b2d_status st = launch_stage(ctx, ctx->slab_plan[s], s, s + 1 == (int)ctx->slab_plan.size());
    if (st != B2D_OK) return st;
    ctx->launches++;
    st = launch_tracers(ctx, ctx->slab_plan[s], true);
    if (st != B2D_OK) return st;
    ctx->slab_next++;
    return B2D_OK;
}

extern "C" b2d_status b2d_slab_end(b2d_ctx* ctx, double* dt_out, b2d_error* err_out)
{
    if (!ctx || ctx->slab_next != (int)ctx->slab_plan.size() || ctx->slab_plan.empty())
        return fail(B2D_ERR_INVALID, "the slab advance has stages left to run");
    b2d_status st = launch_elements(ctx, ctx->slab_fold, ctx->slab_start, (int)ctx->slab_plan.size(), true);
    ctx->slab_next = -1;
    if (st != B2D_OK) return st;
    return finish_advance(ctx, ctx->slab_final, dt_out, err_out);
}

extern "C" b2d_status b2d_slab_rows(b2d_ctx* ctx, int32_t run, int32_t row0, int32_t nrows, double* rows, int32_t put)
{
    if (!ctx || run < 0 || run >= ctx->nruns || !rows || nrows < 1) return fail(B2D_ERR_INVALID, "bad arguments");
    RunHost& r = ctx->runs[run];
    if (nrows > r.N) return fail(B2D_ERR_INVALID, "more rows than the mesh has");
    // the next stage's input slot, or the current state between advances
    const int slot = ctx->slab_next >= 0 && ctx->slab_next < (int)ctx->slab_plan.size()
                         ? ctx->slab_plan[ctx->slab_next].in : ctx->cur;
    const size_t nn = (size_t)r.N * r.N;
    // the stored words as they are: FP64 planes (FP64 and FP64-state contexts),
    // or the hi and lo FP32 planes of the compensated state, so that the
    // receiving context continues with exactly the sender's words
    const int parts = store_of(ctx) == 1 ? 2 : 1;
    const size_t w = store_of(ctx) == 1 ? sizeof(float) : sizeof(double);
    unsigned char* planes = (unsigned char*)r.slot[slot];
    unsigned char* buf = (unsigned char*)rows;
    for (int f = 0; f < ctx->nf; ++f)
        for (int part = 0; part < parts; ++part)
            for (int k = 0; k < nrows; ++k) {
                const int gi = ((row0 + k) % r.N + r.N) % r.N;
                unsigned char* dev = planes + (((size_t)(f * parts + part)) * nn + (size_t)gi * r.N) * w;
                unsigned char* host = buf + (((size_t)(f * parts + part) * nrows + k) * r.N) * w;
                if (put) CUDA_TRY(cudaMemcpyAsync(dev, host, w * r.N, cudaMemcpyHostToDevice, ctx->stream));
                else CUDA_TRY(cudaMemcpyAsync(host, dev, w * r.N, cudaMemcpyDeviceToHost, ctx->stream));
            }
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return B2D_OK;
}

// ---------------------------------------------------------------------------
// One RK stage that allocates nothing.
//
// Some callers cannot call cudaMalloc: a host code that owns a fixed device
// memory pool and forbids allocation by libraries, or an allocator-less
// embedded runtime.  They hand over every input and
// output buffer themselves; the scratch the stage kernel needs (its run
// descriptor, the binary at the stage time, per-tile ledger partials, block
// counters, the max-speed word and the failure key) lives in the file-scope
// array below, which every GPU that loads this library holds until the
// process exits.
constexpr size_t B2D_NOALLOC_SCRATCH_BYTES = 4u << 20;   // 4 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[B2D_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_base[NOALLOC_MAX_DEVICES] = {};
}  // namespace

// Device address of the scratch array on the current device.  The host-side
// name g_noalloc_scratch is only a stand-in for the symbol, never a device
// address: the address comes from cudaGetSymbolAddress, once per device.
static b2d_status noalloc_scratch_base(unsigned char** base)
{
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return fail(B2D_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_base[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(B2D_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_noalloc_base[dev] = (unsigned char*)p;
    }
    *base = g_noalloc_base[dev];
    return B2D_OK;
}

// The binary at the stage time, dt and the stage time, written into scratch.
__global__ void noalloc_setup_kernel(RunDev* rd, double time, double dt)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        kepler_orbit(*rd, time, rd->orbit);
        *rd->dt = dt;
        rd->stage_time[0] = time;
    }
}

extern "C" b2d_status b2d_stage_noalloc(const b2d_config* cfg, const double* d_in, const double* d_background,
                                        const double* d_base, double* d_out, const double* d_ledger_in,
                                        const double* d_ledger_base, double* d_ledger_out, double time, double dt,
                                        double bf, double* d_max_speed, b2d_error* err_out, void* stream_ptr)
{
    if (!cfg || !d_in || !d_background || !d_out || !d_ledger_in || !d_ledger_out || (d_base && !d_ledger_base))
        return fail(B2D_ERR_INVALID, "b2d_stage_noalloc: missing buffer");
    b2d_status st = validate(*cfg, cfg->hydro_kind, cfg->rk_order);
    if (st != B2D_OK) return st;
    cudaStream_t stream = (cudaStream_t)stream_ptr;
    const int nf = cfg->hydro_kind == B2D_EULER ? 4 : 3;
    const int bs = cfg->block_size, nb = cfg->num_blocks, N = bs * nb, nblocks = nb * nb;
    int tw = default_tile_w(bs), th = std::min(64, bs);
    while (bs % th) th /= 2;
    // one thread per tile column: a block width that is not a multiple of 32
    // is its own tile, which the FP64 kernel's 256-thread bound must hold
    if (tw > 256)
        return fail(B2D_ERR_INVALID, "b2d_stage_noalloc: block_size " + std::to_string(bs) +
                                         " must be a multiple of 32 or at most 256");
    const int tiles_per_block = (bs / th) * (bs / tw);
    const int ntiles = (N / th) * (N / tw);

    // scratch layout: run descriptor | control words | counters | tile partials
    const size_t off_run = 0, off_ctl = 2048, off_cnt = 2304;
    const size_t off_part = off_cnt + ((sizeof(unsigned) * (size_t)nblocks + 255) / 256) * 256;
    const size_t need = off_part + sizeof(double) * (size_t)nblocks * tiles_per_block * NITEMS * nf;
    static_assert(sizeof(RunDev) <= 2048, "run descriptor outgrew its scratch slot");
    if (need > B2D_NOALLOC_SCRATCH_BYTES)
        return fail(B2D_ERR_INVALID, "b2d_stage_noalloc: this mesh needs " + std::to_string(need) +
                                         " bytes of scratch; the library holds " +
                                         std::to_string(B2D_NOALLOC_SCRATCH_BYTES) + " (use b2d_create instead)");
    unsigned char* base = nullptr;
    st = noalloc_scratch_base(&base);
    if (st != B2D_OK) return st;

    RunDev* d_run = (RunDev*)(base + off_run);
    double* orbit = (double*)(base + off_ctl);            // 10 doubles
    double* d_dt = orbit + 10;
    double* stime = orbit + 11;
    double* times = orbit + 12;                            // 4 doubles (unused by the stage)
    long long* iters = (long long*)(orbit + 16);           // 4 (unused by the stage)
    unsigned long long* amax = (unsigned long long*)(orbit + 20);
    unsigned long long* err_key = amax + 1;
    unsigned* timeout = (unsigned*)(err_key + 1);
    unsigned* counter = (unsigned*)(base + off_cnt);
    double* partial = (double*)(base + off_part);

    std::vector<double> xc(N), xv((size_t)nb * (bs + 1));
    for (int b = 0; b < nb; ++b) {
        host_cell_centers(cfg, b, xc.data() + (size_t)b * bs);
        host_block_vertices(cfg, b, xv.data() + (size_t)b * (bs + 1));
    }
    // the FP64 kernel reads its geometry from the run descriptor's tables: place
    // them behind the partials in scratch
    const size_t off_geo = ((need + 255) / 256) * 256;
    const size_t need_geo = off_geo + sizeof(double) * (xc.size() + xv.size());
    if (need_geo > B2D_NOALLOC_SCRATCH_BYTES)
        return fail(B2D_ERR_INVALID, "b2d_stage_noalloc: mesh too large for the 4 MiB scratch (use b2d_create instead)");
    double* d_xc = (double*)(base + off_geo);
    double* d_xv = d_xc + xc.size();

    RunDev rd;
    memset(&rd, 0, sizeof rd);
    rd.N = N; rd.bs = bs; rd.nb = nb; rd.nblocks = nblocks;
    rd.tiles_i = N / th; rd.tiles_j = N / tw; rd.ntiles = ntiles; rd.tile_base = 0;
    rd.chunks = rd.tiles_i; rd.chunk0 = 0;
    rd.tiles_per_block = tiles_per_block;
    rd.xc = d_xc; rd.xv = d_xv;
    rd.slot[0] = (void*)d_in; rd.slot[1] = (void*)d_base; rd.slot[2] = d_out; rd.slot[3] = d_out;
    rd.bg = d_background;
    rd.ledger[0] = (double*)d_ledger_in; rd.ledger[1] = (double*)d_ledger_base;
    rd.ledger[2] = d_ledger_out; rd.ledger[3] = d_ledger_out;
    rd.time = times; rd.iter = iters;
    rd.partial = partial; rd.counter = counter;
    rd.dt = d_dt; rd.stage_time = stime; rd.orbit = orbit; rd.amax = amax;
    rd.binary_q = cfg->binary_mass_ratio; rd.binary_e = cfg->binary_eccentricity;
    rd.p = make_params<double>(*cfg);
    rd.pf = make_params<float>(*cfg);

    // every call shares the scratch: reset what must start from zero (or ~0)
    CUDA_TRY(cudaMemcpyAsync(d_run, &rd, sizeof rd, cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(d_xc, xc.data(), sizeof(double) * xc.size(), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(d_xv, xv.data(), sizeof(double) * xv.size(), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(unsigned) * nblocks, stream));
    CUDA_TRY(cudaMemsetAsync(amax, 0, sizeof(unsigned long long), stream));
    CUDA_TRY(cudaMemsetAsync(err_key, 0xff, sizeof(unsigned long long), stream));
    CUDA_TRY(cudaMemsetAsync(timeout, 0, sizeof(unsigned), stream));
    noalloc_setup_kernel<<<1, 32, 0, stream>>>(d_run, time, dt);
    CUDA_TRY(cudaGetLastError());

    StageArgs a;
    a.runs = d_run;
    a.nruns = 1;
    a.th = th;
    a.in_slot = 0;
    a.base_slot = d_base ? 1 : -1;
    a.out_slot = 2;
    a.stage = 0;
    a.amax_flag = d_max_speed ? 1 : 0;
    a.bf = d_base ? bf : 0.0;
    a.w1f = split_df(-a.bf + 1.0);
    a.bff = split_df(a.bf);
    a.err_key = err_key;
    a.timeout_flag = timeout;
    cudaError_t e = launch_stage_f64(nf, a, ntiles, tw, stage_smem_bytes(nf, 8, tw), stream);
    if (e != cudaSuccess) return fail(B2D_ERR_CUDA, std::string("stage kernel launch: ") + cudaGetErrorString(e));
    if (d_max_speed) CUDA_TRY(cudaMemcpyAsync(d_max_speed, amax, sizeof(double), cudaMemcpyDeviceToDevice, stream));

    unsigned long long key = ~0ull;
    CUDA_TRY(cudaMemcpyAsync(&key, err_key, sizeof key, cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (key == ~0ull) return B2D_OK;

    // decode the failure key of the stage (see error_key in stage.cuh)
    b2d_error err;
    memset(&err, 0, sizeof err);
    const int blk = (int)((key >> 30) & 0xffff), order = (int)((key >> 26) & 0xf);
    const int zone = (int)((key >> 2) & 0xffffff);
    err.code = (int)(key & 3);
    err.block_i = (blk / nb + order / 3 - 1 + nb) % nb;
    err.block_j = (blk % nb + order % 3 - 1 + nb) % nb;
    err.zone_i = zone / bs;
    err.zone_j = zone % bs;
    const int gi = err.block_i * bs + err.zone_i, gj = err.block_j * bs + err.zone_j;
    err.x = xc[gi];
    err.y = xc[gj];
    err.time = time;
    double u[4] = {0, 0, 0, 0}, orb[10];
    for (int f = 0; f < nf; ++f)
        CUDA_TRY(cudaMemcpy(&u[f], d_in + (size_t)f * N * N + (size_t)gi * N + gj, sizeof(double),
                            cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(orb, orbit, sizeof orb, cudaMemcpyDeviceToHost));
    err.value = failure_value(*cfg, u, err.code);
    err.binary[0] = orb[1]; err.binary[1] = orb[2]; err.binary[2] = orb[6]; err.binary[3] = orb[7];
    if (err_out) *err_out = err;
    return fail((b2d_status)err.code, "hydro error in b2d_stage_noalloc");
}

// ---------------------------------------------------------------------------
// Orbital-element change per block (BlockState::orbital_elements_change,
// src/state.rs:44-49): [nb][nb][7][4] of (a, M, q, e) per ItemizedChange item.
extern "C" b2d_status b2d_download_elements(b2d_ctx* ctx, int32_t run, double* elements)
{
    if (!ctx || run < 0 || run >= ctx->nruns || !elements) return fail(B2D_ERR_INVALID, "bad arguments");
    RunHost& r = ctx->runs[run];
    CUDA_TRY(cudaMemcpyAsync(elements, r.elements[ctx->cur], sizeof(double) * r.nblocks * NITEMS * 4,
                             cudaMemcpyDeviceToHost, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return B2D_OK;
}

extern "C" b2d_status b2d_upload_elements(b2d_ctx* ctx, int32_t run, const double* elements)
{
    if (!ctx || run < 0 || run >= ctx->nruns || !elements) return fail(B2D_ERR_INVALID, "bad arguments");
    RunHost& r = ctx->runs[run];
    CUDA_TRY(cudaMemcpyAsync(r.elements[ctx->cur], elements, sizeof(double) * r.nblocks * NITEMS * 4,
                             cudaMemcpyHostToDevice, ctx->stream));
    CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return B2D_OK;
}
