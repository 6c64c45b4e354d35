// lbm_capi.cu - C ABI of include/lbm.h: context, geometry classification, stepping, read-back.
//
// Host-side counterpart of the reference's set-up and driver code:
//   geometryMesherBoundary (flag encoding, BC lists, arrayTransfer; geometryMesherBoundary.h),
//   InitializationEquilibriumConstVector (initialisation), SolverTurbulentLES::runSimulation
//   (the step loop), MomentTimeAvg / ErrorQuadratic (monitors).
// Every call returns a status; CUDA errors and inconsistent set-ups are reported, never thrown.

#include "../../include/lbm.h"
#include "lbm_device.cuh"
#include "lbm_aux.cuh"
#include "lbm_launch.h"
#include "lbm_mlp_host.h"
#include "lbm_sync.cuh"

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

using namespace lbm;

static_assert(OUT_INTERPOLATED == LBM_OUTLET_DENSITY_INTERPOLATED && OUT_NEQ == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM &&
                  OUT_NEQ_OMEGA == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA &&
                  OUT_NEQ_OMEGA_RF == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF &&
                  OUT_DENSITY_EQ == LBM_OUTLET_DENSITY_EQUILIBRIUM,
              "device outlet kinds follow lbm.h");

struct lbm_ctx {
    lbm_config cfg{};
    cudaStream_t st = nullptr;
    cudaStream_t st_side = nullptr;    // split step: the remaining rows run here, beside the plain rows
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    long long N = 0;
    size_t esize = 0;  // bytes per stored population
    void* d_f = nullptr;
    uint8_t* d_cls = nullptr;
    int32_t* d_aux = nullptr;
    std::vector<int32_t> flags;
    std::vector<lbm_bc_inlet> inlets;
    std::vector<lbm_bc_outlet> outlets;
    std::vector<lbm_bc_symmetry> syms;
    bool have_flags = false, have_geom = false, initialized = false;
    bool rows_pending = false;                  // build_geometry left the row lists for finish_rows
    std::unique_ptr<uint8_t[]> host_cls;        //   with the class bytes they are built from
    // side tables
    int n_lid = 0, n_in = 0, n_out = 0;
    void* d_lid_state = nullptr;
    float *d_lid_n = nullptr, *d_lid_u = nullptr;
    void* d_in_probe = nullptr;
    float* d_in_u = nullptr;
    int32_t* d_in_dir = nullptr;
    void* d_out_save = nullptr;
    float* d_out_rho = nullptr;
    int32_t* d_out_dir = nullptr;
    int n_ms = 0;                    // neighbour-equilibrium outlets: cells that keep their moments
    void* d_out_msave = nullptr;
    int32_t* d_out_nb = nullptr;
    int n_sym = 0;
    int32_t* d_sym_dir = nullptr;
    int sponge_axis = -1, sponge_begin = 0;
    double sponge_slope = 0.0;
    long long m = 0;  // steps done
    // monitors
    double* d_acc = nullptr;
    bool avg_on = false;
    long long avg_begin = 0, avg_last = -1, avg_count = 0;
    void* d_uerr = nullptr;     // error monitor's previous velocity, 3N of the storage's real type
    double* d_red = nullptr;
    double* d_part = nullptr;  // per-block partial sums of the reductions (read_part_size doubles)
    double *d_rho_out = nullptr, *d_u_out = nullptr, *d_f_out = nullptr;
    double* d_probe = nullptr;
    int32_t* d_bulk_rows = nullptr;   // (y,z) rows whose cells are all bulk fluid
    int32_t* d_other_rows = nullptr;  // the remaining rows
    int n_bulk_rows = 0, n_other_rows = 0;
    int32_t* d_plain_rows = nullptr;  // split step: rows whose pairs all take the packed path
    int32_t* d_rest_rows = nullptr;   // split step: the remaining rows that are not wall rows
    int32_t* d_wall_rows = nullptr;   // split step: rows beside a flat wall (packed, bounce-back by mask)
    uint32_t* d_wall_solid = nullptr; //   their solid-source masks
    int32_t* d_rest_all = nullptr;    // split step: all non-plain rows (closures without the wall kernel)
    int n_plain_rows = 0, n_rest_rows = 0, n_wall_rows = 0, n_rest_all = 0;
    bool split_ok = false;            // the step runs split by rows (FP32 / FP16 storage)
    int* d_err = nullptr;             // device error word
    bool rows_ok = false;             // the row-staged step applies to this lattice
    uint4* d_mlp_frag = nullptr;      // learned closure: fragment table
    MlpNorm mlp_norm{};
    bool have_mlp = false;
    __half* d_nut = nullptr;          // kept nu_t per cell (refresh interval > 1)
    long long mlp_due = 0;            // next step in which the network runs
    std::string err;
};

static std::string g_err;

// a[q[i]] = v[i] for the n listed cells (the side-table indices set at set-up)
__global__ void k_scatter_aux(int32_t* a, const long long* q, const int32_t* v, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[q[i]] = v[i];
}

static lbm_status fail(lbm_ctx* c, lbm_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    g_err = buf;
    return s;
}
#define CU(ctx, call)                                                                                 \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA, "%s: %s (%s:%d)", \
                        #call, cudaGetErrorString(e_), __FILE__, __LINE__);                           \
    } while (0)

static void dfree(void* p) { if (p) cudaFree(p); }

// runs f(begin, end) over [0, n) split into contiguous chunks on the host cores (set-up loops), at
// least `grain` items per chunk (65536 for loops over cells, 65536 / nx for loops over rows of cells);
// each chunk writes only its own range
// compile-time loop over [B, E) for host code: f(std::integral_constant<int, v>) for each v
template <int B, int E, class F>
static inline void sfor_host(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        sfor_host<B + 1, E>(f);
    }
}

template <class F>
static void host_parallel(long long n, F&& f, long long grain = 65536) {
    const unsigned hw = std::thread::hardware_concurrency();
    const long long nth = std::min<long long>(std::max(1u, std::min(hw, 32u)), std::max(1LL, n / std::max(1LL, grain)));
    if (nth <= 1) { f(0LL, n); return; }
    std::vector<std::thread> th;
    for (long long t = 0; t < nth; t++)
        th.emplace_back([&, t] { f(n * t / nth, n * (t + 1) / nth); });
    for (auto& x : th) x.join();
}

static size_t real_size(const lbm_ctx* c) { return c->cfg.storage == LBM_STORAGE_F64 ? 8 : 4; }

static Params make_params(const lbm_ctx* c) {
    Params p;
    std::memset(&p, 0, sizeof(p));
    p.f = c->d_f; p.cls = c->d_cls; p.aux = c->d_aux;
    p.nx = c->cfg.nx; p.ny = c->cfg.ny; p.nz = c->cfg.nz;
    for (int a = 0; a < 3; a++) p.wrap[a] = c->cfg.periodic[a] ? 1 : 0;
    p.N = c->N;
    p.m = (int)c->m;
    p.sr_step_seed = step_seed(p.m);
    p.tau = c->cfg.tau > 0 ? c->cfg.tau : 3.0 * c->cfg.nu + 0.5;
    p.cles18 = 18.0 * c->cfg.cles;
    p.nu = c->cfg.nu;
    for (int a = 0; a < 3; a++) p.F[a] = c->cfg.force[a];
    p.tauf = (float)p.tau; p.cles18f = (float)p.cles18; p.nuf = (float)p.nu;
    p.omega0 = 1.0 / p.tau;
    p.omega0f = (float)p.omega0;
    for (int a = 0; a < 3; a++) p.Ff[a] = (float)p.F[a];
    p.has_force = (p.F[0] != 0.0 || p.F[1] != 0.0 || p.F[2] != 0.0) ? 1 : 0;
    p.rho0 = (float)c->cfg.rho0;
    p.f16_sr = (c->cfg.storage == LBM_STORAGE_F16DEV && !(c->cfg.options & LBM_OPT_F16_ROUND_NEAREST)) ? 1 : 0;
    p.sr_mul = p.f16_sr ? 1u : 0u;
    p.sr_add = p.f16_sr ? 0u : kHalfStep2x;
    for (int v = 0; v < 27; v++) p.sr_off[v] = p.f16_sr ? (uint32_t)v * kSrWeyl : 0u;
    p.scale = std::ldexp(1.0f, c->cfg.f16_scale_log2);
    p.inv_scale = std::ldexp(1.0f, -c->cfg.f16_scale_log2);
    p.scale2 = make_float2(p.scale, p.scale);
    p.inv_scale2 = make_float2(p.inv_scale, p.inv_scale);
    // per-direction addresses of the fast path (bulk cells off the periodic seams)
    const unsigned long long base = (unsigned long long)c->d_f, es = (unsigned long long)c->esize;
    const long long nx = c->cfg.nx, nxy = (long long)c->cfg.nx * c->cfg.ny;
    double raw_rho = 0.0, raw_mdiag = 0.0;
    for (int v = 0; v < 27; v++) {
        const int o = opp(v);
        const long long off = cx(v) + cy(v) * nx + cz(v) * nxy;  // element offset of x + c_v
        p.wr[v] = (float)(wgt(v) * c->cfg.rho0);
        p.nwrs[v] = -(float)(wgt(v) * c->cfg.rho0) * p.scale;
        p.wr2[v] = make_float2(p.wr[v], p.wr[v]);
        raw_rho += (double)p.wr[v];
        raw_mdiag += (double)p.wr[v] * cx(v) * cx(v);
        p.nwrs2[v] = make_float2(p.nwrs[v], p.nwrs[v]);
        p.rd_even[v] = base + (unsigned long long)(v * c->N) * es;
        p.rd_odd[v] = base + (unsigned long long)(o * c->N - off) * es;
        p.wr_even[v] = base + (unsigned long long)(o * c->N) * es;
        p.wr_odd[v] = base + (unsigned long long)(v * c->N + off) * es;
    }
    p.raw_rho = (float)raw_rho;
    p.raw_mdiag = (float)raw_mdiag;
    p.lid_state = c->d_lid_state; p.lid_n = c->d_lid_n; p.lid_u = c->d_lid_u; p.n_lid = c->n_lid;
    p.in_probe = c->d_in_probe; p.in_u = c->d_in_u; p.in_dir = c->d_in_dir; p.n_in = c->n_in;
    p.out_save = c->d_out_save; p.out_rho = c->d_out_rho; p.out_dir = c->d_out_dir; p.n_out = c->n_out;
    p.outlet_kind = c->cfg.outlet_kind;
    p.out_msave = c->d_out_msave; p.out_nb = c->d_out_nb; p.n_ms = c->n_ms;
    p.inlet_zouhe = c->cfg.inlet_kind == LBM_INLET_ZOU_HE ? 1 : 0;
    p.sym_dir = c->d_sym_dir; p.n_sym = c->n_sym;
    p.sponge_axis = c->sponge_axis; p.sponge_begin = c->sponge_begin;
    p.sponge_slope = c->sponge_slope; p.sponge_slopef = (float)c->sponge_slope;
    p.mlp_frag = c->d_mlp_frag;
    p.mlp = c->mlp_norm;
    p.nut = c->d_nut;
    p.mlp_run = 0;
    p.mlp_tc = (c->cfg.options & LBM_OPT_MLP_TCGEN05) ? 1 : 0;
    p.acc = nullptr;
    p.err = c->d_err;
    return p;
}

static cudaError_t do_step(lbm_ctx* c, const Params& p) {
    if (c->rows_ok && p.acc == nullptr && c->cfg.collision == LBM_COLLISION_CUMULANT2015 &&
        c->cfg.storage == LBM_STORAGE_F16DEV)
        return launch_step_rows<StF16>(p, c->cfg.closure, c->d_bulk_rows, c->n_bulk_rows, c->d_other_rows,
                                       c->n_other_rows, c->st);
    RowLists rl;
    rl.plain = c->d_plain_rows; rl.n_plain = c->n_plain_rows;
    rl.other = c->d_rest_rows; rl.n_other = c->n_rest_rows;
    rl.wall = c->d_wall_rows; rl.wall_solid = c->d_wall_solid; rl.n_wall = c->n_wall_rows;
    rl.other_all = c->d_rest_all; rl.n_other_all = c->n_rest_all;
    rl.side = c->st_side; rl.fork = c->ev_fork; rl.join = c->ev_join;
    const RowLists* r = c->split_ok ? &rl : nullptr;
    switch (c->cfg.storage) {
        case LBM_STORAGE_F64: return launch_step<StF64>(p, c->cfg.collision, c->cfg.closure, nullptr, c->st);
        case LBM_STORAGE_F32: return launch_step<StF32>(p, c->cfg.collision, c->cfg.closure, r, c->st);
        default: return launch_step<StF16>(p, c->cfg.collision, c->cfg.closure, r, c->st);
    }
}
static cudaError_t do_read(lbm_ctx* c, const Params& p, const ReadOut& o) {
    switch (c->cfg.storage) {
        case LBM_STORAGE_F64: return launch_read<StF64>(p, o, c->st);
        case LBM_STORAGE_F32: return launch_read<StF32>(p, o, c->st);
        default: return launch_read<StF16>(p, o, c->st);
    }
}
static cudaError_t do_init(lbm_ctx* c, const Params& p, const double* r, const double* u, double r0, const double u0[3],
                           const double* pops) {
    switch (c->cfg.storage) {
        case LBM_STORAGE_F64: return launch_init<StF64>(p, r, u, r0, u0, pops, c->st);
        case LBM_STORAGE_F32: return launch_init<StF32>(p, r, u, r0, u0, pops, c->st);
        default: return launch_init<StF16>(p, r, u, r0, u0, pops, c->st);
    }
}

extern "C" {

int32_t lbm_abi_version(void) { return LBM_ABI_VERSION; }

const char* lbm_status_string(lbm_status s) {
    switch (s) {
        case LBM_OK: return "ok";
        case LBM_ERR_INVALID: return "invalid argument";
        case LBM_ERR_OOM: return "out of memory";
        case LBM_ERR_CUDA: return "CUDA error";
        case LBM_ERR_NONFINITE: return "non-finite populations";
        case LBM_ERR_TIMEOUT: return "device wait timed out";
        case LBM_ERR_STATE: return "call out of order";
        case LBM_ERR_IO: return "I/O error";
        case LBM_ERR_UNSUPPORTED: return "unsupported configuration";
        default: return "unknown status";
    }
}

const char* lbm_last_error(const lbm_ctx* c) { return c ? c->err.c_str() : g_err.c_str(); }

lbm_status lbm_create(const lbm_config* cfg, lbm_ctx** out) {
    if (!cfg || !out) return fail(nullptr, LBM_ERR_INVALID, "lbm_create: null argument");
    *out = nullptr;
    if (cfg->nx < 3 || cfg->ny < 3 || cfg->nz < 3)
        return fail(nullptr, LBM_ERR_INVALID, "lattice must be at least 3 cells per axis (got %d %d %d)", cfg->nx, cfg->ny, cfg->nz);
    long long N = (long long)cfg->nx * cfg->ny * cfg->nz;
    // cell indices are 32-bit in the kernels (signed in the pair path, where an x-wrapped index may
    // exceed the cell by up to nx): N + nx must stay below 2^31; y and z are launch-grid dimensions
    if (cfg->nx > (1 << 21) || N > (1LL << 31) - (1LL << 21) || cfg->ny > 65535 || cfg->nz > 65535)
        return fail(nullptr, LBM_ERR_UNSUPPORTED,
                    "lattice %d x %d x %d: at most 2^31 - 2^21 cells, nx <= 2^21, ny and nz <= 65535",
                    cfg->nx, cfg->ny, cfg->nz);
    if ((cfg->collision == LBM_COLLISION_CUMULANT2017 || cfg->collision == LBM_COLLISION_CUMULANT_COMBINED) &&
        cfg->closure == LBM_CLOSURE_MLP)
        return fail(nullptr, LBM_ERR_UNSUPPORTED, "the learned closure runs with the SRT or cumulant-2015 collision");
    if (cfg->collision != LBM_COLLISION_SRT && cfg->collision != LBM_COLLISION_CUMULANT2015 &&
        cfg->collision != LBM_COLLISION_CUMULANT2017 && cfg->collision != LBM_COLLISION_CUMULANT_COMBINED)
        return fail(nullptr, LBM_ERR_UNSUPPORTED, "collision %d not implemented", cfg->collision);
    if (cfg->closure != LBM_CLOSURE_NONE && cfg->closure != LBM_CLOSURE_SMAGORINSKY && cfg->closure != LBM_CLOSURE_MLP)
        return fail(nullptr, LBM_ERR_UNSUPPORTED, "closure %d not implemented", cfg->closure);
    if (cfg->mlp_interval < 0) return fail(nullptr, LBM_ERR_INVALID, "mlp_interval %d < 0", cfg->mlp_interval);
    if (cfg->inlet_kind < LBM_INLET_MOVING_WALL || cfg->inlet_kind > LBM_INLET_ZOU_HE)
        return fail(nullptr, LBM_ERR_UNSUPPORTED, "inlet kind %d not implemented", cfg->inlet_kind);
    if (cfg->outlet_kind < LBM_OUTLET_DENSITY_INTERPOLATED || cfg->outlet_kind > LBM_OUTLET_DENSITY_EQUILIBRIUM)
        return fail(nullptr, LBM_ERR_UNSUPPORTED, "outlet kind %d not implemented", cfg->outlet_kind);
    if ((cfg->outlet_kind == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA ||
         cfg->outlet_kind == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF) && cfg->closure == LBM_CLOSURE_MLP)
        return fail(nullptr, LBM_ERR_UNSUPPORTED, "the outlet sponge runs with the Smagorinsky or no closure");
    if (cfg->closure == LBM_CLOSURE_MLP && cfg->storage == LBM_STORAGE_F64)
        return fail(nullptr, LBM_ERR_UNSUPPORTED, "the learned closure runs with FP32 or FP16-deviation storage");
    if (cfg->storage < LBM_STORAGE_F64 || cfg->storage > LBM_STORAGE_F16DEV)
        return fail(nullptr, LBM_ERR_INVALID, "storage %d", cfg->storage);
    double tau = cfg->tau > 0 ? cfg->tau : 3.0 * cfg->nu + 0.5;
    if (!(tau > 0.5)) return fail(nullptr, LBM_ERR_INVALID, "tau = %g must exceed 1/2", tau);
    if (cfg->storage == LBM_STORAGE_F16DEV && (cfg->f16_scale_log2 < 0 || cfg->f16_scale_log2 > 20))
        return fail(nullptr, LBM_ERR_INVALID, "f16_scale_log2 = %d out of [0, 20]", cfg->f16_scale_log2);
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(nullptr, LBM_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
    if (cfg->device < 0 || cfg->device >= ndev) return fail(nullptr, LBM_ERR_INVALID, "device %d of %d", cfg->device, ndev);
    lbm_ctx* c = new lbm_ctx;
    c->cfg = *cfg;
    c->N = N;
    c->esize = cfg->storage == LBM_STORAGE_F64 ? 8 : cfg->storage == LBM_STORAGE_F32 ? 4 : 2;
    lbm_status s = LBM_OK;
    int lo_prio = 0, hi_prio = 0;  // the side stream of the split step runs at the highest priority, so
                                   // its slow boundary rows start first and the plain rows fill around them
    if ((e = cudaSetDevice(cfg->device)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio)) != cudaSuccess ||
        (e = cudaStreamCreateWithPriority(&c->st_side, cudaStreamNonBlocking, hi_prio)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaMalloc(&c->d_f, 27 * (size_t)N * c->esize)) != cudaSuccess ||
        (e = cudaMalloc(&c->d_cls, (size_t)N)) != cudaSuccess ||
        (e = cudaMalloc(&c->d_aux, (size_t)N * 4)) != cudaSuccess ||
        (e = cudaMalloc(&c->d_red, RED_COUNT * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&c->d_err, sizeof(int))) != cudaSuccess ||
        (e = cudaMemset(c->d_err, 0, sizeof(int))) != cudaSuccess) {
        s = fail(nullptr, e == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA, "lbm_create: %s", cudaGetErrorString(e));
        lbm_destroy(c);
        return s;
    }
    // default geometry: every cell fluid
    c->flags.assign((size_t)N, 1);
    *out = c;
    return LBM_OK;
}

static void free_side(lbm_ctx* c) {
    dfree(c->d_lid_state); dfree(c->d_lid_n); dfree(c->d_lid_u);
    dfree(c->d_in_probe); dfree(c->d_in_u); dfree(c->d_in_dir);
    dfree(c->d_out_save); dfree(c->d_out_rho); dfree(c->d_out_dir);
    dfree(c->d_out_msave); dfree(c->d_out_nb); dfree(c->d_sym_dir);
    c->d_lid_state = c->d_in_probe = c->d_out_save = c->d_out_msave = nullptr;
    c->d_lid_n = c->d_lid_u = c->d_in_u = c->d_out_rho = nullptr;
    c->d_in_dir = c->d_out_dir = c->d_out_nb = c->d_sym_dir = nullptr;
    c->n_lid = c->n_in = c->n_out = c->n_ms = c->n_sym = 0;
    c->sponge_axis = -1;
}

lbm_status lbm_destroy(lbm_ctx* c) {
    if (!c) return LBM_OK;
    cudaSetDevice(c->cfg.device);
    if (c->st) cudaStreamSynchronize(c->st);
    dfree(c->d_f); dfree(c->d_cls); dfree(c->d_aux);
    free_side(c);
    dfree(c->d_acc); dfree(c->d_uerr); dfree(c->d_red); dfree(c->d_part);
    dfree(c->d_rho_out); dfree(c->d_u_out); dfree(c->d_f_out); dfree(c->d_probe);
    dfree(c->d_bulk_rows); dfree(c->d_other_rows); dfree(c->d_plain_rows); dfree(c->d_rest_rows); dfree(c->d_wall_rows); dfree(c->d_wall_solid); dfree(c->d_rest_all); dfree(c->d_err); dfree(c->d_mlp_frag); dfree(c->d_nut);
    if (c->st) cudaStreamDestroy(c->st);
    if (c->st_side) cudaStreamDestroy(c->st_side);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    delete c;
    return LBM_OK;
}

lbm_status lbm_set_flags(lbm_ctx* c, const int32_t* flags) {
    if (!c || !flags) return fail(c, LBM_ERR_INVALID, "lbm_set_flags: null argument");
    c->flags.resize((size_t)c->N);
    int32_t* dst = c->flags.data();
    host_parallel(c->N, [&](long long q0, long long q1) { std::memcpy(dst + q0, flags + q0, (size_t)(q1 - q0) * 4); });
    c->have_flags = true;
    c->have_geom = false;
    c->initialized = false;
    return LBM_OK;
}

lbm_status lbm_set_bc(lbm_ctx* c, const lbm_bc_inlet* in, int32_t nin, const lbm_bc_outlet* out, int32_t nout) {
    if (!c || nin < 0 || nout < 0 || (nin && !in) || (nout && !out))
        return fail(c, LBM_ERR_INVALID, "lbm_set_bc: bad argument");
    c->inlets.assign(in, in + nin);
    c->outlets.assign(out, out + nout);
    c->syms.clear();
    c->have_geom = false;
    c->initialized = false;
    return LBM_OK;
}

lbm_status lbm_set_symmetry(lbm_ctx* c, const lbm_bc_symmetry* recs, int32_t n) {
    if (!c || n < 0 || (n && !recs)) return fail(c, LBM_ERR_INVALID, "lbm_set_symmetry: bad argument");
    c->syms.assign(recs, recs + n);
    c->have_geom = false;
    c->initialized = false;
    return LBM_OK;
}

// ---- geometry: reference flags + BC records -> class byte, side-table indices, validation -------
// the row lists of the step kernels from the class bytes: the rows the row-staged step may take and the
// split of the rows into plain, wall and remaining rows (host cores), uploaded to the device
static lbm_status build_rows(lbm_ctx* c, const uint8_t* cls) {
    const int nx = c->cfg.nx, ny = c->cfg.ny, nz = c->cfg.nz;
    const int* wrap = c->cfg.periodic;
    auto id = [&](int i, int j, int k) { return (long long)i + (long long)nx * ((long long)j + (long long)ny * k); };
    // rows the row-staged step may take (FP16-deviation storage): every cell bulk fluid, x periodic,
    // segments a multiple of 16 bytes, one thread per x-pair
    {
        const long long nrow = (long long)ny * nz;
        std::vector<int32_t> bulk, other;
        c->rows_ok = (c->cfg.options & LBM_OPT_ROW_STAGING) && c->cfg.closure != LBM_CLOSURE_MLP && c->cfg.storage == LBM_STORAGE_F16DEV && wrap[0] &&
                     nx % 2 == 0 && nx >= 64 && nx <= 1024 &&
                     ((size_t)nx * c->esize) % 16 == 0 && nrow < (1LL << 31);
        for (long long r = 0; r < nrow && c->rows_ok; r++) {
            bool all = true;
            for (int i = 0; i < nx && all; i++) all = (cls[(size_t)(r * nx + i)] & (uint8_t)~BIT_REFBULK) == CLS_BULK;
            (all ? bulk : other).push_back((int32_t)r);
        }
        if (bulk.empty()) c->rows_ok = false;
        dfree(c->d_bulk_rows); dfree(c->d_other_rows);
        c->d_bulk_rows = c->d_other_rows = nullptr;
        c->n_bulk_rows = (int)bulk.size();
        c->n_other_rows = (int)other.size();
        if (c->rows_ok) {
            CU(c, cudaMalloc(&c->d_bulk_rows, bulk.size() * 4));
            CU(c, cudaMemcpy(c->d_bulk_rows, bulk.data(), bulk.size() * 4, cudaMemcpyHostToDevice));
            if (!other.empty()) {
                CU(c, cudaMalloc(&c->d_other_rows, other.size() * 4));
                CU(c, cudaMemcpy(c->d_other_rows, other.data(), other.size() * 4, cudaMemcpyHostToDevice));
            }
        }
    }
    // the step split by rows (FP32 and FP16-deviation storage): plain rows are off the periodic y/z seams
    // with every cell a bulk fluid cell of the packed path (the combined collision packs reference-flag-1
    // cells only); nx even.  LBM_OPT_ONE_LAUNCH keeps one launch over the lattice.
    {
        const long long nrow = (long long)ny * nz;
        const bool comb = c->cfg.collision == LBM_COLLISION_CUMULANT_COMBINED;
        const uint8_t keep = comb ? (uint8_t)0xff : (uint8_t)~BIT_REFBULK;
        const uint8_t want = comb ? (uint8_t)(CLS_BULK | BIT_REFBULK) : (uint8_t)CLS_BULK;
        c->split_ok = c->cfg.storage != LBM_STORAGE_F64 && !(c->cfg.options & LBM_OPT_ONE_LAUNCH) && nrow < (1LL << 31);
        std::vector<uint8_t> plain(c->split_ok ? (size_t)nrow : 0, 0);
        const long long row_grain = std::max(1LL, 65536LL / nx);  // rows of nx cells per thread at least
        if (c->split_ok && !(nx & 1)) {
            host_parallel(nrow, [&](long long r0, long long r1) {
                for (long long r = r0; r < r1; r++) {
                    const int y = (int)(r % ny), z = (int)(r / ny);
                    if ((wrap[1] && (y == 0 || y == ny - 1)) || (wrap[2] && (z == 0 || z == nz - 1))) continue;
                    bool all = true;
                    for (int i = 0; i < nx && all; i++) all = (cls[(size_t)(r * nx + i)] & keep) == want;
                    plain[(size_t)r] = all ? 1 : 0;
                }
            }, row_grain);
        }
        // rows beside a flat wall: every cell an edge cell (no role bit) whose 26 sources are solid or
        // fluid cells of the packed kinds at the same offsets along the whole row, off the periodic y/z
        // seams (the combined collision keeps them on the general path)
        std::vector<uint32_t> wmask(plain.size(), 0);
        std::vector<uint8_t> is_wall(plain.size(), 0);
        if (c->split_ok && !(nx & 1) && !comb && !(c->cfg.options & LBM_OPT_NO_WALL_ROWS)) {
            host_parallel(nrow, [&](long long r0, long long r1) {
                for (long long r = r0; r < r1; r++) {
                    if (plain[(size_t)r]) continue;
                    const int y = (int)(r % ny), z = (int)(r / ny);
                    if ((wrap[1] && (y == 0 || y == ny - 1)) || (wrap[2] && (z == 0 || z == nz - 1))) continue;
                    bool ok = (cls[(size_t)(r * nx)] & (uint8_t)~BIT_REFBULK) == CLS_EDGE;  // cheap early exit
                    // the nine source rows (y - c_y, z - c_z) of the row, inside the lattice (these rows are
                    // off the periodic seams, so a y or z source outside it rules the row out)
                    const uint8_t* src[27];
                    for (int v = 1; v < 27 && ok; v++) {
                        const int b = y - cy(v), e = z - cz(v);
                        if (b < 0 || b >= ny || e < 0 || e >= nz) ok = false;
                        else src[v] = cls + (size_t)id(0, b, e);
                    }
                    if (ok && !wrap[0]) ok = false;  // x sources wrap only on a periodic x axis
                    uint32_t mask = 0;
                    // the solid-source mask of cell i, and whether a source is of a kind other than solid,
                    // bulk or edge (a compile-time loop over the directions; x wraps only at the row ends)
                    auto cell_mask = [&](int i, bool wrapx, uint32_t& other) {
                        uint32_t m = 0;
                        sfor_host<1, 27>([&](auto vc) {
                            constexpr int v = decltype(vc)::value;
                            int a = i - cx(v);
                            if (wrapx) a = a < 0 ? a + nx : a >= nx ? a - nx : a;
                            const int k = src[v][a] & CLS_MASK;
                            m |= (uint32_t)(k == CLS_SOLID) << v;
                            other |= (uint32_t)(k != CLS_SOLID && k != CLS_BULK && k != CLS_EDGE);
                        });
                        return m;
                    };
                    const uint8_t* row = cls + (size_t)r * nx;
                    uint32_t other = 0;
                    if (ok) mask = cell_mask(0, true, other);
                    for (int i = 1; i < nx && ok; i++) {
                        if ((row[i] & (uint8_t)~BIT_REFBULK) != CLS_EDGE) { ok = false; break; }
                        if (cell_mask(i, i == nx - 1, other) != mask) ok = false;
                    }
                    if (other) ok = false;
                    if (ok) { is_wall[(size_t)r] = 1; wmask[(size_t)r] = mask; }
                }
            }, row_grain);
        }
        std::vector<int32_t> pr, rr, wr, ra;
        std::vector<uint32_t> wm;
        for (long long r = 0; r < (long long)plain.size(); r++) {
            if (plain[(size_t)r]) { pr.push_back((int32_t)r); continue; }
            ra.push_back((int32_t)r);
            if (is_wall[(size_t)r]) { wr.push_back((int32_t)r); wm.push_back(wmask[(size_t)r]); }
            else rr.push_back((int32_t)r);
        }
        dfree(c->d_plain_rows); dfree(c->d_rest_rows); dfree(c->d_wall_rows); dfree(c->d_wall_solid); dfree(c->d_rest_all);
        c->d_plain_rows = c->d_rest_rows = c->d_wall_rows = c->d_rest_all = nullptr;
        c->d_wall_solid = nullptr;
        c->n_plain_rows = (int)pr.size();
        c->n_rest_rows = (int)rr.size();
        c->n_wall_rows = (int)wr.size();
        c->n_rest_all = (int)ra.size();
        auto upload = [&](auto** dst, const auto& v) -> lbm_status {
            if (!c->split_ok || v.empty()) return LBM_OK;
            CU(c, cudaMalloc((void**)dst, v.size() * 4));
            CU(c, cudaMemcpy(*dst, v.data(), v.size() * 4, cudaMemcpyHostToDevice));
            return LBM_OK;
        };
        lbm_status us;
        if ((us = upload(&c->d_plain_rows, pr)) || (us = upload(&c->d_rest_rows, rr)) ||
            (us = upload(&c->d_wall_rows, wr)) || (us = upload(&c->d_wall_solid, wm)) || (us = upload(&c->d_rest_all, ra)))
            return us;
    }
    return LBM_OK;
}

// defer_rows: leave the row lists for finish_rows (the class bytes stay on the host until then)
static lbm_status build_geometry(lbm_ctx* c, bool defer_rows = false) {
    const int nx = c->cfg.nx, ny = c->cfg.ny, nz = c->cfg.nz;
    const long long N = c->N;
    const int* wrap = c->cfg.periodic;
    auto id = [&](int i, int j, int k) { return (long long)i + (long long)nx * ((long long)j + (long long)ny * k); };
    auto wrapc = [&](int v, int n, int a, bool& ok) {
        if (v < 0 || v >= n) { if (wrap[a]) v = (v + n) % n; else ok = false; }
        return v;
    };
    // class byte per cell, filled on the host cores; side-table index per cell (-1: none), kept sparse on
    // the host (only boundary nodes and their helper cells have one)
    std::unique_ptr<uint8_t[]> cls_buf(new uint8_t[(size_t)N]);
    uint8_t* cls = cls_buf.get();
    struct SparseIndex {
        std::unordered_map<long long, int32_t> m;
        int32_t operator[](long long q) const { auto it = m.find(q); return it == m.end() ? -1 : it->second; }
        void set(long long q, int32_t v) { m[q] = v; }
    } aux;
    // moving-wall and Zou/He nodes share the 3-level side table: collided, never streamed into
    const bool lid_kind = c->cfg.inlet_kind == LBM_INLET_MOVING_WALL || c->cfg.inlet_kind == LBM_INLET_ZOU_HE;
    const int okind = c->cfg.outlet_kind;
    const bool neq_kind = okind == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM || okind == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA ||
                          okind == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF;
    std::vector<char> is_sym(c->syms.empty() ? 0 : (size_t)N, 0);
    for (const auto& r : c->syms) {
        int i = r.vertex.x, j = r.vertex.y, k = r.vertex.z;
        if (i < 0 || j < 0 || k < 0 || i >= nx || j >= ny || k >= nz)
            return fail(c, LBM_ERR_INVALID, "symmetry record at (%d,%d,%d) is outside the lattice", i, j, k);
        if (c->flags[id(i, j, k)] != -2)
            return fail(c, LBM_ERR_INVALID, "symmetry record at (%d,%d,%d) is not a -2 cell", i, j, k);
        if (is_sym[id(i, j, k)]) return fail(c, LBM_ERR_INVALID, "two symmetry records for (%d,%d,%d)", i, j, k);
        is_sym[id(i, j, k)] = 1;
    }
    // class byte of every cell, in contiguous chunks on the host cores (per-chunk counts and the first
    // bad cell, combined afterwards)
    long long n_flag1 = 0, n_flag2 = 0;  // cells of flag -1 and -2 (each needs one record)
    {
        struct Part { long long n1 = 0, n2 = 0, bad = -1; };
        std::vector<Part> parts(64);
        std::atomic<int> next{0};
        host_parallel(N, [&](long long q0, long long q1) {
            Part& pt = parts[(size_t)next.fetch_add(1)];
            for (long long q = q0; q < q1; q++) {
                const int32_t f = c->flags[q];
                uint8_t k;
                if (f == 0) k = CLS_SOLID;
                else if (f == -1) { k = lid_kind ? CLS_LID : CLS_INLET; pt.n1++; }
                else if (f == -2) { k = (!is_sym.empty() && is_sym[q]) ? CLS_SYM : CLS_OUTLET; pt.n2++; }
                else if (f > 0 || f == -3) k = CLS_BULK;
                else { if (pt.bad < 0) pt.bad = q; k = CLS_SOLID; }
                cls[q] = k | (f == 1 ? BIT_REFBULK : 0);
            }
        });
        long long bad = -1;
        for (const Part& pt : parts) {
            n_flag1 += pt.n1;
            n_flag2 += pt.n2;
            if (pt.bad >= 0 && (bad < 0 || pt.bad < bad)) bad = pt.bad;
        }
        if (bad >= 0)
            return fail(c, LBM_ERR_INVALID, "flag %d at cell %lld is not in the reference encoding", c->flags[bad], bad);
    }
    // -1 records
    std::vector<float> lid_n, lid_u, in_u;
    std::vector<int32_t> in_dir, out_dir;
    std::vector<float> out_rho;
    int n_lid = 0, n_in = 0, n_out = 0;
    for (const auto& r : c->inlets) {
        int i = r.vertex.x, j = r.vertex.y, k = r.vertex.z;
        if (i < 0 || j < 0 || k < 0 || i >= nx || j >= ny || k >= nz)
            return fail(c, LBM_ERR_INVALID, "inlet record at (%d,%d,%d) is outside the lattice", i, j, k);
        long long q = id(i, j, k);
        if (c->flags[q] != -1) return fail(c, LBM_ERR_INVALID, "inlet record at (%d,%d,%d) is not a -1 cell", i, j, k);
        if (aux[q] >= 0) return fail(c, LBM_ERR_INVALID, "two inlet records for (%d,%d,%d)", i, j, k);
        if (lid_kind) {
            aux.set(q, n_lid++);
            for (int a = 0; a < 3; a++) { lid_n.push_back(r.normal[a]); lid_u.push_back(r.velocity[a]); }
        } else {
            int s = (r.normal[0] == 1.f && r.normal[1] == 0.f && r.normal[2] == 0.f) ? 1
                  : (r.normal[0] == -1.f && r.normal[1] == 0.f && r.normal[2] == 0.f) ? -1 : 0;
            if (!s) return fail(c, LBM_ERR_UNSUPPORTED, "equilibrium inlet at (%d,%d,%d): only +-x normals (as the reference)", i, j, k);
            aux.set(q, n_in++);
            in_dir.push_back(s);
            for (int a = 0; a < 3; a++) in_u.push_back(r.velocity[a]);
        }
    }
    for (const auto& r : c->outlets) {
        int i = r.vertex.x, j = r.vertex.y, k = r.vertex.z;
        if (i < 0 || j < 0 || k < 0 || i >= nx || j >= ny || k >= nz)
            return fail(c, LBM_ERR_INVALID, "outlet record at (%d,%d,%d) is outside the lattice", i, j, k);
        long long q = id(i, j, k);
        if (c->flags[q] != -2) return fail(c, LBM_ERR_INVALID, "outlet record at (%d,%d,%d) is not a -2 cell", i, j, k);
        if (aux[q] >= 0) return fail(c, LBM_ERR_INVALID, "two outlet records for (%d,%d,%d)", i, j, k);
        if (!is_sym.empty() && is_sym[q])
            return fail(c, LBM_ERR_INVALID, "(%d,%d,%d) has an outlet and a symmetry record", i, j, k);
        int s = (r.normal[0] == 1.f && r.normal[1] == 0.f && r.normal[2] == 0.f) ? 1
              : (r.normal[0] == -1.f && r.normal[1] == 0.f && r.normal[2] == 0.f) ? -1 : 0;
        if (!s) return fail(c, LBM_ERR_UNSUPPORTED, "outlet at (%d,%d,%d): only +-x normals (as the reference)", i, j, k);
        if (!(r.density > 0)) return fail(c, LBM_ERR_INVALID, "outlet density must be positive");
        aux.set(q, n_out++);
        out_dir.push_back(s);
        out_rho.push_back(r.density);
    }
    // symmetry records: +-y normals only (BounceSymmetryHalf.h:84-133; the x and z branches are commented
    // out), a solid cell across the plane, in-plane sources inside the lattice and streaming normally
    std::vector<int32_t> sym_dir;
    int n_sym = 0;
    for (const auto& r : c->syms) {
        int i = r.vertex.x, j = r.vertex.y, k = r.vertex.z;
        long long q = id(i, j, k);
        int sg = (r.normal[0] == 0.f && r.normal[1] == 1.f && r.normal[2] == 0.f) ? 1
               : (r.normal[0] == 0.f && r.normal[1] == -1.f && r.normal[2] == 0.f) ? -1 : 0;
        if (!sg) return fail(c, LBM_ERR_UNSUPPORTED, "symmetry at (%d,%d,%d): only +-y normals (as the reference)", i, j, k);
        if (wrap[1]) return fail(c, LBM_ERR_UNSUPPORTED, "symmetry planes need a non-periodic y axis");
        if (j + sg < 0 || j + sg >= ny)
            return fail(c, LBM_ERR_UNSUPPORTED, "symmetry at (%d,%d,%d): the row across the plane must be solid", i, j, k);
        for (int dz = -1; dz <= 1; dz++)
            for (int dx = -1; dx <= 1; dx++) {
                bool ok = true;
                int a = wrapc(i + dx, nx, 0, ok), e = wrapc(k + dz, nz, 2, ok);
                if (!ok) return fail(c, LBM_ERR_UNSUPPORTED, "symmetry at (%d,%d,%d) mirrors from outside the lattice", i, j, k);
                if (c->flags[id(a, j + sg, e)] != 0)
                    return fail(c, LBM_ERR_UNSUPPORTED, "symmetry at (%d,%d,%d): the row across the plane must be solid",
                                i, j, k);
                int32_t fs = c->flags[id(a, j, e)];
                if (fs == -1) return fail(c, LBM_ERR_UNSUPPORTED, "symmetry at (%d,%d,%d) mirrors an inlet node", i, j, k);
                if (r.regular && fs == 0)
                    return fail(c, LBM_ERR_INVALID, "symmetry at (%d,%d,%d) is marked regular but has a solid in-plane neighbour", i, j, k);
            }
        aux.set(q, n_sym++);
        sym_dir.push_back(sg);
    }
    // every record names a distinct cell of its flag (checked above), so equal counts mean every -1 and
    // -2 cell has its record; the scan for the culprit runs only when they differ
    if (n_flag1 != (long long)c->inlets.size() || n_flag2 != (long long)(c->outlets.size() + c->syms.size()))
        for (long long q = 0; q < N; q++) {
            int k = cls[q] & CLS_MASK;
            if ((k == CLS_LID || k == CLS_INLET || k == CLS_OUTLET) && aux[q] < 0)
                return fail(c, LBM_ERR_INVALID, "cell %lld has flag %d but no boundary record", q, c->flags[q]);
        }
    std::vector<int32_t> out_nb(neq_kind ? 9 * (size_t)n_out : 0, -1);
    int n_ms = 0;
    // helper roles: probes of the equilibrium inlets, upstream cells of the outlets
    auto set_role = [&](long long q, uint8_t bit, int node, const char* what) -> lbm_status {
        int k = cls[q] & CLS_MASK;
        if (k != CLS_BULK) return fail(c, LBM_ERR_UNSUPPORTED, "%s cell %lld must be a fluid cell", what, q);
        if ((cls[q] & (BIT_PROBE1 | BIT_PROBE2 | BIT_OUTUP)) != 0)
            return fail(c, LBM_ERR_UNSUPPORTED, "cell %lld would serve two boundary nodes", q);
        cls[q] |= bit;
        aux.set(q, node);
        return LBM_OK;
    };
    std::vector<long long> bnodes;  // the inlet and outlet nodes, from their records
    bnodes.reserve(c->inlets.size() + c->outlets.size());
    for (const auto& r : c->inlets) bnodes.push_back(id(r.vertex.x, r.vertex.y, r.vertex.z));
    for (const auto& r : c->outlets) bnodes.push_back(id(r.vertex.x, r.vertex.y, r.vertex.z));
    for (long long q : bnodes) {
        int k = cls[q] & CLS_MASK;
        if (k != CLS_INLET && k != CLS_OUTLET) continue;  // moving-wall and Zou/He nodes have no helpers
        int i = (int)(q % nx), j = (int)((q / nx) % ny), kk = (int)(q / ((long long)nx * ny));
        if (k == CLS_INLET) {
            int s = in_dir[aux[q]];  // interior at -s
            for (int d = 1; d <= 2; d++) {
                bool ok = true;
                int ii = wrapc(i - s * d, nx, 0, ok);
                if (!ok) return fail(c, LBM_ERR_INVALID, "inlet at (%d,%d,%d) has no interior cell %d", i, j, kk, d);
                lbm_status st = set_role(id(ii, j, kk), d == 1 ? BIT_PROBE1 : BIT_PROBE2, aux[q], "inlet probe");
                if (st) return st;
            }
        } else if (k == CLS_OUTLET && okind == LBM_OUTLET_DENSITY_INTERPOLATED) {
            int s = out_dir[aux[q]];
            bool ok = true;
            int ii = wrapc(i - s, nx, 0, ok);
            if (!ok) return fail(c, LBM_ERR_INVALID, "outlet at (%d,%d,%d) has no upstream cell", i, j, kk);
            lbm_status st = set_role(id(ii, j, kk), BIT_OUTUP, aux[q], "outlet upstream");
            if (st) return st;
        } else if (k == CLS_OUTLET && neq_kind) {
            // neighbour-equilibrium outlets read the moments of the 9 cells x + c_v (c_x = -s), which keep
            // them in a side table (one entry per cell, shared by the outlet nodes around it)
            int s = out_dir[aux[q]];
            for (int dz = -1; dz <= 1; dz++)
                for (int dy = -1; dy <= 1; dy++) {
                    bool ok = true;
                    int ii = wrapc(i - s, nx, 0, ok), jj = wrapc(j + dy, ny, 1, ok), ze = wrapc(kk + dz, nz, 2, ok);
                    if (!ok) return fail(c, LBM_ERR_INVALID, "outlet at (%d,%d,%d) has no upstream cell", i, j, kk);
                    long long r = id(ii, jj, ze);
                    if (c->flags[r] <= 0)
                        return fail(c, LBM_ERR_UNSUPPORTED,
                                    "neighbour-equilibrium outlet at (%d,%d,%d): upstream cell (%d,%d,%d) must be fluid",
                                    i, j, kk, ii, jj, ze);
                    if (cls[r] & (BIT_PROBE1 | BIT_PROBE2))
                        return fail(c, LBM_ERR_UNSUPPORTED, "cell %lld would serve two boundary nodes", r);
                    if (!(cls[r] & BIT_OUTUP)) {
                        cls[r] |= BIT_OUTUP;
                        aux.set(r, n_ms++);
                    }
                    out_nb[(size_t)outlet_slot(vid(-s, dy, dz)) * n_out + aux[q]] = aux[r];
                }
        }
    }
    // BULK/EDGE split: fluid cells next to a solid, moving-wall or inlet node stream through
    // per-link rules (visit the 26-neighbourhood of those nodes only).  Chunks of cells on the host
    // cores; a neighbour byte may be marked by two chunks, always from BULK to EDGE with its role bits
    // kept, so the byte accesses are relaxed atomics and the result does not depend on the order
    host_parallel(N, [&](long long q0, long long q1) {
        for (long long q = q0; q < q1; q++) {
            int k = __atomic_load_n(&cls[q], __ATOMIC_RELAXED) & CLS_MASK;
            if (k != CLS_SOLID && k != CLS_LID && k != CLS_INLET) continue;
            int i = (int)(q % nx), j = (int)((q / nx) % ny), kk = (int)(q / ((long long)nx * ny));
            for (int dz = -1; dz <= 1; dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        bool ok = true;
                        int a = wrapc(i + dx, nx, 0, ok), b = wrapc(j + dy, ny, 1, ok), e = wrapc(kk + dz, nz, 2, ok);
                        if (!ok) continue;
                        uint8_t* cr = &cls[(size_t)id(a, b, e)];
                        const uint8_t v = __atomic_load_n(cr, __ATOMIC_RELAXED);
                        if ((v & CLS_MASK) == CLS_BULK) __atomic_store_n(cr, (uint8_t)((v & ~CLS_MASK) | CLS_EDGE), __ATOMIC_RELAXED);
                    }
        }
    });
    // stream targets on a face of a non-periodic axis would stream from outside the lattice;
    // outlets may only do so on their interpolated links, and must not touch solid cells
    auto check_links = [&](long long q) -> lbm_status {
        int k = cls[q] & CLS_MASK;
        if (k != CLS_BULK && k != CLS_EDGE && k != CLS_OUTLET && k != CLS_SYM) return LBM_OK;
        int i = (int)(q % nx), j = (int)((q / nx) % ny), kk = (int)(q / ((long long)nx * ny));
        for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    if (!dx && !dy && !dz) continue;
                    bool ok = true;
                    int a = wrapc(i + dx, nx, 0, ok), b = wrapc(j + dy, ny, 1, ok), e = wrapc(kk + dz, nz, 2, ok);
                    bool interp = (k == CLS_OUTLET) && dx == out_dir[aux[q]];
                    if (!ok) {
                        if (interp) continue;
                        return fail(c, LBM_ERR_UNSUPPORTED,
                                    "cell (%d,%d,%d) streams from outside a non-periodic lattice: add a solid layer "
                                    "(the reference's additional_factor >= 1) or make the axis periodic", i, j, kk);
                    }
                    if (k == CLS_OUTLET && (cls[id(a, b, e)] & CLS_MASK) == CLS_SOLID)
                        return fail(c, LBM_ERR_UNSUPPORTED, "outlet cell (%d,%d,%d) touches a solid cell", i, j, kk);
                }
        return LBM_OK;
    };
    for (int axis = 0; axis < 3; axis++) {
        if (wrap[axis]) continue;
        int n0 = axis == 0 ? nx : axis == 1 ? ny : nz;
        for (int face = 0; face < 2; face++) {
            int fc = face ? n0 - 1 : 0;
            int na = axis == 0 ? ny : nx, nb2 = axis == 2 ? ny : nz;
            for (int u2 = 0; u2 < nb2; u2++)
                for (int u1 = 0; u1 < na; u1++) {
                    int i = axis == 0 ? fc : u1, j = axis == 1 ? fc : (axis == 0 ? u1 : u2), kk = axis == 2 ? fc : u2;
                    lbm_status st = check_links(id(i, j, kk));
                    if (st) return st;
                }
        }
    }
    for (const auto& r : c->outlets) {
        lbm_status st = check_links(id(r.vertex.x, r.vertex.y, r.vertex.z));
        if (st) return st;
    }
    // sponge of OutletNeighbourEquilibriumOmega(RF)::outletOmega (:18-79): along the first outlet's normal
    // axis, the last ceil(0.1 n) planes (the reference's float ceil(n * 0.1f), equal for every n) lose
    // (high - low) / width * (plane - first plane) of their relaxation rate; those cells take the
    // per-cell path (the bit keeps them off the packed pair path)
    int sp_axis = -1, sp_begin = 0;
    double sp_slope = 0.0;
    if ((okind == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA || okind == LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF) &&
        !c->outlets.empty()) {
        sp_axis = 0;  // outlet normals are +-x (checked above)
        const int width = (int)std::ceil((float)nx * 0.1f);
        sp_begin = nx - width;
        sp_slope = (c->cfg.omega_dumping_high - c->cfg.omega_dumping_low) / (double)width;
        if (sp_slope != 0.0)
            for (long long r = 0; r < (long long)ny * nz; r++)
                for (int i = sp_begin; i < nx; i++) {
                    const long long q = r * nx + i;
                    if ((cls[q] & CLS_MASK) != CLS_SOLID) cls[q] |= BIT_SPONGE;
                }
    }
    // upload
    cudaSetDevice(c->cfg.device);
    free_side(c);
    c->sponge_axis = sp_axis; c->sponge_begin = sp_begin; c->sponge_slope = sp_slope;
    CU(c, cudaMemcpyAsync(c->d_cls, cls, (size_t)N, cudaMemcpyHostToDevice, c->st));
    // side-table indices: -1 everywhere (every byte 0xff), then the few set entries scattered on the device
    CU(c, cudaMemsetAsync(c->d_aux, 0xff, (size_t)N * 4, c->st));
    {
        std::vector<long long> sq;
        std::vector<int32_t> sv;
        for (const auto& kv : aux.m) { sq.push_back(kv.first); sv.push_back(kv.second); }
        if (!sq.empty()) {
            long long* d_q = nullptr;
            int32_t* d_v = nullptr;
            CU(c, cudaMalloc(&d_q, sq.size() * sizeof(long long)));
            CU(c, cudaMalloc(&d_v, sv.size() * sizeof(int32_t)));
            CU(c, cudaMemcpyAsync(d_q, sq.data(), sq.size() * sizeof(long long), cudaMemcpyHostToDevice, c->st));
            CU(c, cudaMemcpyAsync(d_v, sv.data(), sv.size() * sizeof(int32_t), cudaMemcpyHostToDevice, c->st));
            const long long n = (long long)sq.size();
            k_scatter_aux<<<(unsigned)((n + 255) / 256), 256, 0, c->st>>>(c->d_aux, d_q, d_v, n);
            cudaError_t e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
            cudaFree(d_q);
            cudaFree(d_v);
            if (e != cudaSuccess) return fail(c, LBM_ERR_CUDA, "side-table index upload: %s", cudaGetErrorString(e));
        }
    }
    const size_t rs = real_size(c);
    c->n_lid = n_lid; c->n_in = n_in; c->n_out = n_out;
    if (n_lid) {
        CU(c, cudaMalloc(&c->d_lid_state, 3 * 27 * (size_t)n_lid * rs));
        CU(c, cudaMalloc(&c->d_lid_n, 3 * (size_t)n_lid * 4));
        CU(c, cudaMalloc(&c->d_lid_u, 3 * (size_t)n_lid * 4));
        std::vector<float> tn(3 * n_lid), tu(3 * n_lid);  // component-major
        for (int e = 0; e < n_lid; e++)
            for (int a = 0; a < 3; a++) { tn[a * n_lid + e] = lid_n[3 * e + a]; tu[a * n_lid + e] = lid_u[3 * e + a]; }
        CU(c, cudaMemcpy(c->d_lid_n, tn.data(), tn.size() * 4, cudaMemcpyHostToDevice));
        CU(c, cudaMemcpy(c->d_lid_u, tu.data(), tu.size() * 4, cudaMemcpyHostToDevice));
    }
    if (n_in) {
        CU(c, cudaMalloc(&c->d_in_probe, 3 * 3 * (size_t)n_in * rs));
        CU(c, cudaMemset(c->d_in_probe, 0, 3 * 3 * (size_t)n_in * rs));
        CU(c, cudaMalloc(&c->d_in_u, 3 * (size_t)n_in * 4));
        CU(c, cudaMalloc(&c->d_in_dir, (size_t)n_in * 4));
        std::vector<float> tu(3 * n_in);
        for (int e = 0; e < n_in; e++)
            for (int a = 0; a < 3; a++) tu[a * n_in + e] = in_u[3 * e + a];
        CU(c, cudaMemcpy(c->d_in_u, tu.data(), tu.size() * 4, cudaMemcpyHostToDevice));
        CU(c, cudaMemcpy(c->d_in_dir, in_dir.data(), (size_t)n_in * 4, cudaMemcpyHostToDevice));
    }
    if (n_out) {
        CU(c, cudaMalloc(&c->d_out_save, 2 * 18 * (size_t)n_out * rs));
        CU(c, cudaMemset(c->d_out_save, 0, 2 * 18 * (size_t)n_out * rs));
        CU(c, cudaMalloc(&c->d_out_rho, (size_t)n_out * 4));
        CU(c, cudaMalloc(&c->d_out_dir, (size_t)n_out * 4));
        CU(c, cudaMemcpy(c->d_out_rho, out_rho.data(), (size_t)n_out * 4, cudaMemcpyHostToDevice));
        CU(c, cudaMemcpy(c->d_out_dir, out_dir.data(), (size_t)n_out * 4, cudaMemcpyHostToDevice));
    }
    c->n_ms = n_ms;
    if (n_ms) {
        CU(c, cudaMalloc(&c->d_out_msave, 2 * 4 * (size_t)n_ms * rs));
        CU(c, cudaMemset(c->d_out_msave, 0, 2 * 4 * (size_t)n_ms * rs));
        CU(c, cudaMalloc(&c->d_out_nb, out_nb.size() * 4));
        CU(c, cudaMemcpy(c->d_out_nb, out_nb.data(), out_nb.size() * 4, cudaMemcpyHostToDevice));
    }
    c->n_sym = n_sym;
    if (n_sym) {
        CU(c, cudaMalloc(&c->d_sym_dir, (size_t)n_sym * 4));
        CU(c, cudaMemcpy(c->d_sym_dir, sym_dir.data(), (size_t)n_sym * 4, cudaMemcpyHostToDevice));
    }
    CU(c, cudaStreamSynchronize(c->st));
    if (defer_rows) {  // the row lists follow in finish_rows, while the init kernel runs
        c->host_cls = std::move(cls_buf);
        c->rows_pending = true;
    } else {
        lbm_status rs = build_rows(c, cls);
        if (rs) return rs;
    }
    c->have_geom = true;
    return LBM_OK;
}

static lbm_status finish_rows(lbm_ctx* c) {
    if (!c->rows_pending) return LBM_OK;
    lbm_status s = build_rows(c, c->host_cls.get());
    c->host_cls.reset();
    c->rows_pending = false;
    return s;
}

static lbm_status ensure_geometry(lbm_ctx* c, bool defer_rows = false) {
    if (c->have_geom) return LBM_OK;
    return build_geometry(c, defer_rows);
}

static lbm_status init_common(lbm_ctx* c, const double* rho, const double* u, double rho0, const double* u0,
                              const double* pops) {
    cudaSetDevice(c->cfg.device);
    lbm_status s = ensure_geometry(c, true);
    if (s) return s;
    double *dr = nullptr, *du = nullptr, *dp = nullptr;  // staging copies (pageable inputs)
    const size_t N = (size_t)c->N;
    // a page-locked host array (cudaHostAlloc / cudaHostRegister) is read by the init kernel where it
    // lies (its device view, over the host link); any other array is copied to a device buffer first
    auto device_view = [&](const double* h, size_t bytes, double** staged, const double** view) -> cudaError_t {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, h) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer) {
            *view = (const double*)a.devicePointer;
            return cudaSuccess;
        }
        cudaGetLastError();  // a pointer the runtime does not know is not an error here
        cudaError_t e = cudaMalloc(staged, bytes);
        if (e == cudaSuccess) e = cudaMemcpyAsync(*staged, h, bytes, cudaMemcpyHostToDevice, c->st);
        *view = *staged;
        return e;
    };
    const double *vr = nullptr, *vu = nullptr, *vp = nullptr;
    if (rho) {
        CU(c, device_view(rho, N * 8, &dr, &vr));
        CU(c, device_view(u, 3 * N * 8, &du, &vu));
    }
    if (pops) CU(c, device_view(pops, 27 * N * 8, &dp, &vp));
    c->m = 0;
    Params p = make_params(c);
    double z3[3] = {0, 0, 0};
    cudaError_t e = do_init(c, p, vr, vu, rho0, u0 ? u0 : z3, vp);
    const lbm_status rs = finish_rows(c);  // host work while the init kernel runs
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    dfree(dr); dfree(du); dfree(dp);
    if (e != cudaSuccess) return fail(c, LBM_ERR_CUDA, "init kernel: %s", cudaGetErrorString(e));
    if (rs) return rs;
    if (c->d_out_save) CU(c, cudaMemset(c->d_out_save, 0, 2 * 18 * (size_t)c->n_out * real_size(c)));
    if (c->d_out_msave) CU(c, cudaMemset(c->d_out_msave, 0, 2 * 4 * (size_t)c->n_ms * real_size(c)));
    c->avg_on = false; c->avg_count = 0; c->avg_last = -1;
    if (c->d_uerr) CU(c, cudaMemset(c->d_uerr, 0, 3 * N * real_size(c)));
    c->initialized = true;
    return LBM_OK;
}

lbm_status lbm_init_equilibrium(lbm_ctx* c, double rho0, const double u0[3]) {
    if (!c || !u0) return fail(c, LBM_ERR_INVALID, "lbm_init_equilibrium: null argument");
    if (!(rho0 > 0)) return fail(c, LBM_ERR_INVALID, "rho0 must be positive");
    return init_common(c, nullptr, nullptr, rho0, u0, nullptr);
}

lbm_status lbm_init_fields(lbm_ctx* c, const double* rho, const double* u) {
    if (!c || !rho || !u) return fail(c, LBM_ERR_INVALID, "lbm_init_fields: null argument");
    return init_common(c, rho, u, 1.0, nullptr, nullptr);
}

lbm_status lbm_set_populations(lbm_ctx* c, const double* f) {
    if (!c || !f) return fail(c, LBM_ERR_INVALID, "lbm_set_populations: null argument");
    return init_common(c, nullptr, nullptr, 1.0, nullptr, f);
}

lbm_status lbm_step(lbm_ctx* c, int32_t n) {
    if (!c || n < 0) return fail(c, LBM_ERR_INVALID, "lbm_step: bad argument");
    if (!c->initialized) return fail(c, LBM_ERR_STATE, "lbm_step before initialisation");
    if (c->cfg.closure == LBM_CLOSURE_MLP && !c->have_mlp)
        return fail(c, LBM_ERR_STATE, "closure LBM_CLOSURE_MLP needs lbm_mlp_load before lbm_step");
    cudaSetDevice(c->cfg.device);
    for (int s = 0; s < n; s++) {
        Params p = make_params(c);
        if (c->avg_on && c->m > c->avg_begin && c->m > c->avg_last) {
            p.acc = c->d_acc;
            c->avg_last = c->m;
            c->avg_count++;
        }
        if (c->d_nut && c->m >= c->mlp_due) {
            p.mlp_run = 1;
            c->mlp_due = c->m + c->cfg.mlp_interval;
        }
        cudaError_t e = do_step(c, p);
        if (e != cudaSuccess) return fail(c, LBM_ERR_CUDA, "step kernel launch: %s", cudaGetErrorString(e));
        c->m++;
    }
    return LBM_OK;
}

lbm_status lbm_step_timed(lbm_ctx* c, int32_t n, double* ms) {
    if (!c || !ms || n < 0) return fail(c, LBM_ERR_INVALID, "lbm_step_timed: bad argument");
    if (!c->initialized) return fail(c, LBM_ERR_STATE, "lbm_step_timed before initialisation");
    cudaSetDevice(c->cfg.device);
    cudaEvent_t e0, e1;
    CU(c, cudaEventCreate(&e0));
    CU(c, cudaEventCreate(&e1));
    CU(c, cudaEventRecord(e0, c->st));
    lbm_status s = lbm_step(c, n);
    cudaError_t e = cudaEventRecord(e1, c->st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float f = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&f, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s) return s;
    if (e != cudaSuccess) return fail(c, LBM_ERR_CUDA, "timing events: %s", cudaGetErrorString(e));
    *ms = f;
    return LBM_OK;
}

lbm_status lbm_step_launches(const lbm_ctx* c, int32_t* per_step) {
    if (!c || !per_step) return fail(nullptr, LBM_ERR_INVALID, "lbm_step_launches: null argument");
    if (!c->initialized) return fail(nullptr, LBM_ERR_STATE, "lbm_step_launches before initialisation");
    if (c->rows_ok && c->cfg.collision == LBM_COLLISION_CUMULANT2015 && c->cfg.storage == LBM_STORAGE_F16DEV)
        *per_step = (c->n_bulk_rows > 0 ? 1 : 0) + (c->n_other_rows > 0 ? 1 : 0);
    else if (c->split_ok && c->cfg.collision == LBM_COLLISION_CUMULANT_COMBINED)
        *per_step = (c->n_plain_rows > 0 ? 1 : 0) + (c->n_rest_all > 0 ? 1 : 0);
    else if (c->split_ok)
        *per_step = (c->n_plain_rows > 0 ? 1 : 0) + (c->n_rest_rows > 0 ? 1 : 0) + (c->n_wall_rows > 0 ? 1 : 0);
    else
        *per_step = 1;
    return LBM_OK;
}

lbm_status lbm_probe(lbm_ctx* c, int32_t x, int32_t y, int32_t z, double out[4]) {
    if (!c || !out) return fail(c, LBM_ERR_INVALID, "lbm_probe: null argument");
    if (x < 0 || y < 0 || z < 0 || x >= c->cfg.nx || y >= c->cfg.ny || z >= c->cfg.nz)
        return fail(c, LBM_ERR_INVALID, "probe (%d,%d,%d) outside the lattice", x, y, z);
    if (!c->initialized) return fail(c, LBM_ERR_STATE, "lbm_probe before initialisation");
    cudaSetDevice(c->cfg.device);
    if (!c->d_probe) CU(c, cudaMalloc(&c->d_probe, 4 * sizeof(double)));
    Params p = make_params(c);
    cudaError_t e;
    switch (c->cfg.storage) {
        case LBM_STORAGE_F64: e = launch_probe<StF64>(p, x, y, z, c->d_probe, c->st); break;
        case LBM_STORAGE_F32: e = launch_probe<StF32>(p, x, y, z, c->d_probe, c->st); break;
        default: e = launch_probe<StF16>(p, x, y, z, c->d_probe, c->st); break;
    }
    if (e != cudaSuccess) return fail(c, LBM_ERR_CUDA, "probe kernel: %s", cudaGetErrorString(e));
    CU(c, cudaMemcpyAsync(out, c->d_probe, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CU(c, cudaStreamSynchronize(c->st));
    return LBM_OK;
}

// a bounded device wait that gave up, or a plain-row pair whose class bytes are not of the packed kind,
// leaves a code in the error word
static lbm_status check_device_error(lbm_ctx* c) {
    int h = 0;
    CU(c, cudaMemcpyAsync(&h, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CU(c, cudaStreamSynchronize(c->st));
    if (h != 0) {
        CU(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), c->st));
        if (h == DEV_ERR_ROW_LIST)
            return fail(c, LBM_ERR_STATE, "a plain-row pair is not a pair of bulk cells: the row lists do not "
                        "match the cell classes (code %d)", h);
        return fail(c, LBM_ERR_TIMEOUT, "%s (code %d)",
                    h == DEV_ERR_MMA_TIMEOUT ? "a step kernel gave up waiting for its tensor-core products"
                                             : "a row-staged step gave up waiting for its bulk copies",
                    h);
    }
    return LBM_OK;
}

lbm_status lbm_synchronize(lbm_ctx* c) {
    if (!c) return fail(c, LBM_ERR_INVALID, "null ctx");
    cudaSetDevice(c->cfg.device);
    CU(c, cudaStreamSynchronize(c->st));
    return check_device_error(c);
}

static lbm_status run_read(lbm_ctx* c, ReadOut& o) {
    Params p = make_params(c);
    if (o.mode & READ_ACC) p.acc = c->d_acc;
    cudaError_t e = do_read(c, p, o);
    if (e != cudaSuccess) return fail(c, LBM_ERR_CUDA, "read kernel: %s", cudaGetErrorString(e));
    return LBM_OK;
}

lbm_status lbm_get_moments(lbm_ctx* c, double* rho, double* u) {
    if (!c || (!rho && !u)) return fail(c, LBM_ERR_INVALID, "lbm_get_moments: null argument");
    if (!c->initialized) return fail(c, LBM_ERR_STATE, "lbm_get_moments before initialisation");
    cudaSetDevice(c->cfg.device);
    const size_t N = (size_t)c->N;
    if (!c->d_rho_out) CU(c, cudaMalloc(&c->d_rho_out, N * 8));
    if (!c->d_u_out) CU(c, cudaMalloc(&c->d_u_out, 3 * N * 8));
    ReadOut o{};
    o.rho = c->d_rho_out; o.u = c->d_u_out; o.mode = READ_MOMENTS;
    lbm_status s = run_read(c, o);
    if (s) return s;
    if (rho) CU(c, cudaMemcpyAsync(rho, c->d_rho_out, N * 8, cudaMemcpyDeviceToHost, c->st));
    if (u) CU(c, cudaMemcpyAsync(u, c->d_u_out, 3 * N * 8, cudaMemcpyDeviceToHost, c->st));
    CU(c, cudaStreamSynchronize(c->st));
    return LBM_OK;
}

lbm_status lbm_get_populations(lbm_ctx* c, double* f) {
    if (!c || !f) return fail(c, LBM_ERR_INVALID, "lbm_get_populations: null argument");
    if (!c->initialized) return fail(c, LBM_ERR_STATE, "lbm_get_populations before initialisation");
    cudaSetDevice(c->cfg.device);
    const size_t N = (size_t)c->N;
    double* d = nullptr;
    CU(c, cudaMalloc(&d, 27 * N * 8));
    ReadOut o{};
    o.f = d; o.mode = READ_POPS;
    lbm_status s = run_read(c, o);
    if (!s) {
        cudaError_t e = cudaMemcpyAsync(f, d, 27 * N * 8, cudaMemcpyDeviceToHost, c->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
        if (e != cudaSuccess) s = fail(c, LBM_ERR_CUDA, "populations copy: %s", cudaGetErrorString(e));
    }
    cudaFree(d);
    return s;
}

lbm_status lbm_reduce(lbm_ctx* c, lbm_diag* out) {
    if (!c || !out) return fail(c, LBM_ERR_INVALID, "lbm_reduce: null argument");
    if (!c->initialized) return fail(c, LBM_ERR_STATE, "lbm_reduce before initialisation");
    cudaSetDevice(c->cfg.device);
    if (!c->d_part) CU(c, cudaMalloc(&c->d_part, read_part_size(c->cfg.nx, c->cfg.ny, c->cfg.nz) * sizeof(double)));
    ReadOut o{};
    o.red = c->d_red; o.part = c->d_part; o.mode = READ_DIAG;
    lbm_status s = run_read(c, o);
    if (s) return s;
    double h[RED_COUNT];
    CU(c, cudaMemcpyAsync(h, c->d_red, sizeof(h), cudaMemcpyDeviceToHost, c->st));
    CU(c, cudaStreamSynchronize(c->st));
    out->mass = h[RED_MASS];
    out->momentum[0] = h[RED_MX]; out->momentum[1] = h[RED_MY]; out->momentum[2] = h[RED_MZ];
    out->drag[0] = h[RED_DX]; out->drag[1] = h[RED_DY]; out->drag[2] = h[RED_DZ];
    out->max_speed = h[RED_VMAX];
    out->nonfinite = (int64_t)h[RED_BAD];
    out->fluid_cells = (int64_t)h[RED_FLUID];
    out->step = c->m;
    lbm_status ds = check_device_error(c);
    if (ds) return ds;
    if (out->nonfinite > 0) return fail(c, LBM_ERR_NONFINITE, "%lld cells hold non-finite populations at step %lld",
                                        (long long)out->nonfinite, (long long)c->m);
    return LBM_OK;
}

lbm_status lbm_error_evaluation(lbm_ctx* c, double* err) {
    if (!c || !err) return fail(c, LBM_ERR_INVALID, "lbm_error_evaluation: null argument");
    if (!c->initialized) return fail(c, LBM_ERR_STATE, "lbm_error_evaluation before initialisation");
    cudaSetDevice(c->cfg.device);
    const size_t N = (size_t)c->N;
    if (!c->d_uerr) {
        CU(c, cudaMalloc(&c->d_uerr, 3 * N * real_size(c)));
        CU(c, cudaMemsetAsync(c->d_uerr, 0, 3 * N * real_size(c), c->st));
    }
    if (!c->d_part) CU(c, cudaMalloc(&c->d_part, read_part_size(c->cfg.nx, c->cfg.ny, c->cfg.nz) * sizeof(double)));
    ReadOut o{};
    o.red = c->d_red; o.part = c->d_part; o.uerr = c->d_uerr; o.mode = READ_ERROR;
    lbm_status s = run_read(c, o);
    if (s) return s;
    double h[RED_COUNT];
    CU(c, cudaMemcpyAsync(h, c->d_red, sizeof(h), cudaMemcpyDeviceToHost, c->st));
    CU(c, cudaStreamSynchronize(c->st));
    *err = std::sqrt(h[RED_ERR1]) / std::sqrt(h[RED_ERR2]);
    if (std::isnan(*err)) return fail(c, LBM_ERR_NONFINITE, "error monitor is NaN at step %lld", (long long)c->m);
    return LBM_OK;
}

lbm_status lbm_timeavg_begin(lbm_ctx* c) {
    if (!c) return fail(c, LBM_ERR_INVALID, "null ctx");
    if (!c->initialized) return fail(c, LBM_ERR_STATE, "lbm_timeavg_begin before initialisation");
    cudaSetDevice(c->cfg.device);
    const size_t N = (size_t)c->N;
    if (!c->d_acc) CU(c, cudaMalloc(&c->d_acc, 10 * N * 8));
    CU(c, cudaMemsetAsync(c->d_acc, 0, 10 * N * 8, c->st));
    c->avg_on = true;
    c->avg_begin = c->m;
    c->avg_last = c->m;
    c->avg_count = 0;
    return LBM_OK;
}

// accumulate the current state if it was produced inside the window and not counted yet
static lbm_status avg_flush(lbm_ctx* c) {
    if (c->avg_on && c->m > c->avg_begin && c->m > c->avg_last) {
        ReadOut o{};
        o.mode = READ_ACC;
        lbm_status s = run_read(c, o);
        if (s) return s;
        c->avg_last = c->m;
        c->avg_count++;
    }
    return LBM_OK;
}

lbm_status lbm_timeavg_end(lbm_ctx* c) {
    if (!c) return fail(c, LBM_ERR_INVALID, "null ctx");
    cudaSetDevice(c->cfg.device);
    lbm_status s = avg_flush(c);
    if (s) return s;
    c->avg_on = false;
    return LBM_OK;
}

lbm_status lbm_timeavg_get(lbm_ctx* c, double* rho, double* u, double* uu, int64_t* count) {
    if (!c) return fail(c, LBM_ERR_INVALID, "null ctx");
    if (!c->d_acc) return fail(c, LBM_ERR_STATE, "lbm_timeavg_get without lbm_timeavg_begin");
    cudaSetDevice(c->cfg.device);
    lbm_status s = avg_flush(c);
    if (s) return s;
    const size_t N = (size_t)c->N;
    std::vector<double> h(10 * N);
    CU(c, cudaMemcpyAsync(h.data(), c->d_acc, 10 * N * 8, cudaMemcpyDeviceToHost, c->st));
    CU(c, cudaStreamSynchronize(c->st));
    const double n = c->avg_count > 0 ? (double)c->avg_count : 1.0;
    for (size_t q = 0; q < N; q++) {
        if (rho) rho[q] = h[q] / n;
        if (u) for (int a = 0; a < 3; a++) u[a * N + q] = h[(1 + a) * N + q] / n;
        if (uu) for (int a = 0; a < 6; a++) uu[a * N + q] = h[(4 + a) * N + q] / n;
    }
    if (count) *count = c->avg_count;
    return LBM_OK;
}

// ---- checkpoint: raw state in storage precision, bit-identical resume ------------------------
static const char kMagic[8] = {'L', 'B', 'M', 'G', 'B', '3', '0', '0'};

lbm_status lbm_checkpoint_save(lbm_ctx* c, const char* path) {
    if (!c || !path) return fail(c, LBM_ERR_INVALID, "lbm_checkpoint_save: null argument");
    if (!c->initialized) return fail(c, LBM_ERR_STATE, "nothing to save before initialisation");
    cudaSetDevice(c->cfg.device);
    CU(c, cudaStreamSynchronize(c->st));
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return fail(c, LBM_ERR_IO, "cannot open %s", path);
    const size_t N = (size_t)c->N, rs = real_size(c);
    auto put = [&](const void* p, size_t n) { return std::fwrite(p, 1, n, fp) == n; };
    auto put_dev = [&](const void* d, size_t n) -> bool {
        if (!n) return true;
        std::vector<char> h(n);
        if (cudaMemcpy(h.data(), d, n, cudaMemcpyDeviceToHost) != cudaSuccess) return false;
        return put(h.data(), n);
    };
    int32_t ver = LBM_ABI_VERSION;
    int64_t m = c->m, nin = (int64_t)c->inlets.size(), nout = (int64_t)c->outlets.size(),
            nsym = (int64_t)c->syms.size();
    bool ok = put(kMagic, 8) && put(&ver, 4) && put(&c->cfg, sizeof(c->cfg)) && put(&m, 8) &&
              put(c->flags.data(), N * 4) && put(&nin, 8) && put(c->inlets.data(), nin * sizeof(lbm_bc_inlet)) &&
              put(&nout, 8) && put(c->outlets.data(), nout * sizeof(lbm_bc_outlet)) &&
              put(&nsym, 8) && put(c->syms.data(), nsym * sizeof(lbm_bc_symmetry)) &&
              put_dev(c->d_f, 27 * N * c->esize) &&
              put_dev(c->d_lid_state, 3 * 27 * (size_t)c->n_lid * rs) &&
              put_dev(c->d_in_probe, 9 * (size_t)c->n_in * rs) &&
              put_dev(c->d_out_save, 36 * (size_t)c->n_out * rs) &&
              put_dev(c->d_out_msave, 8 * (size_t)c->n_ms * rs);
    std::fclose(fp);
    if (!ok) return fail(c, LBM_ERR_IO, "writing %s failed", path);
    return LBM_OK;
}

lbm_status lbm_checkpoint_load(lbm_ctx* c, const char* path) {
    if (!c || !path) return fail(c, LBM_ERR_INVALID, "lbm_checkpoint_load: null argument");
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return fail(c, LBM_ERR_IO, "cannot open %s", path);
    auto get = [&](void* p, size_t n) { return std::fread(p, 1, n, fp) == n; };
    char mg[8];
    int32_t ver = 0;
    lbm_config cfg;
    int64_t m = 0, nin = 0, nout = 0, nsym = 0;
    if (!get(mg, 8) || std::memcmp(mg, kMagic, 8) != 0 || !get(&ver, 4) || ver != LBM_ABI_VERSION ||
        !get(&cfg, sizeof(cfg)) || !get(&m, 8)) {
        std::fclose(fp);
        return fail(c, LBM_ERR_IO, "%s is not a checkpoint of this library version", path);
    }
    if (cfg.nx != c->cfg.nx || cfg.ny != c->cfg.ny || cfg.nz != c->cfg.nz || cfg.storage != c->cfg.storage) {
        std::fclose(fp);
        return fail(c, LBM_ERR_INVALID, "checkpoint lattice/storage differ from this context");
    }
    const size_t N = (size_t)c->N;
    std::vector<int32_t> fl(N);
    bool ok = get(fl.data(), N * 4) && get(&nin, 8);
    std::vector<lbm_bc_inlet> in(ok ? (size_t)nin : 0);
    ok = ok && get(in.data(), nin * sizeof(lbm_bc_inlet)) && get(&nout, 8);
    std::vector<lbm_bc_outlet> out(ok ? (size_t)nout : 0);
    ok = ok && get(out.data(), nout * sizeof(lbm_bc_outlet)) && get(&nsym, 8);
    std::vector<lbm_bc_symmetry> sy(ok ? (size_t)nsym : 0);
    ok = ok && get(sy.data(), nsym * sizeof(lbm_bc_symmetry));
    if (!ok) { std::fclose(fp); return fail(c, LBM_ERR_IO, "truncated checkpoint %s", path); }
    int dev = c->cfg.device;
    c->cfg = cfg;
    c->cfg.device = dev;
    c->flags = fl; c->inlets = in; c->outlets = out; c->syms = sy;
    c->have_flags = true; c->have_geom = false;
    cudaSetDevice(dev);
    lbm_status s = build_geometry(c);
    if (s) { std::fclose(fp); return s; }
    const size_t rs = real_size(c);
    auto get_dev = [&](void* d, size_t n) -> bool {
        if (!n) return true;
        std::vector<char> h(n);
        if (!get(h.data(), n)) return false;
        return cudaMemcpy(d, h.data(), n, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    ok = get_dev(c->d_f, 27 * N * c->esize) && get_dev(c->d_lid_state, 81 * (size_t)c->n_lid * rs) &&
         get_dev(c->d_in_probe, 9 * (size_t)c->n_in * rs) && get_dev(c->d_out_save, 36 * (size_t)c->n_out * rs) &&
         get_dev(c->d_out_msave, 8 * (size_t)c->n_ms * rs);
    std::fclose(fp);
    if (!ok) return fail(c, LBM_ERR_IO, "reading %s failed", path);
    c->m = m;
    c->mlp_due = m;  // kept nu_t are not in the file: the network runs in the next step
    c->initialized = true;
    c->avg_on = false;
    return LBM_OK;
}

// ---- host mesher: geometryMesherBoundary::meshingBoundaryWall (geometryMesherBoundary.h:439-484)
lbm_status lbm_mesher_wall_pass(int32_t* fl, int32_t nx, int32_t ny, int32_t nz) {
    if (!fl || nx <= 0 || ny <= 0 || nz <= 0) return fail(nullptr, LBM_ERR_INVALID, "lbm_mesher_wall_pass: bad argument");
    auto at = [&](int i, int j, int k) -> int32_t& { return fl[(size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k)]; };
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                if (at(i, j, k) <= 0) continue;
                int add = 0;
                for (int n = -1; n <= 1; n++)
                    for (int mm = -1; mm <= 1; mm++)
                        for (int l = -1; l <= 1; l++) {
                            int a = i + l, b = j + mm, e = k + n;
                            if (a >= 0 && b >= 0 && e >= 0 && a < nx && b < ny && e < nz && at(a, b, e) == 0) add++;
                        }
                at(i, j, k) += add;
            }
    return LBM_OK;
}

}  // extern "C"

// ---- learned closure ----------------------------------------------------------------------------------
extern "C" {

lbm_status lbm_mlp_load(lbm_ctx* c, const lbm_mlp_model* m) {
    if (!c || !m) return fail(c, LBM_ERR_INVALID, "lbm_mlp_load: null argument");
    if (c->cfg.closure != LBM_CLOSURE_MLP)
        return fail(c, LBM_ERR_STATE, "lbm_mlp_load: the context was not created with LBM_CLOSURE_MLP");
    if (!mlp_model_valid(m)) return fail(c, LBM_ERR_INVALID, "lbm_mlp_load: non-finite parameters or bad scales");
    cudaSetDevice(c->cfg.device);
    std::vector<uint4> frag(kMlpFragTotal);  // warp fragment table, then the tcgen05 weight image
    MlpNorm nm;
    mlp_pack(*m, frag.data(), nm);
    if (!c->d_mlp_frag) CU(c, cudaMalloc(&c->d_mlp_frag, frag.size() * sizeof(uint4)));
    // ordered after the steps already queued on the context's stream
    CU(c, cudaMemcpyAsync(c->d_mlp_frag, frag.data(), frag.size() * sizeof(uint4), cudaMemcpyHostToDevice, c->st));
    if (c->cfg.mlp_interval > 1 && !c->d_nut) {
        CU(c, cudaMalloc(&c->d_nut, (size_t)c->N * sizeof(__half)));
        CU(c, cudaMemsetAsync(c->d_nut, 0xFF, (size_t)c->N * sizeof(__half), c->st));  // not a number: fallback
    }
    CU(c, cudaStreamSynchronize(c->st));
    c->mlp_norm = nm;
    c->have_mlp = true;
    c->mlp_due = c->m;  // the network runs in the next step
    return LBM_OK;
}

lbm_status lbm_get_eddy_viscosity(lbm_ctx* c, double* nu) {
    if (!c || !nu) return fail(c, LBM_ERR_INVALID, "lbm_get_eddy_viscosity: null argument");
    if (!c->d_nut) return fail(c, LBM_ERR_STATE, "lbm_get_eddy_viscosity: the context keeps no eddy viscosity "
                                                 "(learned closure with mlp_interval > 1 only)");
    cudaSetDevice(c->cfg.device);
    std::vector<__half> h((size_t)c->N);
    CU(c, cudaMemcpyAsync(h.data(), c->d_nut, (size_t)c->N * sizeof(__half), cudaMemcpyDeviceToHost, c->st));
    CU(c, cudaStreamSynchronize(c->st));
    host_parallel(c->N, [&](long long q0, long long q1) {
        for (long long q = q0; q < q1; q++) nu[q] = (double)__half2float(h[(size_t)q]);
    });
    return LBM_OK;
}

lbm_status lbm_les_samples(lbm_ctx* c, int32_t w, float* out, int64_t capacity, int64_t* count) {
    if (!c || !count || w < 1 || capacity < 0 || (capacity > 0 && !out))
        return fail(c, LBM_ERR_INVALID, "lbm_les_samples: bad argument");
    if (!c->initialized) return fail(c, LBM_ERR_STATE, "lbm_les_samples before initialisation");
    const int nx = c->cfg.nx, ny = c->cfg.ny, nz = c->cfg.nz;
    if (nx / w < 3 || ny / w < 3 || nz / w < 3)
        return fail(c, LBM_ERR_INVALID, "lbm_les_samples: fewer than 3 coarse cells per axis");
    cudaSetDevice(c->cfg.device);
    const long long Nc = (long long)(nx / w) * (ny / w) * (nz / w);
    double *d_rho = nullptr, *d_u = nullptr;
    float *d_cf = nullptr, *d_out = nullptr;
    auto cleanup = [&]() { dfree(d_rho); dfree(d_u); dfree(d_cf); dfree(d_out); };
    cudaError_t e = cudaMalloc(&d_rho, (size_t)c->N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_u, 3 * (size_t)c->N * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_cf, 11 * (size_t)Nc * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&d_out, 11 * (size_t)Nc * sizeof(float));
    if (e != cudaSuccess) {
        cleanup();
        return fail(c, e == cudaErrorMemoryAllocation ? LBM_ERR_OOM : LBM_ERR_CUDA, "lbm_les_samples: %s",
                    cudaGetErrorString(e));
    }
    Params p = make_params(c);
    ReadOut o{};
    o.rho = d_rho;
    o.u = d_u;
    o.mode = READ_MOMENTS;
    switch (c->cfg.storage) {
        case LBM_STORAGE_F64: e = launch_read<StF64>(p, o, c->st); break;
        case LBM_STORAGE_F32: e = launch_read<StF32>(p, o, c->st); break;
        default: e = launch_read<StF16>(p, o, c->st); break;
    }
    const int wrap[3] = {p.wrap[0], p.wrap[1], p.wrap[2]};
    if (e == cudaSuccess) e = launch_les_samples(d_rho, d_u, c->d_cls, nx, ny, nz, w, wrap, d_cf, d_out, c->st);
    std::vector<float> h(11 * (size_t)Nc);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d_out, h.size() * sizeof(float), cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    cleanup();
    if (e != cudaSuccess) return fail(c, LBM_ERR_CUDA, "lbm_les_samples: %s", cudaGetErrorString(e));
    long long n = 0;
    for (long long i = 0; i < Nc; i++) {
        const float* r = &h[(size_t)i * 11];
        if (r[10] < 0.5f) continue;
        if (n < capacity) std::memcpy(out + (size_t)n * LBM_MLP_SAMPLE, r, LBM_MLP_SAMPLE * sizeof(float));
        n++;
    }
    *count = n;
    return LBM_OK;
}

}  // extern "C"
