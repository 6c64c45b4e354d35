// lbm_aux.cuh - read-only and set-up kernels that share the step kernel's gather.
#pragma once

#include "lbm_device.cuh"
#include "lbm_step.cuh"

namespace lbm {

// slots of the FP64 reduction buffer filled by k_read in diagnostics mode
enum { RED_MASS = 0, RED_MX, RED_MY, RED_MZ, RED_DX, RED_DY, RED_DZ, RED_VMAX, RED_BAD, RED_FLUID,
       RED_ERR1, RED_ERR2, RED_COUNT };

enum : int {
    READ_MOMENTS = 1,   // write rho_out[N], u_out[3N] (double)
    READ_POPS = 2,      // write f_out[27N] (double)
    READ_DIAG = 4,      // FP64 reductions into red[]
    READ_ERROR = 8,     // ErrorQuadratic sums over reference-bulk cells, then u_err = u
    READ_ACC = 16,      // add the current moments to the time-average accumulators
};

struct ReadOut {
    double* rho;   // N
    double* u;     // 3N
    double* f;     // 27N
    double* red;   // RED_COUNT
    void* uerr;    // 3N of S::R (error monitor's previous velocity)
    double* part;  // READ_DIAG / READ_ERROR: per-block partial sums [RED_COUNT][blocks] (read_part_size)
    int mode;
    int ref_compat_err;  // reproduce the ErrorQuadratic z-term typo
};

// the reading kernels run one thread per x-pair of a (y, kReadZ z-planes) column tile (pairs of bulk
// cells load both cells with the step kernel's packed accesses); the reductions keep per-thread partial
// sums over the tile's cells, one partial per block in part[], and a second kernel adds the partials in
// a fixed order: the result does not depend on scheduling (no atomics)
constexpr int kReadZ = 4;
inline int read_block(int nx) {
    const int half = (nx + 1) / 2;
    return half >= 128 ? 128 : ((half + 31) / 32) * 32;
}
inline dim3 read_grid(int nx, int ny, int nz) {
    const int half = (nx + 1) / 2, b = read_block(nx);
    return dim3((unsigned)((half + b - 1) / b), (unsigned)ny, (unsigned)((nz + kReadZ - 1) / kReadZ));
}
inline long long read_blocks(int nx, int ny, int nz) {
    const dim3 g = read_grid(nx, ny, nz);
    return (long long)g.x * g.y * g.z;
}
inline size_t read_part_size(int nx, int ny, int nz) { return (size_t)RED_COUNT * (size_t)read_blocks(nx, ny, nz); }

LBM_D double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
LBM_D double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// per-thread partial sums of the reductions: FP64 for FP64 storage; for FP32 and FP16 storage a
// compensated FP32 pair per quantity (GB300's FP64 pipe runs about one lane per cycle per SM, which
// made the FP64 sums the read kernel's bound), converted to FP64 once per warp
template <class R>
struct RedAcc {
    double v[RED_COUNT];
    R vmax;
    int nbad, nfluid;
    LBM_D RedAcc() : vmax((R)0), nbad(0), nfluid(0) {
#pragma unroll
        for (int q = 0; q < RED_COUNT; q++) v[q] = 0.0;
    }
    LBM_D void add(int q, double x) { v[q] += x; }
    LBM_D double warp_total(int q) const { return warp_sum(v[q]); }
};
template <>
struct RedAcc<float> {
    FSum v[RED_COUNT];
    float vmax;
    int nbad, nfluid;
    LBM_D RedAcc() : vmax(0.0f), nbad(0), nfluid(0) {
#pragma unroll
        for (int q = 0; q < RED_COUNT; q++) v[q] = FSum{0.0f, 0.0f};
    }
    LBM_D void add(int q, float x) { fsum_add(v[q], x); }
    LBM_D double warp_total(int q) const {
        FSum s = v[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const FSum t{__shfl_xor_sync(0xffffffffu, s.hi, o), __shfl_xor_sync(0xffffffffu, s.lo, o)};
            fsum_merge(s, t);
        }
        return f2d(s.hi) + f2d(s.lo);
    }
};
LBM_D double to_double(double x) { return x; }
LBM_D double to_double(float x) { return f2d(x); }
template <class R> LBM_D R to_real(double x) { if constexpr (std::is_same<R, float>::value) return d2f(x); else return x; }

// block totals of the quantities [Q0, Q1) (the largest |u|^2 for RED_VMAX, counts exact in integers),
// warp by warp and then over the block's warps in a fixed order, written as this block's partial;
// every thread of the block calls it
template <int Q0, int Q1, class R>
LBM_D void block_partials(const RedAcc<R>& a, double* part, long long nblk) {
    __shared__ double sh[RED_COUNT][4];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int q = Q0; q < Q1; q++) {
        double s;
        if (q == RED_VMAX) {
            R m = a.vmax;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const R t = __shfl_xor_sync(0xffffffffu, m, o);
                m = t > m ? t : m;
            }
            s = to_double(m);
        } else if (q == RED_BAD || q == RED_FLUID) {
            s = (double)__reduce_add_sync(0xffffffffu, (unsigned)(q == RED_BAD ? a.nbad : a.nfluid));
        } else {
            s = a.warp_total(q);
        }
        if (lane == 0) sh[q][wid] = s;
    }
    __syncthreads();
    if (threadIdx.x < Q1 - Q0) {
        const int q = Q0 + threadIdx.x;
        double s = sh[q][0];
        for (int w = 1; w < nw; w++) s = q == RED_VMAX ? fmax(s, sh[q][w]) : s + sh[q][w];
        const long long b = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
        part[q * nblk + b] = s;
    }
}

// one cell of the reading kernels: its populations f (gathered as the step kernel does) and drag links
template <class S>
LBM_D void read_cell(const Params& p, const ReadOut& o, RedAcc<typename S::R>& acc, long long idx, uint8_t fl,
                     const typename S::R (&f)[27], const typename S::R (&drag)[3]) {
    using R = typename S::R;
    const int cl = fl & CLS_MASK;
    R rho = 0, jx = 0, jy = 0, jz = 0, ux = 0, uy = 0, uz = 0;
    if (cl != CLS_SOLID) moments(f, p, rho, jx, jy, jz, ux, uy, uz);
    if (o.mode & READ_MOMENTS) {
        o.rho[idx] = to_double(rho);
        o.u[idx] = to_double(ux); o.u[p.N + idx] = to_double(uy); o.u[2 * p.N + idx] = to_double(uz);
    }
    if (o.mode & READ_POPS) {
#pragma unroll
        for (int q = 0; q < 27; q++) o.f[q * p.N + idx] = to_double(f[q]);
    }
    if ((o.mode & READ_ACC) && cl != CLS_SOLID) {
        double* a = p.acc;
        const long long N = p.N;
        a[idx] += rho; a[N + idx] += ux; a[2 * N + idx] += uy; a[3 * N + idx] += uz;
        a[4 * N + idx] += (double)ux * ux; a[5 * N + idx] += (double)uy * uy; a[6 * N + idx] += (double)uz * uz;
        a[7 * N + idx] += (double)ux * uy; a[8 * N + idx] += (double)ux * uz; a[9 * N + idx] += (double)uy * uz;
    }
    if ((o.mode & READ_DIAG) && (cl == CLS_BULK || cl == CLS_EDGE || cl == CLS_OUTLET || cl == CLS_SYM)) {
        // a non-finite population makes rho or the momentum non-finite (a NaN stays NaN, +-Inf
        // give Inf or NaN), so the moments stand for the 27 values
        const bool ok = isfinite(rho) && isfinite(jx) && isfinite(jy) && isfinite(jz);
        acc.add(RED_MASS, rho);
        acc.add(RED_MX, rho * ux); acc.add(RED_MY, rho * uy); acc.add(RED_MZ, rho * uz);
        if (cl != CLS_BULK) {  // only cells beside a solid have momentum-exchange links
            acc.add(RED_DX, drag[0]); acc.add(RED_DY, drag[1]); acc.add(RED_DZ, drag[2]);
        }
        const R u2 = ux * ux + uy * uy + uz * uz;
        if (isfinite(u2) && u2 > acc.vmax) acc.vmax = u2;
        acc.nbad += ok ? 0 : 1;
        acc.nfluid += 1;
    }
    if (o.mode & READ_ERROR) {
        // ErrorQuadratic.h:33-78: sum sqrt|u - u_prev|^2 and sqrt|u|^2 over flag == 1 cells
        R* uerr = (R*)o.uerr;
        if (fl & BIT_REFBULK) {
            const R px = uerr[idx], py = uerr[p.N + idx], pz = uerr[2 * p.N + idx];
            const R dx = ux - px, dy = uy - py;
            const R dz = o.ref_compat_err ? uy - pz : uz - pz;
            const R a1 = dx * dx + dy * dy + dz * dz;
            const R a2 = ux * ux + uy * uy + uz * uz;
            acc.add(RED_ERR1, sqrt(a1));
            acc.add(RED_ERR2, sqrt(a2));
        }
        uerr[idx] = ux; uerr[p.N + idx] = uy; uerr[2 * p.N + idx] = uz;  // copy u -> u_error (:80-90), every cell
    }
}

// a cell of a reading kernel through the general gather
template <class S, bool ODD>
LBM_D void read_cell_general(const Params& p, const ReadOut& o, RedAcc<typename S::R>& acc, int x, int y, int z) {
    using R = typename S::R;
    Cell c;
    make_cell(p, x, y, z, c);
    const uint8_t fl = p.cls[c.idx];
    const int cl = fl & CLS_MASK;
    R f[27];
    R drag[3] = {0, 0, 0};
    if (cl == CLS_SOLID) {
#pragma unroll
        for (int q = 0; q < 27; q++) f[q] = (R)0;
    } else if (cl == CLS_INLET) {
        inlet_state<S>(p, c, f);
    } else if (cl == CLS_BULK && !on_seam(p, c.x, c.y, c.z)) {
        load_fast<S, ODD>(p, (unsigned)c.idx, f);  // the step kernel's per-direction addresses
    } else {
        gather<S, ODD, true>(p, c, cl, f, drag);
    }
    read_cell<S>(p, o, acc, c.idx, fl, f, drag);
}

// one thread per x-pair of a column tile of kReadZ cells along z; gathers df_m exactly as the step kernel.
// Pairs of bulk cells off the periodic y/z seams load through the packed pair accesses (one 32-bit FP16 /
// 64-bit FP32 load per direction for both cells where the AA slot pair is aligned); other pairs cell by cell
template <class S, bool ODD>
__global__ void __launch_bounds__(128, 4) k_read(Params p, ReadOut o) {
    using R = typename S::R;
    const int x0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = blockIdx.y;
    RedAcc<R> acc;
    if (x0 < p.nx) {
        const bool two = x0 + 1 < p.nx;
        const bool yz_seam = (p.wrap[1] && (y == 0 || y == p.ny - 1));
        for (int k = 0; k < kReadZ; k++) {
            const int z = blockIdx.z * kReadZ + k;
            if (z >= p.nz) break;
            const long long idx0 = x0 + (long long)p.nx * (y + (long long)p.ny * z);
            bool pair = false;
            uint8_t f0 = 0, f1 = 0;
            if constexpr (S::kind != 0) {
                f0 = p.cls[idx0];
                f1 = two ? p.cls[idx0 + 1] : (uint8_t)0;
                pair = two && (p.nx & 1) == 0 && !yz_seam && !(p.wrap[2] && (z == 0 || z == p.nz - 1)) &&
                       (f0 & (uint8_t)~BIT_REFBULK) == CLS_BULK && (f1 & (uint8_t)~BIT_REFBULK) == CLS_BULK;
            }
            if constexpr (S::kind != 0) {
                if (pair) {
                    const PairCodec kc = make_codec<S>(p);
                    const PairIdx q = make_pair_idx(p, (int)idx0, x0);
                    F2 f2[27];
                    load_pair<S, ODD, false>(p, q, kc, f2);
                    R fa[27], fb[27];
#pragma unroll
                    for (int v = 0; v < 27; v++) { fa[v] = f2[v].v.x; fb[v] = f2[v].v.y; }
                    const R nod[3] = {0, 0, 0};
                    read_cell<S>(p, o, acc, idx0, f0, fa, nod);
                    read_cell<S>(p, o, acc, idx0 + 1, f1, fb, nod);
                    continue;
                }
            }
            read_cell_general<S, ODD>(p, o, acc, x0, y, z);
            if (two) read_cell_general<S, ODD>(p, o, acc, x0 + 1, y, z);
        }
    }
    const long long nblk = (long long)gridDim.x * gridDim.y * gridDim.z;
    if (o.mode & READ_DIAG) block_partials<RED_MASS, RED_ERR1>(acc, o.part, nblk);
    if (o.mode & READ_ERROR) {
        if (o.mode & READ_DIAG) __syncthreads();
        block_partials<RED_ERR1, RED_COUNT>(acc, o.part, nblk);
    }
}

// the partials of k_read added in a fixed order: one block per quantity q0 + blockIdx.x, a strided pass
// per thread, then a tree over the block's threads; RED_VMAX is the square root of the largest |u|^2
constexpr int kFinalThreads = 1024;
template <class S>
__global__ void __launch_bounds__(kFinalThreads) k_read_final(const double* part, long long nblk, int q0, double* red) {
    __shared__ double sh[kFinalThreads];
    const int q = q0 + blockIdx.x;
    const bool mx = q == RED_VMAX;
    const double* a = part + q * nblk;
    double s = 0.0;
    for (long long b = threadIdx.x; b < nblk; b += kFinalThreads) s = mx ? fmax(s, a[b]) : s + a[b];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kFinalThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] = mx ? fmax(sh[threadIdx.x], sh[threadIdx.x + w]) : sh[threadIdx.x] + sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) red[q] = mx ? sqrt(sh[0]) : sh[0];
}

// one cell's (u_x, u_y, u_z, rho), the reference's per-step probe (SolverTurbulentLES.h:150-177)
template <class S, bool ODD>
__global__ void k_probe(Params p, int x, int y, int z, double* out) {
    using R = typename S::R;
    Cell c;
    make_cell(p, x, y, z, c);
    const int cl = p.cls[c.idx] & CLS_MASK;
    R f[27];
    R drag[3] = {0, 0, 0};
    if (cl == CLS_SOLID) {
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return;
    }
    if (cl == CLS_INLET) inlet_state<S>(p, c, f);
    else gather<S, ODD, false>(p, c, cl, f, drag);
    R rho, jx, jy, jz, ux, uy, uz;
    moments(f, p, rho, jx, jy, jz, ux, uy, uz);
    out[0] = ux; out[1] = uy; out[2] = uz; out[3] = rho;
}

// equilibrium initialisation (InitializationEquilibriumConstVector.h:111-126): state m = 0 in the
// cells' own slots; side tables of the -1 nodes seeded so that the first steps see df_0 there.
template <class S>
__global__ void __launch_bounds__(128) k_init(Params p, const double* rho_f, const double* u_f, double rho0,
                                              double u0x, double u0y, double u0z, const double* pops) {
    using R = typename S::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= p.nx) return;
    Cell c;
    make_cell(p, x, blockIdx.y, blockIdx.z, c);
    const int cl = p.cls[c.idx] & CLS_MASK;
    const long long N = p.N;
    R r, ux, uy, uz;
    if (rho_f) { r = to_real<R>(rho_f[c.idx]); ux = to_real<R>(u_f[c.idx]); uy = to_real<R>(u_f[N + c.idx]); uz = to_real<R>(u_f[2 * N + c.idx]); }
    else { r = to_real<R>(rho0); ux = to_real<R>(u0x); uy = to_real<R>(u0y); uz = to_real<R>(u0z); }
    if (cl == CLS_LID) {
        const int id = p.aux[c.idx];
        ux = p.lid_u[id]; uy = p.lid_u[p.n_lid + id]; uz = p.lid_u[2 * p.n_lid + id];
    } else if (cl == CLS_INLET) {
        const int id = p.aux[c.idx];
        ux = p.in_u[id]; uy = p.in_u[p.n_in + id]; uz = p.in_u[2 * p.n_in + id];
    }
    R f[27];
    const R u2 = ux * ux + uy * uy + uz * uz;
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        f[V] = cl == CLS_SOLID ? (R)0 : (pops ? to_real<R>(pops[V * N + c.idx]) : feq<V>(r, ux, uy, uz, u2));
    });
    if constexpr (S::kind == 2) {
        // FP16 deviations of the initial state: the packed stores' rounding (cvt.rs, lower field) with one
        // seed per cell, a hash of the cell index and this launch's step seed
        const uint32_t s = sr_seed_pair((uint32_t)c.idx, p);
        __half* A = (__half*)p.f;
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            const float e = fmaf(f[V], p.scale, p.nwrs[V]);
            const __half2 h = half2_sr(make_float2(e, 0.0f), s + p.sr_off[V]);
            A[V * N + c.idx] = __low2half(h);
        });
    } else {
        sfor<0, 27>([&](auto vc) {
            constexpr int V = decltype(vc)::value;
            store_at<S, V>(p, V * N + c.idx, f[V]);
        });
    }
    if (cl == CLS_LID) {
        const int id = p.aux[c.idx];
        R* st = (R*)p.lid_state;
        for (int l = 0; l < 3; l++)
            for (int v = 0; v < 27; v++) st[((long long)l * 27 + v) * p.n_lid + id] = f[v];
    } else if (cl == CLS_INLET) {
        // level "step -1": rho1 = rho(I), ux1 = ux2 = u_b  =>  rho_b = rho(I)
        const int id = p.aux[c.idx];
        R rr = 0;
        for (int v = 0; v < 27; v++) rr += f[v];
        if (!pops) rr = r;
        R* pr = (R*)p.in_probe + 2LL * 3 * p.n_in;
        pr[id] = rr; pr[p.n_in + id] = ux; pr[2 * p.n_in + id] = ux;
    }
}

}  // namespace lbm
