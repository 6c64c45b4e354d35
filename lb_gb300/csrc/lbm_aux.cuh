// lbm_aux.cuh - read-only and set-up kernels that share the step kernel's gather.
#pragma once

#include "lbm_device.cuh"

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
    double* uerr;  // 3N (error monitor's previous velocity)
    int mode;
    int ref_compat_err;  // reproduce the ErrorQuadratic z-term typo
};

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

// one thread per cell; gathers df_m exactly as the step kernel would
template <class S, bool ODD>
__global__ void __launch_bounds__(128) k_read(Params p, ReadOut o) {
    using R = typename S::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = x < p.nx;
    Cell c;
    make_cell(p, live ? x : 0, blockIdx.y, blockIdx.z, c);
    const uint8_t fl = live ? p.cls[c.idx] : (uint8_t)0;
    const int cl = fl & CLS_MASK;
    R f[27];
    R drag[3] = {0, 0, 0};
    if (!live || cl == CLS_SOLID) {
#pragma unroll
        for (int v = 0; v < 27; v++) f[v] = (R)0;
    } else if (cl == CLS_INLET) {
        inlet_state<S>(p, c, f);
    } else {
        gather<S, ODD, true>(p, c, cl, f, drag);
    }
    R rho = 0, jx = 0, jy = 0, jz = 0, ux = 0, uy = 0, uz = 0;
    if (live && cl != CLS_SOLID) moments(f, p, rho, jx, jy, jz, ux, uy, uz);
    if (live && (o.mode & READ_MOMENTS)) {
        o.rho[c.idx] = rho;
        o.u[c.idx] = ux; o.u[p.N + c.idx] = uy; o.u[2 * p.N + c.idx] = uz;
    }
    if (live && (o.mode & READ_POPS)) {
#pragma unroll
        for (int v = 0; v < 27; v++) o.f[v * p.N + c.idx] = f[v];
    }
    if (live && (o.mode & READ_ACC) && cl != CLS_SOLID) {
        double* a = p.acc;
        const long long N = p.N;
        a[c.idx] += rho; a[N + c.idx] += ux; a[2 * N + c.idx] += uy; a[3 * N + c.idx] += uz;
        a[4 * N + c.idx] += (double)ux * ux; a[5 * N + c.idx] += (double)uy * uy; a[6 * N + c.idx] += (double)uz * uz;
        a[7 * N + c.idx] += (double)ux * uy; a[8 * N + c.idx] += (double)ux * uz; a[9 * N + c.idx] += (double)uy * uz;
    }
    if (o.mode & READ_DIAG) {
        const bool tgt = live && (cl == CLS_BULK || cl == CLS_EDGE || cl == CLS_OUTLET || cl == CLS_SYM);
        double v[RED_COUNT] = {0};
        if (tgt) {
            bool ok = true;
#pragma unroll
            for (int q = 0; q < 27; q++) ok = ok && isfinite((double)f[q]);
            v[RED_MASS] = rho;
            v[RED_MX] = (double)rho * ux; v[RED_MY] = (double)rho * uy; v[RED_MZ] = (double)rho * uz;
            v[RED_DX] = drag[0]; v[RED_DY] = drag[1]; v[RED_DZ] = drag[2];
            v[RED_VMAX] = sqrt((double)ux * ux + (double)uy * uy + (double)uz * uz);
            if (!isfinite(v[RED_VMAX])) v[RED_VMAX] = 0;
            v[RED_BAD] = ok ? 0.0 : 1.0;
            v[RED_FLUID] = 1.0;
        }
        __shared__ double sh[RED_COUNT][4];
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
        for (int q = 0; q < RED_COUNT; q++) {
            if (q == RED_ERR1 || q == RED_ERR2) continue;
            double s = q == RED_VMAX ? warp_max(v[q]) : warp_sum(v[q]);
            if (lane == 0) sh[q][wid] = s;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int q = 0; q < RED_COUNT; q++) {
                if (q == RED_ERR1 || q == RED_ERR2) continue;
                double s = sh[q][0];
                for (int w = 1; w < nw; w++) s = q == RED_VMAX ? fmax(s, sh[q][w]) : s + sh[q][w];
                if (q == RED_VMAX) {
                    // non-negative doubles order like their bit patterns
                    atomicMax((unsigned long long*)&o.red[q], (unsigned long long)__double_as_longlong(s));
                } else if (s != 0.0) {
                    atomicAdd(&o.red[q], s);
                }
            }
        }
    }
    if (o.mode & READ_ERROR) {
        // ErrorQuadratic.h:33-78: sum sqrt|u - u_prev|^2 and sqrt|u|^2 over flag == 1 cells
        double e1 = 0, e2 = 0;
        if (live && (fl & BIT_REFBULK)) {
            const R px = (R)o.uerr[c.idx], py = (R)o.uerr[p.N + c.idx], pz = (R)o.uerr[2 * p.N + c.idx];
            const R dx = ux - px, dy = uy - py;
            const R dz = o.ref_compat_err ? uy - pz : uz - pz;
            const R a1 = dx * dx + dy * dy + dz * dz;
            const R a2 = ux * ux + uy * uy + uz * uz;
            e1 = (double)sqrt(a1);
            e2 = (double)sqrt(a2);
        }
        if (live) {  // copy u -> u_error (:308-318), every cell
            o.uerr[c.idx] = ux; o.uerr[p.N + c.idx] = uy; o.uerr[2 * p.N + c.idx] = uz;
        }
        e1 = warp_sum(e1);
        e2 = warp_sum(e2);
        if ((threadIdx.x & 31) == 0) {
            if (e1 != 0.0) atomicAdd(&o.red[RED_ERR1], e1);
            if (e2 != 0.0) atomicAdd(&o.red[RED_ERR2], e2);
        }
    }
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
    R r = (R)rho0, ux = (R)u0x, uy = (R)u0y, uz = (R)u0z;
    if (rho_f) { r = (R)rho_f[c.idx]; ux = (R)u_f[c.idx]; uy = (R)u_f[N + c.idx]; uz = (R)u_f[2 * N + c.idx]; }
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
        f[V] = cl == CLS_SOLID ? (R)0 : (pops ? (R)pops[V * N + c.idx] : feq<V>(r, ux, uy, uz, u2));
    });
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        store_at<S, V>(p, V * N + c.idx, f[V]);
    });
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
