// lbm_launch.cuh - definitions of the launchers; included by one .cu per storage type.
#pragma once

#include "lbm_aux.cuh"
#include "lbm_launch.h"
#include "lbm_step.cuh"

namespace lbm {

template <class S, int COLL, int CLOS>
static cudaError_t step_parity(const Params& p, cudaStream_t st) {
    if constexpr (S::kind == 0) {
        dim3 g = cell_grid(p.nx, p.ny, p.nz), b = cell_block(p.nx);
        if (p.m & 1) k_step<S, COLL, CLOS, true><<<g, b, 0, st>>>(p);
        else         k_step<S, COLL, CLOS, false><<<g, b, 0, st>>>(p);
    } else {
        const int half = (p.nx + 1) / 2;  // one thread per x-pair
        dim3 g = cell_grid(half, p.ny, p.nz), b = cell_block(half);
        if (p.m & 1) k_step2<S, COLL, CLOS, true><<<g, b, 0, st>>>(p);
        else         k_step2<S, COLL, CLOS, false><<<g, b, 0, st>>>(p);
    }
    return cudaGetLastError();
}

template <class S>
cudaError_t launch_step(const Params& p, int collision, int closure, cudaStream_t st) {
    if (collision == 0) return closure == 0 ? step_parity<S, 0, 0>(p, st) : step_parity<S, 0, 1>(p, st);
    return closure == 0 ? step_parity<S, 1, 0>(p, st) : step_parity<S, 1, 1>(p, st);
}

template <class S>
cudaError_t launch_read(const Params& p, const ReadOut& o, cudaStream_t st) {
    dim3 g = cell_grid(p.nx, p.ny, p.nz), b = cell_block(p.nx);
    if (p.m & 1) k_read<S, true><<<g, b, 0, st>>>(p, o);
    else         k_read<S, false><<<g, b, 0, st>>>(p, o);
    return cudaGetLastError();
}

template <class S>
cudaError_t launch_init(const Params& p, const double* rho, const double* u, double rho0, const double u0[3],
                        const double* pops, cudaStream_t st) {
    dim3 g = cell_grid(p.nx, p.ny, p.nz), b = cell_block(p.nx);
    k_init<S><<<g, b, 0, st>>>(p, rho, u, rho0, u0[0], u0[1], u0[2], pops);
    return cudaGetLastError();
}

template <class S>
cudaError_t launch_probe(const Params& p, int x, int y, int z, double* out, cudaStream_t st) {
    if (p.m & 1) k_probe<S, true><<<1, 1, 0, st>>>(p, x, y, z, out);
    else         k_probe<S, false><<<1, 1, 0, st>>>(p, x, y, z, out);
    return cudaGetLastError();
}

#define LBM_INSTANTIATE(S)                                                                              \
    template cudaError_t launch_step<S>(const Params&, int, int, cudaStream_t);                         \
    template cudaError_t launch_read<S>(const Params&, const ReadOut&, cudaStream_t);                   \
    template cudaError_t launch_init<S>(const Params&, const double*, const double*, double, const double*, \
                                        const double*, cudaStream_t);                            \
    template cudaError_t launch_probe<S>(const Params&, int, int, int, double*, cudaStream_t);

}  // namespace lbm
