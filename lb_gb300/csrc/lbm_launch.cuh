// lbm_launch.cuh - definitions of the launchers; included by one .cu per storage type.
#pragma once

#include "lbm_aux.cuh"
#include "lbm_launch.h"
#include "lbm_step.cuh"
#include "lbm_step_mlp.cuh"
#include "lbm_tma.cuh"

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
        if constexpr (CLOS == 2) {
            // p.nut == nullptr: network every step; else mlp_run says whether it runs in this step
            if (!p.nut) {
                if (p.m & 1) k_step2_mlp<S, COLL, true, 0><<<g, b, 0, st>>>(p);
                else         k_step2_mlp<S, COLL, false, 0><<<g, b, 0, st>>>(p);
            } else if (p.mlp_run) {
                if (p.m & 1) k_step2_mlp<S, COLL, true, 1><<<g, b, 0, st>>>(p);
                else         k_step2_mlp<S, COLL, false, 1><<<g, b, 0, st>>>(p);
            } else {
                if (p.m & 1) k_step2_mlp<S, COLL, true, 2><<<g, b, 0, st>>>(p);
                else         k_step2_mlp<S, COLL, false, 2><<<g, b, 0, st>>>(p);
            }
        } else {
            if (p.m & 1) k_step2<S, COLL, CLOS, true><<<g, b, 0, st>>>(p);
            else         k_step2<S, COLL, CLOS, false><<<g, b, 0, st>>>(p);
        }
    }
    return cudaGetLastError();
}

// closure 2 (learned) runs on the packed path only: FP32 and FP16-deviation storage
template <class S>
cudaError_t launch_step(const Params& p, int collision, int closure, cudaStream_t st) {
    if (closure == 2) {
        if constexpr (S::kind == 0) return cudaErrorInvalidValue;
        else {
            if (collision >= 2) return cudaErrorInvalidValue;  // learned closure: SRT or cumulant-2015
            return collision == 0 ? step_parity<S, 0, 2>(p, st) : step_parity<S, 1, 2>(p, st);
        }
    }
    if (collision == 0) return closure == 0 ? step_parity<S, 0, 0>(p, st) : step_parity<S, 0, 1>(p, st);
    if (collision == 2) return closure == 0 ? step_parity<S, 2, 0>(p, st) : step_parity<S, 2, 1>(p, st);
    if (collision == 3) return closure == 0 ? step_parity<S, 3, 0>(p, st) : step_parity<S, 3, 1>(p, st);
    return closure == 0 ? step_parity<S, 1, 0>(p, st) : step_parity<S, 1, 1>(p, st);
}

// row-staged step (cumulant collision, FP16-deviation storage); SW = shared elements per segment
template <class S, int CLOS, int SW, bool ODD>
static cudaError_t rows_launch(const Params& p, const int32_t* bulk, int nbulk, cudaStream_t st) {
    const size_t smem = (size_t)kStages * 27 * SW * sizeof(typename S::T) + 64;
    static int grid_of[64] = {};  // persistent grid per device (0: not computed yet)
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 64) return cudaErrorInvalidDevice;
    const int threads = p.nx / 2;
    if (grid_of[dev] == 0) {
        cudaError_t e = cudaFuncSetAttribute(k_step_rows<S, 1, CLOS, ODD, SW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        int per_sm = 0, sms = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_rows<S, 1, CLOS, ODD, SW>, threads, smem);
        if (e != cudaSuccess) return e;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        grid_of[dev] = per_sm > 0 ? per_sm * sms : -1;
    }
    if (grid_of[dev] < 0) return cudaErrorInvalidConfiguration;
    const int g = grid_of[dev] < nbulk ? grid_of[dev] : nbulk;
    k_step_rows<S, 1, CLOS, ODD, SW><<<g, threads, smem, st>>>(p, bulk, nbulk);
    return cudaGetLastError();
}

template <class S, int CLOS, int SW>
static cudaError_t rows_parity(const Params& p, const int32_t* bulk, int nbulk, const int32_t* other, int nother,
                               cudaStream_t st) {
    const bool odd = (p.m & 1) != 0;
    if (nother > 0) {
        dim3 b = cell_block((p.nx + 1) / 2), g(((p.nx + 1) / 2 + b.x - 1) / b.x, nother);
        if (odd) k_step_rowlist<S, 1, CLOS, true><<<g, b, 0, st>>>(p, other);
        else     k_step_rowlist<S, 1, CLOS, false><<<g, b, 0, st>>>(p, other);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (nbulk > 0) return odd ? rows_launch<S, CLOS, SW, true>(p, bulk, nbulk, st) : rows_launch<S, CLOS, SW, false>(p, bulk, nbulk, st);
    return cudaSuccess;
}

template <class S>
cudaError_t launch_step_rows(const Params& p, int closure, const int32_t* bulk, int nbulk, const int32_t* other,
                             int nother, cudaStream_t st) {
    if constexpr (S::kind != 2) {
        return cudaErrorInvalidValue;
    } else {
        constexpr int H = RowGeom<S>::H;
        if (p.nx <= 256)
            return closure == 0 ? rows_parity<S, 0, 256 + 2 * H>(p, bulk, nbulk, other, nother, st)
                                : rows_parity<S, 1, 256 + 2 * H>(p, bulk, nbulk, other, nother, st);
        if (p.nx <= 512)
            return closure == 0 ? rows_parity<S, 0, 512 + 2 * H>(p, bulk, nbulk, other, nother, st)
                                : rows_parity<S, 1, 512 + 2 * H>(p, bulk, nbulk, other, nother, st);
        return closure == 0 ? rows_parity<S, 0, 1024 + 2 * H>(p, bulk, nbulk, other, nother, st)
                            : rows_parity<S, 1, 1024 + 2 * H>(p, bulk, nbulk, other, nother, st);
    }
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
    template cudaError_t launch_probe<S>(const Params&, int, int, int, double*, cudaStream_t);                  \
    template cudaError_t launch_step_rows<S>(const Params&, int, const int32_t*, int, const int32_t*, int, cudaStream_t);

}  // namespace lbm
