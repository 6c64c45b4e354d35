// lbm_launch.cuh - definitions of the launchers; included by one .cu per storage type.
#pragma once

#include "lbm_aux.cuh"
#include "lbm_launch.h"
#include "lbm_step.cuh"
#include "lbm_step_mlp.cuh"
#include "lbm_tma.cuh"

namespace lbm {

using RowKernel = void (*)(Params, const int32_t*, int);

// grid of a row-list launch: x = blocks of 128 x-pairs per row, the n listed rows over y (at most
// 65535) and z
inline dim3 rows_grid(unsigned xb, int n) {
    const unsigned gy = n < 65535 ? (unsigned)n : 65535u;
    return dim3(xb, gy, ((unsigned)n + gy - 1u) / gy);
}

// the learned-closure kernel for this step's parity and network mode (p.nut == nullptr: the network
// runs every step; else p.mlp_run says whether it runs in this step)
template <class S, int COLL, int ROWS>
static RowKernel mlp_kernel(const Params& p) {
    const bool odd = (p.m & 1) != 0;
    if constexpr (ROWS == 1) {  // the plain rows: the network on tcgen05 when the option asks for it
        if (p.mlp_tc && !p.nut) return odd ? k_step2_mlp<S, COLL, true, 0, 1, true> : k_step2_mlp<S, COLL, false, 0, 1, true>;
        if (p.mlp_tc && p.mlp_run) return odd ? k_step2_mlp<S, COLL, true, 1, 1, true> : k_step2_mlp<S, COLL, false, 1, 1, true>;
    }
    if (!p.nut) return odd ? k_step2_mlp<S, COLL, true, 0, ROWS> : k_step2_mlp<S, COLL, false, 0, ROWS>;
    if (p.mlp_run) return odd ? k_step2_mlp<S, COLL, true, 1, ROWS> : k_step2_mlp<S, COLL, false, 1, ROWS>;
    // the plain rows between network steps: the plain-row kernel with the kept nu_t's rate
    if constexpr (ROWS == 1) return odd ? k_step2_plain<S, COLL, 2, true> : k_step2_plain<S, COLL, 2, false>;
    else return odd ? k_step2_mlp<S, COLL, true, 2, ROWS> : k_step2_mlp<S, COLL, false, 2, ROWS>;
}

template <class S, int COLL, int CLOS>
static cudaError_t step_parity(const Params& p, const RowLists* rl, cudaStream_t st) {
    const bool odd = (p.m & 1) != 0;
    if constexpr (S::kind == 0) {
        dim3 g = cell_grid(p.nx, p.ny, p.nz), b = cell_block(p.nx);
        if (odd) k_step<S, COLL, CLOS, true><<<g, b, 0, st>>>(p);
        else     k_step<S, COLL, CLOS, false><<<g, b, 0, st>>>(p);
    } else if (rl) {
        // split step: the wall rows and the remaining rows (side stream) and the plain rows, one thread
        // per x-pair
        const int half = (p.nx + 1) / 2;
        const dim3 b = cell_block(half);
        const unsigned xb = (unsigned)((half + (int)b.x - 1) / (int)b.x);
        // the packed wall kernel serves the collisions whose packed path is their own (not the combined
        // one, which packs reference-flag-1 cells only); with the learned closure (CLOS 2) it runs the
        // Smagorinsky closure, the rate the learned closure gives every cell off the bulk pairs
        constexpr bool WALL = COLL != 3;
        constexpr int WCLOS = CLOS == 2 ? 1 : CLOS;
        const int32_t* other = WALL ? rl->other : rl->other_all;
        const int n_other = WALL ? rl->n_other : rl->n_other_all;
        const int n_wall = WALL ? rl->n_wall : 0;
        RowKernel kp, ko;
        if constexpr (CLOS == 2) {
            kp = mlp_kernel<S, COLL, 1>(p);
            ko = mlp_kernel<S, COLL, 2>(p);
        } else {
            kp = odd ? k_step2_plain<S, COLL, CLOS, true> : k_step2_plain<S, COLL, CLOS, false>;
            ko = odd ? k_step2_list<S, COLL, CLOS, true> : k_step2_list<S, COLL, CLOS, false>;
        }
        const bool fork = rl->side && (n_other > 0 || n_wall > 0) && rl->n_plain > 0;
        cudaStream_t so = fork ? rl->side : st;
        if (fork) {
            cudaError_t e = cudaEventRecord(rl->fork, st);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(rl->side, rl->fork, 0);
            if (e != cudaSuccess) return e;
        }
        if (n_other > 0) {
            ko<<<rows_grid(xb, n_other), b, 0, so>>>(p, other, n_other);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
        if constexpr (WALL) {
            if (n_wall > 0) {
                if (odd) k_step2_wall<S, COLL, WCLOS, true><<<rows_grid(xb, n_wall), b, 0, so>>>(p, rl->wall, rl->wall_solid, n_wall);
                else     k_step2_wall<S, COLL, WCLOS, false><<<rows_grid(xb, n_wall), b, 0, so>>>(p, rl->wall, rl->wall_solid, n_wall);
                cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) return e;
            }
        }
        if (rl->n_plain > 0) kp<<<rows_grid(xb, rl->n_plain), b, 0, st>>>(p, rl->plain, rl->n_plain);
        if (fork) {
            cudaError_t e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaEventRecord(rl->join, rl->side);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(st, rl->join, 0);
            if (e != cudaSuccess) return e;
        }
    } else {
        const int half = (p.nx + 1) / 2;  // one thread per x-pair
        dim3 g = cell_grid(half, p.ny, p.nz), b = cell_block(half);
        if constexpr (CLOS == 2) {
            mlp_kernel<S, COLL, 0>(p)<<<g, b, 0, st>>>(p, nullptr, 0);
        } else {
            if (odd) k_step2<S, COLL, CLOS, true><<<g, b, 0, st>>>(p);
            else     k_step2<S, COLL, CLOS, false><<<g, b, 0, st>>>(p);
        }
    }
    return cudaGetLastError();
}

// one collision's step (instantiated per storage and collision in lbm_step_<storage>_<collision>.cu, so
// the step kernels compile in parallel); closure 2 (learned) runs on the packed path only (FP32 and
// FP16-deviation storage, SRT or cumulant-2015)
template <class S, int COLL>
cudaError_t launch_step_coll(const Params& p, int closure, const RowLists* rl, cudaStream_t st) {
    if (closure == 2) {
        if constexpr (S::kind == 0 || COLL >= 2) return cudaErrorInvalidValue;
        else return step_parity<S, COLL, 2>(p, rl, st);
    }
    return closure == 0 ? step_parity<S, COLL, 0>(p, rl, st) : step_parity<S, COLL, 1>(p, rl, st);
}

template <class S>
cudaError_t launch_step(const Params& p, int collision, int closure, const RowLists* rl, cudaStream_t st) {
    switch (collision) {
        case 0: return launch_step_coll<S, 0>(p, closure, rl, st);
        case 2: return launch_step_coll<S, 2>(p, closure, rl, st);
        case 3: return launch_step_coll<S, 3>(p, closure, rl, st);
        default: return launch_step_coll<S, 1>(p, closure, rl, st);
    }
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
    const dim3 g = read_grid(p.nx, p.ny, p.nz), b((unsigned)read_block(p.nx));
    if (p.m & 1) k_read<S, true><<<g, b, 0, st>>>(p, o);
    else         k_read<S, false><<<g, b, 0, st>>>(p, o);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !(o.mode & (READ_DIAG | READ_ERROR))) return e;
    const int q0 = (o.mode & READ_DIAG) ? RED_MASS : RED_ERR1, q1 = (o.mode & READ_ERROR) ? RED_COUNT : RED_ERR1;
    k_read_final<S><<<q1 - q0, kFinalThreads, 0, st>>>(o.part, (long long)g.x * g.y * g.z, q0, o.red);
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

// the launchers of one storage type except the step kernels (their collisions are compiled in their own
// units: LBM_INSTANTIATE_COLL)
#define LBM_INSTANTIATE(S)                                                                              \
    extern template cudaError_t launch_step_coll<S, 0>(const Params&, int, const RowLists*, cudaStream_t); \
    extern template cudaError_t launch_step_coll<S, 1>(const Params&, int, const RowLists*, cudaStream_t); \
    extern template cudaError_t launch_step_coll<S, 2>(const Params&, int, const RowLists*, cudaStream_t); \
    extern template cudaError_t launch_step_coll<S, 3>(const Params&, int, const RowLists*, cudaStream_t); \
    template cudaError_t launch_step<S>(const Params&, int, int, const RowLists*, cudaStream_t);        \
    template cudaError_t launch_read<S>(const Params&, const ReadOut&, cudaStream_t);                   \
    template cudaError_t launch_init<S>(const Params&, const double*, const double*, double, const double*, \
                                        const double*, cudaStream_t);                                   \
    template cudaError_t launch_probe<S>(const Params&, int, int, int, double*, cudaStream_t);          \
    template cudaError_t launch_step_rows<S>(const Params&, int, const int32_t*, int, const int32_t*, int, cudaStream_t);
#define LBM_INSTANTIATE_COLL(S, C) \
    template cudaError_t launch_step_coll<S, C>(const Params&, int, const RowLists*, cudaStream_t);

}  // namespace lbm
