// lbm_launch.h - host-side launchers of the device kernels, one set per storage type.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace lbm {

struct Params;
struct ReadOut;

// the step split by rows (FP32 and FP16-deviation storage): rows whose pairs all take the packed path
// (every cell bulk fluid of the packed path, the row off the periodic y/z seams, nx even) and the
// remaining rows; row r = y + ny z
struct RowLists {
    const int32_t* plain = nullptr;
    int n_plain = 0;
    const int32_t* other = nullptr;
    int n_other = 0;
    // rows beside a flat wall (every cell an edge cell with the same solid-source mask, `wall_solid`),
    // stepped by the packed wall kernel; closures without it take them with `other` (`other_all` lists
    // both)
    const int32_t* wall = nullptr;
    const uint32_t* wall_solid = nullptr;
    int n_wall = 0;
    const int32_t* other_all = nullptr;
    int n_other_all = 0;
    // the remaining rows run on `side`, forked from and joined back into the step's stream, so their
    // slow per-cell path overlaps the plain rows instead of trailing them (nullptr: same stream)
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

// returns cudaSuccess or the launch error; rl == nullptr: one launch over the lattice
template <class S>
cudaError_t launch_step(const Params& p, int collision, int closure, const RowLists* rl, cudaStream_t st);
template <class S, int COLL>
cudaError_t launch_step_coll(const Params& p, int closure, const RowLists* rl, cudaStream_t st);
template <class S>
cudaError_t launch_read(const Params& p, const ReadOut& o, cudaStream_t st);
template <class S>
cudaError_t launch_init(const Params& p, const double* rho, const double* u, double rho0, const double u0[3],
                        const double* pops, cudaStream_t st);

// row-staged step for rows of bulk cells (cumulant, FP16-deviation storage, periodic x, nx <= 1024):
// `bulk` lists the (y,z) rows whose cells are all bulk fluid, `other` the remaining rows
template <class S>
cudaError_t launch_step_rows(const Params& p, int closure, const int32_t* bulk, int nbulk, const int32_t* other,
                             int nother, cudaStream_t st);
template <class S>
cudaError_t launch_probe(const Params& p, int x, int y, int z, double* out, cudaStream_t st);

inline dim3 cell_block(int nx) {
    int b = nx >= 128 ? 128 : ((nx + 31) / 32) * 32;
    return dim3(b, 1, 1);
}
inline dim3 cell_grid(int nx, int ny, int nz) {
    dim3 b = cell_block(nx);
    return dim3((nx + b.x - 1) / b.x, ny, nz);
}

}  // namespace lbm
