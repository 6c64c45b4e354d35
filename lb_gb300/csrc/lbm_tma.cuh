// lbm_tma.cuh - row-staged step for rows of bulk fluid cells (FP32 and FP16-deviation storage).
//
// One CTA owns one x-row (y, z); each thread owns an x-pair of it.  In the AA pattern the 27 row
// segments a row reads in a step are exactly the 27 it writes: on an even step slot v of the row
// itself; on an odd step slot opp(v) of row (y - c_y, z - c_z), which receives f*_{opp v} of the
// same cells back.  No other CTA touches those segments in that step, so a CTA can
//   1. fetch the 27 segments into shared memory with cp.async.bulk (one thread issues them, an
//      mbarrier counts the bytes),
//   2. collide every pair from shared memory (addresses are compile-time offsets from one base),
//   3. write the post-collision values into the same shared segments (x-shifted on odd steps) and
//   4. store each segment back to where it came from with cp.async.bulk.
// x is periodic in these rows (a row of bulk cells has no x boundary), so the shifted element of
// an odd step that leaves [0, nx) wraps through a one-element halo on each side of the segment.
// Rows holding any other cell class run the per-pair path of k_step2 in a second launch over their list.
// Opt-in (LBM_OPT_ROW_STAGING): on a GB300 it issues fewer instructions per pair than k_step2 but stalls
// on the per-row CTA barriers, so the per-pair kernel stays the default.
#pragma once

#include "lbm_step.cuh"
#include "lbm_sync.cuh"

namespace lbm {

// ---- PTX: bulk copies (the mbarrier helpers are in lbm_sync.cuh) ------------------------------------
LBM_D void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// global -> shared, completion counted on the mbarrier (both addresses and the size 16-byte aligned)
LBM_D void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// shared -> global in the calling thread's bulk group
LBM_D void bulk_s2g(void* dst, const void* src, unsigned bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)), "r"(bytes)
                 : "memory");
}
LBM_D void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
LBM_D void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// velocity table for the copy-issuing thread (runtime direction index)
static __constant__ signed char kVel[27][3] = {
    {0, 0, 0},   {1, 0, 0},   {-1, 0, 0},  {0, 0, -1},  {0, 0, 1},   {0, -1, 0},  {0, 1, 0},
    {1, 0, -1},  {-1, 0, 1},  {1, 0, 1},   {-1, 0, -1}, {-1, -1, 0}, {1, 1, 0},   {0, 1, -1},
    {0, -1, 1},  {-1, 1, 0},  {1, -1, 0},  {0, 1, 1},   {0, -1, -1}, {-1, 1, -1}, {1, -1, 1},
    {-1, -1, 1}, {1, 1, -1},  {1, -1, -1}, {-1, 1, 1},  {-1, -1, -1}, {1, 1, 1}};


// halo of one 16-byte unit on each side of a shared segment (keeps the bulk copies aligned)
template <class S>
struct RowGeom {
    static constexpr int H = 16 / (int)sizeof(typename S::T);
};

// the direction a lane of warp 0 handles (lanes 0..26: V = lane), read once per kernel and kept
// packed in one register: V | (c_x+1) << 8 | (c_y+1) << 10 | (c_z+1) << 12
struct LaneDir {
    int code;
    LBM_D int V() const { return code & 31; }
    LBM_D int cx() const { return ((code >> 8) & 3) - 1; }
    LBM_D int cy() const { return ((code >> 10) & 3) - 1; }
    LBM_D int cz() const { return ((code >> 12) & 3) - 1; }
};
LBM_D LaneDir lane_dir() {
    const int V = threadIdx.x < 27 ? (int)threadIdx.x : 0;
    return LaneDir{V | (kVel[V][0] + 1) << 8 | (kVel[V][1] + 1) << 10 | (kVel[V][2] + 1) << 12};
}

// global segment V of row (y, z): slot V of the row itself on even steps, slot opp(V) of row
// (y - c_y, z - c_z) (periodic) on odd steps; the same segment is read and written back
template <class S, bool ODD>
LBM_D typename S::T* row_segment(const Params& p, const LaneDir& d, int y, int z) {
    using T = typename S::T;
    int slot = d.V(), yy = y, zz = z;
    if (ODD) {
        slot = opp(slot);
        yy = y - d.cy();
        zz = z - d.cz();
        if (yy < 0) yy += p.ny; else if (yy >= p.ny) yy -= p.ny;
        if (zz < 0) zz += p.nz; else if (zz >= p.nz) zz -= p.nz;
    }
    return (T*)p.f + (long long)slot * p.N + ((long long)zz * p.ny + yy) * p.nx;
}

// ---- one row from a shared stage -------------------------------------------------------------------------
// the stage holds the 27 segments of row (y, z) (fetched earlier); collide every pair of the row, write
// the results back into the stage, then store segment V from lane V of warp 0 (one bulk group per row)
template <class S, int COLL, int CLOS, bool ODD, int SW>
LBM_D void row_from_stage(const Params& p, typename S::T* buf, int y, int z, const PairCodec& k, const LaneDir& d) {
    using T = typename S::T;
    constexpr int H = RowGeom<S>::H;
    const int tid = threadIdx.x, nx = p.nx, x0 = 2 * tid;
    if (ODD) {  // periodic halo: x = -1 holds x = nx-1, x = nx holds x = 0
        if (tid < 27) {
            T* seg = buf + d.V() * SW + H;
            if (d.cx() > 0) seg[-1] = seg[nx - 1];
            else if (d.cx() < 0) seg[nx] = seg[0];
        }
        __syncthreads();
    }
    T* base = buf + H + x0;  // this pair's column in every segment
    F2 f[27];
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        constexpr int sh = ODD ? -cx(V) : 0;  // the cell x reads position x - c_x on odd steps
        const T* a = base + V * SW + sh;
        if constexpr (S::kind == 1) {
            if constexpr (sh != 0) f[V] = F2(a[0], a[1]);
            else f[V] = F2(*(const float2*)a);
        } else {
            float2 t;
            if constexpr (sh != 0) t = make_float2(__half2float(a[0]), __half2float(a[1]));
            else t = __half22float2(*(const __half2*)a);
            if constexpr (COLL == 1) f[V] = F2(t);  // moments from the deviations, as step_pair
            else f[V] = lfma(F2(t), k.inv_scale, k.wr[csq(V)]);
        }
    });
    const long long idx0 = ((long long)z * p.ny + y) * nx + x0;
    collide_pair<COLL, CLOS, S::kind == 2 && COLL == 1>(p, f, idx0);
    uint32_t rs = 0;  // stochastic-rounding stream of the pair, as store_pair
    if constexpr (S::kind == 2) rs = sr_seed_pair((uint32_t)idx0, p);
    __syncthreads();  // every pair has read its inputs before any segment is overwritten
    sfor<0, 27>([&](auto vc) {
        constexpr int V = decltype(vc)::value;
        constexpr int sh = ODD ? cx(V) : 0;  // f*_v goes to segment opp(v) at x + c_x (odd) or x (even)
        T* a = base + opp(V) * SW + sh;
        if constexpr (S::kind == 1) {
            if constexpr (sh != 0) { a[0] = f[V].v.x; a[1] = f[V].v.y; }
            else *(float2*)a = f[V].v;
        } else {
            const F2 e = lfma(f[V], k.scale, k.nwrs[csq(V)]);
            const __half2 h = half2_sr(e.v, rs + p.sr_off[V]);
            if constexpr (sh != 0) { a[0] = __low2half(h); a[1] = __high2half(h); }
            else *(__half2*)a = h;
        }
    });
    __syncthreads();
    if (ODD) {  // fold the halo writes back into the periodic row
        if (tid < 27) {
            // segment V received f*_{opp V} shifted by c_x(opp V) = -c_x(V)
            T* seg = buf + d.V() * SW + H;
            if (d.cx() < 0) seg[0] = seg[nx];
            else if (d.cx() > 0) seg[nx - 1] = seg[-1];
        }
        __syncthreads();
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid < 27) {
        bulk_s2g(row_segment<S, ODD>(p, d, y, z), buf + d.V() * SW + H, (unsigned)nx * sizeof(T));
        bulk_commit();
    }
}

// fetch the 27 segments of row (y, z) into a stage: lane 0 of warp 0 arms the barrier with the byte
// count, then lane V issues segment V (called by all of warp 0)
template <class S, bool ODD, int SW>
LBM_D void issue_row_load(const Params& p, typename S::T* buf, uint64_t* bar, int y, int z, const LaneDir& d) {
    constexpr int H = RowGeom<S>::H;
    const unsigned seg_bytes = (unsigned)p.nx * sizeof(typename S::T);
    if (threadIdx.x == 0) mbar_arrive_expect_tx(bar, 27u * seg_bytes);
    __syncwarp();
    if (threadIdx.x < 27) bulk_g2s(buf + d.V() * SW + H, row_segment<S, ODD>(p, d, y, z), seg_bytes, bar);
}

// Persistent CTAs over the list of bulk rows with a 3-stage pipeline: the fetch of row j+2 is issued
// as soon as row j has been stored, into the stage row j-1 used (whose bulk store must have finished
// reading shared memory: wait_group.read 1 in the lane that issued it), so every row's fetch overlaps
// two rows of compute.  SW: elements per shared segment (nx + 2H <= SW).
// Launch bounds: one thread per x-pair, at least 640 threads (20 warps) resident per SM.
constexpr int kStages = 3;
template <class S, int SW>
constexpr int row_threads() { return (SW - 2 * RowGeom<S>::H) / 2; }
template <class S, int COLL, int CLOS, bool ODD, int SW>
__global__ void __launch_bounds__(row_threads<S, SW>(), 640 / row_threads<S, SW>()) k_step_rows(Params p, const int32_t* rows, int nrows) {
    using T = typename S::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* stage = (T*)smem_raw;
    uint64_t* bars = (uint64_t*)(smem_raw + (size_t)kStages * 27 * SW * sizeof(T));
    const int tid = threadIdx.x;
    const int G = gridDim.x;
    const int nj = nrows > (int)blockIdx.x ? (nrows - (int)blockIdx.x + G - 1) / G : 0;
    if (nj == 0) return;
    auto row_of = [&](int j) { return rows[blockIdx.x + j * G]; };
    const LaneDir d = lane_dir();
    if (tid == 0) {
        for (int s = 0; s < kStages; s++) mbar_init(&bars[s], 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (tid < 32) {
        for (int j = 0; j < kStages - 1 && j < nj; j++) {
            const int r = row_of(j);
            issue_row_load<S, ODD, SW>(p, stage + (size_t)j * 27 * SW, &bars[j], r % p.ny, r / p.ny, d);
        }
    }
    PairCodec k;
    if constexpr (S::kind == 2) {
        k.inv_scale = F2(p.inv_scale);
        k.scale = F2(p.scale);
        k.wr[0] = F2(p.wr[0]); k.wr[1] = F2(p.wr[1]); k.wr[2] = F2(p.wr[7]); k.wr[3] = F2(p.wr[19]);
        k.nwrs[0] = F2(p.nwrs[0]); k.nwrs[1] = F2(p.nwrs[1]); k.nwrs[2] = F2(p.nwrs[7]); k.nwrs[3] = F2(p.nwrs[19]);
    }
    for (int j = 0; j < nj; j++) {
        const int s = j % kStages;
        const unsigned phase = (unsigned)(j / kStages) & 1u;
        T* buf = stage + (size_t)s * 27 * SW;
        bool ok = false;
        for (int it = 0; it < kWaitLimit && !ok; it++) ok = mbar_try_wait(&bars[s], phase);
        if (!__syncthreads_and(ok)) {
            // the copies did not land: report, give the fetches in flight one more bounded wait, stop
            if (tid == 0) {
                atomicExch(p.err, DEV_ERR_TMA_TIMEOUT);
                for (int q = j; q < j + kStages - 1 && q < nj; q++) {
                    bool done = false;
                    for (int it = 0; it < kWaitLimit && !done; it++)
                        done = mbar_try_wait(&bars[q % kStages], (unsigned)(q / kStages) & 1u);
                }
            }
            if (tid < 32) bulk_wait_all();
            return;
        }
        const int r = row_of(j);
        row_from_stage<S, COLL, CLOS, ODD, SW>(p, buf, r % p.ny, r / p.ny, k, d);
        if (tid < 32 && j + kStages - 1 < nj) {
            const int jn = j + kStages - 1, sn = jn % kStages;  // the stage row j-1 used
            asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
            const int rn = row_of(jn);
            issue_row_load<S, ODD, SW>(p, stage + (size_t)sn * 27 * SW, &bars[sn], rn % p.ny, rn / p.ny, d);
        }
    }
    if (tid < 32) bulk_wait_all();
}

// the rows that are not all bulk fluid: the per-pair path over a list of rows
template <class S, int COLL, int CLOS, bool ODD>
__global__ void __launch_bounds__(128) k_step_rowlist(Params p, const int32_t* rows) {
    const int x0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (x0 >= p.nx) return;
    const int r = rows[blockIdx.y];
    step_pair<S, COLL, CLOS, ODD>(p, x0, r % p.ny, r / p.ny);
}

}  // namespace lbm
