// voxelizer.cu - GPU point-in-polyhedron voxelizer for OFF meshes (C ABI in include/lbm.h).
//
// Replaces the reference preprocessor (3D/preprocess/src/geometry/geometryMesherOFF.h:45-112 with
// geometryHandlerOFF.h:63-182), which asks a CGAL AABB tree, cell by cell on one host thread, for
// the distinct intersection points of the segment [cell centre, outside point] and marks the cell
// inside when their number is odd.  Here every (y, z) column of cells casts a +x ray: the column
// collects the x of every triangle whose (y, z) projection contains it, and a cell is inside when an
// odd number of crossings lie before its x.  A CTA owns a 4 x 4 tile of columns and runs the exact
// test only on the triangles whose bounding box meets the tile (k_columns).  For a closed
// mesh and a cell not on the surface both counts have the same parity, so the flags agree with the
// reference; the grid (dimensions, float-rounded bounding box and sample points) follows the
// reference arithmetic exactly.  Ties (a column through an edge or a vertex of the projection) use
// a half-open rule on canonically ordered edges, so a shared edge is counted by exactly one of the
// triangles that cross there and by none or both at a silhouette; the reference instead merges
// coincident intersection points (|d|^2 <= 1e-10, geometryHandlerOFF.h:174).
#include "../../include/lbm.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

namespace {

bool next_data_line(std::istream& in, std::string& line) {
    while (std::getline(in, line)) {
        size_t h = line.find('#');
        if (h != std::string::npos) line.resize(h);
        if (line.find_first_not_of(" \t\r\n") != std::string::npos) return true;
    }
    return false;
}

// OFF / NOFF / COFF: header word containing "OFF", counts (same or next line), vertex lines whose
// first three numbers are the position, face lines "n i0 .. i(n-1) [colour]" (fan-triangulated)
bool read_off(const char* path, std::vector<double>& V, std::vector<int32_t>& T) {
    std::ifstream in(path);
    if (!in) return false;
    std::string line;
    if (!next_data_line(in, line)) return false;
    std::istringstream hs(line);
    std::string head;
    hs >> head;
    if (head.find("OFF") == std::string::npos) return false;
    long nv = -1, nf = -1;
    if (!(hs >> nv >> nf)) {
        if (!next_data_line(in, line)) return false;
        std::istringstream cs(line);
        if (!(cs >> nv >> nf)) return false;
    }
    if (nv <= 0 || nf <= 0) return false;
    V.resize(3 * (size_t)nv);
    for (long i = 0; i < nv; i++) {
        if (!next_data_line(in, line)) return false;
        std::istringstream vs(line);
        if (!(vs >> V[3 * i] >> V[3 * i + 1] >> V[3 * i + 2])) return false;
    }
    for (long f = 0; f < nf; f++) {
        if (!next_data_line(in, line)) return false;
        std::istringstream fs(line);
        int k;
        if (!(fs >> k) || k < 3) return false;
        std::vector<int32_t> idx(k);
        for (int a = 0; a < k; a++)
            if (!(fs >> idx[a]) || idx[a] < 0 || idx[a] >= nv) return false;
        for (int a = 1; a + 1 < k; a++) { T.push_back(idx[0]); T.push_back(idx[a]); T.push_back(idx[a + 1]); }
    }
    return true;
}

// prepared triangle: projected (y, z) vertices ordered counter-clockwise, x of each vertex
struct Tri {
    double y[3], z[3], x[3];
};

constexpr int kMaxCross = 256;  // crossings kept per column
constexpr int kTileJ = 4, kTileK = 4, kTileCols = kTileJ * kTileK;  // columns of one CTA (y x z)
constexpr int kVoxThreads = 256;
constexpr int kChunk = 2048;  // triangles filtered per pass of a CTA

// the (y, z) bounding box of a prepared triangle's projection in float, rounded outwards, so that a
// float sample point outside it is outside the exact box by at least one float step; NaN coordinates
// (triangles parallel to the rays) give NaN bounds, which no comparison passes
struct __align__(16) Box {
    float y0, y1, z0, z1;
};
__host__ __device__ inline float round_down(double v) {
    float f = (float)v;
#ifdef __CUDA_ARCH__
    if ((double)f > v) f = nextafterf(f, -INFINITY);
#else
    if ((double)f > v) f = std::nextafter(f, -INFINITY);
#endif
    return f;
}
__host__ __device__ inline float round_up(double v) {
    float f = (float)v;
#ifdef __CUDA_ARCH__
    if ((double)f < v) f = nextafterf(f, INFINITY);
#else
    if ((double)f < v) f = std::nextafter(f, INFINITY);
#endif
    return f;
}
__host__ __device__ inline Box box_of(const Tri& r) {
    const double y0 = fmin(r.y[0], fmin(r.y[1], r.y[2])), y1 = fmax(r.y[0], fmax(r.y[1], r.y[2]));
    const double z0 = fmin(r.z[0], fmin(r.z[1], r.z[2])), z1 = fmax(r.z[0], fmax(r.z[1], r.z[2]));
    return Box{round_down(y0), round_up(y1), round_down(z0), round_up(z1)};
}

// edge function of p against the edge (a -> b), evaluated on the canonically ordered endpoints so
// that the reversed edge gives exactly the negated value
__device__ __forceinline__ double edge_fn(double ay, double az, double by, double bz, double py, double pz,
                                          bool& incl) {
    bool swap = (ay > by) || (ay == by && az > bz);
    double sy = swap ? by : ay, sz = swap ? bz : az, ty = swap ? ay : by, tz = swap ? az : bz;
    double e = (ty - sy) * (pz - sz) - (tz - sz) * (py - sy);
    // half-open rule: a point on the edge belongs to the side the directed edge "includes";
    // d and -d never both include it
    double dy = by - ay, dz = bz - az;
    incl = (dz > 0) || (dz == 0 && dy > 0);
    return swap ? -e : e;
}

// x of the crossing of the +x ray through (py, pz) with triangle T, or NaN when the ray misses it
__device__ __forceinline__ double crossing(const Tri& T, double py, double pz) {
    bool i0, i1, i2;
    const double e0 = edge_fn(T.y[1], T.z[1], T.y[2], T.z[2], py, pz, i0);  // opposite vertex 0
    const double e1 = edge_fn(T.y[2], T.z[2], T.y[0], T.z[0], py, pz, i1);  // opposite vertex 1
    const double e2 = edge_fn(T.y[0], T.z[0], T.y[1], T.z[1], py, pz, i2);  // opposite vertex 2
    const bool in = (e0 > 0 || (e0 == 0 && i0)) && (e1 > 0 || (e1 == 0 && i1)) && (e2 > 0 || (e2 == 0 && i2));
    const double area = e0 + e1 + e2;
    if (!in || !(area > 0)) return NAN;
    return (e0 * T.x[0] + e1 * T.x[1] + e2 * T.x[2]) / area;
}

// One CTA per tile of kTileJ x kTileK (y, z) columns.  Per chunk of triangles, the CTA keeps those
// whose float box meets the tile's range of sample points (a conservative filter: the exact test can
// only accept a point inside the exact box), then tests every (candidate, column) pair whose sample
// lies in the candidate's box with the exact FP64 edge functions and appends the crossing x to the
// column's list in shared memory.  Last, one warp per column writes the cells: a cell is inside when
// an odd number of crossings lie before its x (the order of the list does not matter).
__global__ void __launch_bounds__(kVoxThreads) k_columns(const Tri* tris, const Box* boxes, int nt, const float* ys,
                                                         const float* zs, const float* xs, int nx, int ny, int nz,
                                                         int32_t* flags, int* overflow) {
    __shared__ double cross[kTileCols][kMaxCross];
    __shared__ int ncross[kTileCols];
    __shared__ int cand[kChunk];
    __shared__ int ncand;
    const int j0 = blockIdx.x * kTileJ, k0 = blockIdx.y * kTileK;
    const int j1 = min(j0 + kTileJ, ny) - 1, k1 = min(k0 + kTileK, nz) - 1;
    // sample coordinates increase with the index: the tile's samples lie in [ys[j0], ys[j1]] x [zs[k0], zs[k1]]
    const float ty0 = ys[j0], ty1 = ys[j1], tz0 = zs[k0], tz1 = zs[k1];
    if (threadIdx.x < kTileCols) ncross[threadIdx.x] = 0;
    for (int base = 0; base < nt; base += kChunk) {
        if (threadIdx.x == 0) ncand = 0;
        __syncthreads();
        const int cnt = min(kChunk, nt - base);
        for (int t = threadIdx.x; t < cnt; t += kVoxThreads) {
            const Box b = boxes[base + t];
            if (b.y0 <= ty1 && b.y1 >= ty0 && b.z0 <= tz1 && b.z1 >= tz0) cand[atomicAdd(&ncand, 1)] = base + t;
        }
        __syncthreads();
        const int nc = ncand;
        for (int w = threadIdx.x; w < nc * kTileCols; w += kVoxThreads) {
            const int c = w % kTileCols, ti = cand[w / kTileCols];
            const int j = j0 + c % kTileJ, k = k0 + c / kTileJ;
            if (j >= ny || k >= nz) continue;
            const float fy = ys[j], fz = zs[k];
            const Box b = boxes[ti];
            if (!(fy >= b.y0 && fy <= b.y1 && fz >= b.z0 && fz <= b.z1)) continue;
            const double xc = crossing(tris[ti], (double)fy, (double)fz);
            if (xc != xc) continue;
            const int slot = atomicAdd(&ncross[c], 1);
            if (slot < kMaxCross) cross[c][slot] = xc;
            else atomicExch(overflow, 1);
        }
        __syncthreads();  // the candidate list is refilled by the next chunk
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int c = warp; c < kTileCols; c += kVoxThreads / 32) {
        const int j = j0 + c % kTileJ, k = k0 + c / kTileJ;
        if (j >= ny || k >= nz) continue;
        const int n = min(ncross[c], kMaxCross);
        int32_t* row = flags + (size_t)nx * ((size_t)j + (size_t)ny * k);
        for (int i = lane; i < nx; i += 32) {
            const double px = xs[i];
            int q = 0;
            for (int a = 0; a < n; a++) q += cross[c][a] < px;
            row[i] = q & 1;
        }
    }
}

dim3 column_grid(int ny, int nz) { return dim3((ny + kTileJ - 1) / kTileJ, (nz + kTileK - 1) / kTileK); }

}  // namespace

extern "C" {

lbm_status lbm_voxelize_mesh(const double* verts, int32_t nv, const int32_t* tris, int32_t nt, double res, double add,
                             int32_t* flags_out, int32_t dims_out[3], double bbox_out[6], int32_t device) {
    if (!verts || !tris || nv <= 0 || nt <= 0 || !dims_out || !(res > 0) || add < 0) return LBM_ERR_INVALID;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < nv; i++)
        for (int a = 0; a < 3; a++) { lo[a] = std::min(lo[a], verts[3 * i + a]); hi[a] = std::max(hi[a], verts[3 * i + a]); }
    // the reference keeps BB, resolution and additional factor as float (LBMConstants.h:9-19)
    const float resf = (float)res, addf = (float)add;
    float blo[3], bhi[3];
    for (int a = 0; a < 3; a++) { blo[a] = (float)lo[a]; bhi[a] = (float)hi[a]; }
    for (int a = 0; a < 3; a++) dims_out[a] = (int32_t)std::ceil((bhi[a] - blo[a]) * resf + 2 * addf);
    if (bbox_out) for (int a = 0; a < 3; a++) { bbox_out[a] = blo[a]; bbox_out[3 + a] = bhi[a]; }
    if (!flags_out) return LBM_OK;
    const int nx = dims_out[0], ny = dims_out[1], nz = dims_out[2];
    if (nx <= 0 || ny <= 0 || nz <= 0) return LBM_ERR_INVALID;
    // sample coordinates (geometryMesherOFF.h:94-96, stored in float `lookx`)
    std::vector<float> s[3];
    for (int a = 0; a < 3; a++) {
        s[a].resize(dims_out[a]);
        for (int i = 0; i < dims_out[a]; i++)
            s[a][i] = (float)(((double)i + 0.5 - (double)addf) / (double)resf + (double)blo[a]);
    }
    // prepare triangles: drop index errors, orient projections counter-clockwise
    std::vector<Tri> T;
    std::vector<Box> B;
    T.reserve(nt);
    for (int t = 0; t < nt; t++) {
        int i0 = tris[3 * t], i1 = tris[3 * t + 1], i2 = tris[3 * t + 2];
        if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= nv || i1 >= nv || i2 >= nv) return LBM_ERR_INVALID;
        Tri r;
        int id[3] = {i0, i1, i2};
        for (int a = 0; a < 3; a++) { r.x[a] = verts[3 * id[a]]; r.y[a] = verts[3 * id[a] + 1]; r.z[a] = verts[3 * id[a] + 2]; }
        double ar = (r.y[1] - r.y[0]) * (r.z[2] - r.z[0]) - (r.z[1] - r.z[0]) * (r.y[2] - r.y[0]);
        if (ar == 0) continue;  // parallel to the rays: never crossed
        if (ar < 0) { std::swap(r.x[1], r.x[2]); std::swap(r.y[1], r.y[2]); std::swap(r.z[1], r.z[2]); }
        T.push_back(r);
        B.push_back(box_of(r));
    }
    if (cudaSetDevice(device) != cudaSuccess) return LBM_ERR_CUDA;
    Tri* dT = nullptr;
    Box* dB = nullptr;
    float *dy = nullptr, *dz = nullptr, *dx = nullptr;
    int32_t* dflags = nullptr;
    int* dovf = nullptr;
    const size_t ncell = (size_t)nx * ny * nz;
    lbm_status st = LBM_OK;
    if (cudaMalloc(&dT, std::max<size_t>(1, T.size()) * sizeof(Tri)) != cudaSuccess ||
        cudaMalloc(&dB, std::max<size_t>(1, B.size()) * sizeof(Box)) != cudaSuccess ||
        cudaMalloc(&dx, nx * 4) != cudaSuccess || cudaMalloc(&dy, ny * 4) != cudaSuccess ||
        cudaMalloc(&dz, nz * 4) != cudaSuccess || cudaMalloc(&dflags, ncell * 4) != cudaSuccess ||
        cudaMalloc(&dovf, 4) != cudaSuccess) {
        st = LBM_ERR_OOM;
    } else {
        cudaMemcpy(dT, T.data(), T.size() * sizeof(Tri), cudaMemcpyHostToDevice);
        cudaMemcpy(dB, B.data(), B.size() * sizeof(Box), cudaMemcpyHostToDevice);
        cudaMemcpy(dx, s[0].data(), nx * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dy, s[1].data(), ny * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dz, s[2].data(), nz * 4, cudaMemcpyHostToDevice);
        cudaMemset(dovf, 0, 4);
        k_columns<<<column_grid(ny, nz), kVoxThreads>>>(dT, dB, (int)T.size(), dy, dz, dx, nx, ny, nz, dflags, dovf);
        int ovf = 0;
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(&ovf, dovf, 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(flags_out, dflags, ncell * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = LBM_ERR_CUDA;
        else if (ovf)
            st = LBM_ERR_UNSUPPORTED;  // more than kMaxCross crossings on one column
    }
    cudaFree(dT); cudaFree(dB); cudaFree(dx); cudaFree(dy); cudaFree(dz); cudaFree(dflags); cudaFree(dovf);
    return st;
}

}  // extern "C"

// ---- allocation-free variant ------------------------------------------------------------------------
// Everything the column kernel needs besides the caller's output lives in one file-scope device
// array: the raw mesh copied from the host, the oriented triangle records, the sample coordinates
// and two status words.  Each process holds it once per device that loads this library.
namespace {

struct VoxScratch {
    double verts[3 * LBM_VOXELIZE_NOALLOC_MAX_VERTICES];
    int32_t tris[3 * LBM_VOXELIZE_NOALLOC_MAX_TRIANGLES];
    Tri prepared[LBM_VOXELIZE_NOALLOC_MAX_TRIANGLES];
    Box boxes[LBM_VOXELIZE_NOALLOC_MAX_TRIANGLES];
    float xs[LBM_VOXELIZE_NOALLOC_MAX_DIM], ys[LBM_VOXELIZE_NOALLOC_MAX_DIM], zs[LBM_VOXELIZE_NOALLOC_MAX_DIM];
    int overflow;   // a column met more crossings than the kernel keeps
    int bad_index;  // a triangle referenced a vertex outside [0, nv)
};

static __device__ __align__(256) unsigned char g_vox_scratch[sizeof(VoxScratch)];

constexpr int kMaxDevices = 64;
std::mutex g_vox_mutex;                      // one call at a time per process

// orient each triangle's (y, z) projection counter-clockwise, as the allocating path does on the
// host; a triangle parallel to the rays gets NaN coordinates so that no column ever meets it
__global__ void k_prepare(VoxScratch* s, int nv, int nt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const int id[3] = {s->tris[3 * t], s->tris[3 * t + 1], s->tris[3 * t + 2]};
    Tri r;
    for (int a = 0; a < 3; a++) {
        if (id[a] < 0 || id[a] >= nv) {
            s->bad_index = 1;
            for (int b = 0; b < 3; b++) r.x[b] = r.y[b] = r.z[b] = nan("");
            s->prepared[t] = r;
            s->boxes[t] = box_of(r);
            return;
        }
        r.x[a] = s->verts[3 * id[a]];
        r.y[a] = s->verts[3 * id[a] + 1];
        r.z[a] = s->verts[3 * id[a] + 2];
    }
    // the same products as the host path, without FMA contraction
    const double ar = __dsub_rn(__dmul_rn(__dsub_rn(r.y[1], r.y[0]), __dsub_rn(r.z[2], r.z[0])),
                                __dmul_rn(__dsub_rn(r.z[1], r.z[0]), __dsub_rn(r.y[2], r.y[0])));
    if (ar == 0) {
        for (int b = 0; b < 3; b++) r.y[b] = r.z[b] = nan("");
    } else if (ar < 0) {
        double tx = r.x[1], ty = r.y[1], tz = r.z[1];
        r.x[1] = r.x[2]; r.y[1] = r.y[2]; r.z[1] = r.z[2];
        r.x[2] = tx; r.y[2] = ty; r.z[2] = tz;
    }
    s->prepared[t] = r;
    s->boxes[t] = box_of(r);
}

// sample coordinates of geometryMesherOFF.h:94-96 (double arithmetic, stored as float)
__global__ void k_samples(VoxScratch* s, int nx, int ny, int nz, float resf, float addf, float bx, float by, float bz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nx) s->xs[i] = (float)__dadd_rn(__ddiv_rn(__dsub_rn((double)i + 0.5, (double)addf), (double)resf), (double)bx);
    if (i < ny) s->ys[i] = (float)__dadd_rn(__ddiv_rn(__dsub_rn((double)i + 0.5, (double)addf), (double)resf), (double)by);
    if (i < nz) s->zs[i] = (float)__dadd_rn(__ddiv_rn(__dsub_rn((double)i + 0.5, (double)addf), (double)resf), (double)bz);
}

}  // namespace

extern "C" {

lbm_status lbm_voxelize_mesh_noalloc(const double* verts, int32_t nv, const int32_t* tris, int32_t nt, double res,
                                     double add, int32_t* flags_out_device, int32_t dims_out[3], double bbox_out[6],
                                     int32_t device) {
    if (!verts || !tris || nv <= 0 || nt <= 0 || !dims_out || !(res > 0) || add < 0) return LBM_ERR_INVALID;
    if (nv > LBM_VOXELIZE_NOALLOC_MAX_VERTICES || nt > LBM_VOXELIZE_NOALLOC_MAX_TRIANGLES) return LBM_ERR_UNSUPPORTED;
    if (device < 0 || device >= kMaxDevices) return LBM_ERR_INVALID;
    // grid exactly as lbm_voxelize_mesh (float BB, resolution and additional factor)
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < nv; i++)
        for (int a = 0; a < 3; a++) { lo[a] = std::min(lo[a], verts[3 * i + a]); hi[a] = std::max(hi[a], verts[3 * i + a]); }
    const float resf = (float)res, addf = (float)add;
    float blo[3], bhi[3];
    for (int a = 0; a < 3; a++) { blo[a] = (float)lo[a]; bhi[a] = (float)hi[a]; }
    for (int a = 0; a < 3; a++) dims_out[a] = (int32_t)std::ceil((bhi[a] - blo[a]) * resf + 2 * addf);
    if (bbox_out) for (int a = 0; a < 3; a++) { bbox_out[a] = blo[a]; bbox_out[3 + a] = bhi[a]; }
    if (!flags_out_device) return LBM_OK;
    const int nx = dims_out[0], ny = dims_out[1], nz = dims_out[2];
    if (nx <= 0 || ny <= 0 || nz <= 0) return LBM_ERR_INVALID;
    if (nx > LBM_VOXELIZE_NOALLOC_MAX_DIM || ny > LBM_VOXELIZE_NOALLOC_MAX_DIM || nz > LBM_VOXELIZE_NOALLOC_MAX_DIM)
        return LBM_ERR_UNSUPPORTED;

    // every triangle index must name a vertex: checked here, before any device work, so a bad mesh
    // leaves the caller's buffer untouched (as lbm_voxelize_mesh does)
    for (long long i = 0; i < 3LL * nt; i++)
        if (tris[i] < 0 || tris[i] >= nv) return LBM_ERR_INVALID;

    std::lock_guard<std::mutex> lock(g_vox_mutex);
    if (cudaSetDevice(device) != cudaSuccess) return LBM_ERR_CUDA;
    // the scratch array's device address on this device, looked up on every call (a context torn
    // down with cudaDeviceReset reloads the module at a new address)
    void* sp = nullptr;
    if (cudaGetSymbolAddress(&sp, g_vox_scratch) != cudaSuccess || !sp) return LBM_ERR_CUDA;
    VoxScratch* s = (VoxScratch*)sp;
    // the status words start at zero; verts, tris, prepared and samples are overwritten for the
    // ranges this call reads
    if (cudaMemset(&s->overflow, 0, 2 * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(s->verts, verts, 3 * sizeof(double) * (size_t)nv, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(s->tris, tris, 3 * sizeof(int32_t) * (size_t)nt, cudaMemcpyHostToDevice) != cudaSuccess)
        return LBM_ERR_CUDA;
    const int bs = 128;
    k_prepare<<<(nt + bs - 1) / bs, bs>>>(s, nv, nt);
    const int nmax = std::max(nx, std::max(ny, nz));
    k_samples<<<(nmax + bs - 1) / bs, bs>>>(s, nx, ny, nz, resf, addf, blo[0], blo[1], blo[2]);
    k_columns<<<column_grid(ny, nz), kVoxThreads>>>(s->prepared, s->boxes, nt, s->ys, s->zs, s->xs, nx, ny, nz,
                                                    flags_out_device, &s->overflow);
    int status[2] = {0, 0};
    if (cudaGetLastError() != cudaSuccess || cudaMemcpy(status, &s->overflow, sizeof(status), cudaMemcpyDeviceToHost) != cudaSuccess)
        return LBM_ERR_CUDA;
    if (status[1]) return LBM_ERR_INVALID;      // a triangle index outside [0, nv)
    if (status[0]) return LBM_ERR_UNSUPPORTED;  // more than kMaxCross crossings on one column
    return LBM_OK;
}

lbm_status lbm_voxelize_off(const char* path, double res, double add, const double outside[3], int32_t* flags_out,
                            int32_t dims_out[3], double bbox_out[6], int32_t device) {
    (void)outside;
    if (!path || !dims_out) return LBM_ERR_INVALID;
    std::vector<double> V;
    std::vector<int32_t> T;
    if (!read_off(path, V, T)) return LBM_ERR_IO;
    return lbm_voxelize_mesh(V.data(), (int32_t)(V.size() / 3), T.data(), (int32_t)(T.size() / 3), res, add, flags_out,
                             dims_out, bbox_out, device);
}

}  // extern "C"
