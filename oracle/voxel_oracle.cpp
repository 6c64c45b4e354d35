// voxel_oracle.cpp - CPU ORACLE of the reference OFF voxelizer.  TEST INFRASTRUCTURE ONLY.
//
// Restates 3D/preprocess/src/geometry/geometryMesherOFF.h:45-112 (grid dimensions and cell
// sampling) and 3D/preprocess/src/geometry/geometryHandlerOFF.h:63-182 (OFF reading, bounding
// box, point-in-polyhedron by the parity of distinct segment/triangle intersection points).
//
// The reference answers the segment query with CGAL (Simple_cartesian<double> AABB_tree,
// `all_intersections`, version not pinned in the reference; not vendored).  CGAL is absent here,
// so the query is restated from its published definition: a segment [p,q] meets a triangle when
// p and q are not strictly on the same side of the triangle's plane and the line pq passes
// through the closed triangle (signs of the three scalar triple products).  Only single-point
// results are kept (the reference drops non-point results with CGAL::assign, :162); a segment
// lying in a triangle's plane is therefore dropped as well.  Distinct points are those more than
// 1e-10 apart in squared length (:174).  Parity is pinned by the committed golden mesh matrix
// 3D/simulation/results/BackwardStepLaminar.txt (tests/golden/).
//
// The grid arithmetic follows the reference's types: LBMConstants holds float BB, resolution
// and additional factors (preprocess/src/data/LBMConstants.h:9-19) and the sample coordinates
// are float (`RealType lookx`, geometryMesherOFF.h:83), so both are rounded to float here.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace vox {

struct Mesh {
    std::vector<double> V;  // 3 per vertex
    std::vector<int> T;     // 3 per triangle
};

static bool next_data_line(std::istream& in, std::string& line) {
    while (std::getline(in, line)) {
        size_t h = line.find('#');
        if (h != std::string::npos) line = line.substr(0, h);
        bool blank = true;
        for (char ch : line) if (!std::isspace((unsigned char)ch)) { blank = false; break; }
        if (!blank) return true;
    }
    return false;
}

// OFF / NOFF / COFF reader; vertex lines may carry normals or colours, face lines trailing colours
static bool read_off(const char* path, Mesh& m) {
    std::ifstream in(path);
    if (!in) return false;
    std::string line;
    if (!next_data_line(in, line)) return false;
    std::istringstream hs(line);
    std::string head;
    hs >> head;
    if (head.find("OFF") == std::string::npos) return false;
    long nv = -1, nf = -1, ne = 0;
    if (!(hs >> nv >> nf >> ne)) {
        if (!next_data_line(in, line)) return false;
        std::istringstream cs(line);
        if (!(cs >> nv >> nf)) return false;
    }
    if (nv <= 0 || nf <= 0) return false;
    m.V.resize(3 * nv);
    for (long i = 0; i < nv; i++) {
        if (!next_data_line(in, line)) return false;
        std::istringstream vs(line);
        if (!(vs >> m.V[3 * i] >> m.V[3 * i + 1] >> m.V[3 * i + 2])) return false;
    }
    for (long f = 0; f < nf; f++) {
        if (!next_data_line(in, line)) return false;
        std::istringstream fs(line);
        int k;
        if (!(fs >> k) || k < 3) return false;
        std::vector<int> idx(k);
        for (int a = 0; a < k; a++) { if (!(fs >> idx[a])) return false; if (idx[a] < 0 || idx[a] >= nv) return false; }
        for (int a = 1; a + 1 < k; a++) { m.T.push_back(idx[0]); m.T.push_back(idx[a]); m.T.push_back(idx[a + 1]); }
    }
    return true;
}

static inline double triple(const double* a, const double* b, const double* c, const double* d) {
    // orientation of d w.r.t. plane (a,b,c): (b-a) x (c-a) . (d-a)
    double ux = b[0] - a[0], uy = b[1] - a[1], uz = b[2] - a[2];
    double vx = c[0] - a[0], vy = c[1] - a[1], vz = c[2] - a[2];
    double wx = d[0] - a[0], wy = d[1] - a[1], wz = d[2] - a[2];
    return ux * (vy * wz - vz * wy) - uy * (vx * wz - vz * wx) + uz * (vx * wy - vy * wx);
}
static inline int sgn(double x) { return (x > 0) - (x < 0); }

// single-point intersection of segment [p,q] with triangle (a,b,c); false if none or not a point
static bool seg_tri(const double* p, const double* q, const double* a, const double* b, const double* c,
                    double* out) {
    int sp = sgn(triple(a, b, c, p)), sq = sgn(triple(a, b, c, q));
    if (sp == sq) return false;  // both strictly on one side, or both in the plane (non-point result)
    // the line pq must pass through the closed triangle: the three edge orientations agree
    int s1 = sgn(triple(p, q, a, b)), s2 = sgn(triple(p, q, b, c)), s3 = sgn(triple(p, q, c, a));
    bool pos = s1 >= 0 && s2 >= 0 && s3 >= 0, neg = s1 <= 0 && s2 <= 0 && s3 <= 0;
    if (!(pos || neg)) return false;
    // line/plane intersection point
    double n[3] = {(b[1] - a[1]) * (c[2] - a[2]) - (b[2] - a[2]) * (c[1] - a[1]),
                   (b[2] - a[2]) * (c[0] - a[0]) - (b[0] - a[0]) * (c[2] - a[2]),
                   (b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0])};
    double dpq[3] = {q[0] - p[0], q[1] - p[1], q[2] - p[2]};
    double den = n[0] * dpq[0] + n[1] * dpq[1] + n[2] * dpq[2];
    if (den == 0) return false;
    double t = (n[0] * (a[0] - p[0]) + n[1] * (a[1] - p[1]) + n[2] * (a[2] - p[2])) / den;
    for (int k = 0; k < 3; k++) out[k] = p[k] + t * dpq[k];
    return true;
}

// geometryHandlerOFF::polyhedronInside, geometryHandlerOFF.h:135-182
static bool inside(const Mesh& m, const std::vector<double>& tb, const double* p, const double* o) {
    if (p[0] == o[0] && p[1] == o[1] && p[2] == o[2]) return false;
    double lo[3], hi[3];
    for (int k = 0; k < 3; k++) { lo[k] = std::min(p[k], o[k]); hi[k] = std::max(p[k], o[k]); }
    std::vector<double> pts;
    size_t nt = m.T.size() / 3;
    for (size_t t = 0; t < nt; t++) {
        const double* bb = &tb[6 * t];
        if (bb[0] > hi[0] || bb[3] < lo[0] || bb[1] > hi[1] || bb[4] < lo[1] || bb[2] > hi[2] || bb[5] < lo[2]) continue;
        double x[3];
        if (seg_tri(p, o, &m.V[3 * m.T[3 * t]], &m.V[3 * m.T[3 * t + 1]], &m.V[3 * m.T[3 * t + 2]], x))
            pts.insert(pts.end(), x, x + 3);
    }
    size_t np = pts.size() / 3;
    int ndist = 0;
    for (size_t i = 0; i < np; i++) {
        bool distinct = true;
        for (size_t j = 0; j < i; j++) {
            double dx = pts[3 * i] - pts[3 * j], dy = pts[3 * i + 1] - pts[3 * j + 1], dz = pts[3 * i + 2] - pts[3 * j + 2];
            distinct = (dx * dx + dy * dy + dz * dz) > 1e-10;
            if (!distinct) break;
        }
        if (distinct) ndist++;
    }
    return ndist % 2 == 1;
}

static int voxelize(const Mesh& m, double res, double add, const double* outside, int32_t* flags,
                    int32_t* dims, double* bbox) {
    size_t nv = m.V.size() / 3;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (size_t i = 0; i < nv; i++)
        for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], m.V[3 * i + k]); hi[k] = std::max(hi[k], m.V[3 * i + k]); }
    // LBMConstants stores BB, resolution and additional factor as float
    float blo[3], bhi[3], resf = (float)res, addf = (float)add;
    for (int k = 0; k < 3; k++) { blo[k] = (float)lo[k]; bhi[k] = (float)hi[k]; }
    for (int k = 0; k < 3; k++) dims[k] = (int32_t)std::ceil((bhi[k] - blo[k]) * resf + 2 * addf);  // :147-155
    if (bbox) for (int k = 0; k < 3; k++) { bbox[k] = blo[k]; bbox[3 + k] = bhi[k]; }
    if (!flags) return 0;
    size_t nt = m.T.size() / 3;
    std::vector<double> tb(6 * nt);
    for (size_t t = 0; t < nt; t++)
        for (int k = 0; k < 3; k++) {
            double a = m.V[3 * m.T[3 * t] + k], b = m.V[3 * m.T[3 * t + 1] + k], c = m.V[3 * m.T[3 * t + 2] + k];
            tb[6 * t + k] = std::min(a, std::min(b, c));
            tb[6 * t + 3 + k] = std::max(a, std::max(b, c));
        }
    int X = dims[0], Y = dims[1], Z = dims[2];
#pragma omp parallel for collapse(2) schedule(dynamic, 1)
    for (int k = 0; k < Z; k++)
        for (int j = 0; j < Y; j++)
            for (int i = 0; i < X; i++) {
                // sample point, geometryMesherOFF.h:94-96 (float `lookx`)
                float lx = (float)(((double)i + 0.5 - (double)addf) / (double)resf + (double)blo[0]);
                float ly = (float)(((double)j + 0.5 - (double)addf) / (double)resf + (double)blo[1]);
                float lz = (float)(((double)k + 0.5 - (double)addf) / (double)resf + (double)blo[2]);
                double p[3] = {lx, ly, lz};
                flags[(size_t)i + (size_t)X * ((size_t)j + (size_t)Y * k)] = inside(m, tb, p, outside) ? 1 : 0;
            }
    return 0;
}

}  // namespace vox

extern "C" {

// returns 0 on success, -7 if the file cannot be read; flags may be NULL to query dims/bbox
int orc_voxelize_off(const char* path, double res, double add, const double* outside, int32_t* flags,
                     int32_t* dims, double* bbox) {
    vox::Mesh m;
    if (!vox::read_off(path, m)) return -7;
    return vox::voxelize(m, res, add, outside, flags, dims, bbox);
}
int orc_voxelize_mesh(const double* verts, int nv, const int32_t* tris, int nt, double res, double add,
                      const double* outside, int32_t* flags, int32_t* dims, double* bbox) {
    vox::Mesh m;
    m.V.assign(verts, verts + 3 * (size_t)nv);
    m.T.assign(tris, tris + 3 * (size_t)nt);
    return vox::voxelize(m, res, add, outside, flags, dims, bbox);
}
int orc_read_off_counts(const char* path, int* nv, int* nt) {
    vox::Mesh m;
    if (!vox::read_off(path, m)) return -7;
    *nv = (int)(m.V.size() / 3); *nt = (int)(m.T.size() / 3);
    return 0;
}

}  // extern "C"
