// mesh_io.cu - host code: the reference's mesh-matrix text files (outputerMesh::MeshMatrixOut and
// ::MeshMatrixIn, 3D/simulation/src/postprocesors/outputerMesh.h:19-211), so flag matrices pass
// between this library and the reference's toolchain unchanged.
//
// Format: "Dimensions: nx ny nz " then one line each for the resolution factor, the additional factor,
// BBmaxx/y/z and BBminx/y/z, written as the reference writes its float fields through an ostream
// (6 significant digits); then the values with x fastest, a space after every value, one line per
// (y, z) and an empty line after every z slice.
#include "../../include/lbm.h"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

namespace {
std::string g_io_err;

lbm_status io_fail(lbm_status s, const std::string& m) {
    g_io_err = m;
    return s;
}
}  // namespace

extern "C" {

const char* lbm_mesh_matrix_last_error(void) { return g_io_err.c_str(); }

lbm_status lbm_mesh_matrix_write(const char* path, const int32_t* flags, const int32_t dims[3], double resolution,
                                 double additional, const double bbox[6]) {
    if (!path || !flags || !dims || !bbox || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
        return io_fail(LBM_ERR_INVALID, "lbm_mesh_matrix_write: bad argument");
    std::ofstream out(path);
    if (!out.is_open()) return io_fail(LBM_ERR_IO, std::string("cannot write ") + path);
    // the reference's constants are float (LBMTraits.h:72), printed with the stream defaults
    auto f = [](double v) { return (float)v; };
    out << "Dimensions: " << dims[0] << " " << dims[1] << " " << dims[2] << " " << "\n";
    out << "Resolution Factor: " << f(resolution) << "\n";
    out << "Additional Factor: " << f(additional) << "\n";
    out << "BBmaxx: " << f(bbox[3]) << "\n";
    out << "BBmaxy: " << f(bbox[4]) << "\n";
    out << "BBmaxz: " << f(bbox[5]) << "\n";
    out << "BBminx: " << f(bbox[0]) << "\n";
    out << "BBminy: " << f(bbox[1]) << "\n";
    out << "BBminz: " << f(bbox[2]) << "\n";
    std::string row;
    char num[16];
    const size_t nx = (size_t)dims[0];
    for (int z = 0; z < dims[2]; ++z) {
        for (int y = 0; y < dims[1]; ++y) {
            row.clear();
            const int32_t* r = flags + nx * ((size_t)y + (size_t)dims[1] * z);
            for (size_t x = 0; x < nx; ++x) {
                const int n = std::snprintf(num, sizeof(num), "%d ", r[x]);
                row.append(num, (size_t)n);
            }
            row.push_back('\n');
            out << row;
        }
        out << "\n";
    }
    out.close();
    if (!out) return io_fail(LBM_ERR_IO, std::string("writing ") + path + " failed");
    return LBM_OK;
}

lbm_status lbm_mesh_matrix_read(const char* path, int32_t* flags, int64_t capacity, int32_t dims[3],
                                double* resolution, double* additional, double bbox[6]) {
    if (!path || !dims) return io_fail(LBM_ERR_INVALID, "lbm_mesh_matrix_read: bad argument");
    std::ifstream in(path);
    if (!in.is_open()) return io_fail(LBM_ERR_IO, std::string("cannot read ") + path);
    // header fields are found by keyword; the header ends with BBminz (outputerMesh.h:166-170)
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // resolution, additional, maxx, maxy, maxz, minx, miny, minz
    const char* keys[8] = {"Resolution Factor:", "Additional Factor:", "BBmaxx:", "BBmaxy:",
                           "BBmaxz:", "BBminx:", "BBminy:", "BBminz:"};
    int d[3] = {0, 0, 0};
    bool have_dims = false, done = false;
    std::string line;
    while (!done && std::getline(in, line)) {
        if (line.find("Dimensions:") != std::string::npos) {
            have_dims = std::sscanf(line.c_str() + line.find("Dimensions:") + 11, "%d %d %d", &d[0], &d[1], &d[2]) == 3;
            continue;
        }
        for (int k = 0; k < 8; k++) {
            const size_t at = line.find(keys[k]);
            if (at == std::string::npos) continue;
            std::sscanf(line.c_str() + at + std::strlen(keys[k]), "%lf", &v[k]);
            if (k == 7) done = true;
            break;
        }
    }
    if (!have_dims || !done || d[0] <= 0 || d[1] <= 0 || d[2] <= 0)
        return io_fail(LBM_ERR_IO, std::string(path) + ": not a mesh-matrix file (header)");
    for (int a = 0; a < 3; a++) dims[a] = d[a];
    if (resolution) *resolution = v[0];
    if (additional) *additional = v[1];
    if (bbox) {
        bbox[0] = v[5]; bbox[1] = v[6]; bbox[2] = v[7];
        bbox[3] = v[2]; bbox[4] = v[3]; bbox[5] = v[4];
    }
    if (!flags) return LBM_OK;
    const long long n = (long long)d[0] * d[1] * d[2];
    if (capacity < n) return io_fail(LBM_ERR_INVALID, "lbm_mesh_matrix_read: flags buffer too small");
    for (long long i = 0; i < n; i++) {
        int h;
        if (!(in >> h)) return io_fail(LBM_ERR_IO, std::string(path) + ": fewer values than nx*ny*nz");
        flags[i] = h;
    }
    return LBM_OK;
}

}  // extern "C"
