// vtk_io.cu - host code: the reference's legacy VTK field files (outputerVTK, postprocesors/outputerVTK.h:
// 26-823) and its probe CSV (outputerVTK::probeWriteOut, :824-851), so field dumps open in the same
// post-processing as the reference's; and the restart read of InitializationEquilibriumVariables
// (initializations/InitializationEquilibriumVariables.h:47-113).
//
// VTK layout (every writer of the reference): "# vtk DataFile Version 2.0", a title line, "ASCII",
// "DATASET STRUCTURED_POINTS", "DIMENSIONS nx ny nz", "ASPECT_RATIO" 1/res three times (float),
// "ORIGIN" bbmin - (additional - 0.5) / res per axis, "POINT_DATA N", then per field
// "SCALARS <name> double 1" + "LOOKUP_TABLE default" or "VECTORS <name> double", one line per point
// with x fastest.  The reference's fields are float and its constants float, printed through an
// ostream with the default 6 significant digits; values are rounded to float first here as well.
#include "../../include/lbm.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

namespace {
std::string g_vtk_err;

lbm_status vtk_fail(lbm_status s, const std::string& m) {
    g_vtk_err = m;
    return s;
}

// an ostream's default rendering of a float (precision 6, %g style)
int put_float(char* buf, size_t n, float v) { return std::snprintf(buf, n, "%.6g", (double)v); }
int put_double(char* buf, size_t n, double v) { return std::snprintf(buf, n, "%.6g", v); }

struct File {
    FILE* f = nullptr;
    std::string buf;
    explicit File(const char* path) : f(std::fopen(path, "w")) {}
    ~File() {
        if (f) std::fclose(f);
    }
    void flush() {
        if (!buf.empty()) std::fwrite(buf.data(), 1, buf.size(), f);
        buf.clear();
    }
    void add(const char* s, size_t n) {
        buf.append(s, n);
        if (buf.size() > (1u << 20)) flush();
    }
    void add(const std::string& s) { add(s.data(), s.size()); }
};
}  // namespace

extern "C" {

const char* lbm_vtk_last_error(void) { return g_vtk_err.c_str(); }

lbm_status lbm_vtk_write(const char* path, const char* title, const int32_t dims[3], double resolution,
                         double additional, const double bbmin[3], const lbm_vtk_field* fields, int32_t nfields) {
    if (!path || !dims || !bbmin || nfields < 0 || (nfields && !fields) || dims[0] <= 0 || dims[1] <= 0 ||
        dims[2] <= 0 || !(resolution > 0))
        return vtk_fail(LBM_ERR_INVALID, "lbm_vtk_write: bad argument");
    for (int i = 0; i < nfields; i++) {
        const lbm_vtk_field& fd = fields[i];
        if (!fd.name || !fd.data || (fd.components != 1 && fd.components != 3) || std::strchr(fd.name, ' ') ||
            std::strchr(fd.name, '\n'))
            return vtk_fail(LBM_ERR_INVALID, "lbm_vtk_write: field " + std::to_string(i) + " is malformed");
    }
    File out(path);
    if (!out.f) return vtk_fail(LBM_ERR_IO, std::string("cannot write ") + path);
    const long long N = (long long)dims[0] * dims[1] * dims[2];
    char num[64];
    const float res = (float)resolution, add = (float)additional;
    out.add("# vtk DataFile Version 2.0\n");
    out.add(std::string(title ? title : "LBE variables") + "\n");
    out.add("ASCII\nDATASET STRUCTURED_POINTS\n");
    out.add("DIMENSIONS " + std::to_string(dims[0]) + " " + std::to_string(dims[1]) + " " + std::to_string(dims[2]) +
            "\n");
    const float asp = 1.f / res;
    std::string line = "ASPECT_RATIO ";
    for (int a = 0; a < 3; a++) {
        int n = put_float(num, sizeof(num), asp);
        line.append(num, (size_t)n);
        line += a < 2 ? " " : "\n";
    }
    out.add(line);
    line = "ORIGIN ";
    for (int a = 0; a < 3; a++) {
        // float BBmin - (float additional - 0.5) / float res, evaluated in double as the reference's
        // expression promotes at the double literal
        const double o = (double)(float)bbmin[a] - ((double)add - 0.5) / (double)res;
        int n = put_double(num, sizeof(num), o);
        line.append(num, (size_t)n);
        line += a < 2 ? " " : "\n";
    }
    out.add(line);
    out.add("POINT_DATA " + std::to_string(N) + "\n");
    for (int i = 0; i < nfields; i++) {
        const lbm_vtk_field& fd = fields[i];
        const float sc = (float)fd.scale;
        if (fd.components == 1) {
            out.add(std::string("SCALARS ") + fd.name + " double 1\nLOOKUP_TABLE default\n");
            for (long long q = 0; q < N; q++) {
                int n = put_float(num, sizeof(num), (float)fd.data[q] * sc);
                num[n++] = '\n';
                out.add(num, (size_t)n);
            }
        } else {
            out.add(std::string("VECTORS ") + fd.name + " double\n");
            for (long long q = 0; q < N; q++) {
                int n = 0;
                for (int a = 0; a < 3; a++) {
                    n += put_float(num + n, sizeof(num) - (size_t)n, (float)fd.data[a * N + q] * sc);
                    num[n++] = a < 2 ? ' ' : '\n';
                }
                out.add(num, (size_t)n);
            }
        }
    }
    out.flush();
    if (std::ferror(out.f)) return vtk_fail(LBM_ERR_IO, std::string("writing ") + path + " failed");
    return LBM_OK;
}

lbm_status lbm_probe_csv_append(const char* path, double sampling_period, const double sample[4], double cu,
                                double crho, double cpressure) {
    if (!path || !sample) return vtk_fail(LBM_ERR_INVALID, "lbm_probe_csv_append: bad argument");
    FILE* probe = std::fopen(path, "r");
    const bool exists = probe != nullptr;
    if (probe) std::fclose(probe);
    FILE* f = std::fopen(path, "a");
    if (!f) return vtk_fail(LBM_ERR_IO, std::string("cannot append to ") + path);
    char num[64];
    std::string s;
    if (!exists) {
        int n = put_float(num, sizeof(num), (float)sampling_period);
        s += "Sampling frequency is: " + std::string(num, (size_t)n) + "\nux,uy,uz,rho,pressure\n";
    }
    // probeWriteOut multiplies float fields by float constants (:843-847); cs2 = 1/3 in float
    const float cs2 = 1.f / 3.f;
    auto mul = [](double a, double b) { return (float)((double)(float)a * (double)(float)b); };
    const float vals[5] = {mul(sample[0], cu), mul(sample[1], cu), mul(sample[2], cu), mul(sample[3], crho),
                           (float)sample[3] * cs2 * (float)cpressure};
    for (int i = 0; i < 5; i++) {
        int n = put_float(num, sizeof(num), vals[i]);
        s.append(num, (size_t)n);
        s += i < 4 ? "," : "\n";
    }
    const bool ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
    std::fclose(f);
    if (!ok) return vtk_fail(LBM_ERR_IO, std::string("appending to ") + path + " failed");
    return LBM_OK;
}

lbm_status lbm_vtk_read_variables(const char* path, const int32_t dims[3], double* rho, double* u) {
    if (!path || !dims || !rho || !u || dims[0] <= 0 || dims[1] <= 0 || dims[2] <= 0)
        return vtk_fail(LBM_ERR_INVALID, "lbm_vtk_read_variables: bad argument");
    std::ifstream in(path);
    if (!in.is_open()) return vtk_fail(LBM_ERR_IO, std::string("cannot open ") + path);
    const long long N = (long long)dims[0] * dims[1] * dims[2];
    std::string line;
    bool found = false;
    while (std::getline(in, line)) {
        if (line.compare(0, 10, "DIMENSIONS") == 0) {
            std::istringstream d(line.substr(10));
            long long a = 0, b = 0, c = 0;
            if (!(d >> a >> b >> c) || a != dims[0] || b != dims[1] || c != dims[2])
                return vtk_fail(LBM_ERR_INVALID, std::string(path) + ": " + line + " does not match the lattice");
        }
        if (line.find("LOOKUP_TABLE default") != std::string::npos) {
            found = true;
            break;
        }
    }
    if (!found) return vtk_fail(LBM_ERR_INVALID, std::string(path) + ": no LOOKUP_TABLE default line");
    // the reference reads into its float RealType (operator>> on float)
    float v = 0.f;
    for (long long q = 0; q < N; q++) {
        if (!(in >> v)) return vtk_fail(LBM_ERR_INVALID, std::string(path) + ": short density data");
        rho[q] = v;
    }
    found = false;
    while (std::getline(in, line))
        if (line.find("VECTORS U double") != std::string::npos) {
            found = true;
            break;
        }
    if (!found) return vtk_fail(LBM_ERR_INVALID, std::string(path) + ": no VECTORS U double line");
    float x = 0.f, y = 0.f, z = 0.f;
    for (long long q = 0; q < N; q++) {
        if (!(in >> x >> y >> z)) return vtk_fail(LBM_ERR_INVALID, std::string(path) + ": short velocity data");
        u[q] = x; u[N + q] = y; u[2 * N + q] = z;
    }
    return LBM_OK;
}

}  // extern "C"
