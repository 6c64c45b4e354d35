// mesher.cu - host code: the cuboid boundary passes of the reference's geometry mesher
// (geometryMesherBoundary::meshingBoundaryCondition*, 3D/simulation/src/geometry/geometryMesherBoundary.h:
// 47-437, with geometryObjectCuboid::isInside, geometryObjectCuboid.h:20-38), so a case built the way the
// reference's main.cu builds one gives the same flag field and boundary records.
//
// Arithmetic as the reference's: the look coordinate (i + 0.5 - additional) / resolution + bbmin is formed
// in double from float constants; the inlet passes keep it in a float (RealType) variable, the others in
// a double; cuboid corners are doubles.  The reference's neighboursFluidSearch always returns true
// (geometryMesherBoundary.h:621-656), so the inlet pass has no neighbour test.
#include "../../include/lbm.h"

#include <cmath>
#include <string>
#include <vector>

namespace {
std::string g_mesher_err;

lbm_status mfail(lbm_status s, const std::string& m) {
    g_mesher_err = m;
    return s;
}

bool inside(const lbm_cuboid& c, const double p[3]) {
    for (int a = 0; a < 3; a++) {
        const double lo = std::fmin(c.x1[a], std::fmin(c.x2[a], c.x3[a]));
        const double hi = std::fmax(c.x1[a], std::fmax(c.x2[a], c.x3[a]));
        if (!(p[a] >= lo && p[a] <= hi)) return false;
    }
    return true;
}

double look(const lbm_mesh_frame& f, int i, int a) {
    return ((double)i + 0.5 - (double)f.additional_factor) / (double)f.resolution_factor + (double)f.bbmin[a];
}

// the centre of cell (i, j, k); as float-rounded coordinates for the inlet passes
void centre(const lbm_mesh_frame& f, int i, int j, int k, bool as_float, double p[3]) {
    const int ijk[3] = {i, j, k};
    for (int a = 0; a < 3; a++) p[a] = as_float ? (double)(float)look(f, ijk[a], a) : look(f, ijk[a], a);
}

lbm_status check_args(const lbm_mesh_frame* f, const int32_t* flags, const lbm_cuboid* c, const void* rec,
                      int64_t cap, const int64_t* n, const char* who) {
    if (!f || !flags || !c || !n || (cap > 0 && !rec) || *n < 0 || *n > cap || f->dims[0] <= 0 || f->dims[1] <= 0 ||
        f->dims[2] <= 0 || !(f->resolution_factor > 0))
        return mfail(LBM_ERR_INVALID, std::string(who) + ": bad argument");
    return LBM_OK;
}

// cells the pass takes (flag > 0 for inlets, != 0 otherwise) in the reference's k, j, i loop order
std::vector<long long> take(const lbm_mesh_frame& f, const int32_t* flags, const lbm_cuboid& c, bool inlet) {
    std::vector<long long> out;
    double p[3];
    for (int k = 0; k < f.dims[2]; k++)
        for (int j = 0; j < f.dims[1]; j++)
            for (int i = 0; i < f.dims[0]; i++) {
                const long long q = ((long long)k * f.dims[1] + j) * f.dims[0] + i;
                const int32_t fl = flags[q];
                if (inlet ? fl <= 0 : fl == 0) continue;
                centre(f, i, j, k, inlet, p);
                if (inside(c, p)) out.push_back(q);
            }
    return out;
}

lbm_vertex vertex_of(const lbm_mesh_frame& f, long long q) {
    lbm_vertex v;
    v.x = (int32_t)(q % f.dims[0]);
    v.y = (int32_t)((q / f.dims[0]) % f.dims[1]);
    v.z = (int32_t)(q / ((long long)f.dims[0] * f.dims[1]));
    return v;
}

lbm_status inlet_pass(const lbm_mesh_frame* f, int32_t* flags, const lbm_cuboid* c, const float normal[3],
                      const float velocity[3], lbm_bc_inlet* rec, int64_t cap, int64_t* n, const char* who) {
    const std::vector<long long> cells = take(*f, flags, *c, true);
    if ((int64_t)cells.size() > cap - *n)
        return mfail(LBM_ERR_INVALID, std::string(who) + ": " + std::to_string(cells.size()) +
                                          " inlet records do not fit");
    for (long long q : cells) {
        lbm_bc_inlet& r = rec[(*n)++];
        r.vertex = vertex_of(*f, q);
        for (int a = 0; a < 3; a++) { r.normal[a] = normal[a]; r.velocity[a] = velocity[a]; }
        r.regular = flags[q] > 10 ? 0 : 1;
        flags[q] = c->id;
    }
    return LBM_OK;
}

template <class Rec, class Fill>
lbm_status plain_pass(const lbm_mesh_frame* f, int32_t* flags, const lbm_cuboid* c, Rec* rec, int64_t cap, int64_t* n,
                      const char* who, Fill fill) {
    lbm_status s = check_args(f, flags, c, rec, cap, n, who);
    if (s) return s;
    const std::vector<long long> cells = take(*f, flags, *c, false);
    if ((int64_t)cells.size() > cap - *n)
        return mfail(LBM_ERR_INVALID, std::string(who) + ": " + std::to_string(cells.size()) + " records do not fit");
    for (long long q : cells) {
        Rec& r = rec[(*n)++];
        r.vertex = vertex_of(*f, q);
        fill(r);
        r.regular = flags[q] == 10 ? 1 : 0;
        flags[q] = c->id;
    }
    return LBM_OK;
}
}  // namespace

extern "C" {

const char* lbm_mesher_last_error(void) { return g_mesher_err.c_str(); }

lbm_status lbm_mesher_inlet_uniform(const lbm_mesh_frame* frame, int32_t* flags, const lbm_cuboid* cuboid,
                                    const float normal[3], const float velocity[3], lbm_bc_inlet* records,
                                    int64_t capacity, int64_t* n) {
    lbm_status s = check_args(frame, flags, cuboid, records, capacity, n, "lbm_mesher_inlet_uniform");
    if (s) return s;
    if (!normal || !velocity) return mfail(LBM_ERR_INVALID, "lbm_mesher_inlet_uniform: bad argument");
    if (velocity[0] == velocity[1] && velocity[0] == velocity[2])
        return mfail(LBM_ERR_INVALID, "Expected a 3D vector for velocity_in (three equal components)");
    return inlet_pass(frame, flags, cuboid, normal, velocity, records, capacity, n, "lbm_mesher_inlet_uniform");
}

lbm_status lbm_mesher_inlet_paraboloid_circle(const lbm_mesh_frame* frame, int32_t* flags, const lbm_cuboid* cuboid,
                                              const double center[3], float radius, const float normal[3],
                                              float mean_velocity, lbm_bc_inlet* records, int64_t capacity,
                                              int64_t* n) {
    const char* who = "lbm_mesher_inlet_paraboloid_circle";
    lbm_status s = check_args(frame, flags, cuboid, records, capacity, n, who);
    if (s) return s;
    if (!center || !normal || !(radius > 0)) return mfail(LBM_ERR_INVALID, std::string(who) + ": bad argument");
    const float zero[3] = {0.f, 0.f, 0.f};
    s = inlet_pass(frame, flags, cuboid, normal, zero, records, capacity, n, who);
    if (s) return s;
    for (int64_t e = 0; e < *n; e++) {
        lbm_bc_inlet& r = records[e];
        double p[3];
        centre(*frame, r.vertex.x, r.vertex.y, r.vertex.z, true, p);
        if (!inside(*cuboid, p)) continue;
        const float d = (float)std::sqrt(std::pow(p[0] - center[0], 2) + std::pow(p[1] - center[1], 2) +
                                         std::pow(p[2] - center[2], 2));
        if (!(d <= radius)) continue;
        // 3 * mean (float) times (1.0 - pow(d / radius, 2)) in double, stored as float
        float v = (float)((double)(3 * mean_velocity) * (1.0 - std::pow((double)(d / radius), 2)));
        if (v < 0) v = 0;
        for (int a = 0; a < 3; a++) r.velocity[a] = -v * normal[a];
    }
    return LBM_OK;
}

lbm_status lbm_mesher_inlet_paraboloid_rectangle(const lbm_mesh_frame* frame, int32_t* flags,
                                                 const lbm_cuboid* cuboid, const double center[3],
                                                 float inlet_dims[3], const float normal[3], float mean_velocity,
                                                 lbm_bc_inlet* records, int64_t capacity, int64_t* n) {
    const char* who = "lbm_mesher_inlet_paraboloid_rectangle";
    lbm_status s = check_args(frame, flags, cuboid, records, capacity, n, who);
    if (s) return s;
    if (!center || !normal || !inlet_dims) return mfail(LBM_ERR_INVALID, std::string(who) + ": bad argument");
    const float zero[3] = {0.f, 0.f, 0.f};
    s = inlet_pass(frame, flags, cuboid, normal, zero, records, capacity, n, who);
    if (s) return s;
    for (int64_t e = 0; e < *n; e++) {
        lbm_bc_inlet& r = records[e];
        double p[3];
        centre(*frame, r.vertex.x, r.vertex.y, r.vertex.z, true, p);
        if (!inside(*cuboid, p)) continue;
        float part[3];
        for (int a = 0; a < 3; a++) {
            // distance from the face's low corner: float look - (double centre - float D / 2), stored as float
            const float dist = (float)(p[a] - (center[a] - (double)(inlet_dims[a] / 2)));
            if (normal[a] == 0) {
                part[a] = dist * (inlet_dims[a] - dist);
            } else {
                part[a] = 1.f;
                inlet_dims[a] = 1.f;
            }
        }
        const float D = inlet_dims[0] * inlet_dims[1] * inlet_dims[2] * inlet_dims[0] * inlet_dims[1] * inlet_dims[2];
        const float k = D / 16;
        float v = 2 * mean_velocity * part[0] * part[1] * part[2] / k;
        if (v < 0) v = 0;
        for (int a = 0; a < 3; a++) r.velocity[a] = -v * normal[a];
    }
    return LBM_OK;
}

lbm_status lbm_mesher_outlet(const lbm_mesh_frame* frame, int32_t* flags, const lbm_cuboid* cuboid,
                             const float normal[3], float density, lbm_bc_outlet* records, int64_t capacity,
                             int64_t* n) {
    if (!normal) return mfail(LBM_ERR_INVALID, "lbm_mesher_outlet: bad argument");
    return plain_pass(frame, flags, cuboid, records, capacity, n, "lbm_mesher_outlet", [&](lbm_bc_outlet& r) {
        for (int a = 0; a < 3; a++) r.normal[a] = normal[a];
        r.density = density;
    });
}

lbm_status lbm_mesher_symmetry(const lbm_mesh_frame* frame, int32_t* flags, const lbm_cuboid* cuboid,
                               const float normal[3], lbm_bc_symmetry* records, int64_t capacity, int64_t* n) {
    if (!normal) return mfail(LBM_ERR_INVALID, "lbm_mesher_symmetry: bad argument");
    return plain_pass(frame, flags, cuboid, records, capacity, n, "lbm_mesher_symmetry", [&](lbm_bc_symmetry& r) {
        for (int a = 0; a < 3; a++) r.normal[a] = normal[a];
    });
}

lbm_status lbm_mesher_periodic(const lbm_mesh_frame* frame, int32_t* flags, const lbm_cuboid* cuboid,
                               const float normal[3], int32_t periodic_index, lbm_bc_periodic* records,
                               int64_t capacity, int64_t* n) {
    if (!normal) return mfail(LBM_ERR_INVALID, "lbm_mesher_periodic: bad argument");
    return plain_pass(frame, flags, cuboid, records, capacity, n, "lbm_mesher_periodic", [&](lbm_bc_periodic& r) {
        for (int a = 0; a < 3; a++) r.normal[a] = normal[a];
        r.periodic_index = periodic_index;
    });
}

}  // extern "C"
