// config_io.cu - host code: lbm_config defaults and the key = value case file.  The reference has no
// configuration file (its cases are set by assigning LBMConstants fields in main.cu:84-165 and choosing
// policy typedefs, main.cu:37-52); the names accepted here are those policy names and the field names
// of lbm_config, so a case reads like the reference's main.cu set-up.
#include "../../include/lbm.h"

#include <cerrno>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

namespace {
std::string g_cfg_err;

struct Name {
    const char* name;
    int32_t code;
};
const Name kCollision[] = {{"srt", LBM_COLLISION_SRT},
                           {"CollisionSRTTurbulent", LBM_COLLISION_SRT},
                           {"CollisionSRTLaminar", LBM_COLLISION_SRT},
                           {"CollisionSRTunroll", LBM_COLLISION_SRT},
                           {"cumulant2015", LBM_COLLISION_CUMULANT2015},
                           {"CollisionCumD3Q27Turbulent2015", LBM_COLLISION_CUMULANT2015},
                           {"CollisionCumD3Q27Laminar", LBM_COLLISION_CUMULANT2015},
                           {"cumulant2017", LBM_COLLISION_CUMULANT2017},
                           {"CollisionCumD3Q27Turbulent2017", LBM_COLLISION_CUMULANT2017},
                           {"combined", LBM_COLLISION_CUMULANT_COMBINED},
                           {"CollisionCumD3Q27TurbulentCombined", LBM_COLLISION_CUMULANT_COMBINED}};
const Name kClosure[] = {{"none", LBM_CLOSURE_NONE},
                         {"OmegaNo", LBM_CLOSURE_NONE},
                         {"smagorinsky", LBM_CLOSURE_SMAGORINSKY},
                         {"OmegaLES", LBM_CLOSURE_SMAGORINSKY},
                         {"mlp", LBM_CLOSURE_MLP},
                         {"OmegaMLP", LBM_CLOSURE_MLP}};
const Name kStorage[] = {{"f64", LBM_STORAGE_F64}, {"f32", LBM_STORAGE_F32}, {"f16dev", LBM_STORAGE_F16DEV}};
const Name kInlet[] = {{"moving_wall", LBM_INLET_MOVING_WALL},
                       {"InletVelocityMovingWall", LBM_INLET_MOVING_WALL},
                       {"equilibrium", LBM_INLET_EQUILIBRIUM},
                       {"InletVelocityEquilibrium", LBM_INLET_EQUILIBRIUM},
                       {"zou_he", LBM_INLET_ZOU_HE},
                       {"InletVelocityZouHe", LBM_INLET_ZOU_HE}};
const Name kOutlet[] = {{"density_interpolated", LBM_OUTLET_DENSITY_INTERPOLATED},
                        {"OutletDensityInterpolated", LBM_OUTLET_DENSITY_INTERPOLATED},
                        {"neighbour_equilibrium", LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM},
                        {"OutletNeighbourEquilibrium", LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM},
                        {"neighbour_equilibrium_omega", LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA},
                        {"OutletNeighbourEquilibriumOmega", LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA},
                        {"neighbour_equilibrium_omega_rf", LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF},
                        {"OutletNeighbourEquilibriumOmegaRF", LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF},
                        {"density_equilibrium", LBM_OUTLET_DENSITY_EQUILIBRIUM},
                        {"OutletDensityEquilibrium", LBM_OUTLET_DENSITY_EQUILIBRIUM}};

bool to_int(const std::string& t, int32_t& v) {
    errno = 0;
    char* end = nullptr;
    const long x = std::strtol(t.c_str(), &end, 10);
    if (errno || end == t.c_str() || *end || x < INT32_MIN || x > INT32_MAX) return false;
    v = (int32_t)x;
    return true;
}
bool to_double(const std::string& t, double& v) {
    errno = 0;
    char* end = nullptr;
    v = std::strtod(t.c_str(), &end);
    return !errno && end != t.c_str() && !*end;
}
template <size_t K>
bool to_code(const std::string& t, const Name (&names)[K], int32_t& v) {
    for (const Name& n : names)
        if (t == n.name) {
            v = n.code;
            return true;
        }
    return to_int(t, v);
}
}  // namespace

extern "C" {

const char* lbm_config_last_error(void) { return g_cfg_err.c_str(); }

lbm_status lbm_config_defaults(lbm_config* c) {
    if (!c) return LBM_ERR_INVALID;
    std::memset(c, 0, sizeof(*c));
    c->collision = LBM_COLLISION_CUMULANT2015;
    c->closure = LBM_CLOSURE_NONE;
    c->storage = LBM_STORAGE_F32;
    c->inlet_kind = LBM_INLET_MOVING_WALL;
    c->outlet_kind = LBM_OUTLET_DENSITY_INTERPOLATED;
    c->nu = 1.0 / 6.0;
    c->cles = 0.173;
    c->rho0 = 1.0;
    c->f16_scale_log2 = 10;
    c->mlp_interval = 1;
    c->omega_dumping_low = -1.0;
    c->omega_dumping_high = -1.0;
    return LBM_OK;
}

lbm_status lbm_config_parse(const char* text, lbm_config* cfg) {
    if (!text || !cfg) {
        g_cfg_err = "lbm_config_parse: null argument";
        return LBM_ERR_INVALID;
    }
    lbm_config c = *cfg;
    std::istringstream in(text);
    std::string line;
    int ln = 0;
    while (std::getline(in, line)) {
        ln++;
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        for (char& ch : line)
            if (ch == '=' || ch == ',' || ch == '\t' || ch == '\r') ch = ' ';
        std::istringstream ls(line);
        std::string key, t;
        if (!(ls >> key)) continue;
        std::vector<std::string> v;
        while (ls >> t) v.push_back(t);
        auto bad = [&](const char* why) {
            g_cfg_err = "line " + std::to_string(ln) + " (" + key + "): " + why;
            return LBM_ERR_INVALID;
        };
        auto ints = [&](int32_t* dst, size_t n) {
            if (v.size() != n) return false;
            for (size_t i = 0; i < n; i++)
                if (!to_int(v[i], dst[i])) return false;
            return true;
        };
        auto reals = [&](double* dst, size_t n) {
            if (v.size() != n) return false;
            for (size_t i = 0; i < n; i++)
                if (!to_double(v[i], dst[i])) return false;
            return true;
        };
        bool ok;
        if (key == "nx") ok = ints(&c.nx, 1);
        else if (key == "ny") ok = ints(&c.ny, 1);
        else if (key == "nz") ok = ints(&c.nz, 1);
        else if (key == "periodic") ok = ints(c.periodic, 3);
        else if (key == "collision") ok = v.size() == 1 && to_code(v[0], kCollision, c.collision);
        else if (key == "closure") ok = v.size() == 1 && to_code(v[0], kClosure, c.closure);
        else if (key == "storage") ok = v.size() == 1 && to_code(v[0], kStorage, c.storage);
        else if (key == "inlet" || key == "inlet_kind") ok = v.size() == 1 && to_code(v[0], kInlet, c.inlet_kind);
        else if (key == "outlet" || key == "outlet_kind") ok = v.size() == 1 && to_code(v[0], kOutlet, c.outlet_kind);
        else if (key == "nu") ok = reals(&c.nu, 1);
        else if (key == "tau") ok = reals(&c.tau, 1);
        else if (key == "cles") ok = reals(&c.cles, 1);
        else if (key == "force") ok = reals(c.force, 3);
        else if (key == "rho0") ok = reals(&c.rho0, 1);
        else if (key == "f16_scale_log2") ok = ints(&c.f16_scale_log2, 1);
        else if (key == "device") ok = ints(&c.device, 1);
        else if (key == "options") ok = ints(&c.options, 1);
        else if (key == "mlp_interval") ok = ints(&c.mlp_interval, 1);
        else if (key == "omega_dumping") {
            double d[2];
            ok = reals(d, 2);
            if (ok) { c.omega_dumping_low = d[0]; c.omega_dumping_high = d[1]; }
        } else if (key == "omega_dumping_low") ok = reals(&c.omega_dumping_low, 1);
        else if (key == "omega_dumping_high") ok = reals(&c.omega_dumping_high, 1);
        else return bad("unknown key");
        if (!ok) return bad("bad value");
    }
    *cfg = c;
    return LBM_OK;
}

}  // extern "C"
