/*
 * lbm.h - C ABI of the GB300 (sm_103a) D3Q27 lattice-Boltzmann solver core.
 *
 * Plain C types only: every buffer crossing this boundary is a host pointer plus
 * sizes, owned by the caller and copied by the call.  One context owns one CUDA
 * stream on one device; a context is not thread-safe (one host thread at a time).
 * Every function returns lbm_status (0 = LBM_OK, negative = error); nothing throws
 * across the boundary.  lbm_last_error() gives the message of the last failure.
 *
 * Reference interfaces replaced (stloufra/LB, paths inside that project):
 *  - the compile-time policy hooks `static void hook(LBMDataPointer&, LBMConstantsPointer&)`
 *    composed by SolverTurbulentLES (3D/simulation/src/solvers/SolverTurbulentLES.h:67-82);
 *  - the data carriers LBMData / LBMConstants (3D/simulation/src/data/LBMData.h:3-77,
 *    3D/simulation/src/data/LBMConstants.h:4-113);
 *  - the boundary-condition records (3D/simulation/src/traits/LBMTraits.h:17-61);
 *  - the OFF voxelizer (3D/preprocess/src/geometry/geometryMesherOFF.h:45-112 and
 *    3D/preprocess/src/geometry/geometryHandlerOFF.h:63-182).
 *
 * Lattice: D3Q27 in the reference's velocity order (3D/simulation/src/solvers/models/
 * D3Q27/D3Q27.h:81-111).  Scalar fields are (x,y,z) with x fastest; populations are
 * SoA [v][z][y][x] (the reference NDArray layout, LBMTraits.h:84-85,177-180).
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LBM_ABI_VERSION 3

typedef int32_t lbm_status;
#define LBM_OK                 0
#define LBM_ERR_INVALID       -1  /* bad argument or inconsistent set-up */
#define LBM_ERR_OOM           -2  /* device or host allocation failed */
#define LBM_ERR_CUDA          -3  /* CUDA runtime error (message in lbm_last_error) */
#define LBM_ERR_NONFINITE     -4  /* a population became NaN/Inf (reference: NaN break,
                                     SolverTurbulentLES.h:233-239) */
#define LBM_ERR_TIMEOUT       -5  /* a bounded device wait gave up */
#define LBM_ERR_STATE         -6  /* call out of order (e.g. step before flags) */
#define LBM_ERR_IO            -7  /* file could not be read or written */
#define LBM_ERR_UNSUPPORTED   -8  /* configuration the kernels do not implement */

/* collision operator (reference: solvers/collisions/) */
#define LBM_COLLISION_SRT            0  /* CollisionSRTTurbulent.h:20-81 */
#define LBM_COLLISION_CUMULANT2015   1  /* CollisionCumD3Q27Turbulent2015.h:19-537 */
#define LBM_COLLISION_CUMULANT2017   2  /* CollisionCumD3Q27Turbulent2017.h:19-594, with the omega_210
                                           limiters on C210 +- C012, the bulk term -k000 and eq. 44 driven
                                           by Dyv + Dzw - 2 Dxu (the reference reads C120 +- C102, -(rho - 1)
                                           and Dxu + Dyv - 2 Dzw, :256-266, :295, :351) */
#define LBM_COLLISION_CUMULANT_COMBINED 3  /* CollisionCumD3Q27TurbulentCombined.h:19-1087: cumulant-2015 on
                                           cells of flag 1, cumulant-2017 (corrected as above) on every other
                                           fluid or boundary cell (:1066-1078); the reference's 2017 copy
                                           there subtracts 1 + rho in Dxu (:295) */

/* eddy-viscosity closure (reference: solvers/turbulence/) */
#define LBM_CLOSURE_NONE         0  /* OmegaNo.h:25-48 : omega = 1/tau */
#define LBM_CLOSURE_SMAGORINSKY  1  /* OmegaLES.h:25-137 */
#define LBM_CLOSURE_MLP          2  /* learned closure; no reference counterpart */

/* population storage in HBM; the collision always runs in FP32 (FP64 for F64) */
#define LBM_STORAGE_F64     0
#define LBM_STORAGE_F32     1
#define LBM_STORAGE_F16DEV  2  /* half(h), f = w_v*rho0 + h*2^-s */

/* what the reference's flag -1 nodes are (its INLETTYPE policy) */
#define LBM_INLET_MOVING_WALL  0  /* Inlet/InletVelocityMovingWall.h:18-60 */
#define LBM_INLET_EQUILIBRIUM  1  /* Inlet/InletVelocityEquilibrium.h:18-108 */
#define LBM_INLET_ZOU_HE       2  /* Inlet/InletVelocityZouHe.h:18-104: the node is collided, never streamed
                                     into, and for n.c_v > 0 sets df(opp v) = f*_v - f_eq_v(rho, u)
                                     + f_eq_{opp v}(rho, u_b) (rho, u: the node's moments) */

/* what the reference's flag -2 outlet nodes do (its OUTLETTYPE policy); outlet normals +-x */
#define LBM_OUTLET_DENSITY_INTERPOLATED        0  /* Outlet/OutletDensityInterpolated.h:20-257 */
#define LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM       1  /* Outlet/OutletNeighbourEquilibrium.h:20-127: for the 9
                                                     links entering against the normal, f_v = f_eq_v(u, rho_b)
                                                     + (f_eq_v - f_v)(x+c_v), u the node's velocity and
                                                     f_v(x+c_v) the value the node streamed there */
#define LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA 2  /* the same + the sponge of OutletNeighbourEquilibriumOmega.h:
                                                     18-79: over the last ceil(10 %) of the lattice along the
                                                     first outlet's normal axis, omega -= (high - low) / width
                                                     * (distance from the sponge's start) */
#define LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA_RF 3  /* the same + OutletNeighbourEquilibriumOmegaRF.h:151-155:
                                                     rho_b *= 1 - u_x^2 / 2 where the node's u_x < 0 */
#define LBM_OUTLET_DENSITY_EQUILIBRIUM         4  /* Outlet/OutletDensityEquilibrium.h:20-79: the 9 entering
                                                     links set to f_eq(u, rho_b) of their own direction (the
                                                     reference writes f_eq of the opposite, outgoing one, :66) */

typedef struct lbm_config {
    int32_t nx, ny, nz;       /* lattice size: at most 2^31 - 2^21 cells, nx <= 2^21, ny, nz <= 65535 */
    int32_t periodic[3];      /* 1 = wrap this axis by index (replaces Periodic.h ghost planes) */
    int32_t collision;        /* LBM_COLLISION_* */
    int32_t closure;          /* LBM_CLOSURE_* */
    int32_t storage;          /* LBM_STORAGE_* */
    int32_t inlet_kind;       /* LBM_INLET_* */
    double  nu;               /* lattice kinematic viscosity; tau = 3 nu + 1/2 */
    double  tau;              /* if > 0, overrides the tau derived from nu */
    double  cles;             /* Smagorinsky constant; coefficient 18*cles (OmegaLES.h:119) */
    double  force[3];         /* body force density (lattice units); no reference counterpart */
    double  rho0;             /* reference density of the FP16-deviation encoding */
    int32_t f16_scale_log2;   /* s of the FP16-deviation encoding (10 => 2^10) */
    int32_t device;           /* CUDA device ordinal */
    int32_t options;          /* LBM_OPT_* bits (0: defaults) */
    int32_t mlp_interval;     /* learned closure: the network runs every k-th step (0, 1: every step);
                                 in between each cell relaxes with its last nu_t (kept in FP16) */
    int32_t outlet_kind;      /* LBM_OUTLET_* */
    double  omega_dumping_low;   /* sponge of LBM_OUTLET_NEIGHBOUR_EQUILIBRIUM_OMEGA(_RF): omegaDumpingLow, */
    double  omega_dumping_high;  /* omegaDumpingHigh (LBMConstants.h:74-76, set in main.cu:137-138) */
} lbm_config;

/* The defaults the Python mirror uses: cumulant-2015, no closure, FP32, moving-wall inlet, density-
 * interpolated outlet, nu = 1/6, cles = 0.173 (LBMConstants.h:70), rho0 = 1, s = 10, mlp_interval = 1,
 * no sponge (-1), nothing periodic; the lattice size is left 0. */
lbm_status lbm_config_defaults(lbm_config* cfg);
/* A case file as text: one "key = value" (or "key value") per line, '#' to the end of a line is a
 * comment.  Keys are the field names of lbm_config (periodic, force and omega_dumping take three, three
 * and two numbers); collision, closure, storage, inlet and outlet take a number or a name: the
 * reference's policy name (CollisionCumD3Q27Turbulent2015, OmegaLES, InletVelocityZouHe,
 * OutletNeighbourEquilibriumOmega, ...) or srt, cumulant2015, cumulant2017, combined; none,
 * smagorinsky, mlp; f64, f32, f16dev; moving_wall, equilibrium, zou_he; density_interpolated,
 * neighbour_equilibrium, neighbour_equilibrium_omega, neighbour_equilibrium_omega_rf,
 * density_equilibrium.  Fields not named keep their value in cfg.  LBM_ERR_INVALID on an unknown key
 * or a bad value (cfg unchanged then; the reason in lbm_config_last_error). */
lbm_status lbm_config_parse(const char* text, lbm_config* cfg);
const char* lbm_config_last_error(void);

/* implementation options */
#define LBM_OPT_ROW_STAGING  1  /* FP16 storage: rows of bulk cells through the shared-memory row-staged step
                                   (identical results) */
#define LBM_OPT_F16_ROUND_NEAREST 2  /* FP16 storage: round stores to nearest (ties away from zero).  Default:
                                   stochastic rounding
                                   (unbiased; keeps per-step increments below one FP16 step, such as a weak
                                   body force, in expectation; reproducible: the random bits are a hash of
                                   the element and the step) */

#define LBM_OPT_ONE_LAUNCH 4  /* FP32 / FP16 storage: one step launch over the whole lattice instead of the
                                  default split (rows whose pairs all take the packed path, then the
                                  remaining rows); identical results */

#define LBM_OPT_NO_WALL_ROWS 8  /* FP32 / FP16 storage: rows beside a flat wall take the general per-cell path
                                    instead of the packed wall kernel (the per-cell and packed paths round
                                    differently; this keeps the split step bit-identical to one launch) */

#define LBM_OPT_MLP_TCGEN05 16  /* learned closure (LBM_CLOSURE_MLP): the network of the plain-row step
                                   kernel runs on tcgen05.mma with TMEM accumulators (one CTA's 256 cells
                                   per product) instead of warp-level mma.sync; same inputs, weights and
                                   activation, FP32 accumulation in another order */

/* boundary-condition records, mirroring LBMTraits.h:17-43 */
typedef struct lbm_vertex { int32_t x, y, z; } lbm_vertex;

typedef struct lbm_bc_inlet {       /* boundaryConditionInlet, LBMTraits.h:31-36 */
    lbm_vertex vertex;
    float normal[3];                /* outward normal */
    float velocity[3];              /* lattice units */
    int32_t regular;
} lbm_bc_inlet;

typedef struct lbm_bc_outlet {      /* boundaryConditionOutlet, LBMTraits.h:38-43 */
    lbm_vertex vertex;
    float normal[3];                /* outward normal, +-x only (as the reference) */
    float density;                  /* lattice units */
    int32_t regular;
} lbm_bc_outlet;

typedef struct lbm_bc_symmetry {    /* boundaryConditionSymmetry, LBMTraits.h:45-49 */
    lbm_vertex vertex;
    float normal[3];                /* outward normal, +-y only (the reference's x and z branches are
                                       commented out, BounceSymmetryHalf.h:58-81, :135-157) */
    int32_t regular;                /* 1: the node's wall-pass flag was 10 (a flat face) */
} lbm_bc_symmetry;

/* diagnostics of the current state, reduced in FP64 on the device */
typedef struct lbm_diag {
    double  mass;            /* sum of rho over stream-target cells */
    double  momentum[3];     /* sum of rho*u over the same cells */
    double  drag[3];         /* momentum exchange on solid links by the last completed step */
    double  max_speed;       /* max |u| */
    int64_t nonfinite;       /* cells whose populations are not all finite */
    int64_t fluid_cells;     /* number of stream-target cells */
    int64_t step;            /* time steps done */
} lbm_diag;

typedef struct lbm_ctx lbm_ctx;

/* ---- lifecycle --------------------------------------------------------------- */
lbm_status  lbm_create(const lbm_config* cfg, lbm_ctx** out);
lbm_status  lbm_destroy(lbm_ctx* ctx);
const char* lbm_status_string(lbm_status s);
const char* lbm_last_error(const lbm_ctx* ctx);   /* ctx may be NULL: last global error */
int32_t     lbm_abi_version(void);

/* ---- set-up (replaces geometryMesherBoundary::arrayTransfer, geometryMesherBoundary.h:602-617) */
/* flags: nx*ny*nz int32 in the reference encoding (geometryMesherBoundary.h:439-484,
 * main.cu:95-97): 0 solid, >0 fluid, -1 inlet/moving wall, -2 outlet, -3 periodic
 * (treated as fluid; periodicity comes from cfg.periodic). */
lbm_status lbm_set_flags(lbm_ctx* ctx, const int32_t* flags);
/* per-node records of the -1 and -2 nodes (compileBoundaryArrayInlets/Outlets). */
lbm_status lbm_set_bc(lbm_ctx* ctx, const lbm_bc_inlet* inlets, int32_t n_inlets,
                      const lbm_bc_outlet* outlets, int32_t n_outlets);
/* half-way specular reflection on -2 nodes listed here (Symmetry/BounceSymmetryHalf.h:18-178,
 * compileBoundaryArraySymmetry, geometryMesherBoundary.h:563-580): for the links entering across the
 * plane, f_v(x) = f*_{sym v}(x - c_v parallel), sym mirroring the normal component.  The cell across
 * the plane must be solid; a link whose in-plane source is solid bounces back.  Call after lbm_set_bc
 * (which clears the list). */
lbm_status lbm_set_symmetry(lbm_ctx* ctx, const lbm_bc_symmetry* records, int32_t n);

/* ---- initialisation (InitializationEquilibriumConstVector.h:20-141) ---------- */
lbm_status lbm_init_equilibrium(lbm_ctx* ctx, double rho0, const double u0[3]);
/* rho: N doubles, u: 3*N doubles component-major (ux[N], uy[N], uz[N]) */
lbm_status lbm_init_fields(lbm_ctx* ctx, const double* rho, const double* u);

/* ---- time stepping (SolverTurbulentLES::runSimulation body, :186-226) ---------- */
lbm_status lbm_step(lbm_ctx* ctx, int32_t nsteps);
/* waits for the context's stream; LBM_ERR_TIMEOUT when a bounded device wait gave up, LBM_ERR_STATE when
 * an FP16 plain-row step met a pair whose class bytes are not of the packed kind (the row lists of the
 * split step no longer match the cell classes; no sequence of calls of this header produces that) */
lbm_status lbm_synchronize(lbm_ctx* ctx);
/* nsteps steps bracketed by CUDA events on the context's stream; *ms = elapsed device time */
lbm_status lbm_step_timed(lbm_ctx* ctx, int32_t nsteps, double* ms);
/* kernel launches one lbm_step step issues on this context (after initialisation): 1 to 3 (the split
   step launches the plain rows, the rows beside flat walls and the remaining rows separately; a kind with
   no rows is not launched).
   No reference counterpart (the reference runs one launch per hook) */
lbm_status lbm_step_launches(const lbm_ctx* ctx, int32_t* per_step);

/* ---- read-back (host copies, caller-owned) ----------------------------------- */
/* moments of the current pre-collision state (MomentDensityVelocityN27.h:27-83) */
lbm_status lbm_get_moments(lbm_ctx* ctx, double* rho, double* u);
/* the current pre-collision populations df[v][z][y][x] in reference velocity order */
lbm_status lbm_get_populations(lbm_ctx* ctx, double* f);
lbm_status lbm_set_populations(lbm_ctx* ctx, const double* f);
lbm_status lbm_reduce(lbm_ctx* ctx, lbm_diag* out);
/* u_x, u_y, u_z, rho of one cell (SolverTurbulentLES::probeWrite, SolverTurbulentLES.h:150-177) */
lbm_status lbm_probe(lbm_ctx* ctx, int32_t x, int32_t y, int32_t z, double out[4]);

/* relative velocity change since the previous call (ErrorQuadratic.h:19-91) */
lbm_status lbm_error_evaluation(lbm_ctx* ctx, double* err);

/* ---- time averaging (MomentTimeAvg.h:19-80, extended with <u_i u_j>) ------------ */
lbm_status lbm_timeavg_begin(lbm_ctx* ctx);   /* zero accumulators, accumulate each step */
lbm_status lbm_timeavg_end(lbm_ctx* ctx);     /* stop accumulating */
/* means over the accumulated steps; uu: 6*N doubles (xx,yy,zz,xy,xz,yz); count may be NULL */
lbm_status lbm_timeavg_get(lbm_ctx* ctx, double* rho_mean, double* u_mean,
                           double* uu_mean, int64_t* count);

/* ---- checkpoint / resume: bit-identical continuation ------------------------- */
lbm_status lbm_checkpoint_save(lbm_ctx* ctx, const char* path);
lbm_status lbm_checkpoint_load(lbm_ctx* ctx, const char* path);

/* ---- host mesher (geometryMesherBoundary.h:439-484 wall pass) ---------------- */
/* in place: every fluid cell (>0) gets 1 + number of solid cells in its 26-neighbourhood */
lbm_status lbm_mesher_wall_pass(int32_t* flags, int32_t nx, int32_t ny, int32_t nz);

/* ---- host mesher, cuboid boundary passes (geometryMesherBoundary.h:47-437) ---------------------
 * The sampling frame of the mesher (LBMConstants): cell (i, j, k) is tested at its centre
 * (i + 0.5 - additional) / resolution + bbmin per axis (in double, rounded to float for the inlet passes as
 * the reference's RealType look coordinates are).  A cuboid (geometryObjectCuboid.h:9-52) is the axis box
 * spanned by three corners, closed on every face; its id (a negative flag: -1 inlet, -2 outlet or
 * symmetry, -3 periodic) replaces the flag of every cell a pass takes.  Each pass appends records at
 * records[*n] (room for capacity records in all) and advances *n; LBM_ERR_INVALID when they do not fit
 * (nothing is written then).  Run the wall pass first: the regular field is read off the wall-pass
 * count (inlets: 1 unless the flag is above 10; outlets, symmetry, periodic: 1 only for a flag of 10). */
typedef struct lbm_mesh_frame {
    int32_t dims[3];
    float resolution_factor, additional_factor;
    float bbmin[3];
} lbm_mesh_frame;
typedef struct lbm_cuboid {
    double x1[3], x2[3], x3[3];
    int32_t id;
} lbm_cuboid;
typedef struct lbm_bc_periodic {    /* boundaryConditionPeriodic (LBMTraits.h): mesher output only; the
                                       kernels wrap periodic axes by index (lbm_config.periodic) */
    lbm_vertex vertex;
    float normal[3];
    int32_t periodic_index;
    int32_t regular;
} lbm_bc_periodic;
/* meshingBoundaryConditionInletUniform (:47-108): cells with flag > 0.  As the reference, a velocity with
 * three equal components is refused (LBM_ERR_INVALID: the reference's guard against a scalar passed as a
 * vector). */
lbm_status lbm_mesher_inlet_uniform(const lbm_mesh_frame* frame, int32_t* flags, const lbm_cuboid* cuboid,
                                    const float normal[3], const float velocity[3], lbm_bc_inlet* records,
                                    int64_t capacity, int64_t* n);
/* meshingBoundaryConditionInletParaboloidCircle (:111-177): the uniform pass at zero velocity, then every
 * inlet record so far whose cell centre lies in the cuboid and within radius of center gets
 * -3 u_mean (1 - (d / radius)^2) normal (clipped at 0).  The reference's own zero-velocity call trips the
 * guard above and throws; the pass here skips that guard. */
lbm_status lbm_mesher_inlet_paraboloid_circle(const lbm_mesh_frame* frame, int32_t* flags, const lbm_cuboid* cuboid,
                                              const double center[3], float radius, const float normal[3],
                                              float mean_velocity, lbm_bc_inlet* records, int64_t capacity,
                                              int64_t* n);
/* meshingBoundaryConditionInletParaboloidRectangle (:179-274): as above with the product profile
 * 2 u_mean prod_a s_a (D_a - s_a) / (prod_a D_a^2 / 16) over the two in-plane axes (s_a measured from the
 * face's low corner center - D/2); inlet_dims[a] along the normal is set to 1 on return, as the
 * reference does to its by-reference arguments. */
lbm_status lbm_mesher_inlet_paraboloid_rectangle(const lbm_mesh_frame* frame, int32_t* flags,
                                                 const lbm_cuboid* cuboid, const double center[3],
                                                 float inlet_dims[3], const float normal[3], float mean_velocity,
                                                 lbm_bc_inlet* records, int64_t capacity, int64_t* n);
/* meshingBoundaryConditionOutlet (:276-325), ...Symmetry (:327-377), ...Periodic (:379-437): cells with a
 * nonzero flag (earlier boundary ids included). */
lbm_status lbm_mesher_outlet(const lbm_mesh_frame* frame, int32_t* flags, const lbm_cuboid* cuboid,
                             const float normal[3], float density, lbm_bc_outlet* records, int64_t capacity,
                             int64_t* n);
lbm_status lbm_mesher_symmetry(const lbm_mesh_frame* frame, int32_t* flags, const lbm_cuboid* cuboid,
                               const float normal[3], lbm_bc_symmetry* records, int64_t capacity, int64_t* n);
lbm_status lbm_mesher_periodic(const lbm_mesh_frame* frame, int32_t* flags, const lbm_cuboid* cuboid,
                               const float normal[3], int32_t periodic_index, lbm_bc_periodic* records,
                               int64_t capacity, int64_t* n);
const char* lbm_mesher_last_error(void);

/* ---- mesh-matrix text files (postprocesors/outputerMesh.h:19-211) ------------ */
/* Writes the reference's format (outputerMesh::MeshMatrixOut): the header "Dimensions: nx ny nz ",
 * resolution and additional factors, BBmax x/y/z, BBmin x/y/z (as the reference's float fields print
 * through an ostream, 6 significant digits), then the flags with x fastest, one line per (y, z) with a
 * space after every value, an empty line after every z slice.  bbox: xmin, ymin, zmin, xmax, ymax,
 * zmax (the order of lbm_voxelize_off).  The path is used as given (the reference prepends results/). */
lbm_status lbm_mesh_matrix_write(const char* path, const int32_t* flags, const int32_t dims[3],
                                 double resolution, double additional, const double bbox[6]);
/* Reads it back (outputerMesh::MeshMatrixIn): header fields by keyword, then nx*ny*nz integers into
 * flags (nullable: header only; capacity in elements).  resolution, additional, bbox are nullable. */
lbm_status lbm_mesh_matrix_read(const char* path, int32_t* flags, int64_t capacity, int32_t dims[3],
                                double* resolution, double* additional, double bbox[6]);
const char* lbm_mesh_matrix_last_error(void);

/* ---- legacy VTK field files and the probe CSV (postprocesors/outputerVTK.h:26-851) ----------------
 * lbm_vtk_write gives the reference's structured-points layout: "# vtk DataFile Version 2.0", the title
 * (the reference writes "LBE variables", or "LBE <name>" for the mesh), "ASCII", "DATASET
 * STRUCTURED_POINTS", "DIMENSIONS nx ny nz", "ASPECT_RATIO" 1/resolution three times, "ORIGIN"
 * bbmin - (additional - 0.5)/resolution per axis, "POINT_DATA N", then per field "SCALARS <name> double 1"
 * + "LOOKUP_TABLE default" or "VECTORS <name> double", one point per line, x fastest.  Each value is
 * the field rounded to float times the float scale (the reference's Crho, Cpressure, Cu; 1 for lattice
 * units), printed as an ostream prints a float (6 significant digits).  The writers of the reference map
 * onto fields as: MeshVTK {object: flags}; variablesVTK {rho*Crho, p*Cpressure, U*Cu};
 * variablesLatticeVTK {rho, pressure, U}; the time-averaged ones the same on the means, with pressure
 * rho*cs2; omegaVTK {Omega}; distributionFunctionVTK and tauVTK one scalar each. */
typedef struct lbm_vtk_field {
    const char* name;        /* no spaces */
    int32_t components;      /* 1: SCALARS; 3: VECTORS, data component-major (x[N], y[N], z[N]) */
    const double* data;      /* N (or 3N) values, x fastest */
    double scale;
} lbm_vtk_field;
lbm_status lbm_vtk_write(const char* path, const char* title, const int32_t dims[3], double resolution,
                         double additional, const double bbmin[3], const lbm_vtk_field* fields, int32_t nfields);
/* probeWriteOut: appends "ux,uy,uz,rho,pressure" of one lbm_probe sample (u_x, u_y, u_z, rho) times Cu,
 * Crho and cs2*Cpressure; a new file starts with "Sampling frequency is: <Ct * probe_every_it>" and the
 * column line.  The path is used as given (the reference writes ./results/probeData.csv). */
lbm_status lbm_probe_csv_append(const char* path, double sampling_period, const double sample[4], double cu,
                                double crho, double cpressure);
/* InitializationEquilibriumVariables (initializations/InitializationEquilibriumVariables.h:47-113): the
 * restart read of a variables file.  Skips lines up to the first one holding "LOOKUP_TABLE default",
 * reads nx*ny*nz values (x fastest) as float into rho, skips lines up to one holding "VECTORS U double"
 * and reads three floats per point into u (component-major: x[N], y[N], z[N]).  No conversion factor is
 * applied (the reference reads the numbers as they stand), so the file to restart from is a lattice-unit
 * one (variablesLatticeVTK).  A DIMENSIONS line ahead of the data must match dims.  LBM_ERR_IO when the
 * file does not open, LBM_ERR_INVALID when a marker is missing or the data run short. */
lbm_status lbm_vtk_read_variables(const char* path, const int32_t dims[3], double* rho, double* u);
const char* lbm_vtk_last_error(void);

/* ---- OFF voxelizer on the GPU (preprocess geometryMesherOFF.h:45-112) -------- */
/* Reads an OFF/NOFF file; dims_out = ceil((BBmax-BBmin)*res + 2*add) per axis and bbox_out
 * (xmin,ymin,zmin,xmax,ymax,zmax).  flags_out (nullable: query dims only) receives
 * dims_out[0]*dims_out[1]*dims_out[2] int32, x fastest: 1 inside, 0 outside.
 * `outside` is accepted for interface parity with polyhedronInside() and otherwise unused:
 * the GPU casts +x rays. */
lbm_status lbm_voxelize_off(const char* path, double res, double add, const double outside[3],
                            int32_t* flags_out, int32_t dims_out[3], double bbox_out[6],
                            int32_t device);
/* the same on an in-memory triangle soup: verts 3*nv doubles, tris 3*nt int32 */
lbm_status lbm_voxelize_mesh(const double* verts, int32_t nv, const int32_t* tris, int32_t nt,
                             double res, double add, int32_t* flags_out, int32_t dims_out[3],
                             double bbox_out[6], int32_t device);

/* ---- the same voxelizer for callers that cannot allocate device memory ---------------------
 * No counterpart in the reference.  Some callers may not call cudaMalloc: an application whose
 * memory manager has reserved the whole device heap for its own pool, or a real-time loop where an
 * allocation's latency or failure is not acceptable.  This entry point gives the flags of
 * lbm_voxelize_mesh without allocating anything: the caller passes the output as device memory
 * (flags_out_device, dims[0]*dims[1]*dims[2] int32 on `device`; NULL queries dims and bbox only), and
 * the library's own scratch is one fixed array compiled into the library (about 4.1 MB, held on every
 * device that loads the library until the process exits).  Limits: at most
 * LBM_VOXELIZE_NOALLOC_MAX_VERTICES vertices, LBM_VOXELIZE_NOALLOC_MAX_TRIANGLES triangles and
 * LBM_VOXELIZE_NOALLOC_MAX_DIM cells per axis; larger inputs return LBM_ERR_UNSUPPORTED before any
 * device work, as do triangle indices outside [0, nv) (LBM_ERR_INVALID, the output untouched).  Each
 * call looks up that array's device address on `device`, so make the first call before capturing any
 * CUDA stream.  All calls in a process share the array: calls that overlapped on the GPU would race,
 * so this function holds a lock and returns only after its kernels finished.  Its copies and kernels
 * run on the legacy default stream of `device`: a caller that wrote flags_out_device (or will read it)
 * on a non-blocking stream must synchronise that stream first. */
#define LBM_VOXELIZE_NOALLOC_MAX_VERTICES  32768
#define LBM_VOXELIZE_NOALLOC_MAX_TRIANGLES 32768
#define LBM_VOXELIZE_NOALLOC_MAX_DIM       4096
lbm_status lbm_voxelize_mesh_noalloc(const double* verts, int32_t nv, const int32_t* tris, int32_t nt,
                                     double res, double add, int32_t* flags_out_device,
                                     int32_t dims_out[3], double bbox_out[6], int32_t device);

/* ---- learned LES closure (no reference counterpart; the reference has OmegaLES only) -----------
 * A per-cell MLP  x(7) -> 32 -> 32 -> 1  maps strain-rate invariants and density to the eddy
 * viscosity:  nu_t = out_scale * softplus(z).  Hidden activation: GELU in its sigmoid form
 * x * sigmoid(1.702 x).  Inputs, from the strain-rate tensor S (lattice units) and rho:
 *   0 tr S, 1 I2 = (tr^2 S - S:S)/2, 2 I3 = det S, 3 Lode parameter 3 sqrt(6) det(S_d)/|S_d|^3,
 *   4 S_d:S_d / S:S, 5 rho, 6 |S| = sqrt(2 S:S)        (S_d: deviatoric part)
 * normalised as (x - in_mean) / in_std before the first layer.  Training keeps FP32 parameters;
 * the step kernel evaluates FP16 copies on the tensor cores with FP32 accumulation and relaxes with
 * tau = tau_0 + 3 nu_t.  In the step kernel S is estimated locally from the non-equilibrium stress,
 * S = -3 Pi / (2 rho tau_S), tau_S being the Smagorinsky relaxation time; a cell whose raw input lies
 * outside [in_lo, in_hi] (the training range), or that is not a bulk cell, relaxes with tau_S.
 * params layout: w1[32][7], b1[32], w2[32][32], b2[32], w3[32], b3 (out x in, row-major). */
#define LBM_MLP_INPUTS  7
#define LBM_MLP_HIDDEN  32
#define LBM_MLP_PARAMS  1345  /* H^2 + 10 H + 1 for H = LBM_MLP_HIDDEN */
#define LBM_MLP_SAMPLE  10   /* floats per training sample: x[7], a, b, c */
typedef struct lbm_mlp_model {
    float params[LBM_MLP_PARAMS];
    float in_mean[LBM_MLP_INPUTS], in_std[LBM_MLP_INPUTS];
    float in_lo[LBM_MLP_INPUTS], in_hi[LBM_MLP_INPUTS];
    float out_scale;
} lbm_mlp_model;

/* model of a context created with closure LBM_CLOSURE_MLP (FP32 or FP16DEV storage); required before
 * the first lbm_step of such a context; may be replaced between steps */
lbm_status lbm_mlp_load(lbm_ctx* ctx, const lbm_mlp_model* model);

/* the eddy viscosity each cell keeps between network evaluations (contexts with mlp_interval > 1):
 * nu[N] doubles, the value of the last step that ran the network (-1 where that cell's inputs were out
 * of the training range and it relaxed with the Smagorinsky rate; NaN where it never ran the network:
 * cells off the packed bulk path, or before the first network step).
 * LBM_ERR_STATE without a kept value.  No reference counterpart (OmegaLES keeps omega, not nu_t). */
lbm_status lbm_get_eddy_viscosity(lbm_ctx* ctx, double* nu);

/* training samples from the current state of a run on a 4x-finer (generally width-x-finer) lattice:
 * box filter of `width` fine cells per coarse cell, strain rate of the filtered velocity by central
 * differences in coarse lattice units, filtered stress tau = <u u> - <u><u>.  A sample is
 *   x[7] (the inputs above, of the filtered S and rho), a = tau_d:S_d, b = S_d:S_d, c = tau_d:tau_d,
 * so that |tau_d + 2 nu_t S_d|^2 = c + 4 nu_t a + 4 nu_t^2 b is the subgrid-stress error of nu_t.
 * Coarse cells whose 3x3x3 stencil touches a solid fine cell are left out.  Samples are written in
 * coarse-cell order (x fastest) to out (LBM_MLP_SAMPLE floats each, nullable), at most `capacity`;
 * *count receives the number of samples of the state (which may exceed capacity). */
lbm_status lbm_les_samples(lbm_ctx* fine, int32_t width, float* out, int64_t capacity, int64_t* count);

/* nu_t of n raw input vectors (x: n*7 floats) through the step kernel's FP16 tensor-core path;
 * in_range (nullable) receives 1 where every input lies in [in_lo, in_hi] */
lbm_status lbm_mlp_eval(const lbm_mlp_model* model, const float* x, int64_t n, float* nu,
                        int32_t* in_range, int32_t device);
/* the same through a chosen product path: LBM_MLP_PATH_WARP_MMA (warp-level mma.sync, the default of
 * the step kernel) or LBM_MLP_PATH_TCGEN05 (tcgen05.mma with TMEM accumulators, one CTA per 256 inputs;
 * the path LBM_OPT_MLP_TCGEN05 selects in the step kernel).  LBM_ERR_TIMEOUT if a CTA gave up waiting
 * for its products. */
#define LBM_MLP_PATH_WARP_MMA 0
#define LBM_MLP_PATH_TCGEN05  1
lbm_status lbm_mlp_eval_path(const lbm_mlp_model* model, const float* x, int64_t n, float* nu,
                             int32_t* in_range, int32_t path, int32_t device);

/* GPU trainer: the samples (n * LBM_MLP_SAMPLE floats) are copied to the device once.  Loss of a set
 * of samples: the mean of (c + 4 nu_t a + 4 nu_t^2 b) / K with K the mean of c over all the trainer's
 * samples (loss 1 = the error of nu_t = 0). */
typedef struct lbm_mlp_trainer lbm_mlp_trainer;
lbm_status lbm_mlp_trainer_create(const float* samples, int64_t n, int32_t device, lbm_mlp_trainer** out);
lbm_status lbm_mlp_trainer_destroy(lbm_mlp_trainer* trainer);
double     lbm_mlp_trainer_norm(const lbm_mlp_trainer* trainer);   /* K */
/* loss and its gradient (LBM_MLP_PARAMS floats, params layout) over samples [first, first+count),
 * FP32 forward and backward kernels */
lbm_status lbm_mlp_gradient(lbm_mlp_trainer* trainer, const lbm_mlp_model* model, int64_t first,
                            int64_t count, float* grad, double* loss);
/* `epochs` passes of Adam (beta 0.9, 0.999) over minibatches of `batch` samples (a multiple of 128)
 * in a seeded random order; model->params is updated in place; loss_per_epoch (nullable, epochs
 * floats) receives the mean minibatch loss of each epoch */
lbm_status lbm_mlp_train(lbm_mlp_trainer* trainer, lbm_mlp_model* model, int32_t epochs, int32_t batch,
                         float lr, uint64_t seed, float* loss_per_epoch);
const char* lbm_mlp_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* LBM_GB300_H */
