/*
 * ff.h -- C ABI of libff, the GB300 (sm_103a) implementation of fluxflow's
 * grid-fluid hot path.  This is the drop-in boundary: a Node N-API addon (or
 * any FFI: ctypes, cffi, JNI) binds exactly these symbols.  Plain pointers,
 * sizes and opaque handles; no C++ or torch types cross it.
 *
 * Conventions
 *   - Every function returns an int status: 0 ok, negative FF_E_* on error.
 *     ff_last_error() gives a one-line description (thread-local).
 *   - Handles are opaque.  Device buffers are owned by the library and freed
 *     by the matching *_destroy (the reference has no disposal API,
 *     fluxflow src/linalg/linalg.js:43-53; this is an addition).
 *   - One CUDA stream per context.  A context is not thread-safe, matching
 *     the reference's single JS thread.
 *   - Layout is the reference's i-fastest layout (tsl_array_n
 *     src/array.js:24-38): element (i,j,k) of shape (nx,ny,nz) is at
 *     i + nx*(j + ny*k).  MAC faces: u is (nx+1,ny,nz), v (nx,ny+1,nz),
 *     w (nx,ny,nz+1) (fluxflow src/grid/grid_data3.js:121-176).
 *   - There is no CPU fallback: without a CUDA device every entry point that
 *     needs one returns FF_E_CUDA.
 */
#ifndef FF_H
#define FF_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define FF_OK 0
#define FF_E_ARG (-1)      /* bad argument / shape mismatch (reference throws) */
#define FF_E_CUDA (-2)     /* CUDA runtime error or no device                 */
#define FF_E_NOMEM (-3)
#define FF_E_STATE (-4)    /* call out of order                               */
#define FF_E_LIMIT (-5)    /* size beyond a stated limit                      */

typedef struct ff_ctx_s *ff_ctx;
typedef struct ff_field_s *ff_field;
typedef struct ff_pressure_s *ff_pressure;

const char *ff_last_error(void);
/* Library build identification ("ff <version> sm_103a"). */
const char *ff_version(void);

/* ---- context: replaces tsl_array_n init() (src/context.js:74-132), which
 * brings up a WebGPU device; here it selects a CUDA device and stream. ---- */
int ff_ctx_create(int device, ff_ctx *out);
int ff_ctx_destroy(ff_ctx ctx);
int ff_ctx_synchronize(ff_ctx ctx);
/* The compute stream waits for everything enqueued so far on the context's
 * copy streams (ff_pressure3_project_host's uploads and downloads), so an
 * event recorded after it covers them. */
int ff_ctx_join_copies(ff_ctx ctx);
/* Page-locked host memory for fast uploads/downloads (no reference
 * counterpart; the reference's host arrays are JS TypedArrays). */
int ff_host_alloc(size_t bytes, void **out);
int ff_host_free(void *p);
/* CUDA events on the context stream, for device-side timing by callers
 * (replaces the WebGPU timestamp queries of fluxflow src/profiling.js:302-330).
 * Slots 0..15.  elapsed waits for event b.                                  */
int ff_ctx_event_record(ff_ctx ctx, int slot);
int ff_ctx_event_elapsed(ff_ctx ctx, int slot_a, int slot_b, float *ms);

/* ---- fields: replace tsl_array_n arrayN (src/array.js:94-133) ---------- */
#define FF_FLOAT 0   /* 'float'  -> f32          */
#define FF_INT 1     /* 'int'    -> i32          */
#define FF_UINT8 2   /* masks    -> u8           */
#define FF_VEC3 3    /* 'vec3'   -> 3 x f32, AoS */
/* arrayN(type, shape): ndim 1..3 (array.js:4-20 rejects 4D) */
int ff_field_create(ff_ctx ctx, int dtype, int ndim, const int *shape, ff_field *out);
int ff_field_destroy(ff_field f);
/* fromArray (array.js:124-129): host -> device, bytes must equal the field size */
int ff_field_upload(ff_field f, const void *host, size_t bytes);
/* toArray (array.js:114-122): device -> host; synchronous like the awaited promise */
int ff_field_download(ff_field f, void *host, size_t bytes);
/* Asynchronous variants on the context stream (host memory should be pinned). */
int ff_field_upload_async(ff_field f, const void *host, size_t bytes);
int ff_field_download_async(ff_field f, void *host, size_t bytes);
int ff_field_fill(ff_field f, float value);
/* device-to-device copy between fields of one type and size              */
int ff_field_copy(ff_field dst, ff_field src);
int ff_field_info(ff_field f, int *dtype, int *ndim, int *shape3, int64_t *count);
void *ff_field_device_ptr(ff_field f);

/* ---- pressure projection: replaces createGridPressureSolver3
 * (fluxflow src/grid/grid_pressure_solver3.js:66-574) and, with nz == 1,
 * createGridPressureSolver2 (grid_pressure_solver2.js:223-981). ---------- */
#define FF_PRE_MULTIGRID 0
#define FF_PRE_JACOBI 1
#define FF_PRE_NONE 2
#define FF_COARSE_SWEEPS 0   /* numberOfCoarsestIterations RB sweeps (reference) */
#define FF_COARSE_DIRECT 1   /* FP64 direct solve of the coarsest level          */
#define FF_STORE_FP32 0      /* V-cycle arrays in FP32                            */
#define FF_STORE_BF16 1      /* V-cycle arrays in BF16, FP32 arithmetic           */
#define FF_ITERATE_FP32 0    /* CG iterate x in FP32 (reference)                  */
#define FF_ITERATE_DS 1      /* x as hi+lo FP32 pair, compensated residual        */

typedef struct {
    int resolution[3];          /* nz == 1 selects the 2D solver              */
    double grid_spacing[3];
    double origin[3];
    int preconditioner;         /* FF_PRE_*                       (:72)       */
    double tolerance;           /* default 1e-6                   (:73)       */
    int max_iterations;         /* <=0: ceil(factor*max(res)*(3D?1:4)) (:133) */
    double max_iterations_factor;   /* default 1.5                (:76)       */
    int relative_tolerance;     /* default 1                      (:77)       */
    double max_plausible_pressure;  /* default 1e6                (:36)       */
    /* multigrid options (multigrid.js:1186-1250) */
    int mg_levels;              /* numberOfLevels, default 1                   */
    int mg_down, mg_up;         /* numberOfSmoothingIterationsDown/Up, 2       */
    int mg_coarsest;            /* numberOfCoarsestIterations, 20              */
    int mg_final;               /* numberOfFinalIterations, 2                  */
    double mg_sor;              /* sorFactor, 1.0                              */
    int mg_coarsen_mask;        /* coarsenDirichletMask, 1                     */
    int mg_coarsen_weights;     /* coarsenFaceWeights, 1                       */
    int mg_coarse_mode;         /* FF_COARSE_*                                 */
    /* precision (no reference counterpart: the reference is FP32 only) */
    int vcycle_storage;         /* FF_STORE_*                                  */
    int iterate;                /* FF_ITERATE_*                                */
} ff_pressure_desc;

/* Fills the reference defaults for a resolution/spacing. */
void ff_pressure_desc_default(ff_pressure_desc *d, const int *resolution, const double *spacing);

typedef struct {
    int converged;              /* diagnostics.converged                       */
    int rejected;               /* circuit breaker fired (:547-554)            */
    int iterations;             /* diagnostics.iterations                      */
    int stopped_by;             /* FF_STOP_* (linalg.js:1056-1103)             */
    double residual;            /* sqrt|r.r| of the last true residual         */
    double b_norm;              /* sqrt(b.b)                                   */
    int bad_cells;              /* non-finite or |p| > maxPlausiblePressure    */
    int max_iterations;         /* the cap that applied                        */
    int kernel_launches;        /* libff kernels launched by the call          */
    int warm_start;             /* -1 none, 0 previous pressure kept, 1 network guess used */
    /* reportNoiseFloor diagnostics (grid_pressure_solver3.js:517-542,
     * linalg.js:884-905), filled when the setting is on, else 0: */
    int report_floor;           /* 1 when the fields below were measured       */
    int tolerance_below_floor;  /* toleranceBelowFloor: threshold < floor      */
    double max_residual;        /* maxResidual: max |r| of the last residual   */
    double noise_floor;         /* noiseFloor: 2^-24 * sum(2/h^2) * |x0|       */
    double noise_floor_relative;/* noiseFloorRelative: noise_floor / |b|       */
    double floor_threshold;     /* the stop threshold it is compared with      */
} ff_diag;

#define FF_STOP_NONE 0
#define FF_STOP_DEGENERATE_PAP 1
#define FF_STOP_PAP_GROWTH 2
#define FF_STOP_ALPHA_MAGNITUDE 3
#define FF_STOP_DEGENERATE_OLD_RZ 4
#define FF_STOP_CONVERGED 5
#define FF_STOP_RESIDUAL_GROWING 6

int ff_pressure3_create(ff_ctx ctx, const ff_pressure_desc *desc, ff_pressure *out);
int ff_pressure3_destroy(ff_pressure ps);
/* colliderWeights {u,v,w} (:69, :163-230): face fields, or NULL to clear.  */
int ff_pressure3_set_collider_weights(ff_pressure ps, ff_field u, ff_field v, ff_field w);
/* faceWeights {u,v,w} (beta, :68, :217-229), or NULL to clear.            */
int ff_pressure3_set_face_weights(ff_pressure ps, ff_field u, ff_field v, ff_field w);
/* dirichlet(pos) -> {active, target} (:68, :171-206) evaluated per cell:
 * active is a FF_UINT8 cell field, target a FF_FLOAT cell field (or NULL
 * for 0).  active == NULL clears the Dirichlet condition.                 */
int ff_pressure3_set_dirichlet(ff_pressure ps, ff_field active, ff_field target);
/* project() with the velocity taken from and returned to host memory (no
 * reference counterpart: the reference's host arrays reach the GPU through
 * field.fromArray / toArray, array.js:114-129).  Uploads hu, hv, hw into the
 * input fields on a copy stream, projects into the output fields, downloads
 * them into hu_out, hv_out, hw_out on a second copy stream; the upload of one
 * call overlaps the download of the previous one.  Host buffers should be
 * page-locked (ff_host_alloc); outputs are in place after
 * ff_ctx_synchronize.  2D solvers take w_in/w_out/hw/hw_out NULL. */
int ff_pressure3_project_host(ff_pressure ps, ff_field u_in, ff_field v_in, ff_field w_in, const void *hu,
                              const void *hv, const void *hw, ff_field u_out, ff_field v_out, ff_field w_out,
                              void *hu_out, void *hv_out, void *hw_out, ff_diag *diag);
/* Runtime settings object (:135): key names as in the reference
 * ("tolerance", "maxIterations", "relativeTolerance", "checkBadCells",
 * "preconditioner", "sorFactor", "reportNoiseFloor"), plus "useGraph",
 * "useTma" and "coarseTail" for this implementation's paths. */
int ff_pressure3_set(ff_pressure ps, const char *key, double value);
/* project(inGrid, outGrid)() (:339-556).  u_out may equal u_in.  The
 * pressure field persists between calls and is the warm start.           */
int ff_pressure3_project(ff_pressure ps, ff_field u_in, ff_field v_in, ff_field w_in,
                         ff_field u_out, ff_field v_out, ff_field w_out, ff_diag *diag);
/* PCG solve of A p = b for a caller-given b on the solver's current system
 * (createPreconditionedConjugateGradientSolver(...).solve, linalg.js:2176
 * with the GPU-resident path of :1651).  The pressure field is the initial
 * guess and the result; the circuit breaker applies as in project().      */
int ff_pressure3_solve(ff_pressure ps, ff_field b, ff_diag *diag);
/* The solver's own fields: pressure (:142), b (:143), dirichletMask and
 * ventMask (:572, as u8 here).  Borrowed handles, valid until destroy.     */
int ff_pressure3_fields(ff_pressure ps, ff_field *pressure, ff_field *b,
                        ff_field *dirichlet_mask, ff_field *vent_mask);

/* ---- static SDF collider: replaces createSDFStaticCollider3.addShapes
 * (fluxflow src/grid/sdf_collider3.js:69-99) and computeFaceWeights
 * (:131-254), which the reference runs on the CPU; here FP64 on the device.
 * phi: cell field (nx,ny,nz) of signed distance (solid where phi < 0);
 * wu/wv/ww: face-open fractions (MIN_FACE_WEIGHT 0.01, :23).  Any of the
 * output fields may be NULL.                                              */
#define FF_SHAPE_SPHERE 0
#define FF_SHAPE_BOX 1
typedef struct {
    int type;                 /* FF_SHAPE_*   (primitive_sdf3.js:169-200) */
    int has_rotation;
    double center[3];
    double radius;            /* sphere */
    double half_extents[3];   /* box    */
    double rotation_axis[3];
    double rotation_angle;
} ff_shape;
int ff_collider3_bake(ff_ctx ctx, const ff_shape *shapes, int nshapes, int invert,
                      const int *resolution, const double *grid_spacing, const double *origin,
                      ff_field phi, ff_field wu, ff_field wv, ff_field ww);
/* ff_collider3_bake without any device allocation (no counterpart in the
 * reference, which bakes on the CPU).  For hosts that may not allocate device
 * memory while they run: a process whose device memory is owned by an outside
 * pool, or a frame loop that cannot take the implicit device-wide
 * synchronisation of cudaMalloc/cudaFree.  The shape table lives in one
 * fixed device array of FF_BAKE_NOALLOC_MAX_SHAPES entries per device; more
 * shapes return FF_E_LIMIT.  The first call on a device looks the array up
 * (make it before any stream capture).  The table reaches the device as a
 * kernel parameter, so the call copies nothing from host memory and returns
 * without waiting for its kernels.  The array is shared by every caller on
 * the device, so calls must be ordered on the GPU: issue them on the same
 * stream, or make the next caller wait for the previous call's stream (an
 * event or a synchronize) first; unordered calls (two contexts' streams, two
 * threads) race on it.  The caller's current device is restored on return.
 * Same arguments, outputs and errors as ff_collider3_bake.                */
#define FF_BAKE_NOALLOC_MAX_SHAPES 64
int ff_collider3_bake_noalloc(ff_ctx ctx, const ff_shape *shapes, int nshapes, int invert,
                              const int *resolution, const double *grid_spacing, const double *origin,
                              ff_field phi, ff_field wu, ff_field wv, ff_field ww);

/* ---- semi-Lagrangian advection: replaces createSemiLagrangianAdvectionSolver3
 * (fluxflow src/grid/advection_solver3.js:67-364).  The trace is backTrace
 * (:20-62): RK2 midpoint substeps of at most one cell (h = min spacing),
 * at most max_substeps, stopping on the collider SDF with a linear blend.
 * The final sample is the monotone tricubic of grid_math3.js:137-215.  FP32
 * with every operation rounded on its own, as the reference's WGSL.       */
typedef struct ff_advect_s *ff_advect;
typedef struct {
    int resolution[3];
    double grid_spacing[3];
    double origin[3];
    double dt;                  /* dt (:67)                            */
    int max_substeps;           /* maxSubsteps, default 32             */
    int order;                  /* 1 semi-Lagrangian, 2 MacCormack     */
} ff_advect_desc;
int ff_advect3_create(ff_ctx ctx, const ff_advect_desc *desc, ff_advect *out);
int ff_advect3_destroy(ff_advect a);
int ff_advect3_set_dt(ff_advect a, double dt);
/* collider: cell-centred SDF field sampled trilinearly (sdf_collider3.js:33),
 * or NULL (boundary sample 1 everywhere).  Borrowed.                       */
int ff_advect3_set_collider(ff_advect a, ff_field phi);
/* advectFaceCentered3(input, output) (:130-178): every face whose position
 * samples the collider > 0 gets the cubic sample of `in` at trace(position)
 * through the velocity (vu, vv, vw); other faces keep the output's value. */
int ff_advect3_faces(ff_advect a, ff_field vu, ff_field vv, ff_field vw, ff_field in_u, ff_field in_v,
                     ff_field in_w, ff_field out_u, ff_field out_v, ff_field out_w);
/* advectScalar3 (:304-360) of a cell-centred scalar */
int ff_advect3_scalar(ff_advect a, ff_field vu, ff_field vv, ff_field vw, ff_field s_in, ff_field s_out);
/* trace(start, direction) (:363) of FF_VEC3 points; direction 1 traces
 * back in time, -1 forward (the FLIP particle advection).                 */
int ff_advect3_trace(ff_advect a, ff_field vu, ff_field vv, ff_field vw, ff_field p_in, ff_field p_out,
                     int direction);

/* ---- velocity constraint: replaces createGridBlockedBoundaryConditionSolver3
 * (fluxflow src/grid/grid_blocked_boundary_condition_solver3.js:48-490).    */
#define FF_DIRECTION_LEFT 1
#define FF_DIRECTION_RIGHT 2
#define FF_DIRECTION_DOWN 4
#define FF_DIRECTION_UP 8
#define FF_DIRECTION_BACK 16
#define FF_DIRECTION_FRONT 32
#define FF_DIRECTION_ALL_3D 63      /* constant.js:24-38 */
typedef struct ff_bc_s *ff_bc;
int ff_bc3_create(ff_ctx ctx, const int *resolution, const double *grid_spacing, const double *origin,
                  ff_bc *out);
int ff_bc3_destroy(ff_bc b);
/* setCollider (:390-404): a static SDF collider (cell field, solid where
 * phi < 0, friction 0.5) and optionally its face weights (colliderFaceWeights,
 * :60-62), which then decide the closed faces.  NULL phi removes it.       */
int ff_bc3_set_collider(ff_bc b, ff_field phi, ff_field wu, ff_field wv, ff_field ww);
/* closedDomainBoundaryFlag (:102), FF_DIRECTION_* bits, default ALL_3D    */
int ff_bc3_set_closed(ff_bc b, int flags);
/* setInflows (:138-146): n inflow SDFs (cell fields, inside where < 0),
 * velocities (3 per inflow) and modes (0 'set', 1 'add'); n == 0 clears.   */
int ff_bc3_set_inflows(ff_bc b, int n, const ff_field *phis, const double *velocities, const int *modes);
/* constrainVelocity(extrapolationDepth = 5) (:445-477), in place          */
int ff_bc3_constrain(ff_bc b, ff_field u, ff_field v, ff_field w, int depth);

/* ---- external force: createExternalForceSolver3 (fluxflow
 * src/grid/external_force_solver3.js:7-29) for a uniform force; every face
 * of each component gains force.x * dt (.y, .z).                           */
int ff_velocity3_add_force(ff_ctx ctx, const int *resolution, ff_field u, ff_field v, ff_field w, double fx,
                           double fy, double fz, double dt);

/* ---- explicit viscosity (no counterpart: grid_solver3.js:104 leaves
 * computeViscosity a no-op): out = in + dt nu lap(in) on the faces strictly
 * inside each component's own axis range, Neumann at the array ends.       */
int ff_viscosity3_apply(ff_ctx ctx, const int *resolution, const double *grid_spacing, ff_field u, ff_field v,
                        ff_field w, double nu, double dt, ff_field u_out, ff_field v_out, ff_field w_out);

/* ---- outflow: replaces createGridOutflowSolver3 (fluxflow
 * src/grid/grid_outflow_solver3.js:79-210) with createSDFOutflow3
 * (sdf_inflow_outflow3.js:25-29, an SDF baked like a static collider).
 * Each outflow is a float cell SDF (borrowed) on its own grid:
 * phi_resolution / phi_spacing / phi_origin hold 3 entries per outflow
 * (phi_origin may be NULL: zeros).  At most 64 outflows.                  */
typedef struct ff_outflow_s *ff_outflow;
int ff_outflow3_create(ff_ctx ctx, const int *resolution, const double *grid_spacing, const double *origin, int n,
                       const ff_field *phis, const int *phi_resolution, const double *phi_spacing,
                       const double *phi_origin, double dt, int apply_velocity_bc, ff_outflow *out);
int ff_outflow3_destroy(ff_outflow o);
int ff_outflow3_set_dt(ff_outflow o, double dt);
/* applyOutflowVelocityBC (:153-170): per outflow, u then v then w, faces
 * inside relax toward the velocity one spacing upstream by the Courant
 * number of the outward bulk speed (convective condition, :98-133); a
 * no-op when created with apply_velocity_bc = 0                           */
int ff_outflow3_apply_velocity_bc(ff_outflow o, ff_field u, ff_field v, ff_field w);
/* clearOutflowScalarField(scalarGrid)() (:174-196): cells of a
 * cell-centred scalar grid (its own geometry) inside an outflow become 0  */
int ff_outflow3_clear_scalar(ff_outflow o, ff_field scalar, const int *resolution, const double *grid_spacing,
                             const double *origin);
/* the `dirichlet` closure (createOutflowPressureDirichlet3, :44-64)
 * evaluated at the cell centres of a pressure grid: active (uint8) = 1
 * where an outflow holds the centre, target (float) = target everywhere;
 * pass both to ff_pressure3_set_dirichlet                                 */
int ff_outflow3_dirichlet(ff_outflow o, const int *resolution, const double *grid_spacing, const double *origin,
                          double target, ff_field active, ff_field target_field);

/* ---- FLIP: replaces createGridFlipSolver3 (fluxflow
 * src/grid/grid_flip_solver3.js:135-1157), resampling included.  Particles
 * are FF_VEC3 positions and velocities (AoS, as the reference's vec3
 * arrays); P2G accumulates round(v w S) and round(w S) in int32 (S =
 * p2gAtomicScale, :508-530), so the transfer does not depend on the
 * order particles arrive in.                                               */
typedef struct ff_flip_s *ff_flip;
typedef struct {
    int resolution[3];
    double grid_spacing[3];
    double origin[3];
    int max_particles;             /* maxParticles (required)             */
    double dt;                     /* dt                                   */
    double gravity[3];             /* default (0, -9.81, 0)                */
    int reduced_pressure;          /* reducedPressure, default 1           */
    double flip_ratio;             /* flipRatio, default 0.97              */
    double velocity_damping;       /* velocityDamping, default 0.02        */
    double p2g_atomic_scale;       /* p2gAtomicScale, default 65536        */
    double weight_epsilon;         /* weightEpsilon, default 1e-4          */
    int closed_flags;              /* closedDomainBoundaryFlag             */
    int max_substeps;              /* of the particle trace, default 32    */
    double collider_push_thresh;   /* colliderPushThresh, default 0        */
    double collider_push_shift;    /* colliderPushShift, default 0         */
    int carry_concentration;       /* carryConcentration, default 0        */
    double mixing, fade;           /* default 0, 0                         */
    double concentration_atomic_scale;   /* default 4096                   */
    double ambient_density;        /* > 0 with component_density: the      */
    double component_density;      /* variable-density coupling (:265-359) */
    int extrapolation_depth;       /* default 5                            */
    ff_pressure_desc pressure;     /* the projection's options (`pressure`)*/
    int resample_enabled;          /* resample.enabled, default 1 (:178)   */
    int min_particles_per_cell;    /* resample.minParticlesPerCell, 4      */
    int max_particles_per_cell;    /* resample.maxParticlesPerCell, 8      */
} ff_flip_desc;
void ff_flip_desc_default(ff_flip_desc *d, const int *resolution, const double *grid_spacing, int max_particles,
                          double dt);
/* u, v, w: the velocity grid the solver works on (borrowed)              */
int ff_flip3_create(ff_ctx ctx, const ff_flip_desc *desc, ff_field u, ff_field v, ff_field w, ff_flip *out);
int ff_flip3_destroy(ff_flip f);
/* collider SDF (cell field, borrowed) or NULL                             */
int ff_flip3_set_collider(ff_flip f, ff_field phi);
/* number of live particles (<= max_particles); the first n are stepped   */
int ff_flip3_set_count(ff_flip f, int n);
/* borrowed handles: positions, velocities (FF_VEC3), concentration (or
 * NULL), fluidMask (float cells) and the projection's pressure solver    */
int ff_flip3_fields(ff_flip f, ff_field *positions, ff_field *velocities, ff_field *concentration,
                    ff_field *fluid_mask, ff_pressure *pressure);
/* borrowed handles of the grid-side state: cellConcentration and
 * cellDensity (cells), the beta faces, and the Dirichlet active/target
 * fields the projection used (any may be NULL when not in use)           */
int ff_flip3_grid_fields(ff_flip f, ff_field *cell_concentration, ff_field *cell_density, ff_field *beta_u,
                         ff_field *beta_v, ff_field *beta_w, ff_field *dirichlet_active, ff_field *dirichlet_target);
/* stages of onAdvanceTimeStep (:1110-1150), for tests and custom steps   */
#define FF_FLIP_ADVECT_PARTICLES 0        /* advectParticles + pushOutOfCollider */
#define FF_FLIP_P2G 1                     /* reset, scatter, finalize            */
#define FF_FLIP_SNAPSHOT 2                /* snapshotOldU/V/W                    */
#define FF_FLIP_EXTRAPOLATE_WEIGHT 3      /* extrapolateWeightU/V/W              */
#define FF_FLIP_CONSTRAIN 4               /* boundarySolver.constrainVelocity    */
#define FF_FLIP_MARK_FLUID 5              /* clear + markFluidCells + adjacency  */
#define FF_FLIP_CONCENTRATION_GRID 6      /* cell concentration, density, beta   */
#define FF_FLIP_GRAVITY 7                 /* applyGravity / applyReducedGravity  */
#define FF_FLIP_PROJECT 8                 /* Dirichlet air cells + projection    */
#define FF_FLIP_EXTRAPOLATE_PRESSURE 9    /* extrapolatePressureU/V/W            */
#define FF_FLIP_G2P 10                    /* g2pUpdate                           */
#define FF_FLIP_CONCENTRATION_PARTICLE 11 /* mixAndFade                          */
#define FF_FLIP_RESAMPLE 12               /* resamplePass, then markFluidCells   */
int ff_flip3_stage(ff_flip f, int stage);
/* the last resamplePass (:621-820): donors = particles in cells above
 * max_particles_per_cell, requested = the slots under-full cells asked
 * for; min(donors, requested) particles moved.  Synchronises the stream. */
int ff_flip3_resample_stats(ff_flip f, int64_t *donors, int64_t *requested);
/* onAdvanceTimeStep(): every stage in the reference's order; diag is the
 * projection's diagnostics                                                */
int ff_flip3_step(ff_flip f, ff_diag *diag);
/* ---- 2D two-phase FLIP: replaces createGridTwoPhaseFlipSolver2 (fluxflow
 * src/grid/grid_two_phase_flip_solver2.js:479-1622), run on a
 * one-cell-thick grid (u, v: the 2D face arrays; particles on the plane
 * through the cell centres).  Every cell is fluid; density and beta faces
 * follow the particles' concentration; the pressure is pinned to 0 at
 * pin_cell (pressurePin; {-1, -1} = null).                                 */
typedef struct ff_twophase_s *ff_twophase;
typedef struct {
    int resolution[2];
    double grid_spacing[2];
    double origin[2];
    int max_particles;             /* maxParticles (required)             */
    double dt;
    double gravity[2];             /* default (0, -9.81)                   */
    double ambient_density;        /* gasDensity / ambientDensity, 0.01    */
    double component_density;      /* liquidDensity / componentDensity, 1  */
    double mixing, fade;           /* default 0, 0                         */
    double concentration_atomic_scale;   /* default 4096                   */
    double flip_ratio;             /* default 0.97                         */
    double gas_flip_ratio;         /* default 0.90                         */
    double velocity_damping;       /* default 0.02                         */
    double p2g_atomic_scale;       /* default 65536                        */
    double weight_epsilon;         /* default 1e-4                         */
    int closed_flags;              /* closedDomainBoundaryFlag, default 15 */
    int max_substeps;              /* of the particle trace, default 32    */
    double collider_push_thresh, collider_push_shift;
    int pin_cell[2];               /* default topCenter (nx/2, ny-1)       */
    int resample_enabled;          /* resample.enabled, default 1          */
    int min_particles_per_cell;    /* default 3                            */
    int max_particles_per_cell;    /* default 8                            */
    int extrapolation_depth;       /* default 5                            */
    ff_pressure_desc pressure;     /* multigrid levels default: deepest of
                                      up to 4 the resolution divides into  */
} ff_twophase_desc;
void ff_twophase_desc_default(ff_twophase_desc *d, const int *resolution, const double *grid_spacing,
                              int max_particles, double dt);
int ff_twophase2_create(ff_ctx ctx, const ff_twophase_desc *desc, ff_field u, ff_field v, ff_twophase *out);
int ff_twophase2_destroy(ff_twophase t);
int ff_twophase2_set_collider(ff_twophase t, ff_field phi);
int ff_twophase2_set_count(ff_twophase t, int n);
/* positions / velocities as 2D pairs (x, y), phase (concentration) per
 * particle; NULL leaves that array alone                                  */
int ff_twophase2_set_particles(ff_twophase t, int n, const float *xy, const float *vxy, const float *phase);
int ff_twophase2_get_particles(ff_twophase t, int n, float *xy, float *vxy, float *phase);
/* borrowed handles: phase (= concentration), liquidFraction, density
 * (cells), betaU, betaV (faces), and the pressure solver                   */
int ff_twophase2_fields(ff_twophase t, ff_field *phase, ff_field *liquid_fraction, ff_field *density,
                        ff_field *beta_u, ff_field *beta_v, ff_pressure *pressure);
#define FF_TP_ADVECT 0             /* advectParticles + pushOutOfCollider  */
#define FF_TP_DENSITY 1            /* countPhases, density, betaU/V        */
#define FF_TP_P2G 2                /* scatter + finalize U/V               */
#define FF_TP_SNAPSHOT 3           /* snapshotOldU/V                       */
#define FF_TP_EXTRAPOLATE_WEIGHT 4 /* extrapolateWeightU/V                 */
#define FF_TP_CONSTRAIN 5          /* boundarySolver.constrainVelocity     */
#define FF_TP_GRAVITY 6            /* applyGravityU/V                      */
#define FF_TP_PROJECT 7            /* the variable-density projection      */
#define FF_TP_G2P 8                /* g2pUpdate (per-phase blend)          */
#define FF_TP_MIX 9                /* mixConcentration (mixing / fade)     */
#define FF_TP_RESAMPLE 10          /* per-phase resamplePass               */
int ff_twophase2_stage(ff_twophase t, int stage);
/* onAdvanceTimeStep(): every stage in the reference's order               */
int ff_twophase2_step(ff_twophase t, ff_diag *diag);
/* the last resampling pass: {liquid donors, liquid cells' need, gas
 * donors, gas cells' need}.  Synchronises the stream.                      */
int ff_twophase2_resample_stats(ff_twophase t, int64_t *out4);
/* ---- 3D two-phase FLIP: no counterpart in the reference, whose two-phase
 * solver is 2D only (grid_two_phase_flip_solver2.js:479-1622).  The same
 * stages on a full 3D grid: u, v, w face arrays (borrowed), particles in 3D,
 * density and beta on all three face sets (the 3D FLIP solver's beta,
 * grid_flip_solver3.js:298-359, with every cell fluid), the pressure pinned
 * at pin_cell, and resampling recipients with at least 3 of their 6 clamped
 * face neighbours full (the 3D single-phase rule, grid_flip_solver3.js:
 * 700-724).  Stages are the FF_TP_* codes; the handle type is ff_twophase. */
typedef struct {
    int resolution[3];
    double grid_spacing[3];
    double origin[3];
    int max_particles;             /* required                            */
    double dt;
    double gravity[3];             /* default (0, -9.81, 0)               */
    double ambient_density;        /* concentration 0 (gas), default 0.01 */
    double component_density;      /* concentration 1 (liquid), 1         */
    double mixing, fade;           /* default 0, 0                        */
    double concentration_atomic_scale;   /* default 4096                  */
    double flip_ratio;             /* default 0.97                        */
    double gas_flip_ratio;         /* default 0.90                        */
    double velocity_damping;       /* default 0.02                        */
    double p2g_atomic_scale;       /* default 65536                       */
    double weight_epsilon;         /* default 1e-4                        */
    int closed_flags;              /* default 63 (all six walls)          */
    int max_substeps;              /* default 32                          */
    double collider_push_thresh, collider_push_shift;
    int pin_cell[3];               /* default top centre (nx/2, ny-1, nz/2); {-1,..} = none */
    int resample_enabled;          /* default 1                           */
    int min_particles_per_cell;    /* default 3                           */
    int max_particles_per_cell;    /* default 8                           */
    int extrapolation_depth;       /* default 5                           */
    ff_pressure_desc pressure;     /* multigrid: deepest of up to 5 levels the resolution divides into */
} ff_twophase3_desc;
void ff_twophase3_desc_default(ff_twophase3_desc *d, const int *resolution, const double *grid_spacing,
                               int max_particles, double dt);
int ff_twophase3_create(ff_ctx ctx, const ff_twophase3_desc *desc, ff_field u, ff_field v, ff_field w,
                        ff_twophase *out);
/* positions and velocities as (x, y, z) triples, phase per particle; NULL
 * leaves that array alone                                                  */
int ff_twophase3_set_particles(ff_twophase t, int n, const float *xyz, const float *vxyz, const float *phase);
int ff_twophase3_get_particles(ff_twophase t, int n, float *xyz, float *vxyz, float *phase);
/* borrowed handles: phase, liquidFraction, density (cells), beta on the u,
 * v, w faces, and the pressure solver                                      */
int ff_twophase3_fields(ff_twophase t, ff_field *phase, ff_field *liquid_fraction, ff_field *density,
                        ff_field *beta_u, ff_field *beta_v, ff_field *beta_w, ff_pressure *pressure);
/* the per-cell particle count and fixed-point concentration sum of the last
 * density stage (int32 arrays of nx ny nz), for tests.  Synchronises.      */
int ff_twophase3_cell_counts(ff_twophase t, int32_t *count, int32_t *sum);
/* destroy, set_collider, set_count, stage, step and resample_stats of a 3D
 * solver are the ff_twophase2_* calls on its handle.                       */

/* computeFlipBoxSeed3 (:70-130): per_axis^3 jittered particles per cell,
 * mulberry32(seed) (jitter_random.js:29-46), in doubles as JavaScript.
 * positions NULL: only *count.  FF_E_LIMIT when capacity is too small.    */
int ff_flip_box_seed3(const double *box_min, const double *box_max, const double *grid_spacing, int per_axis,
                      double jitter, uint32_t seed, float *positions, int64_t capacity, int64_t *count);
/* createJitterRandom(seed): the first n values                           */
int ff_jitter_random(uint32_t seed, int n, double *out);

/* ---- learned warm start (no reference counterpart): a 3-level 3D U-Net
 * (16/32/64 channels, 3x3x3 convolutions, GELU, 2x average pooling, nearest
 * upsampling with skip concatenation, a 1x1 output) mapping (divergence b,
 * solid mask, previous pressure) to a pressure guess.  BF16 weights and
 * activations, FP32 accumulation, FP32 master weights and Adam.  Inputs are
 * normalised by rms(b) and rms(p_prev) (or rms(b) L^2 / 4 pi^2 when p_prev
 * is zero); the output is in pressure units.  Resolutions must be multiples
 * of 4.  Parameters are one FP32 vector: per convolution W[27][cin][cout]
 * (tap = (dz+1) 9 + (dy+1) 3 + (dx+1)) then bias[cout], in network order,
 * then the output layer's 16 weights and bias.                            */
typedef struct ff_unet_s *ff_unet;
int ff_unet_create(ff_ctx ctx, uint32_t seed, ff_unet *out);
int ff_unet_destroy(ff_unet u);
int ff_unet_param_count(ff_unet u, int64_t *n);
int ff_unet_get_params(ff_unet u, float *host, int64_t n);
int ff_unet_set_params(ff_unet u, const float *host, int64_t n);   /* resets Adam */
int ff_unet_get_grads(ff_unet u, float *host, int64_t n);
/* p_prev and mask may be NULL; out: float cell field                     */
int ff_unet_forward(ff_unet u, const int *resolution, double grid_spacing, ff_field b, ff_field mask,
                    ff_field p_prev, ff_field out);
/* forward, MSE against target (normalised units), backward into the
 * gradient buffer (overwritten), loss in *loss                            */
int ff_unet_loss_backward(ff_unet u, const int *resolution, double grid_spacing, ff_field b, ff_field mask,
                          ff_field p_prev, ff_field target, double *loss);
int ff_unet_adam_step(ff_unet u, double lr, double beta1, double beta2, double eps);
/* Use `net` (borrowed; NULL to stop) for the initial guess of every later
 * project()/solve(): after the system is built, the network predicts p0
 * from (b, Dirichlet mask, current pressure); p0 replaces the current
 * pressure only when ||b - A p0|| < ||b - A p_prev||, and Dirichlet cells
 * keep their targets.  ff_diag.warm_start reports the choice.             */
int ff_pressure3_set_warm_start(ff_pressure ps, ff_unet net);

/* ---- test hooks mirroring the exported multigrid.js / linalg.js pieces -- */
/* createLaplacianOperator (multigrid.js:457-471): y = A x with the solver's
 * current level-0 system (call ff_pressure3_prepare first).                 */
int ff_pressure3_prepare(ff_pressure ps, ff_field u_in, ff_field v_in, ff_field w_in);
int ff_laplacian_apply(ff_pressure ps, ff_field x, ff_field y);
/* One application of the preconditioner z = M r (the V-cycle,
 * multigrid.js:1589-1642, or Jacobi / identity, :568-619).                 */
int ff_precondition_apply(ff_pressure ps, ff_field r, ff_field z);
/* buildRestrictKernel / buildCorrectKernel (multigrid.js:866-914, 990-1040)
 * on a level of the prepared hierarchy: coarse = R fine, fine += P coarse.  */
int ff_mg_restrict(ff_pressure ps, int fine_level, ff_field fine, ff_field coarse);
int ff_mg_prolong_add(ff_pressure ps, int fine_level, ff_field coarse, ff_field fine);
/* Coarsened mask / weights of a level (refreshCoarseLevels, :1416-1452).   */
int ff_mg_level_info(ff_pressure ps, int level, int *shape3);
/* Average device time (CUDA events, context stream) of one launch of a
 * kernel family on the solver's level-0 buffers: the per-dispatch timing of
 * fluxflow src/profiling.js:92-149.  Call after a project() or prepare().  */
#define FF_PROF_P_PAP 0          /* p = z + beta p, A p, p.Ap           */
#define FF_PROF_X_RESIDUAL 1     /* x += alpha p, r = b - A x, r.r      */
#define FF_PROF_RELAX 2          /* one red-black colour pass, level 0  */
#define FF_PROF_RESIDUAL 3       /* V-cycle residual, level 0           */
#define FF_PROF_RESTRICT 4       /* level 0 -> 1                        */
#define FF_PROF_PROLONG 5        /* level 1 -> 0                        */
#define FF_PROF_RZ 6             /* r.z and beta                        */
#define FF_PROF_PRECONDITIONER 7 /* one whole V-cycle                   */
#define FF_PROF_ITERATION 8      /* one whole PCG iteration             */
int ff_pressure3_profile(ff_pressure ps, int which, int reps, float *avg_ms);
int ff_mg_level_download(ff_pressure ps, int level, uint8_t *mask, float *wu, float *wv, float *ww);

#ifdef __cplusplus
}
#endif
#endif
