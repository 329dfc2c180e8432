/*
 * ff_oracle -- FP64 CPU restatement of the fluxflow grid-fluid hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library (libff.so) links,
 * loads or calls this code.  Only tests/, __graft_entry__.smoke() and the CPU
 * baseline arm of bench.py use it, and only to check or time against it.
 *
 * Every function restates one piece of the reference (bertJcW/tsl_array_n,
 * package fluxflow) and cites the file:line it follows.  Layout everywhere is
 * the reference's i-fastest layout (tsl_array_n src/array.js:24-38):
 *   cell (i,j,k)        -> i + nx*(j + ny*k)
 *   u face (i,j,k)      -> i + (nx+1)*(j + ny*k)      shape (nx+1, ny, nz)
 *   v face (i,j,k)      -> i + nx*(j + (ny+1)*k)      shape (nx, ny+1, nz)
 *   w face (i,j,k)      -> i + nx*(j + ny*k)          shape (nx, ny, nz+1)
 * A 2D grid is nz == 1 and is treated as having no third axis.
 */
#ifndef FF_ORACLE_H
#define FF_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- operator (multigrid.js:273-339, :399-437) -------------------------- */
void orc_laplacian(int nx, int ny, int nz, double hx, double hy, double hz,
                   const double *x, const uint8_t *mask,
                   const double *wu, const double *wv, const double *ww,
                   double *out);
void orc_laplacian_diag(int nx, int ny, int nz, double hx, double hy, double hz,
                        const uint8_t *mask, const double *wu, const double *wv,
                        const double *ww, double *out);

/* cpu_reference.mjs:58-90 applyA, with optional float32 rounding of every
 * step (Math.fround).  2D only, no weights. */
void orc_cpuref_apply(int nx, int ny, double hx, double hy, const double *x,
                      const uint8_t *pinned, double *out, int round_f32);
/* cpu_reference.mjs:183-248 cg(): returns iterations, writes final relative
 * residual.  dot_kind: 0 double, 1 f32 lanes(256), 2 f32 naive. */
int orc_cpuref_cg(int nx, int ny, double hx, double hy, const double *b,
                  const uint8_t *pinned, const double *x0, double *x_out,
                  int round_f32, int dot_kind, int max_iter, int recompute_every,
                  double *final_rel);

/* ---- multigrid preconditioner (multigrid.js:1213-1735) ------------------ */
typedef struct orc_mg orc_mg;
typedef struct {
    int levels, down, up, coarsest, final_iters;
    double sor;
    int coarsen_mask, coarsen_weights;
    int coarse_direct;   /* 0: coarsest RB sweeps (reference); 1: FP64 direct */
    int store_bf16;      /* emulate BF16 storage of V-cycle arrays            */
} orc_mg_opts;

orc_mg *orc_mg_create(int nx, int ny, int nz, double hx, double hy, double hz,
                      const orc_mg_opts *opts);
void orc_mg_destroy(orc_mg *mg);
/* mask / vent: u8 cell arrays or NULL; wu/wv/ww: face arrays or NULL.  The
 * arrays are copied.  refresh coarsens masks and weights per level
 * (refreshCoarseLevels, multigrid.js:1416-1452). */
int orc_mg_set_system(orc_mg *mg, const uint8_t *mask, const uint8_t *vent,
                      const double *wu, const double *wv, const double *ww);
void orc_mg_refresh(orc_mg *mg);
void orc_mg_apply(orc_mg *mg, const double *r, double *z);
/* level introspection for tests */
int orc_mg_level_shape(orc_mg *mg, int level, int *shape3);
int orc_mg_level_mask(orc_mg *mg, int level, uint8_t *out);
int orc_mg_level_weights(orc_mg *mg, int level, int axis, double *out);
/* restrict (multigrid.js:866-914) and correct (:990-1040) in isolation */
void orc_restrict(int fnx, int fny, int fnz, const double *fine,
                  const uint8_t *fine_mask, const uint8_t *coarse_mask,
                  double *coarse);
void orc_prolong_add(int fnx, int fny, int fnz, const double *coarse,
                     const uint8_t *fine_mask, double *fine);

/* ---- PCG (linalg.js:782-2469, GPU-resident chunked path) ---------------- */
typedef struct {
    int converged, iterations, stop_code, stopped_by;
    double rr, bb, residual;
} orc_pcg_result;
enum { ORC_PRE_MG = 0, ORC_PRE_JACOBI = 1, ORC_PRE_NONE = 2 };
/* x is the initial guess and the output.  last_iters is the chunk-size
 * memory of the previous solve (linalg.js:942-951); pass 4 for a fresh
 * solver.  mg may be NULL unless pre == ORC_PRE_MG. */
int orc_pcg_solve(int nx, int ny, int nz, double hx, double hy, double hz,
                  const uint8_t *mask, const double *wu, const double *wv,
                  const double *ww, orc_mg *mg, int pre, const double *b,
                  double *x, double tol, int max_iter, int relative,
                  int *last_iters, orc_pcg_result *res);

/* ---- pressure projection (grid_pressure_solver3.js) --------------------- */
/* updateDirichletFields (:163-206): active/target may be NULL; cw* collider
 * weights may be NULL.  Writes mask/target/vent (u8, f64, u8). */
void orc_dirichlet_fields(int nx, int ny, int nz, const uint8_t *active,
                          const double *target, const double *cwu,
                          const double *cwv, const double *cww, uint8_t *mask,
                          double *tgt, uint8_t *vent);
/* dispatchBuildSystem (:350-453): writes b and pins p. */
void orc_build_system(int nx, int ny, int nz, double hx, double hy, double hz,
                      const double *u, const double *v, const double *w,
                      const double *cwu, const double *cwv, const double *cww,
                      const double *fwu, const double *fwv, const double *fww,
                      const uint8_t *mask, const double *tgt, double *b,
                      double *p);
/* dispatchCorrectU/V/W (:457-494): interior faces only. */
void orc_correct(int nx, int ny, int nz, double hx, double hy, double hz,
                 const double *p, const double *fwu, const double *fwv,
                 const double *fww, const double *cwu, const double *cwv,
                 const double *cww, const double *uin, const double *vin,
                 const double *win, double *uout, double *vout, double *wout);
/* countBadPressureCells (:297-304) */
int orc_count_bad(int n, const double *p, double max_plausible);

/* collider bake (sdf_collider3.js:69-99, 131-254): shapes are 13 doubles
 * each [type(0 sphere,1 box), cx, cy, cz, radius, hx, hy, hz, has_rot, ax,
 * ay, az, angle]; any output may be NULL. */
double orc_fraction_inside(double bl, double br, double tl, double tr);
void orc_collider_bake(const double *shapes, int nshapes, int invert, int nx, int ny, int nz,
                       double hx, double hy, double hz, double ox, double oy, double oz,
                       float *phi, float *wu, float *wv, float *ww);

/* float32 guards (float_guards.js) */
int orc_is_nonfinite_f32(float v);
float orc_round_bf16(float v);

#ifdef __cplusplus
}
#endif
#endif
