/*
 * ff_oracle.c -- FP64 CPU restatement of the fluxflow pressure-projection
 * path.  TEST INFRASTRUCTURE ONLY (see ff_oracle.h).
 *
 * Reference files restated here (paths inside bertJcW/tsl_array_n):
 *   packages/fluxflow/src/linalg/multigrid.js    operator, V-cycle, coarsening
 *   packages/fluxflow/src/linalg/linalg.js       PCG with guards and stop codes
 *   packages/fluxflow/src/grid/grid_pressure_solver3.js  build / correct / breaker
 *   cpu_reference.mjs                            applyA and plain CG arms
 */
#include "ff_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#define IDX(i, j, k, nx, ny) ((size_t)(i) + (size_t)(nx) * ((size_t)(j) + (size_t)(ny) * (size_t)(k)))

static inline size_t cells_of(int nx, int ny, int nz) { return (size_t)nx * ny * nz; }

/* ------------------------------------------------------------------------ */
/* float guards (float_guards.js:78-111): non-finite means exponent all ones */
int orc_is_nonfinite_f32(float v) {
    uint32_t u; memcpy(&u, &v, 4);
    return (u & 0x7f800000u) == 0x7f800000u;
}
static int nonfinite_or_above(double v, double limit) {
    /* isNonFiniteOrAbove: non-finite, or NOT(|v| <= limit) */
    return !isfinite(v) || !(fabs(v) <= limit);
}

float orc_round_bf16(float v) {
    uint32_t u; memcpy(&u, &v, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) { /* inf / nan pass through */
        if (u & 0x007fffffu) u |= 0x00400000u;
        u &= 0xffff0000u; memcpy(&v, &u, 4); return v;
    }
    uint32_t lsb = (u >> 16) & 1u;
    u += 0x7fffu + lsb;          /* round to nearest even */
    u &= 0xffff0000u;
    memcpy(&v, &u, 4);
    return v;
}

/* ------------------------------------------------------------------------ */
/* laplacianAt (multigrid.js:273-339).  The row of a masked cell is -x.  A
 * masked neighbour is eliminated: dLower -> center, dUpper -> -center.  Face
 * weights multiply after the substitution.  Edges drop the term. */
static inline double wt(const double *w, size_t idx) { return w ? w[idx] : 1.0; }

void orc_laplacian(int nx, int ny, int nz, double hx, double hy, double hz,
                   const double *x, const uint8_t *mask,
                   const double *wu, const double *wv, const double *ww,
                   double *out) {
    const double ihx = 1.0 / (hx * hx), ihy = 1.0 / (hy * hy), ihz = 1.0 / (hz * hz);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t c = IDX(i, j, k, nx, ny);
                double center = x[c];
                if (mask && mask[c]) { out[c] = -center; continue; }
                double sum = 0.0, dl, du;
                /* x axis: u faces (nx+1, ny, nz) */
                dl = 0.0; du = 0.0;
                if (i > 0) dl = (mask && mask[c - 1]) ? center : center - x[c - 1];
                if (i < nx - 1) du = (mask && mask[c + 1]) ? -center : x[c + 1] - center;
                if (wu) { size_t f = IDX(i, j, k, nx + 1, ny); dl *= wu[f]; du *= wu[f + 1]; }
                sum += (du - dl) * ihx;
                /* y axis: v faces (nx, ny+1, nz) */
                dl = 0.0; du = 0.0;
                if (j > 0) dl = (mask && mask[c - nx]) ? center : center - x[c - nx];
                if (j < ny - 1) du = (mask && mask[c + nx]) ? -center : x[c + nx] - center;
                if (wv) { size_t f = IDX(i, j, k, nx, ny + 1); dl *= wv[f]; du *= wv[f + nx]; }
                sum += (du - dl) * ihy;
                /* z axis: w faces (nx, ny, nz+1); absent in 2D (nz == 1) */
                if (nz > 1) {
                    size_t s = (size_t)nx * ny;
                    dl = 0.0; du = 0.0;
                    if (k > 0) dl = (mask && mask[c - s]) ? center : center - x[c - s];
                    if (k < nz - 1) du = (mask && mask[c + s]) ? -center : x[c + s] - center;
                    if (ww) { size_t f = c; dl *= ww[f]; du *= ww[f + s]; }
                    sum += (du - dl) * ihz;
                }
                out[c] = sum;
            }
}

/* laplacianDiagonalAt (multigrid.js:399-437): -(sum of present face
 * weights)/h^2; a masked neighbour still counts; a masked row is -1. */
void orc_laplacian_diag(int nx, int ny, int nz, double hx, double hy, double hz,
                        const uint8_t *mask, const double *wu, const double *wv,
                        const double *ww, double *out) {
    const double ihx = 1.0 / (hx * hx), ihy = 1.0 / (hy * hy), ihz = 1.0 / (hz * hz);
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t c = IDX(i, j, k, nx, ny);
                if (mask && mask[c]) { out[c] = -1.0; continue; }
                size_t fu = IDX(i, j, k, nx + 1, ny), fv = IDX(i, j, k, nx, ny + 1);
                double s = 0.0;
                s += ((i > 0 ? wt(wu, fu) : 0.0) + (i < nx - 1 ? wt(wu, fu + 1) : 0.0)) * ihx;
                s += ((j > 0 ? wt(wv, fv) : 0.0) + (j < ny - 1 ? wt(wv, fv + nx) : 0.0)) * ihy;
                if (nz > 1) {
                    size_t sl = (size_t)nx * ny;
                    s += ((k > 0 ? wt(ww, c) : 0.0) + (k < nz - 1 ? wt(ww, c + sl) : 0.0)) * ihz;
                }
                out[c] = -s;
            }
}

/* ------------------------------------------------------------------------ */
/* cpu_reference.mjs:58-90 -- 2D applyA, Math.fround on every step when
 * round_f32 is set. */
static inline double fr(double v, int r) { return r ? (double)(float)v : v; }

void orc_cpuref_apply(int nx, int ny, double hx, double hy, const double *x,
                      const uint8_t *pinned, double *out, int r) {
    const double ihx2 = fr(1.0 / (hx * hx), r), ihy2 = fr(1.0 / (hy * hy), r);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            size_t c = (size_t)i + (size_t)nx * j;
            double center = x[c];
            if (pinned[c]) { out[c] = fr(-center, r); continue; }
            double dl = 0, du = 0;
            if (i > 0) dl = pinned[c - 1] ? center : fr(center - x[c - 1], r);
            if (i < nx - 1) du = pinned[c + 1] ? -center : fr(x[c + 1] - center, r);
            double sum = fr(fr(du - dl, r) * ihx2, r);
            dl = 0; du = 0;
            if (j > 0) dl = pinned[c - nx] ? center : fr(center - x[c - nx], r);
            if (j < ny - 1) du = pinned[c + nx] ? -center : fr(x[c + nx] - center, r);
            sum = fr(sum + fr(fr(du - dl, r) * ihy2, r), r);
            out[c] = sum;
        }
}

/* cpu_reference.mjs:106-126: the three dot flavours */
static double dot_d(size_t n, const double *a, const double *c) {
    double s = 0; for (size_t i = 0; i < n; ++i) s += a[i] * c[i]; return s;
}
static double dot_f32_naive(size_t n, const double *a, const double *c) {
    float s = 0; for (size_t i = 0; i < n; ++i) s = (float)(s + (float)(a[i] * c[i])); return s;
}
static double dot_f32_lanes(size_t n, const double *a, const double *c) {
    float part[256]; memset(part, 0, sizeof part);
    for (size_t i = 0; i < n; ++i) part[i % 256] = (float)(part[i % 256] + (float)(a[i] * c[i]));
    float s = 0; for (int l = 0; l < 256; ++l) s = (float)(s + part[l]);
    return s;
}

/* cpu_reference.mjs:183-248 */
int orc_cpuref_cg(int nx, int ny, double hx, double hy, const double *b,
                  const uint8_t *pinned, const double *x0, double *x_out,
                  int r, int dot_kind, int max_iter, int recompute_every,
                  double *final_rel) {
    size_t n = (size_t)nx * ny;
    double (*dotf)(size_t, const double *, const double *) =
        dot_kind == 1 ? dot_f32_lanes : dot_kind == 2 ? dot_f32_naive : dot_d;
    double *x = calloc(n, 8), *rv = calloc(n, 8), *p = calloc(n, 8), *Ap = calloc(n, 8), *Ax = calloc(n, 8);
    if (x0) {
        memcpy(x, x0, n * 8);
        orc_cpuref_apply(nx, ny, hx, hy, x, pinned, Ax, r);
        for (size_t i = 0; i < n; ++i) { rv[i] = fr(b[i] - Ax[i], r); p[i] = rv[i]; }
    } else {
        for (size_t i = 0; i < n; ++i) { rv[i] = fr(b[i], r); p[i] = rv[i]; }
    }
    double rr = dotf(n, rv, rv);
    double bnorm = sqrt(dot_d(n, b, b));
    double target = 1e-6 * bnorm;
    int iters = 0;
    for (int k = 0; k < max_iter; ++k) {
        orc_cpuref_apply(nx, ny, hx, hy, p, pinned, Ap, r);
        double pAp = dotf(n, p, Ap);
        if (!isfinite(pAp) || pAp == 0) break;
        double alpha = fr(rr / pAp, r);
        for (size_t i = 0; i < n; ++i) { x[i] = fr(x[i] + alpha * p[i], r); rv[i] = fr(rv[i] - alpha * Ap[i], r); }
        if (recompute_every > 0 && (k + 1) % recompute_every == 0) {
            orc_cpuref_apply(nx, ny, hx, hy, x, pinned, Ax, r);
            for (size_t i = 0; i < n; ++i) rv[i] = fr(b[i] - Ax[i], r);
        }
        double rrn = dotf(n, rv, rv);
        double res = sqrt(fabs(rrn));
        iters = k + 1;
        if (res < target) break;
        double beta = fr(rrn / rr, r);
        for (size_t i = 0; i < n; ++i) p[i] = fr(rv[i] + beta * p[i], r);
        rr = rrn;
    }
    if (final_rel) *final_rel = sqrt(fabs(dot_d(n, rv, rv))) / bnorm;
    if (x_out) memcpy(x_out, x, n * 8);
    free(x); free(rv); free(p); free(Ap); free(Ax);
    return iters;
}

/* ------------------------------------------------------------------------ */
/* Multigrid (multigrid.js:1213-1735)                                        */
typedef struct {
    int nx, ny, nz;
    double hx, hy, hz;
    uint8_t *mask;        /* NULL: no mask at this level */
    double *w[3];         /* NULL: unweighted */
    double *x, *b, *buf, *diag;
    int own_mask, own_w;
} level_t;

struct orc_mg {
    int dims, L;
    orc_mg_opts o;
    level_t lv[16];
    uint8_t *vent;        /* coarseDirichletMask source */
    int has_mask, has_w, coarsening_masks;
    /* dense FP64 coarsest factorisation: B = -A = L D L^T, semidefinite */
    int nc;
    double *Lf, *Df;
    int direct_ready;
};

/* store_bf16 bits: 1 level-0 x, 2 coarse-level x and b, 4 residual buffers */
static void store_round(const orc_mg *mg, int bit, double *a, size_t n) {
    if (!(mg->o.store_bf16 & bit)) return;
    for (size_t i = 0; i < n; ++i) a[i] = (double)orc_round_bf16((float)a[i]);
}

orc_mg *orc_mg_create(int nx, int ny, int nz, double hx, double hy, double hz,
                      const orc_mg_opts *opts) {
    orc_mg *mg = calloc(1, sizeof *mg);
    mg->o = *opts;
    mg->dims = nz > 1 ? 3 : 2;
    mg->L = opts->levels < 1 ? 1 : opts->levels;
    int div = 1 << (mg->L - 1);
    if (nx % div || ny % div || (mg->dims == 3 && nz % div)) { free(mg); return NULL; }
    for (int l = 0; l < mg->L; ++l) {
        level_t *v = &mg->lv[l];
        int s = 1 << l;
        v->nx = nx / s; v->ny = ny / s; v->nz = mg->dims == 3 ? nz / s : 1;
        v->hx = hx * s; v->hy = hy * s; v->hz = hz * s;
        size_t n = cells_of(v->nx, v->ny, v->nz);
        v->x = calloc(n, 8); v->b = calloc(n, 8); v->buf = calloc(n, 8); v->diag = calloc(n, 8);
    }
    return mg;
}

void orc_mg_destroy(orc_mg *mg) {
    if (!mg) return;
    for (int l = 0; l < mg->L; ++l) {
        level_t *v = &mg->lv[l];
        free(v->x); free(v->b); free(v->buf); free(v->diag);
        free(v->mask);
        for (int a = 0; a < 3; ++a) free(v->w[a]);
    }
    free(mg->vent); free(mg->Lf); free(mg->Df);
    free(mg);
}

static size_t face_count(const level_t *v, int axis) {
    return (size_t)(v->nx + (axis == 0)) * (v->ny + (axis == 1)) * (v->nz + (axis == 2));
}

int orc_mg_set_system(orc_mg *mg, const uint8_t *mask, const uint8_t *vent,
                      const double *wu, const double *wv, const double *ww) {
    level_t *v0 = &mg->lv[0];
    size_t n0 = cells_of(v0->nx, v0->ny, v0->nz);
    mg->has_mask = mask != NULL;
    mg->has_w = wu != NULL;
    free(v0->mask); v0->mask = NULL;
    if (mask) { v0->mask = malloc(n0); memcpy(v0->mask, mask, n0); }
    free(mg->vent); mg->vent = NULL;
    /* coarseDirichletMask defaults to the whole mask (multigrid.js:278) */
    if (mask) { mg->vent = malloc(n0); memcpy(mg->vent, vent ? vent : mask, n0); }
    const double *src[3] = { wu, wv, ww };
    for (int a = 0; a < 3; ++a) {
        free(v0->w[a]); v0->w[a] = NULL;
        if (wu && (a < 2 || mg->dims == 3)) {
            size_t nf = face_count(v0, a);
            v0->w[a] = malloc(nf * 8); memcpy(v0->w[a], src[a], nf * 8);
        }
    }
    /* coarseningMasks (multigrid.js:335) */
    mg->coarsening_masks = (mg->has_mask && mg->o.coarsen_mask) || (mg->has_w && mg->o.coarsen_weights);
    for (int l = 1; l < mg->L; ++l) {
        level_t *v = &mg->lv[l];
        size_t n = cells_of(v->nx, v->ny, v->nz);
        free(v->mask); v->mask = NULL;
        if (mg->coarsening_masks) v->mask = calloc(n, 1);   /* zero: nothing pinned */
        for (int a = 0; a < 3; ++a) {
            free(v->w[a]); v->w[a] = NULL;
            if (mg->has_w && mg->o.coarsen_weights && (a < 2 || mg->dims == 3)) {
                size_t nf = face_count(v, a);
                v->w[a] = malloc(nf * 8);
                for (size_t q = 0; q < nf; ++q) v->w[a][q] = 1.0;   /* one: open */
            }
        }
    }
    mg->direct_ready = 0;
    return 0;
}

/* buildFaceWeightCoarsenKernel (multigrid.js:1138-1184): mean of the
 * 2^(d-1) fine faces under each coarse face. */
static void coarsen_weights(const orc_mg *mg, const level_t *f, level_t *c, int axis) {
    int cx = c->nx + (axis == 0), cy = c->ny + (axis == 1), cz = c->nz + (axis == 2);
    int fx = f->nx + (axis == 0), fy = f->ny + (axis == 1);
    const double *fw = f->w[axis];
    for (int k = 0; k < cz; ++k)
        for (int j = 0; j < cy; ++j)
            for (int i = 0; i < cx; ++i) {
                double s = 0; int cnt = 0;
                int ni = axis == 0 ? 1 : 2, nj = axis == 1 ? 1 : 2;
                int nk = (mg->dims == 2) ? 1 : (axis == 2 ? 1 : 2);
                for (int dk = 0; dk < nk; ++dk)
                    for (int dj = 0; dj < nj; ++dj)
                        for (int di = 0; di < ni; ++di) {
                            int fi = 2 * i + di, fj = 2 * j + dj;
                            int fk = mg->dims == 2 ? 0 : 2 * k + dk;
                            s += fw[IDX(fi, fj, fk, fx, fy)];
                            cnt++;
                        }
                c->w[axis][IDX(i, j, k, cx, cy)] = s / cnt;
            }
}

/* buildMaskCoarsenKernel (multigrid.js:1066-1122): ALL children pinned, or
 * the coarse cell is enclosed (sum of its 2d coarse face weights < 1e-6). */
static void coarsen_mask(const orc_mg *mg, const level_t *f, const uint8_t *src, level_t *c) {
    for (int k = 0; k < c->nz; ++k)
        for (int j = 0; j < c->ny; ++j)
            for (int i = 0; i < c->nx; ++i) {
                int masked = -1;
                if (src) {
                    int all = 1;
                    int nk = mg->dims == 2 ? 1 : 2;
                    for (int dk = 0; dk < nk; ++dk)
                        for (int dj = 0; dj < 2; ++dj)
                            for (int di = 0; di < 2; ++di) {
                                int fk = mg->dims == 2 ? 0 : 2 * k + dk;
                                if (!src[IDX(2 * i + di, 2 * j + dj, fk, f->nx, f->ny)]) all = 0;
                            }
                    masked = all;
                }
                if (c->w[0]) {
                    double t = c->w[0][IDX(i, j, k, c->nx + 1, c->ny)] + c->w[0][IDX(i + 1, j, k, c->nx + 1, c->ny)]
                             + c->w[1][IDX(i, j, k, c->nx, c->ny + 1)] + c->w[1][IDX(i, j + 1, k, c->nx, c->ny + 1)];
                    if (mg->dims == 3)
                        t += c->w[2][IDX(i, j, k, c->nx, c->ny)] + c->w[2][IDX(i, j, k + 1, c->nx, c->ny)];
                    int enclosed = t < 1e-6;
                    masked = masked < 0 ? enclosed : (masked || enclosed);
                }
                c->mask[IDX(i, j, k, c->nx, c->ny)] = masked > 0;
            }
}

static void factor_coarsest(orc_mg *mg);

void orc_mg_refresh(orc_mg *mg) {
    /* order: weights of a level before its mask (multigrid.js:416-438) */
    for (int l = 1; l < mg->L; ++l) {
        level_t *f = &mg->lv[l - 1], *c = &mg->lv[l];
        if (mg->has_w && mg->o.coarsen_weights)
            for (int a = 0; a < mg->dims; ++a) coarsen_weights(mg, f, c, a);
        if (!mg->coarsening_masks) continue;
        const uint8_t *src = (!mg->has_mask || !mg->o.coarsen_mask) ? NULL
                             : (l == 1 ? mg->vent : f->mask);
        coarsen_mask(mg, f, src, c);
    }
    mg->direct_ready = 0;
}

int orc_mg_level_shape(orc_mg *mg, int level, int *s) {
    if (level < 0 || level >= mg->L) return -1;
    s[0] = mg->lv[level].nx; s[1] = mg->lv[level].ny; s[2] = mg->lv[level].nz;
    return 0;
}
int orc_mg_level_mask(orc_mg *mg, int level, uint8_t *out) {
    level_t *v = &mg->lv[level];
    size_t n = cells_of(v->nx, v->ny, v->nz);
    if (!v->mask) { memset(out, 0, n); return 0; }
    memcpy(out, v->mask, n); return 1;
}
int orc_mg_level_weights(orc_mg *mg, int level, int axis, double *out) {
    level_t *v = &mg->lv[level];
    size_t nf = face_count(v, axis);
    if (!v->w[axis]) { for (size_t q = 0; q < nf; ++q) out[q] = 1.0; return 0; }
    memcpy(out, v->w[axis], nf * 8); return 1;
}

static void level_apply(const level_t *v, const double *x, double *out) {
    orc_laplacian(v->nx, v->ny, v->nz, v->hx, v->hy, v->hz, x, v->mask,
                  v->w[0], v->w[1], v->w[2], out);
}

/* buildRelaxKernel (multigrid.js:626-640): one colour, x += sor (b-Ax)/diag */
static void relax_colour(orc_mg *mg, level_t *v, int colour) {
    size_t n = cells_of(v->nx, v->ny, v->nz);
    level_apply(v, v->x, v->buf);   /* buf used as scratch for Ax */
#pragma omp parallel for schedule(static)
    for (int k = 0; k < v->nz; ++k)
        for (int j = 0; j < v->ny; ++j)
            for (int i = 0; i < v->nx; ++i) {
                if (((i + j + k) & 1) != colour) continue;
                size_t c = IDX(i, j, k, v->nx, v->ny);
                double upd = v->x[c] + (v->b[c] - v->buf[c]) / v->diag[c] * mg->o.sor;
                int bit = v == &mg->lv[0] ? 1 : 2;
                v->x[c] = (mg->o.store_bf16 & bit) ? (double)orc_round_bf16((float)upd) : upd;
            }
    (void)n;
}

static void relax(orc_mg *mg, int l, int iters, int reversed) {
    level_t *v = &mg->lv[l];
    for (int it = 0; it < iters; ++it) {
        relax_colour(mg, v, reversed ? 1 : 0);
        relax_colour(mg, v, reversed ? 0 : 1);
    }
}

/* restrictionTapsForAxis (multigrid.js:847-864) */
static void rtaps(int c, int nc, int *idx, double *w) {
    idx[0] = c > 0 ? 2 * c - 1 : 2 * c; w[0] = 0.125;
    idx[1] = 2 * c;                      w[1] = 0.375;
    idx[2] = 2 * c + 1;                  w[2] = 0.375;
    idx[3] = c + 1 < nc ? 2 * c + 2 : 2 * c + 1; w[3] = 0.125;
}

/* buildRestrictKernel (multigrid.js:866-914): fine-masked values read as 0,
 * coarse-masked results are 0. */
void orc_restrict(int fnx, int fny, int fnz, const double *fine,
                  const uint8_t *fine_mask, const uint8_t *coarse_mask,
                  double *coarse) {
    int d3 = fnz > 1;
    int cnx = fnx / 2, cny = fny / 2, cnz = d3 ? fnz / 2 : 1;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < cnz; ++k)
        for (int j = 0; j < cny; ++j)
            for (int i = 0; i < cnx; ++i) {
                int ii[4], jj[4], kk[4]; double wi[4], wj[4], wk[4];
                rtaps(i, cnx, ii, wi); rtaps(j, cny, jj, wj);
                int nk = 1;
                if (d3) { rtaps(k, cnz, kk, wk); nk = 4; } else { kk[0] = 0; wk[0] = 1.0; }
                double s = 0;
                for (int a = 0; a < nk; ++a)
                    for (int b2 = 0; b2 < 4; ++b2)
                        for (int q = 0; q < 4; ++q) {
                            size_t f = IDX(ii[q], jj[b2], kk[a], fnx, fny);
                            double val = (fine_mask && fine_mask[f]) ? 0.0 : fine[f];
                            s += val * (wi[q] * wj[b2] * wk[a]);
                        }
                size_t cc = IDX(i, j, k, cnx, cny);
                coarse[cc] = (coarse_mask && coarse_mask[cc]) ? 0.0 : s;
            }
}

/* correctionTapsForAxis (multigrid.js:924-938) */
static void ptaps(int f, int nc, int *idx, double *w) {
    int ci = f / 2, even = (f % 2) == 0;
    int lo = ci > 0 ? ci - 1 : ci, hi = ci < nc - 1 ? ci + 1 : ci;
    if (even) { idx[0] = lo; w[0] = 0.25; idx[1] = ci; w[1] = 0.75; }
    else      { idx[0] = ci; w[0] = 0.75; idx[1] = hi; w[1] = 0.25; }
}

/* buildCorrectKernel (multigrid.js:990-1040): fine += P coarse, skipped on
 * fine-masked cells. */
void orc_prolong_add(int fnx, int fny, int fnz, const double *coarse,
                     const uint8_t *fine_mask, double *fine) {
    int d3 = fnz > 1;
    int cnx = fnx / 2, cny = fny / 2, cnz = d3 ? fnz / 2 : 1;
#pragma omp parallel for schedule(static)
    for (int k = 0; k < fnz; ++k)
        for (int j = 0; j < fny; ++j)
            for (int i = 0; i < fnx; ++i) {
                size_t f = IDX(i, j, k, fnx, fny);
                if (fine_mask && fine_mask[f]) continue;
                int ii[2], jj[2], kk[2]; double wi[2], wj[2], wk[2];
                ptaps(i, cnx, ii, wi); ptaps(j, cny, jj, wj);
                int nk = 1;
                if (d3) { ptaps(k, cnz, kk, wk); nk = 2; } else { kk[0] = 0; wk[0] = 1.0; }
                double s = 0;
                for (int a = 0; a < nk; ++a)
                    for (int b2 = 0; b2 < 2; ++b2)
                        for (int q = 0; q < 2; ++q)
                            s += coarse[IDX(ii[q], jj[b2], kk[a], cnx, cny)] * (wi[q] * wj[b2] * wk[a]);
                fine[f] += s;
            }
}

/* FP64 direct coarsest solve: B = -A (positive semidefinite), factored as
 * L D L^T without pivoting; a pivot that vanishes (relative to the original
 * diagonal) marks a null direction and its D^+ entry is 0.  The resulting
 * generalised inverse -L^-T D^+ L^-1 is symmetric, as PCG needs. */
static void factor_coarsest(orc_mg *mg) {
    level_t *v = &mg->lv[mg->L - 1];
    int n = (int)cells_of(v->nx, v->ny, v->nz);
    mg->nc = n;
    free(mg->Lf); free(mg->Df);
    mg->Lf = calloc((size_t)n * n, 8); mg->Df = calloc(n, 8);
    double *B = mg->Lf, *e = calloc(n, 8), *col = calloc(n, 8);
    for (int q = 0; q < n; ++q) {
        memset(e, 0, n * 8); e[q] = 1.0;
        level_apply(v, e, col);
        for (int p = 0; p < n; ++p) B[(size_t)p * n + q] = -col[p];
    }
    double *orig = calloc(n, 8);
    for (int j = 0; j < n; ++j) orig[j] = B[(size_t)j * n + j];
    /* in-place LDL^T in the lower triangle; B[j][j] holds d_j */
    for (int j = 0; j < n; ++j) {
        double d = B[(size_t)j * n + j];
        for (int k = 0; k < j; ++k) d -= B[(size_t)j * n + k] * B[(size_t)j * n + k] * mg->Df[k];
        int zero = !(d > 1e-10 * fabs(orig[j])) || orig[j] == 0.0;
        mg->Df[j] = zero ? 0.0 : d;
        for (int i = j + 1; i < n; ++i) {
            if (zero) { B[(size_t)i * n + j] = 0.0; continue; }
            double s = B[(size_t)i * n + j];
            for (int k = 0; k < j; ++k) s -= B[(size_t)i * n + k] * B[(size_t)j * n + k] * mg->Df[k];
            B[(size_t)i * n + j] = s / d;
        }
    }
    free(e); free(col); free(orig);
    mg->direct_ready = 1;
}

static void coarse_direct(orc_mg *mg) {
    if (!mg->direct_ready) factor_coarsest(mg);
    level_t *v = &mg->lv[mg->L - 1];
    int n = mg->nc;
    double *y = calloc(n, 8);
    const double *L = mg->Lf;
    /* B y = -b  (A x = b with A = -B, x = y) */
    for (int i = 0; i < n; ++i) {
        double s = -v->b[i];
        for (int k = 0; k < i; ++k) s -= L[(size_t)i * n + k] * y[k];
        y[i] = s;
    }
    for (int i = 0; i < n; ++i) y[i] = mg->Df[i] > 0 ? y[i] / mg->Df[i] : 0.0;
    for (int i = n - 1; i >= 0; --i) {
        double s = y[i];
        for (int k = i + 1; k < n; ++k) s -= L[(size_t)k * n + i] * y[k];
        y[i] = s;
    }
    for (int i = 0; i < n; ++i) v->x[i] = y[i];
    store_round(mg, mg->L == 1 ? 1 : 2, v->x, n);
    free(y);
}

static void vcycle(orc_mg *mg, int l) {
    level_t *v = &mg->lv[l];
    size_t n = cells_of(v->nx, v->ny, v->nz);
    if (l == mg->L - 1) {
        if (mg->o.coarse_direct) coarse_direct(mg);
        else relax(mg, l, mg->o.coarsest, 0);
        return;
    }
    level_t *c = &mg->lv[l + 1];
    relax(mg, l, mg->o.down, 0);
    /* buildResidualKernel (multigrid.js:741-749) */
    level_apply(v, v->x, v->buf);
    for (size_t q = 0; q < n; ++q) v->buf[q] = v->b[q] - v->buf[q];
    store_round(mg, 4, v->buf, n);
    orc_restrict(v->nx, v->ny, v->nz, v->buf, v->mask, c->mask, c->b);
    size_t nc = cells_of(c->nx, c->ny, c->nz);
    store_round(mg, 2, c->b, nc);
    memset(c->x, 0, nc * 8);
    vcycle(mg, l + 1);
    orc_prolong_add(v->nx, v->ny, v->nz, c->x, v->mask, v->x);
    store_round(mg, l == 0 ? 1 : 2, v->x, n);
    relax(mg, l, l > 0 ? mg->o.up : mg->o.final_iters, 1);
}

void orc_mg_apply(orc_mg *mg, const double *r, double *z) {
    level_t *v = &mg->lv[0];
    size_t n = cells_of(v->nx, v->ny, v->nz);
    for (int l = 0; l < mg->L; ++l) {
        level_t *q = &mg->lv[l];
        orc_laplacian_diag(q->nx, q->ny, q->nz, q->hx, q->hy, q->hz, q->mask,
                           q->w[0], q->w[1], q->w[2], q->diag);
    }
    memcpy(v->b, r, n * 8);
    memset(v->x, 0, n * 8);
    vcycle(mg, 0);
    memcpy(z, v->x, n * 8);
}

/* ------------------------------------------------------------------------ */
/* PCG, GPU-resident chunked path (linalg.js:1030-1311, 1651-1911).          */
enum { STOP_NONE = 0, STOP_DEGENERATE_PAP = 1, STOP_PAP_GROWTH = 2,
       STOP_ALPHA_MAGNITUDE = 3, STOP_DEGENERATE_OLD_RZ = 4, STOP_CONVERGED = 5,
       STOP_RESIDUAL_GROWING = 6 };

static double par_dot(size_t n, const double *a, const double *b) {
    double s = 0;
#pragma omp parallel for reduction(+:s) schedule(static)
    for (size_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

int orc_pcg_solve(int nx, int ny, int nz, double hx, double hy, double hz,
                  const uint8_t *mask, const double *wu, const double *wv,
                  const double *ww, orc_mg *mg, int pre, const double *b,
                  double *x, double tol, int max_iter, int relative,
                  int *last_iters, orc_pcg_result *res) {
    size_t n = cells_of(nx, ny, nz);
    double *r = malloc(n * 8), *z = malloc(n * 8), *p = calloc(n, 8), *Ap = malloc(n * 8),
           *Ax = malloc(n * 8), *dg = NULL;
    if (pre == ORC_PRE_JACOBI) {
        dg = malloc(n * 8);
        orc_laplacian_diag(nx, ny, nz, hx, hy, hz, mask, wu, wv, nz > 1 ? ww : NULL, dg);
    }
    const double *w3 = nz > 1 ? ww : NULL;
#define APPLY(in, out) orc_laplacian(nx, ny, nz, hx, hy, hz, in, mask, wu, wv, w3, out)
#define PRECOND() do { \
        if (pre == ORC_PRE_MG) orc_mg_apply(mg, r, z); \
        else if (pre == ORC_PRE_JACOBI) { for (size_t q = 0; q < n; ++q) z[q] = fabs(dg[q]) > 0 ? r[q] / dg[q] : r[q]; } \
        else memcpy(z, r, n * 8); } while (0)

    /* setup sequence (linalg.js:1627-1637) */
    APPLY(x, Ax);
    for (size_t q = 0; q < n; ++q) r[q] = b[q] - Ax[q];
    double rr = par_dot(n, r, r), bb = par_dot(n, b, b);
    PRECOND();
    double rz = par_dot(n, r, z);
    for (size_t q = 0; q < n; ++q) p[q] = z[q];
    double rz_old = rz, baseline = fmax(fabs(rr), 1e-12);
    int stop = STOP_NONE, iter = 0, stop_iter = 0;
    double thr = relative ? fmax(tol * sqrt(fabs(bb)), tol) : tol;

    int ran = 0, result = 0, stopped_by = STOP_NONE;
    double best = -1;
    int last = last_iters ? *last_iters : 4;
    while (ran < max_iter) {
        int target = last + 2 > 4 ? last + 2 : 4;
        int chunk = target - ran > 4 ? target - ran : 4;
        if (chunk > max_iter - ran) chunk = max_iter - ran;
        for (int it = 0; it < chunk; ++it) {
            /* Ap, pAp, alpha kernel (linalg.js:1147-1199) */
            APPLY(p, Ap);
            double pAp = par_dot(n, p, Ap);
            double value = rz_old / pAp;
            int code = STOP_NONE;
            if (!isfinite(pAp) || pAp == 0) code = STOP_DEGENERATE_PAP;
            else if (fabs(pAp) > baseline * 1e8) code = STOP_PAP_GROWTH;
            else if (nonfinite_or_above(value, 1e6)) code = STOP_ALPHA_MAGNITUDE;
            double alpha = (stop != STOP_NONE || code != STOP_NONE) ? 0.0 : value;
            if (stop == STOP_NONE) stop = code;
            for (size_t q = 0; q < n; ++q) x[q] += alpha * p[q];
            APPLY(x, Ax);
            for (size_t q = 0; q < n; ++q) r[q] = b[q] - Ax[q];
            rr = par_dot(n, r, r);
            PRECOND();
            rz = par_dot(n, r, z);
            /* beta kernel (linalg.js:1201-1240) */
            double bval = rz / rz_old;
            int degenerate = !isfinite(rz_old) || rz_old == 0;
            int restart = (rz_old * rz < 0) || nonfinite_or_above(bval, 10.0);
            int already = stop != STOP_NONE;
            double beta = (already || restart) ? 0.0 : bval;
            if (degenerate && stop == STOP_NONE) stop = STOP_DEGENERATE_OLD_RZ;
            rz_old = rz;
            for (size_t q = 0; q < n; ++q) p[q] = z[q] + beta * p[q];
            /* convergence kernel (linalg.js:1283-1311) */
            iter++;
            double resid = sqrt(fabs(rr));
            int conv = !nonfinite_or_above(resid, thr);
            if (conv && stop == STOP_NONE) { stop = STOP_CONVERGED; stop_iter = iter; }
        }
        ran += chunk;
        /* host chunk read (linalg.js:1839-1905) */
        if (isfinite(rr)) {
            if (best < 0 || fabs(rr) < best) best = fabs(rr);
            else if (best > 0 && fabs(rr) > best * 100 && stop != STOP_CONVERGED) {
                stopped_by = STOP_RESIDUAL_GROWING; last = ran; result = 0;
                res->iterations = ran; goto done;
            }
        }
        if (stop == STOP_CONVERGED) {
            res->iterations = stop_iter; last = stop_iter; result = 1; goto done;
        }
        if (stop != STOP_NONE) {
            if (!(sqrt(fabs(rr)) < thr)) stopped_by = stop;
            last = ran; result = 0; res->iterations = ran; goto done;
        }
    }
    last = ran; result = 0; res->iterations = ran;
done:
    if (last_iters) *last_iters = last;
    res->converged = result;
    res->stop_code = stop;
    res->stopped_by = stopped_by;
    res->rr = rr; res->bb = bb; res->residual = sqrt(fabs(rr));
    free(r); free(z); free(p); free(Ap); free(Ax); free(dg);
#undef APPLY
#undef PRECOND
    return result;
}

/* ------------------------------------------------------------------------ */
/* grid_pressure_solver3.js                                                  */
void orc_dirichlet_fields(int nx, int ny, int nz, const uint8_t *active,
                          const double *target, const double *cwu,
                          const double *cwv, const double *cww, uint8_t *mask,
                          double *tgt, uint8_t *vent) {
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t c = IDX(i, j, k, nx, ny);
                int enclosed = 0;
                if (cwu) {
                    /* totalColliderWeight (:163-169) */
                    double t = cwu[IDX(i, j, k, nx + 1, ny)] + cwu[IDX(i + 1, j, k, nx + 1, ny)]
                             + cwv[IDX(i, j, k, nx, ny + 1)] + cwv[IDX(i, j + 1, k, nx, ny + 1)];
                    if (nz > 1) t += cww[c] + cww[c + (size_t)nx * ny];
                    enclosed = t < 1e-6;
                }
                int act = active ? active[c] != 0 : 0;
                mask[c] = act || enclosed;
                tgt[c] = act ? (target ? target[c] : 0.0) : 0.0;
                vent[c] = act;
            }
}

void orc_build_system(int nx, int ny, int nz, double hx, double hy, double hz,
                      const double *u, const double *v, const double *w,
                      const double *cwu, const double *cwv, const double *cww,
                      const double *fwu, const double *fwv, const double *fww,
                      const uint8_t *mask, const double *tgt, double *b,
                      double *p) {
    const double ihx = 1 / (hx * hx), ihy = 1 / (hy * hy), ihz = 1 / (hz * hz);
    size_t s = (size_t)nx * ny;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                size_t c = IDX(i, j, k, nx, ny);
                size_t fu = IDX(i, j, k, nx + 1, ny), fv = IDX(i, j, k, nx, ny + 1), fw = c;
                /* weightedDivergence (:412-427) */
                double lu = u[fu] * (cwu ? cwu[fu] : 1), ru = u[fu + 1] * (cwu ? cwu[fu + 1] : 1);
                double lv = v[fv] * (cwv ? cwv[fv] : 1), rv = v[fv + nx] * (cwv ? cwv[fv + nx] : 1);
                double div = (ru - lu) / hx + (rv - lv) / hy;
                if (nz > 1) {
                    double lw = w[fw] * (cww ? cww[fw] : 1), rw = w[fw + s] * (cww ? cww[fw + s] : 1);
                    div += (rw - lw) / hz;
                }
                if (!mask) { b[c] = div; continue; }
                if (mask[c]) { b[c] = -tgt[c]; p[c] = tgt[c]; continue; }
                /* neighbourDirichletContribution (:350-394): system weight
                 * = faceWeight * colliderWeight */
#define SW(fwx, cwx, f) (((fwx) ? (fwx)[f] : 1.0) * ((cwx) ? (cwx)[f] : 1.0))
                int hasw = fwu || cwu;
                double acc = 0;
                if (i > 0 && mask[c - 1]) acc += (hasw ? SW(fwu, cwu, fu) : 1.0) * tgt[c - 1] * ihx;
                if (i < nx - 1 && mask[c + 1]) acc += (hasw ? SW(fwu, cwu, fu + 1) : 1.0) * tgt[c + 1] * ihx;
                if (j > 0 && mask[c - nx]) acc += (hasw ? SW(fwv, cwv, fv) : 1.0) * tgt[c - nx] * ihy;
                if (j < ny - 1 && mask[c + nx]) acc += (hasw ? SW(fwv, cwv, fv + nx) : 1.0) * tgt[c + nx] * ihy;
                if (nz > 1) {
                    if (k > 0 && mask[c - s]) acc += (hasw ? SW(fww, cww, fw) : 1.0) * tgt[c - s] * ihz;
                    if (k < nz - 1 && mask[c + s]) acc += (hasw ? SW(fww, cww, fw + s) : 1.0) * tgt[c + s] * ihz;
                }
#undef SW
                b[c] = div - acc;
            }
}

void orc_correct(int nx, int ny, int nz, double hx, double hy, double hz,
                 const double *p, const double *fwu, const double *fwv,
                 const double *fww, const double *cwu, const double *cwv,
                 const double *cww, const double *uin, const double *vin,
                 const double *win, double *uout, double *vout, double *wout) {
    size_t s = (size_t)nx * ny;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int m = 1; m < nx; ++m) {
                size_t f = IDX(m, j, k, nx + 1, ny);
                double g = (p[IDX(m, j, k, nx, ny)] - p[IDX(m - 1, j, k, nx, ny)]) / hx;
                if (fwu) g *= fwu[f];
                if (cwu) g *= cwu[f] > 0 ? 1.0 : 0.0;
                uout[f] = uin[f] - g;
            }
    for (int k = 0; k < nz; ++k)
        for (int m = 1; m < ny; ++m)
            for (int i = 0; i < nx; ++i) {
                size_t f = IDX(i, m, k, nx, ny + 1);
                double g = (p[IDX(i, m, k, nx, ny)] - p[IDX(i, m - 1, k, nx, ny)]) / hy;
                if (fwv) g *= fwv[f];
                if (cwv) g *= cwv[f] > 0 ? 1.0 : 0.0;
                vout[f] = vin[f] - g;
            }
    if (nz > 1)
        for (int m = 1; m < nz; ++m)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    size_t f = IDX(i, j, m, nx, ny);
                    double g = (p[f] - p[f - s]) / hz;
                    if (fww) g *= fww[f];
                    if (cww) g *= cww[f] > 0 ? 1.0 : 0.0;
                    wout[f] = win[f] - g;
                }
}

int orc_count_bad(int n, const double *p, double max_plausible) {
    int cnt = 0;
    for (int i = 0; i < n; ++i) cnt += nonfinite_or_above(p[i], max_plausible);
    return cnt;
}

/* ------------------------------------------------------------------------ */
/* Collider SDF bake and face weights (sdf_collider3.js:69-99, 131-254;     */
/* level_set_utils.js:51-161; primitive_sdf3.js:169-208), FP64 like the     */
/* reference's CPU code, stored f32.  shapes: n x 12 doubles                 */
/* [type, cx, cy, cz, radius, hx, hy, hz, has_rot, ax, ay, az] + angle at    */
/* index 12 (13 per shape).                                                  */
static double orc_prim_distance(const double *s, double x, double y, double z) {
    double lx = x - s[1], ly = y - s[2], lz = z - s[3];
    if (s[0] == 0) return sqrt(lx * lx + ly * ly + lz * lz) - s[4];
    double qx = lx, qy = ly, qz = lz;
    if (s[8] != 0) {
        double len = sqrt(s[9] * s[9] + s[10] * s[10] + s[11] * s[11]);
        double kx = len > 0 ? s[9] / len : 0, ky = len > 0 ? s[10] / len : 0, kz = len > 0 ? s[11] / len : 1;
        double a = -s[12], c = cos(a), sn = sin(a);
        double cx = ky * lz - kz * ly, cy = kz * lx - kx * lz, cz = kx * ly - ky * lx;
        double kd = kx * lx + ky * ly + kz * lz;
        qx = lx * c + cx * sn + kx * kd * (1 - c);
        qy = ly * c + cy * sn + ky * kd * (1 - c);
        qz = lz * c + cz * sn + kz * kd * (1 - c);
    }
    double dx = fabs(qx) - s[5], dy = fabs(qy) - s[6], dz = fabs(qz) - s[7];
    double mx = fmax(dx, 0), my = fmax(dy, 0), mz = fmax(dz, 0);
    return sqrt(mx * mx + my * my + mz * mz) + fmin(fmax(dx, fmax(dy, dz)), 0.0);
}

static double orc_shapes_distance(const double *sh, int n, double x, double y, double z) {
    double d = INFINITY;
    for (int q = 0; q < n; ++q) d = fmin(d, orc_prim_distance(sh + 13 * q, x, y, z));
    return d;
}

static double frac_sdf(double p0, double p1) {
    int i0 = p0 < 0, i1 = p1 < 0;
    if (i0 && i1) return 1;
    if (i0 && !i1) return p0 / (p0 - p1);
    if (!i0 && i1) return p1 / (p1 - p0);
    return 0;
}

static void cycle4(double *a) { double t = a[0]; a[0] = a[1]; a[1] = a[2]; a[2] = a[3]; a[3] = t; }

double orc_fraction_inside(double bl, double br, double tl, double tr) {
    int cnt = (bl < 0) + (tl < 0) + (br < 0) + (tr < 0);
    double L[4] = { bl, br, tr, tl };
    if (cnt == 4) return 1;
    if (cnt == 3) {
        for (int g = 0; g < 4 && L[0] < 0; ++g) cycle4(L);
        double s0 = 1 - frac_sdf(L[0], L[3]), s1 = 1 - frac_sdf(L[0], L[1]);
        return 1 - 0.5 * s0 * s1;
    }
    if (cnt == 2) {
        for (int g = 0; g < 4 && (L[0] >= 0 || !(L[1] < 0 || L[2] < 0)); ++g) cycle4(L);
        if (L[1] < 0) return 0.5 * (frac_sdf(L[0], L[3]) + frac_sdf(L[1], L[2]));
        double mid = 0.25 * (L[0] + L[1] + L[2] + L[3]);
        if (mid < 0) {
            double area = 0.5 * (1 - frac_sdf(L[0], L[3])) * (1 - frac_sdf(L[2], L[3]));
            area += 0.5 * (1 - frac_sdf(L[0], L[1])) * (1 - frac_sdf(L[2], L[1]));
            return 1 - area;
        }
        double area = 0.5 * frac_sdf(L[0], L[1]) * frac_sdf(L[0], L[3]);
        area += 0.5 * frac_sdf(L[2], L[1]) * frac_sdf(L[2], L[3]);
        return area;
    }
    if (cnt == 1) {
        for (int g = 0; g < 4 && L[0] >= 0; ++g) cycle4(L);
        return 0.5 * frac_sdf(L[0], L[3]) * frac_sdf(L[0], L[1]);
    }
    return 0;
}

void orc_collider_bake(const double *shapes, int nshapes, int invert, int nx, int ny, int nz,
                       double hx, double hy, double hz, double ox, double oy, double oz,
                       float *phi, float *wu, float *wv, float *ww) {
    const double sign = invert ? -1.0 : 1.0;
    if (phi) {
#pragma omp parallel for schedule(static)
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    double x = (ox + 0.5 * hx) + i * hx, y = (oy + 0.5 * hy) + j * hy, z = (oz + 0.5 * hz) + k * hz;
                    phi[IDX(i, j, k, nx, ny)] = (float)(sign * orc_shapes_distance(shapes, nshapes, x, y, z));
                }
    }
    float *outs[3] = { wu, wv, ww };
    const double hh[3] = { 0.5 * hx, 0.5 * hy, 0.5 * hz };
    for (int a = 0; a < 3; ++a) {
        float *w = outs[a];
        if (!w) continue;
        int fx = nx + (a == 0), fy = ny + (a == 1), fz = nz + (a == 2);
        double o[3] = { ox + (a != 0 ? hh[0] : 0), oy + (a != 1 ? hh[1] : 0), oz + (a != 2 ? hh[2] : 0) };
        double off[4][3];
        if (a == 0) { double t[4][3] = {{0,-hh[1],-hh[2]},{0,hh[1],-hh[2]},{0,-hh[1],hh[2]},{0,hh[1],hh[2]}}; memcpy(off, t, sizeof t); }
        else if (a == 1) { double t[4][3] = {{-hh[0],0,-hh[2]},{hh[0],0,-hh[2]},{-hh[0],0,hh[2]},{hh[0],0,hh[2]}}; memcpy(off, t, sizeof t); }
        else { double t[4][3] = {{-hh[0],-hh[1],0},{hh[0],-hh[1],0},{-hh[0],hh[1],0},{hh[0],hh[1],0}}; memcpy(off, t, sizeof t); }
#pragma omp parallel for schedule(static)
        for (int k = 0; k < fz; ++k)
            for (int j = 0; j < fy; ++j)
                for (int i = 0; i < fx; ++i) {
                    double x = o[0] + i * hx, y = o[1] + j * hy, z = o[2] + k * hz, c[4];
                    for (int q = 0; q < 4; ++q)
                        c[q] = sign * orc_shapes_distance(shapes, nshapes, x + off[q][0], y + off[q][1], z + off[q][2]);
                    double frac = orc_fraction_inside(c[0], c[1], c[2], c[3]);
                    double wv2 = fmin(1.0, fmax(0.0, 1.0 - frac));
                    if (c[0] <= 0 && c[1] <= 0 && c[2] <= 0 && c[3] <= 0) wv2 = 0;
                    else if (wv2 > 0 && wv2 < 0.01) wv2 = 0.01;
                    w[IDX(i, j, k, fx, fy)] = (float)wv2;
                }
    }
}
