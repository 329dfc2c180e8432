/*
 * Oracle (test infrastructure only): CPU restatement of fluxflow's 3D FLIP
 * stages (src/grid/grid_flip_solver3.js) in FP32, one IEEE operation at a
 * time (built with -ffp-contract=off), and of its seeding in doubles as
 * JavaScript computes it.
 *
 *   mulberry32                      jitter_random.js:29-46
 *   computeFlipBoxSeed3             grid_flip_solver3.js:70-130
 *   cellIndexOf / markFluidCells    :227-245
 *   dirichlet(pos)                  :252-259 (reduced pressure target)
 *   P2G scatter / finalize          :508-568 (int32 fixed point, wraps)
 *   fluid-adjacent faces            :586-618
 *   concentration, cell density, beta faces, reduced gravity, mix/fade
 *                                   :265-359, :848-884, :960-1049
 *   G2P                             :909-922
 *   advectParticles, pushOutOfCollider :925-957
 *   resamplePass                    :621-820
 * and of the 2D two-phase solver (grid_two_phase_flip_solver2.js):
 *   countPhases / density / beta    :646-762
 *   g2pUpdate (per-phase blend)     :966-992
 *   mixConcentration                :1055-1073
 *   per-phase resamplePass          :1226-1494
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ---- mulberry32 (jitter_random.js:29-41) ---------------------------- */
typedef struct {
    uint32_t state;
} orc_rng;

static double rng_next(orc_rng *r) {
    r->state = r->state + 0x6D2B79F5u;
    uint32_t t = r->state;
    t = (t ^ (t >> 15)) * (t | 1u);
    t ^= t + (t ^ (t >> 7)) * (t | 61u);
    return (double)(t ^ (t >> 14)) / 4294967296.0;
}

void orc_jitter_random(uint32_t seed, int n, double *out) {
    orc_rng r = {seed};
    for (int q = 0; q < n; ++q) out[q] = rng_next(&r);
}

/* computeFlipBoxSeed3: k^3 particles per cell, jittered by +-jitter of the
 * sub-spacing; positions in doubles, stored as float.  Returns the count;
 * writes at most `capacity` points when `out` is not NULL. */
int64_t orc_flip_box_seed(const double *bmin, const double *bmax, const double *h, int k, double jitter,
                          uint32_t seed, float *out, int64_t capacity) {
    int64_t cells[3];
    double sub[3];
    for (int a = 0; a < 3; ++a) {
        double c = floor((bmax[a] - bmin[a]) / h[a] + 0.5);   /* Math.round */
        cells[a] = c < 1 ? 1 : (int64_t)c;
        sub[a] = h[a] / k;
    }
    orc_rng r = {seed};
    int64_t n = 0;
    for (int64_t ck = 0; ck < cells[2]; ++ck)
        for (int64_t cj = 0; cj < cells[1]; ++cj)
            for (int64_t ci = 0; ci < cells[0]; ++ci)
                for (int sk = 0; sk < k; ++sk)
                    for (int sj = 0; sj < k; ++sj)
                        for (int si = 0; si < k; ++si) {
                            double jx = (rng_next(&r) * 2 - 1) * jitter * sub[0];
                            double jy = (rng_next(&r) * 2 - 1) * jitter * sub[1];
                            double jz = (rng_next(&r) * 2 - 1) * jitter * sub[2];
                            double x = bmin[0] + (double)ci * h[0] + (si + 0.5) * sub[0] + jx;
                            double y = bmin[1] + (double)cj * h[1] + (sj + 0.5) * sub[1] + jy;
                            double z = bmin[2] + (double)ck * h[2] + (sk + 0.5) * sub[2] + jz;
                            if (out && n < capacity) {
                                out[3 * n] = (float)x;
                                out[3 * n + 1] = (float)y;
                                out[3 * n + 2] = (float)z;
                            }
                            ++n;
                        }
    return n;
}

/* ---- shared FP32 helpers (same forms as ff_oracle_grid.c) ------------ */
typedef struct {
    int nx, ny, nz;
    float hx, hy, hz, ox, oy, oz;
} fg;

static inline int iclamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline float gclamp(float g) { return fminf(fmaxf(g, -1.0e8f), 1.0e8f); }
static inline int nonfinite(float v) { return isnan(v) || isinf(v); }
/* float -> int32 after rounding, saturating out of range and NaN -> 0 (the
 * conversion the device performs) */
static inline int32_t sat_i32(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x < -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}

static fg make_fg(const int *res, const float *h, const float *o) {
    fg g = {res[0], res[1], res[2], h[0], h[1], h[2], o[0], o[1], o[2]};
    return g;
}
static void shape_of(const fg *g, int a, int *s) {
    s[0] = g->nx + (a == 0);
    s[1] = g->ny + (a == 1);
    s[2] = g->nz + (a == 2);
}
static void origin_of(const fg *g, int a, float *o) {
    o[0] = g->ox + (a == 0 ? 0.0f : g->hx * 0.5f);
    o[1] = g->oy + (a == 1 ? 0.0f : g->hy * 0.5f);
    o[2] = g->oz + (a == 2 ? 0.0f : g->hz * 0.5f);
}

typedef struct {
    int i0c, i1c, j0c, j1c, k0c, k1c;
    float w[8];
} tri;

/* trilinearCoordsAndWeights3 (grid_math3.js:61-101) */
static tri tri_coords(const fg *g, const int *s, const float *o, const float *p) {
    tri t;
    float gx = gclamp((p[0] - o[0]) / g->hx), gy = gclamp((p[1] - o[1]) / g->hy), gz = gclamp((p[2] - o[2]) / g->hz);
    int i0 = (int)floorf(gx), j0 = (int)floorf(gy), k0 = (int)floorf(gz);
    float fx = gx - (float)i0, fy = gy - (float)j0, fz = gz - (float)k0;
    t.i0c = iclamp(i0, 0, s[0] - 1);
    t.i1c = iclamp(i0 + 1, 0, s[0] - 1);
    t.j0c = iclamp(j0, 0, s[1] - 1);
    t.j1c = iclamp(j0 + 1, 0, s[1] - 1);
    t.k0c = iclamp(k0, 0, s[2] - 1);
    t.k1c = iclamp(k0 + 1, 0, s[2] - 1);
    float ux = 1.0f - fx, uy = 1.0f - fy, uz = 1.0f - fz;
    t.w[0] = ux * uy * uz;
    t.w[1] = fx * uy * uz;
    t.w[2] = ux * fy * uz;
    t.w[3] = fx * fy * uz;
    t.w[4] = ux * uy * fz;
    t.w[5] = fx * uy * fz;
    t.w[6] = ux * fy * fz;
    t.w[7] = fx * fy * fz;
    return t;
}
static inline int64_t corner(const tri *t, const int *s, int c) {
    int i = (c & 1) ? t->i1c : t->i0c, j = (c & 2) ? t->j1c : t->j0c, k = (c & 4) ? t->k1c : t->k0c;
    return i + (int64_t)s[0] * (j + (int64_t)s[1] * k);
}
static float tri_sample(const float *d, const fg *g, const int *s, const float *o, const float *p) {
    tri t = tri_coords(g, s, o, p);
    float acc = d[corner(&t, s, 0)] * t.w[0];
    for (int c = 1; c < 8; ++c) acc = acc + d[corner(&t, s, c)] * t.w[c];
    return acc;
}

/* cellIndexOf (:227-235) */
static int64_t cell_index(const fg *g, const float *p) {
    float cx = gclamp((p[0] - g->ox) / g->hx), cy = gclamp((p[1] - g->oy) / g->hy), cz = gclamp((p[2] - g->oz) / g->hz);
    int i = iclamp((int)floorf(cx), 0, g->nx - 1), j = iclamp((int)floorf(cy), 0, g->ny - 1),
        k = iclamp((int)floorf(cz), 0, g->nz - 1);
    return i + (int64_t)g->nx * (j + (int64_t)g->ny * k);
}

void orc_flip_cell_index(const int *res, const float *h, const float *o, int64_t n, const float *pos, int64_t *out) {
    fg g = make_fg(res, h, o);
    for (int64_t p = 0; p < n; ++p) out[p] = cell_index(&g, pos + 3 * p);
}

/* clearFluidMask + markFluidCellsKernel (:237-245) */
void orc_flip_mark_fluid(const int *res, const float *h, const float *o, int64_t n, const float *pos, float *mask) {
    fg g = make_fg(res, h, o);
    memset(mask, 0, sizeof(float) * (size_t)g.nx * g.ny * g.nz);
    for (int64_t p = 0; p < n; ++p) mask[cell_index(&g, pos + 3 * p)] = 1.0f;
}

/* dirichlet(pos) at the cell centres (:252-259): air cells (trilinear mask
 * < 0.5) are Dirichlet with target -dt (g . pos) under reduced pressure */
void orc_flip_dirichlet(const int *res, const float *h, const float *o, const float *mask, const float *grav, float dt,
                        int reduced, uint8_t *active, float *target) {
    fg g = make_fg(res, h, o);
    int s[3] = {g.nx, g.ny, g.nz};
    float oc[3];
    origin_of(&g, 3, oc);
    for (int k = 0; k < g.nz; ++k)
        for (int j = 0; j < g.ny; ++j)
            for (int i = 0; i < g.nx; ++i) {
                int64_t c = i + (int64_t)g.nx * (j + (int64_t)g.ny * k);
                float p[3] = {oc[0] + g.hx * (float)i, oc[1] + g.hy * (float)j, oc[2] + g.hz * (float)k};
                float m = tri_sample(mask, &g, s, oc, p);
                active[c] = m < 0.5f;
                target[c] = reduced ? -((grav[0] * p[0] + grav[1] * p[1] + grav[2] * p[2]) * dt) : 0.0f;
            }
}

/* P2G: buildScatter + buildFinalize (:508-568).  Accumulators are int32 and
 * wrap on overflow like the reference's i32 atomics. */
void orc_flip_p2g(const int *res, const float *h, const float *o, int64_t n, const float *pos, const float *vel,
                  float scale, float eps, float *u, float *v, float *w, int32_t *vu, int32_t *vv, int32_t *vw) {
    fg g = make_fg(res, h, o);
    float *out[3] = {u, v, w};
    int32_t *valid[3] = {vu, vv, vw};
    for (int a = 0; a < 3; ++a) {
        int s[3];
        float oa[3];
        shape_of(&g, a, s);
        origin_of(&g, a, oa);
        const int64_t nf = (int64_t)s[0] * s[1] * s[2];
        uint32_t *num = (uint32_t *)calloc((size_t)nf, 4), *den = (uint32_t *)calloc((size_t)nf, 4);
        for (int64_t p = 0; p < n; ++p) {
            const float value = vel[3 * p + a];
            tri t = tri_coords(&g, s, oa, pos + 3 * p);
            for (int c = 0; c < 8; ++c) {
                const int64_t f = corner(&t, s, c);
                num[f] += (uint32_t)sat_i32(rintf(value * t.w[c] * scale));
                den[f] += (uint32_t)sat_i32(rintf(t.w[c] * scale));
            }
        }
        for (int64_t f = 0; f < nf; ++f) {
            const float numer = (float)(int32_t)num[f] / scale;
            const float denom = (float)(int32_t)den[f] / scale;
            if (denom > eps) {
                out[a][f] = numer / denom;
                valid[a][f] = 1;
            } else {
                out[a][f] = 0.0f;
                valid[a][f] = 0;
            }
        }
        free(num);
        free(den);
    }
}

/* computeU/V/WFluidAdjacent (:586-618) */
void orc_flip_fluid_adjacent(const int *res, const float *mask, int32_t *au, int32_t *av, int32_t *aw) {
    const int nx = res[0], ny = res[1], nz = res[2];
    int32_t *out[3] = {au, av, aw};
    for (int a = 0; a < 3; ++a) {
        int s[3] = {nx + (a == 0), ny + (a == 1), nz + (a == 2)};
        for (int k = 0; k < s[2]; ++k)
            for (int j = 0; j < s[1]; ++j)
                for (int i = 0; i < s[0]; ++i) {
                    int lo[3] = {i, j, k}, hi[3] = {i, j, k};
                    int idx = a == 0 ? i : (a == 1 ? j : k), n = a == 0 ? nx : (a == 1 ? ny : nz);
                    lo[a] = iclamp(idx - 1, 0, n - 1);
                    hi[a] = iclamp(idx, 0, n - 1);
                    float ml = mask[lo[0] + (int64_t)nx * (lo[1] + (int64_t)ny * lo[2])];
                    float mh = mask[hi[0] + (int64_t)nx * (hi[1] + (int64_t)ny * hi[2])];
                    out[a][i + (int64_t)s[0] * (j + (int64_t)s[1] * k)] = (ml > 0.5f || mh > 0.5f) ? 1 : 0;
                }
    }
}

/* g2pUpdate (:909-922) */
void orc_flip_g2p(const int *res, const float *h, const float *o, int64_t n, const float *pos, float *vel,
                  const float *u, const float *v, const float *w, const float *uo, const float *vo, const float *wo,
                  float flip_ratio, float damping) {
    fg g = make_fg(res, h, o);
    const float *nw[3] = {u, v, w}, *od[3] = {uo, vo, wo};
    const float damp = fminf(fmaxf(damping, 0.0f), 1.0f);
    for (int64_t p = 0; p < n; ++p) {
        float nv[3], ov[3], out[3];
        for (int a = 0; a < 3; ++a) {
            int s[3];
            float oa[3];
            shape_of(&g, a, s);
            origin_of(&g, a, oa);
            nv[a] = tri_sample(nw[a], &g, s, oa, pos + 3 * p);
            ov[a] = tri_sample(od[a], &g, s, oa, pos + 3 * p);
        }
        int bad = 0;
        for (int a = 0; a < 3; ++a) {
            float delta = nv[a] - ov[a];
            float flipv = vel[3 * p + a] + delta;
            float blended = flipv * flip_ratio + nv[a] * (1.0f - flip_ratio);
            out[a] = blended * (1.0f - damp);
            bad |= nonfinite(out[a]);
        }
        for (int a = 0; a < 3; ++a) vel[3 * p + a] = bad ? 0.0f : fminf(fmaxf(out[a], -500.0f), 500.0f);
    }
}

/* concentration grid pass (:989-1020): per-cell mean of clamped particle
 * concentration in fixed point (scale cscale), cell density and, when the
 * density coupling is on, the beta faces (:298-359) */
void orc_flip_concentration_grid(const int *res, const float *h, const float *o, int64_t n, const float *pos,
                                 const float *conc, float cscale, const float *mask, int density, float rho0,
                                 float rho1, float *cell_conc, float *cell_rho, float *bu, float *bv, float *bw) {
    fg g = make_fg(res, h, o);
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int64_t nc = (int64_t)nx * ny * nz;
    uint32_t *cnt = (uint32_t *)calloc((size_t)nc, 4), *acc = (uint32_t *)calloc((size_t)nc, 4);
    for (int64_t p = 0; p < n; ++p) {
        int64_t c = cell_index(&g, pos + 3 * p);
        cnt[c] += 1;
        float cc = fminf(fmaxf(conc[p], 0.0f), 1.0f);
        acc[c] += (uint32_t)sat_i32(rintf(cc * cscale));
    }
    const float r0 = fmaxf(rho0, 1e-4f), r1 = fmaxf(rho1, 1e-4f), rref = fmaxf(r0, r1);
    for (int64_t c = 0; c < nc; ++c) {
        float total = (float)(int32_t)cnt[c];
        float sum = (float)(int32_t)acc[c] / cscale;
        float mean = sum / fmaxf(total, 1.0f);
        float cv = total > 0.5f ? fminf(fmaxf(mean, 0.0f), 1.0f) : 0.0f;
        cell_conc[c] = cv;
        if (density) cell_rho[c] = r0 + (r1 - r0) * cv;
    }
    free(cnt);
    free(acc);
    if (!density) return;
    float *beta[3] = {bu, bv, bw};
    for (int a = 0; a < 3; ++a) {
        int s[3] = {nx + (a == 0), ny + (a == 1), nz + (a == 2)};
        for (int k = 0; k < s[2]; ++k)
            for (int j = 0; j < s[1]; ++j)
                for (int i = 0; i < s[0]; ++i) {
                    int A[3] = {i, j, k}, B[3] = {i, j, k};
                    int idx = a == 0 ? i : (a == 1 ? j : k), nn = a == 0 ? nx : (a == 1 ? ny : nz);
                    A[a] = iclamp(idx - 1, 0, nn - 1);
                    B[a] = iclamp(idx, 0, nn - 1);
                    int64_t ca = A[0] + (int64_t)nx * (A[1] + (int64_t)ny * A[2]);
                    int64_t cb = B[0] + (int64_t)nx * (B[1] + (int64_t)ny * B[2]);
                    float ra = cell_rho[ca], rb = cell_rho[cb];
                    int fa = mask[ca] > 0.5f, fb = mask[cb] > 0.5f;
                    float rf = (fa && fb) ? (ra + rb) * 0.5f : ((fa || fb) ? (fa ? ra : rb) : rref);
                    beta[a][i + (int64_t)s[0] * (j + (int64_t)s[1] * k)] = rref / fmaxf(rf, 1e-4f);
                }
    }
}

/* applyReducedGravityU/V/W (:848-884) */
void orc_flip_reduced_gravity(const int *res, const float *h, const float *o, const float *cell_rho, const float *bu,
                              const float *bv, const float *bw, const float *grav, float dt, float rref, float *u,
                              float *v, float *w) {
    const int nx = res[0], ny = res[1], nz = res[2];
    const float *beta[3] = {bu, bv, bw};
    float *data[3] = {u, v, w};
    for (int a = 0; a < 3; ++a) {
        int s[3] = {nx + (a == 0), ny + (a == 1), nz + (a == 2)};
        for (int k = 0; k < s[2]; ++k)
            for (int j = 0; j < s[1]; ++j)
                for (int i = 0; i < s[0]; ++i) {
                    float p[3];
                    p[0] = o[0] + (a == 0 ? (float)i * h[0] : ((float)i + 0.5f) * h[0]);
                    p[1] = o[1] + (a == 1 ? (float)j * h[1] : ((float)j + 0.5f) * h[1]);
                    p[2] = o[2] + (a == 2 ? (float)k * h[2] : ((float)k + 0.5f) * h[2]);
                    int A[3] = {i, j, k}, B[3] = {i, j, k};
                    int idx = a == 0 ? i : (a == 1 ? j : k), nn = a == 0 ? nx : (a == 1 ? ny : nz);
                    B[a] = iclamp(idx, 0, nn - 1);
                    A[a] = iclamp(idx - 1, 0, nn - 1);
                    float rb = cell_rho[B[0] + (int64_t)nx * (B[1] + (int64_t)ny * B[2])];
                    float ra = cell_rho[A[0] + (int64_t)nx * (A[1] + (int64_t)ny * A[2])];
                    float drho = (rb - ra) / h[a];
                    int64_t f = i + (int64_t)s[0] * (j + (int64_t)s[1] * k);
                    float gp = grav[0] * p[0] + grav[1] * p[1] + grav[2] * p[2];
                    float term = beta[a][f] * dt / rref * gp * drho;
                    data[a][f] = data[a][f] - term;
                }
    }
}

/* mixAndFade (:1022-1029) */
void orc_flip_mix_fade(const int *res, const float *h, const float *o, int64_t n, const float *pos,
                       const float *cell_conc, float mixing, float fade, float *conc) {
    fg g = make_fg(res, h, o);
    int s[3] = {g.nx, g.ny, g.nz};
    float oc[3];
    origin_of(&g, 3, oc);
    const float mx = fminf(fmaxf(mixing, 0.0f), 1.0f), fd = fminf(fmaxf(fade, 0.0f), 1.0f);
    for (int64_t p = 0; p < n; ++p) {
        float sampled = tri_sample(cell_conc, &g, s, oc, pos + 3 * p);
        float c = fminf(fmaxf(conc[p], 0.0f), 1.0f);
        float local = nonfinite(sampled) ? c : sampled;
        float blended = c + (local - c) * mx;
        conc[p] = fminf(fmaxf(blended * (1.0f - fd), 0.0f), 1.0f);
    }
}

/* trace from ff_oracle_grid.c */
void orc_trace(const int *res, const float *h, const float *o, const float *u, const float *v, const float *w,
               const float *phi, float dt, int max_substeps, float dirn, int64_t n, const float *pin, float *pout);

/* advectParticles + pushOutOfCollider (:925-957).  box_max: origin + the
 * domain extent (computed by the caller as the reference does: extent in
 * doubles, stored as float). */
void orc_flip_advect(const int *res, const float *h, const float *o, const float *u, const float *v, const float *w,
                     const float *phi, float dt, int max_substeps, int64_t n, float *pos, const float *extent,
                     float push_thresh, float push_shift) {
    float *traced = (float *)malloc(sizeof(float) * 3 * (size_t)(n > 0 ? n : 1));
    orc_trace(res, h, o, u, v, w, phi, dt, max_substeps, -1.0f, n, pos, traced);
    float mn[3], mx[3];
    for (int a = 0; a < 3; ++a) {
        mn[a] = o[a] + 1e-4f;
        mx[a] = (o[a] + extent[a]) - 1e-4f;
    }
    for (int64_t p = 0; p < n; ++p) {
        float *q = traced + 3 * p;
        int bad = nonfinite(q[0]) || nonfinite(q[1]) || nonfinite(q[2]);
        for (int a = 0; a < 3; ++a) {
            float sv = bad ? pos[3 * p + a] : q[a];
            pos[3 * p + a] = fminf(fmaxf(sv, mn[a]), mx[a]);
        }
    }
    free(traced);
    if (!phi) return;
    fg g = make_fg(res, h, o);
    int s[3] = {g.nx, g.ny, g.nz};
    float oc[3];
    origin_of(&g, 3, oc);
    for (int64_t p = 0; p < n; ++p) {
        float *q = pos + 3 * p;
        float val = tri_sample(phi, &g, s, oc, q);
        if (!(val < push_thresh)) continue;
        /* trilinearGradientAtPosition3 (grid_math3.js:295-352) */
        float coord[3] = {gclamp((q[0] - oc[0]) / g.hx), gclamp((q[1] - oc[1]) / g.hy), gclamp((q[2] - oc[2]) / g.hz)};
        int lo[3], hi[3];
        float t[3];
        for (int a = 0; a < 3; ++a) {
            int idx = (int)floorf(coord[a]);
            int lim = s[a] - 2;
            lo[a] = idx < lim ? idx : lim;
            if (lo[a] < 0) lo[a] = 0;
            hi[a] = lo[a] + 1 < s[a] - 1 ? lo[a] + 1 : s[a] - 1;
            t[a] = fminf(fmaxf(coord[a] - (float)lo[a], 0.0f), 1.0f);
        }
#define V(i, j, k) phi[(i) + (int64_t)g.nx * ((j) + (int64_t)g.ny * (k))]
        float v000 = V(lo[0], lo[1], lo[2]), v100 = V(hi[0], lo[1], lo[2]), v010 = V(lo[0], hi[1], lo[2]);
        float v110 = V(hi[0], hi[1], lo[2]), v001 = V(lo[0], lo[1], hi[2]), v101 = V(hi[0], lo[1], hi[2]);
        float v011 = V(lo[0], hi[1], hi[2]), v111 = V(hi[0], hi[1], hi[2]);
#undef V
        float tx = t[0], ty = t[1], tz = t[2], gr[3], sacc;
        sacc = (1.0f - ty) * (1.0f - tz) * (v100 - v000);
        sacc = sacc + ty * (1.0f - tz) * (v110 - v010);
        sacc = sacc + (1.0f - ty) * tz * (v101 - v001);
        sacc = sacc + ty * tz * (v111 - v011);
        gr[0] = sacc / g.hx;
        sacc = (1.0f - tx) * (1.0f - tz) * (v010 - v000);
        sacc = sacc + tx * (1.0f - tz) * (v110 - v100);
        sacc = sacc + (1.0f - tx) * tz * (v011 - v001);
        sacc = sacc + tx * tz * (v111 - v101);
        gr[1] = sacc / g.hy;
        sacc = (1.0f - tx) * (1.0f - ty) * (v001 - v000);
        sacc = sacc + tx * (1.0f - ty) * (v101 - v100);
        sacc = sacc + (1.0f - tx) * ty * (v011 - v010);
        sacc = sacc + tx * ty * (v111 - v110);
        gr[2] = sacc / g.hz;
        float gl = sqrtf(gr[0] * gr[0] + gr[1] * gr[1] + gr[2] * gr[2]);
        if (!(gl > 0.0f)) continue;
        float shift = (push_thresh - val) + push_shift;
        for (int a = 0; a < 3; ++a) q[a] = q[a] + gr[a] / gl * shift;
    }
}

/* resamplePass (:621-820): particles in cells holding more than max_pc are
 * donors, ranked in particle order; cells holding fewer than min_pc with
 * at least 3 of their 6 clamped face neighbours at min_pc or more ask for
 * min_pc - count, and claim donor slots in flat cell order (i fastest).  A
 * claimed donor moves to the claiming cell's centre, cellCenterOrigin +
 * (i, j, k) h, and takes the face-centred velocity sampled there
 * (faceCenteredValueAtPosition3).  The pass then rebuilds the fluid mask
 * (markFluidCells, run again by the caller).  Returns the number of
 * particles moved. */
int64_t orc_flip_resample(const int *res, const float *h, const float *o, int64_t n, float *pos, float *vel,
                          const float *u, const float *v, const float *w, int min_pc, int max_pc) {
    fg g = make_fg(res, h, o);
    const int64_t nc = (int64_t)g.nx * g.ny * g.nz;
    int32_t *cnt = (int32_t *)calloc((size_t)nc, sizeof(int32_t));
    int64_t *pool = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    int64_t *cell = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t p = 0; p < n; ++p) {
        cell[p] = cell_index(&g, pos + 3 * p);
        cnt[cell[p]] += 1;
    }
    int64_t donors = 0;
    for (int64_t p = 0; p < n; ++p)
        if (cnt[cell[p]] > max_pc) pool[donors++] = p;
    const float *comp[3] = {u, v, w};
    const float cc[3] = {g.ox + g.hx * 0.5f, g.oy + g.hy * 0.5f, g.oz + g.hz * 0.5f};
    int64_t base = 0, moved = 0;
    for (int k = 0; k < g.nz; ++k)
        for (int j = 0; j < g.ny; ++j)
            for (int i = 0; i < g.nx; ++i) {
                const int64_t c = i + (int64_t)g.nx * (j + (int64_t)g.ny * k);
                const int32_t count = cnt[c];
#define ORC_CNT(ii, jj, kk) cnt[(ii) + (int64_t)g.nx * ((jj) + (int64_t)g.ny * (kk))]
                const int nb = (ORC_CNT(i > 0 ? i - 1 : 0, j, k) >= min_pc) +
                               (ORC_CNT(i < g.nx - 1 ? i + 1 : g.nx - 1, j, k) >= min_pc) +
                               (ORC_CNT(i, j > 0 ? j - 1 : 0, k) >= min_pc) +
                               (ORC_CNT(i, j < g.ny - 1 ? j + 1 : g.ny - 1, k) >= min_pc) +
                               (ORC_CNT(i, j, k > 0 ? k - 1 : 0) >= min_pc) +
                               (ORC_CNT(i, j, k < g.nz - 1 ? k + 1 : g.nz - 1) >= min_pc);
#undef ORC_CNT
                const int need = (count < min_pc && nb >= 3) ? min_pc - count : 0;
                for (int q = 0; q < need; ++q) {
                    const int64_t slot = base + q;
                    if (slot >= donors) break;
                    const int64_t d = pool[slot];
                    float np[3] = {cc[0] + (float)i * g.hx, cc[1] + (float)j * g.hy, cc[2] + (float)k * g.hz};
                    for (int a = 0; a < 3; ++a) {
                        int s[3];
                        float oa[3];
                        shape_of(&g, a, s);
                        origin_of(&g, a, oa);
                        vel[3 * d + a] = tri_sample(comp[a], &g, s, oa, np);
                    }
                    for (int a = 0; a < 3; ++a) pos[3 * d + a] = np[a];
                    ++moved;
                }
                base += need;
            }
    free(cnt);
    free(pool);
    free(cell);
    return moved;
}

/* ==== 2D two-phase FLIP (grid_two_phase_flip_solver2.js) =================
 * Written in 2D with (x, y) pairs, independently of the one-cell-thick 3D
 * layout the device runs it on. */
typedef struct {
    int nx, ny;
    float hx, hy, ox, oy;
} fg2;

/* cellIndexOf (:608-614) */
static int64_t cell2(const fg2 *g, const float *p) {
    float cx = gclamp((p[0] - g->ox) / g->hx), cy = gclamp((p[1] - g->oy) / g->hy);
    int i = iclamp((int)floorf(cx), 0, g->nx - 1), j = iclamp((int)floorf(cy), 0, g->ny - 1);
    return i + (int64_t)g->nx * j;
}
/* collocatedValueAtPosition2 (grid_math.js:35-73) */
static float bilinear2(const float *d, int sx, int sy, float ox, float oy, float hx, float hy, float x, float y) {
    float gx = gclamp((x - ox) / hx), gy = gclamp((y - oy) / hy);
    int i0 = (int)floorf(gx), j0 = (int)floorf(gy);
    float fx = gx - (float)i0, fy = gy - (float)j0;
    int i0c = iclamp(i0, 0, sx - 1), i1c = iclamp(i0 + 1, 0, sx - 1);
    int j0c = iclamp(j0, 0, sy - 1), j1c = iclamp(j0 + 1, 0, sy - 1);
    float ux = 1.0f - fx, uy = 1.0f - fy;
    float s = d[i0c + (int64_t)sx * j0c] * (ux * uy);
    s = s + d[i1c + (int64_t)sx * j0c] * (fx * uy);
    s = s + d[i0c + (int64_t)sx * j1c] * (ux * fy);
    s = s + d[i1c + (int64_t)sx * j1c] * (fx * fy);
    return s;
}
/* faceCenteredValueAtPosition2 (grid_math.js:75-90) */
static void face2(const fg2 *g, const float *u, const float *v, float x, float y, float *out) {
    out[0] = bilinear2(u, g->nx + 1, g->ny, g->ox, g->oy + g->hy * 0.5f, g->hx, g->hy, x, y);
    out[1] = bilinear2(v, g->nx, g->ny + 1, g->ox + g->hx * 0.5f, g->oy, g->hx, g->hy, x, y);
}

/* countPhasesKernel, computeDensityKernel, computeBetaU/V (:646-762) */
void orc_tp_density(const int *res, const float *h, const float *o, int64_t n, const float *pos, const float *phase,
                    float cscale, float rho0, float rho1, int32_t *cnt, int32_t *acc, float *frac, float *rho,
                    float *bu, float *bv) {
    fg2 g = {res[0], res[1], h[0], h[1], o[0], o[1]};
    const int nx = g.nx, ny = g.ny;
    const int64_t nc = (int64_t)nx * ny;
    memset(cnt, 0, 4 * (size_t)nc);
    memset(acc, 0, 4 * (size_t)nc);
    for (int64_t p = 0; p < n; ++p) {
        int64_t c = cell2(&g, pos + 2 * p);
        cnt[c] = (int32_t)((uint32_t)cnt[c] + 1u);
        acc[c] = (int32_t)((uint32_t)acc[c] + (uint32_t)sat_i32(rintf(fminf(fmaxf(phase[p], 0.0f), 1.0f) * cscale)));
    }
    const float r0 = fmaxf(rho0, 1e-4f), r1 = fmaxf(rho1, 1e-4f), rref = fmaxf(r0, r1);
    for (int64_t c = 0; c < nc; ++c) {
        float total = (float)cnt[c], sum = (float)acc[c] / cscale;
        float mean = sum / fmaxf(total, 1.0f);
        float f = total > 0.5f ? fminf(fmaxf(mean, 0.0f), 1.0f) : 0.0f;
        frac[c] = f;
        rho[c] = r0 + (r1 - r0) * f;
    }
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i <= nx; ++i)
            bu[i + (int64_t)(nx + 1) * j] =
                rref / fmaxf((rho[iclamp(i - 1, 0, nx - 1) + (int64_t)nx * j] + rho[iclamp(i, 0, nx - 1) + (int64_t)nx * j]) *
                                 0.5f, 1e-4f);
    for (int j = 0; j <= ny; ++j)
        for (int i = 0; i < nx; ++i)
            bv[i + (int64_t)nx * j] =
                rref / fmaxf((rho[i + (int64_t)nx * iclamp(j - 1, 0, ny - 1)] + rho[i + (int64_t)nx * iclamp(j, 0, ny - 1)]) *
                                 0.5f, 1e-4f);
}

/* g2pUpdate (:966-992): the FLIP/PIC blend ratio runs from gas_ratio at
 * concentration 0 to flip_ratio at 1 */
void orc_tp_g2p(const int *res, const float *h, const float *o, int64_t n, const float *pos, float *vel,
                const float *phase, const float *u, const float *v, const float *uo, const float *vo, float flip_ratio,
                float gas_ratio, float damping) {
    fg2 g = {res[0], res[1], h[0], h[1], o[0], o[1]};
    const float fr = fminf(fmaxf(flip_ratio, 0.0f), 1.0f), gr = fminf(fmaxf(gas_ratio, 0.0f), 1.0f);
    const float damp = fminf(fmaxf(damping, 0.0f), 1.0f);
    for (int64_t p = 0; p < n; ++p) {
        float nv[2], ov[2], out[2];
        face2(&g, u, v, pos[2 * p], pos[2 * p + 1], nv);
        face2(&g, uo, vo, pos[2 * p], pos[2 * p + 1], ov);
        const float c = fminf(fmaxf(phase[p], 0.0f), 1.0f);
        const float ratio = gr + (fr - gr) * c;
        int bad = 0;
        for (int a = 0; a < 2; ++a) {
            float delta = nv[a] - ov[a];
            float flipv = vel[2 * p + a] + delta;
            float blended = flipv * ratio + nv[a] * (1.0f - ratio);
            out[a] = blended * (1.0f - damp);
            bad |= nonfinite(out[a]);
        }
        for (int a = 0; a < 2; ++a) vel[2 * p + a] = bad ? 0.0f : fminf(fmaxf(out[a], -500.0f), 500.0f);
    }
}

/* mixConcentration (:1055-1073) */
void orc_tp_mix(const int *res, const float *h, const float *o, int64_t n, const float *pos, const float *frac,
                float mixing, float fade, float *phase) {
    fg2 g = {res[0], res[1], h[0], h[1], o[0], o[1]};
    const float mx = fminf(fmaxf(mixing, 0.0f), 1.0f), fd = fminf(fmaxf(fade, 0.0f), 1.0f);
    for (int64_t p = 0; p < n; ++p) {
        float sampled = bilinear2(frac, g.nx, g.ny, g.ox + g.hx * 0.5f, g.oy + g.hy * 0.5f, g.hx, g.hy, pos[2 * p],
                                  pos[2 * p + 1]);
        float c = fminf(fmaxf(phase[p], 0.0f), 1.0f);
        float local = nonfinite(sampled) ? c : sampled;
        float blended = c + (local - c) * mx;
        phase[p] = fminf(fmaxf(blended * (1.0f - fd), 0.0f), 1.0f);
    }
}

/* resamplePassNow (:1226-1494) on the counts (cnt, acc) of orc_tp_density:
 * recipients' signed need, liquid / gas donor ranks in particle order in a
 * pool filled from both ends (each half capped at max(1, maxParticles/2)),
 * claims in flat cell order.  stats: liquid donors, liquid need, gas
 * donors, gas need.  Returns the number of particles moved. */
int64_t orc_tp_resample(const int *res, const float *h, const float *o, int64_t n, int max_particles, float *pos,
                        float *vel, const float *phase, const float *u, const float *v, const int32_t *cnt,
                        const int32_t *acc, float cscale, int min_pc, int max_pc, int64_t *stats) {
    fg2 g = {res[0], res[1], h[0], h[1], o[0], o[1]};
    const int nx = g.nx, ny = g.ny;
    const int64_t nc = (int64_t)nx * ny;
    int32_t *need = (int32_t *)malloc(4 * (size_t)nc);
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int64_t c = i + (int64_t)nx * j;
            const int64_t l = i > 0 ? c - 1 : c, r = i < nx - 1 ? c + 1 : c, d = j > 0 ? c - nx : c,
                          up = j < ny - 1 ? c + nx : c;
            const int count = cnt[c];
            const int nb = (cnt[l] >= min_pc) + (cnt[r] >= min_pc) + (cnt[d] >= min_pc) + (cnt[up] >= min_pc);
            const float total = (float)count, sum = (float)acc[c] / cscale;
            const float ntot = (float)(int32_t)((uint32_t)cnt[l] + (uint32_t)cnt[r] + (uint32_t)cnt[d] + (uint32_t)cnt[up]);
            const float nsum =
                (float)(int32_t)((uint32_t)acc[l] + (uint32_t)acc[r] + (uint32_t)acc[d] + (uint32_t)acc[up]) / cscale;
            const float own = sum / fmaxf(total, 1.0f), around = nsum / fmaxf(ntot, 1.0f);
            const int liquid = total > 0.5f ? own > 0.5f : around > 0.5f;
            const int needed = min_pc - count;
            need[c] = (count < min_pc && nb >= 2) ? (liquid ? needed : -needed) : 0;
        }
    const int64_t half = max_particles / 2 > 1 ? max_particles / 2 : 1, top = max_particles - 1;
    int *pool = (int *)malloc(sizeof(int) * (size_t)(max_particles > 0 ? max_particles : 1));
    int64_t nl = 0, ng = 0;
    for (int64_t p = 0; p < n; ++p) {
        if (!(cnt[cell2(&g, pos + 2 * p)] > max_pc)) continue;
        if (phase[p] > 0.5f) {
            if (nl < half) pool[nl] = (int)p;
            ++nl;
        } else {
            if (ng < half) pool[top - ng] = (int)p;
            ++ng;
        }
    }
    const int64_t avl = nl < half ? nl : half, avg = ng < half ? ng : half;
    int64_t bl = 0, bg = 0, moved = 0;
    const float ccx = g.ox + g.hx * 0.5f, ccy = g.oy + g.hy * 0.5f;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int q = need[i + (int64_t)nx * j];
            if (q == 0) continue;
            const int liquid = q > 0;
            const int64_t needed = liquid ? q : -q, base = liquid ? bl : bg, avail = liquid ? avl : avg;
            if (liquid) bl += needed;
            else bg += needed;
            for (int64_t m = 0; m < needed && base + m < avail; ++m) {
                const int64_t dnr = pool[liquid ? base + m : top - (base + m)];
                const float x = ccx + (float)i * g.hx, y = ccy + (float)j * g.hy;
                float vv[2];
                face2(&g, u, v, x, y, vv);
                pos[2 * dnr] = x;
                pos[2 * dnr + 1] = y;
                vel[2 * dnr] = vv[0];
                vel[2 * dnr + 1] = vv[1];
                ++moved;
            }
        }
    if (stats) {
        stats[0] = nl;
        stats[1] = bl;
        stats[2] = ng;
        stats[3] = bg;
    }
    free(need);
    free(pool);
    return moved;
}

/* ---- 3D two-phase solver (the 2D two-phase stages on a full grid) ---- */

/* per-cell particle count and fixed-point concentration sum (countPhases,
 * grid_two_phase_flip_solver2.js:646-680, on 3D cells) */
void orc_tp3_counts(const int *res, const float *h, const float *o, int64_t n, const float *pos, const float *phase,
                    float cscale, int32_t *cnt, int32_t *acc) {
    fg g = make_fg(res, h, o);
    const int64_t nc = (int64_t)g.nx * g.ny * g.nz;
    memset(cnt, 0, 4 * (size_t)nc);
    memset(acc, 0, 4 * (size_t)nc);
    for (int64_t p = 0; p < n; ++p) {
        const int64_t c = cell_index(&g, pos + 3 * p);
        cnt[c] = (int32_t)((uint32_t)cnt[c] + 1u);
        acc[c] = (int32_t)((uint32_t)acc[c] + (uint32_t)sat_i32(rintf(fminf(fmaxf(phase[p], 0.0f), 1.0f) * cscale)));
    }
}

/* g2pUpdate (:966-992) with all three components: the FLIP/PIC blend runs
 * from gas_ratio at concentration 0 to flip_ratio at 1 */
void orc_tp3_g2p(const int *res, const float *h, const float *o, int64_t n, const float *pos, float *vel,
                 const float *phase, const float *u, const float *v, const float *w, const float *uo, const float *vo,
                 const float *wo, float flip_ratio, float gas_ratio, float damping) {
    fg g = make_fg(res, h, o);
    const float *nw[3] = {u, v, w}, *od[3] = {uo, vo, wo};
    const float fr = fminf(fmaxf(flip_ratio, 0.0f), 1.0f), gr = fminf(fmaxf(gas_ratio, 0.0f), 1.0f);
    const float damp = fminf(fmaxf(damping, 0.0f), 1.0f);
    for (int64_t p = 0; p < n; ++p) {
        float nv[3], ov[3], out[3];
        for (int a = 0; a < 3; ++a) {
            int s[3];
            float oa[3];
            shape_of(&g, a, s);
            origin_of(&g, a, oa);
            nv[a] = tri_sample(nw[a], &g, s, oa, pos + 3 * p);
            ov[a] = tri_sample(od[a], &g, s, oa, pos + 3 * p);
        }
        const float c = fminf(fmaxf(phase[p], 0.0f), 1.0f);
        const float ratio = gr + (fr - gr) * c;
        int bad = 0;
        for (int a = 0; a < 3; ++a) {
            float delta = nv[a] - ov[a];
            float flipv = vel[3 * p + a] + delta;
            float blended = flipv * ratio + nv[a] * (1.0f - ratio);
            out[a] = blended * (1.0f - damp);
            bad |= nonfinite(out[a]);
        }
        for (int a = 0; a < 3; ++a) vel[3 * p + a] = bad ? 0.0f : fminf(fmaxf(out[a], -500.0f), 500.0f);
    }
}

/* the per-phase resampling pass (:1226-1494) on 3D cells: a recipient is
 * below min_pc with at least 3 of its 6 clamped face neighbours at min_pc or
 * more (the 3D single-phase rule, grid_flip_solver3.js:700-724), its phase
 * its own majority or, empty, its neighbours'; donors rank in particle
 * order into a pool filled from both ends; claims in flat cell order move
 * a donor to the cell centre with the face velocity there.  stats as
 * orc_tp_resample's.  Returns the number of particles moved. */
int64_t orc_tp3_resample(const int *res, const float *h, const float *o, int64_t n, int max_particles, float *pos,
                         float *vel, const float *phase, const float *u, const float *v, const float *w,
                         const int32_t *cnt, const int32_t *acc, float cscale, int min_pc, int max_pc,
                         int64_t *stats) {
    fg g = make_fg(res, h, o);
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const int64_t plane = (int64_t)nx * ny, nc = plane * nz;
    int32_t *need = (int32_t *)malloc(4 * (size_t)nc);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t c = i + (int64_t)nx * j + plane * k;
                const int64_t nb6[6] = {i > 0 ? c - 1 : c,      i < nx - 1 ? c + 1 : c,     j > 0 ? c - nx : c,
                                        j < ny - 1 ? c + nx : c, k > 0 ? c - plane : c, k < nz - 1 ? c + plane : c};
                const int count = cnt[c];
                int nb = 0;
                uint32_t ct = 0, at = 0;
                for (int q = 0; q < 6; ++q) {
                    nb += cnt[nb6[q]] >= min_pc;
                    ct += (uint32_t)cnt[nb6[q]];
                    at += (uint32_t)acc[nb6[q]];
                }
                const float total = (float)count, sum = (float)acc[c] / cscale;
                const float ntot = (float)(int32_t)ct, nsum = (float)(int32_t)at / cscale;
                const float own = sum / fmaxf(total, 1.0f), around = nsum / fmaxf(ntot, 1.0f);
                const int liquid = total > 0.5f ? own > 0.5f : around > 0.5f;
                const int needed = min_pc - count;
                need[c] = (count < min_pc && nb >= 3) ? (liquid ? needed : -needed) : 0;
            }
    const int64_t half = max_particles / 2 > 1 ? max_particles / 2 : 1, top = max_particles - 1;
    int *pool = (int *)malloc(sizeof(int) * (size_t)(max_particles > 0 ? max_particles : 1));
    int64_t nl = 0, ng = 0;
    for (int64_t p = 0; p < n; ++p) {
        if (!(cnt[cell_index(&g, pos + 3 * p)] > max_pc)) continue;
        if (phase[p] > 0.5f) {
            if (nl < half) pool[nl] = (int)p;
            ++nl;
        } else {
            if (ng < half) pool[top - ng] = (int)p;
            ++ng;
        }
    }
    const int64_t avl = nl < half ? nl : half, avg = ng < half ? ng : half;
    int64_t bl = 0, bg = 0, moved = 0;
    const float *comp[3] = {u, v, w};
    const float ccx = g.ox + g.hx * 0.5f, ccy = g.oy + g.hy * 0.5f, ccz = g.oz + g.hz * 0.5f;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int q = need[i + (int64_t)nx * j + plane * k];
                if (q == 0) continue;
                const int liquid = q > 0;
                const int64_t needed = liquid ? q : -q, base = liquid ? bl : bg, avail = liquid ? avl : avg;
                if (liquid) bl += needed;
                else bg += needed;
                const float pt[3] = {ccx + g.hx * (float)i, ccy + g.hy * (float)j, ccz + g.hz * (float)k};
                float vq[3];
                for (int a = 0; a < 3; ++a) {
                    int s[3];
                    float oa[3];
                    shape_of(&g, a, s);
                    origin_of(&g, a, oa);
                    vq[a] = tri_sample(comp[a], &g, s, oa, pt);
                }
                for (int64_t m = 0; m < needed && base + m < avail; ++m) {
                    const int64_t dnr = pool[liquid ? base + m : top - (base + m)];
                    for (int a = 0; a < 3; ++a) {
                        pos[3 * dnr + a] = pt[a];
                        vel[3 * dnr + a] = vq[a];
                    }
                    ++moved;
                }
            }
    if (stats) {
        stats[0] = nl;
        stats[1] = bl;
        stats[2] = ng;
        stats[3] = bg;
    }
    free(need);
    free(pool);
    return moved;
}
