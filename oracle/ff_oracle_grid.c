/*
 * Oracle (test infrastructure only): FP32 CPU restatement of fluxflow's
 * grid-velocity kernels around the pressure projection.  The reference runs
 * them as WGSL in f32; this file does the same arithmetic in C floats, one
 * IEEE operation at a time (built with -ffp-contract=off), in the order the
 * reference's expressions evaluate.
 *
 *   sampling          grid_math3.js:61-230 (trilinear, monotone tricubic),
 *                     :295-352 (trilinear gradient), grid_data3.js:121-176
 *   backTrace / trace advection_solver3.js:20-62
 *   advectFaceCentered3 / advectScalar3, orders 1 and 2 (MacCormack)
 *                     advection_solver3.js:67-364
 *   constrainVelocity grid_blocked_boundary_condition_solver3.js:30-477,
 *                     array_utils3.js:88-228 (Jacobi extrapolation),
 *                     level_set_utils.js:5-40 (fractionInsideSdf)
 *   outflow           grid_outflow_solver3.js:79-210 (convective velocity
 *                     condition, scalar clearing), sdf_inflow_outflow3.js:44-64
 *                     (pressure Dirichlet of the outflow cells)
 *   explicit viscosity (no reference counterpart: grid_solver3.js:104 is a
 *                     no-op) u += dt nu lap(u) on interior faces, Neumann
 *                     at the array ends.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int nx, ny, nz;
    float hx, hy, hz, ox, oy, oz;
} og_geom;

typedef struct {
    float x, y, z;
} f3;

static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int iclamp(int v, int lo, int hi) { return imax(lo, imin(v, hi)); }
/* keeps float->int conversion defined for absurd or non-finite positions */
static inline float gclamp(float g) { return fminf(fmaxf(g, -1.0e8f), 1.0e8f); }

static void comp_shape(const og_geom *g, int a, int *sx, int *sy, int *sz) {
    *sx = g->nx + (a == 0);
    *sy = g->ny + (a == 1);
    *sz = g->nz + (a == 2);
}
/* dataOriginU/V/W (grid_data3.js:131-133); a == 3: cell centres */
static f3 comp_origin(const og_geom *g, int a) {
    f3 o;
    o.x = g->ox + (a == 0 ? 0.0f : g->hx * 0.5f);
    o.y = g->oy + (a == 1 ? 0.0f : g->hy * 0.5f);
    o.z = g->oz + (a == 2 ? 0.0f : g->hz * 0.5f);
    return o;
}
static f3 index_pos(const og_geom *g, f3 o, int i, int j, int k) {
    f3 p;
    p.x = o.x + g->hx * (float)i;
    p.y = o.y + g->hy * (float)j;
    p.z = o.z + g->hz * (float)k;
    return p;
}

static float trilinear(const float *d, int sx, int sy, int sz, const og_geom *g, f3 o, f3 pos) {
    float gx = gclamp((pos.x - o.x) / g->hx), gy = gclamp((pos.y - o.y) / g->hy), gz = gclamp((pos.z - o.z) / g->hz);
    int i0 = (int)floorf(gx), j0 = (int)floorf(gy), k0 = (int)floorf(gz);
    float fx = gx - (float)i0, fy = gy - (float)j0, fz = gz - (float)k0;
    int i0c = iclamp(i0, 0, sx - 1), i1c = iclamp(i0 + 1, 0, sx - 1);
    int j0c = iclamp(j0, 0, sy - 1), j1c = iclamp(j0 + 1, 0, sy - 1);
    int k0c = iclamp(k0, 0, sz - 1), k1c = iclamp(k0 + 1, 0, sz - 1);
    float ux = 1.0f - fx, uy = 1.0f - fy, uz = 1.0f - fz;
    float w000 = ux * uy * uz, w100 = fx * uy * uz, w010 = ux * fy * uz, w110 = fx * fy * uz;
    float w001 = ux * uy * fz, w101 = fx * uy * fz, w011 = ux * fy * fz, w111 = fx * fy * fz;
#define D(i, j, k) d[(i) + (int64_t)sx * ((j) + (int64_t)sy * (k))]
    float s = D(i0c, j0c, k0c) * w000;
    s = s + D(i1c, j0c, k0c) * w100;
    s = s + D(i0c, j1c, k0c) * w010;
    s = s + D(i1c, j1c, k0c) * w110;
    s = s + D(i0c, j0c, k1c) * w001;
    s = s + D(i1c, j0c, k1c) * w101;
    s = s + D(i0c, j1c, k1c) * w011;
    s = s + D(i1c, j1c, k1c) * w111;
    return s;
}

static float mono_cubic(float f0, float f1, float f2, float f3v, float f) {
    float D1 = f2 - f1;
    float rawD1 = (f2 - f0) * 0.5f, rawD2 = (f3v - f1) * 0.5f;
    int flat = fabsf(D1) < 1e-12f;
    float d1 = (flat || rawD1 * D1 < 0.0f) ? 0.0f : rawD1;
    float d2 = (flat || rawD2 * D1 < 0.0f) ? 0.0f : rawD2;
    float a3 = (d1 + d2) - D1 * 2.0f;
    float a2 = (D1 * 3.0f - d1 * 2.0f) - d2;
    float a1 = d1, a0 = f1;
    float t = a3 * f * f * f;
    t = t + a2 * f * f;
    t = t + a1 * f;
    return t + a0;
}

static void cubic_idx(float coord, int n, int idx[4], float *f) {
    int i0 = (int)floorf(coord);
    *f = coord - (float)i0;
    idx[0] = iclamp(i0 - 1, 0, n - 1);
    idx[1] = iclamp(i0, 0, n - 1);
    idx[2] = iclamp(i0 + 1, 0, n - 1);
    idx[3] = iclamp(i0 + 2, 0, n - 1);
}

static float tricubic(const float *d, int sx, int sy, int sz, const og_geom *g, f3 o, f3 pos) {
    float gx = gclamp((pos.x - o.x) / g->hx), gy = gclamp((pos.y - o.y) / g->hy), gz = gclamp((pos.z - o.z) / g->hz);
    int xi[4], yi[4], zi[4];
    float fx, fy, fz;
    cubic_idx(gx, sx, xi, &fx);
    cubic_idx(gy, sy, yi, &fy);
    cubic_idx(gz, sz, zi, &fz);
    float zv[4];
    for (int c = 0; c < 4; ++c) {
        float row[4];
        for (int b = 0; b < 4; ++b)
            row[b] = mono_cubic(D(xi[0], yi[b], zi[c]), D(xi[1], yi[b], zi[c]), D(xi[2], yi[b], zi[c]),
                                D(xi[3], yi[b], zi[c]), fx);
        zv[c] = mono_cubic(row[0], row[1], row[2], row[3], fy);
    }
    return mono_cubic(zv[0], zv[1], zv[2], zv[3], fz);
}
#undef D

typedef struct {
    og_geom g;
    const float *u, *v, *w, *phi;
} og_field;

static f3 sample_vel(const og_field *F, f3 pos) {
    f3 r;
    int sx, sy, sz;
    comp_shape(&F->g, 0, &sx, &sy, &sz);
    r.x = trilinear(F->u, sx, sy, sz, &F->g, comp_origin(&F->g, 0), pos);
    comp_shape(&F->g, 1, &sx, &sy, &sz);
    r.y = trilinear(F->v, sx, sy, sz, &F->g, comp_origin(&F->g, 1), pos);
    comp_shape(&F->g, 2, &sx, &sy, &sz);
    r.z = trilinear(F->w, sx, sy, sz, &F->g, comp_origin(&F->g, 2), pos);
    return r;
}
static float sample_phi(const og_field *F, f3 pos) {
    if (!F->phi) return 1.0f;
    return trilinear(F->phi, F->g.nx, F->g.ny, F->g.nz, &F->g, comp_origin(&F->g, 3), pos);
}

/* backTrace (advection_solver3.js:20-62) */
static f3 back_trace(const og_field *F, f3 pos, float dt, float dirn, int max_substeps) {
    const float h = fminf(F->g.hx, fminf(F->g.hy, F->g.hz));
    f3 pt = pos;
    float T = dt;
    for (int s = 0; s < max_substeps; ++s) {
        if (T <= 1e-6f) break;
        f3 v0 = sample_vel(F, pt);
        float len = sqrtf(v0.x * v0.x + v0.y * v0.y + v0.z * v0.z);
        float nsub = fmaxf(ceilf(len * T / h), 1.0f);
        float sdt = T / nsub;
        float hs = sdt * 0.5f;
        f3 mid = {pt.x - v0.x * hs * dirn, pt.y - v0.y * hs * dirn, pt.z - v0.z * hs * dirn};
        f3 mv = sample_vel(F, mid);
        f3 nxt = {pt.x - mv.x * sdt * dirn, pt.y - mv.y * sdt * dirn, pt.z - mv.z * sdt * dirn};
        float phi0 = sample_phi(F, pt), phi1 = sample_phi(F, nxt);
        if (phi1 <= 0.0f) {
            float w = fabsf(phi1) / (fabsf(phi0) + fabsf(phi1));
            float wm = 1.0f - w;
            pt.x = pt.x * w + nxt.x * wm;
            pt.y = pt.y * w + nxt.y * wm;
            pt.z = pt.z * w + nxt.z * wm;
            break;
        }
        T = T - sdt;
        pt = nxt;
    }
    return pt;
}

static og_field make_field(const int *res, const float *h, const float *o, const float *u, const float *v,
                           const float *w, const float *phi) {
    og_field F;
    F.g.nx = res[0];
    F.g.ny = res[1];
    F.g.nz = res[2];
    F.g.hx = h[0];
    F.g.hy = h[1];
    F.g.hz = h[2];
    F.g.ox = o[0];
    F.g.oy = o[1];
    F.g.oz = o[2];
    F.u = u;
    F.v = v;
    F.w = w;
    F.phi = phi;
    return F;
}

/* trace(start, direction) for a list of points (xyz interleaved) */
void orc_trace(const int *res, const float *h, const float *o, const float *u, const float *v, const float *w,
               const float *phi, float dt, int max_substeps, float dirn, int64_t n, const float *pin, float *pout) {
    og_field F = make_field(res, h, o, u, v, w, phi);
    for (int64_t q = 0; q < n; ++q) {
        f3 p = {pin[3 * q], pin[3 * q + 1], pin[3 * q + 2]};
        f3 r = back_trace(&F, p, dt, dirn, max_substeps);
        pout[3 * q] = r.x;
        pout[3 * q + 1] = r.y;
        pout[3 * q + 2] = r.z;
    }
}

/* min/max of `data` over the 8 trilinear corners around `traced`, counting
 * only corners whose own position samples the boundary > 0
 * (advection_solver3.js gatherLocalMinMax / clampCorrection) */
static float clamp_correction(const og_field *F, const float *data, int a, int sx, int sy, int sz, f3 o,
                              f3 traced, float corrected, float fwd) {
    const og_geom *g = &F->g;
    float gx = gclamp((traced.x - o.x) / g->hx), gy = gclamp((traced.y - o.y) / g->hy),
          gz = gclamp((traced.z - o.z) / g->hz);
    int i0 = (int)floorf(gx), j0 = (int)floorf(gy), k0 = (int)floorf(gz);
    int ic[2] = {iclamp(i0, 0, sx - 1), iclamp(i0 + 1, 0, sx - 1)};
    int jc[2] = {iclamp(j0, 0, sy - 1), iclamp(j0 + 1, 0, sy - 1)};
    int kc[2] = {iclamp(k0, 0, sz - 1), iclamp(k0 + 1, 0, sz - 1)};
    float mn = 1e30f, mx = -1e30f;
    int have = 0;
    (void)a;
    for (int c = 0; c < 8; ++c) {
        int ni = ic[c & 1], nj = jc[(c >> 1) & 1], nk = kc[(c >> 2) & 1];
        f3 p = index_pos(g, o, ni, nj, nk);
        int valid = sample_phi(F, p) > 0.0f;
        float val = data[ni + (int64_t)sx * (nj + (int64_t)sy * nk)];
        if (valid) {
            mn = fminf(mn, val);
            mx = fmaxf(mx, val);
            have = 1;
        }
    }
    int in_range = corrected >= mn && corrected <= mx;
    return (have && in_range) ? corrected : fwd;
}

/* advectFaceCentered3 (order 1 or 2) of (u, v, w) -> (uo, vo, wo); faces
 * whose own position samples the boundary <= 0 keep the output's value */
void orc_advect_faces(const int *res, const float *h, const float *o, const float *u, const float *v,
                      const float *w, const float *phi, float dt, int max_substeps, int order, float *uo, float *vo,
                      float *wo) {
    og_field F = make_field(res, h, o, u, v, w, phi);
    const float *in[3] = {u, v, w};
    float *out[3] = {uo, vo, wo};
    for (int a = 0; a < 3; ++a) {
        int sx, sy, sz;
        comp_shape(&F.g, a, &sx, &sy, &sz);
        f3 oa = comp_origin(&F.g, a);
        const int64_t n = (int64_t)sx * sy * sz;
        if (order == 1) {
            for (int64_t f = 0; f < n; ++f) {
                int i = (int)(f % sx), j = (int)((f / sx) % sy), k = (int)(f / ((int64_t)sx * sy));
                f3 pos = index_pos(&F.g, oa, i, j, k);
                if (sample_phi(&F, pos) > 0.0f)
                    out[a][f] = tricubic(in[a], sx, sy, sz, &F.g, oa, back_trace(&F, pos, dt, 1.0f, max_substeps));
            }
            continue;
        }
        float *fwd = (float *)malloc(sizeof(float) * n), *bwd = (float *)malloc(sizeof(float) * n);
        for (int64_t f = 0; f < n; ++f) {
            int i = (int)(f % sx), j = (int)((f / sx) % sy), k = (int)(f / ((int64_t)sx * sy));
            f3 pos = index_pos(&F.g, oa, i, j, k);
            fwd[f] = sample_phi(&F, pos) > 0.0f
                         ? tricubic(in[a], sx, sy, sz, &F.g, oa, back_trace(&F, pos, dt, 1.0f, max_substeps))
                         : in[a][f];
        }
        for (int64_t f = 0; f < n; ++f) {
            int i = (int)(f % sx), j = (int)((f / sx) % sy), k = (int)(f / ((int64_t)sx * sy));
            f3 pos = index_pos(&F.g, oa, i, j, k);
            bwd[f] = sample_phi(&F, pos) > 0.0f
                         ? tricubic(fwd, sx, sy, sz, &F.g, oa, back_trace(&F, pos, dt, -1.0f, max_substeps))
                         : fwd[f];
        }
        for (int64_t f = 0; f < n; ++f) {
            int i = (int)(f % sx), j = (int)((f / sx) % sy), k = (int)(f / ((int64_t)sx * sy));
            f3 pos = index_pos(&F.g, oa, i, j, k);
            if (!(sample_phi(&F, pos) > 0.0f)) continue;
            f3 tr = back_trace(&F, pos, dt, 1.0f, max_substeps);
            float fv = fwd[f];
            float corr = fv + (in[a][f] - bwd[f]) * 0.5f;
            out[a][f] = clamp_correction(&F, in[a], a, sx, sy, sz, oa, tr, corr, fv);
        }
        free(fwd);
        free(bwd);
    }
}

/* advectScalar3 of a cell-centred scalar (order 1 or 2) */
void orc_advect_scalar(const int *res, const float *h, const float *o, const float *u, const float *v,
                       const float *w, const float *phi, float dt, int max_substeps, int order, const float *s,
                       float *so) {
    og_field F = make_field(res, h, o, u, v, w, phi);
    const int sx = F.g.nx, sy = F.g.ny, sz = F.g.nz;
    const int64_t n = (int64_t)sx * sy * sz;
    f3 oc = comp_origin(&F.g, 3);
    if (order == 1) {
        for (int64_t c = 0; c < n; ++c) {
            int i = (int)(c % sx), j = (int)((c / sx) % sy), k = (int)(c / ((int64_t)sx * sy));
            f3 pos = index_pos(&F.g, oc, i, j, k);
            if (sample_phi(&F, pos) > 0.0f)
                so[c] = tricubic(s, sx, sy, sz, &F.g, oc, back_trace(&F, pos, dt, 1.0f, max_substeps));
        }
        return;
    }
    float *fwd = (float *)malloc(sizeof(float) * n), *bwd = (float *)malloc(sizeof(float) * n);
    for (int64_t c = 0; c < n; ++c) {
        int i = (int)(c % sx), j = (int)((c / sx) % sy), k = (int)(c / ((int64_t)sx * sy));
        f3 pos = index_pos(&F.g, oc, i, j, k);
        fwd[c] = sample_phi(&F, pos) > 0.0f
                     ? tricubic(s, sx, sy, sz, &F.g, oc, back_trace(&F, pos, dt, 1.0f, max_substeps))
                     : s[c];
    }
    for (int64_t c = 0; c < n; ++c) {
        int i = (int)(c % sx), j = (int)((c / sx) % sy), k = (int)(c / ((int64_t)sx * sy));
        f3 pos = index_pos(&F.g, oc, i, j, k);
        bwd[c] = sample_phi(&F, pos) > 0.0f
                     ? tricubic(fwd, sx, sy, sz, &F.g, oc, back_trace(&F, pos, dt, -1.0f, max_substeps))
                     : fwd[c];
    }
    for (int64_t c = 0; c < n; ++c) {
        int i = (int)(c % sx), j = (int)((c / sx) % sy), k = (int)(c / ((int64_t)sx * sy));
        f3 pos = index_pos(&F.g, oc, i, j, k);
        if (!(sample_phi(&F, pos) > 0.0f)) continue;
        f3 tr = back_trace(&F, pos, dt, 1.0f, max_substeps);
        float fv = fwd[c];
        float corr = fv + (s[c] - bwd[c]) * 0.5f;
        so[c] = clamp_correction(&F, s, 3, sx, sy, sz, oc, tr, corr, fv);
    }
    free(fwd);
    free(bwd);
}

/* ---- constrainVelocity ------------------------------------------------ */
static float frac_inside_sdf(float p0, float p1) {
    int a = p0 < 0.0f, b = p1 < 0.0f;
    if (a && b) return 1.0f;
    if (a) return p0 / (p0 - p1);
    if (b) return p1 / (p1 - p0);
    return 0.0f;
}

static f3 trilinear_gradient(const float *d, const og_geom *g, f3 o, f3 pos) {
    const int n[3] = {g->nx, g->ny, g->nz};
    float coord[3] = {gclamp((pos.x - o.x) / g->hx), gclamp((pos.y - o.y) / g->hy), gclamp((pos.z - o.z) / g->hz)};
    int lo[3], hi[3];
    float t[3];
    for (int a = 0; a < 3; ++a) {
        int idx = (int)floorf(coord[a]);
        lo[a] = imax(0, imin(idx, n[a] - 2));
        hi[a] = imin(lo[a] + 1, n[a] - 1);
        t[a] = fminf(fmaxf(coord[a] - (float)lo[a], 0.0f), 1.0f);
    }
#define V(i, j, k) d[(i) + (int64_t)g->nx * ((j) + (int64_t)g->ny * (k))]
    float v000 = V(lo[0], lo[1], lo[2]), v100 = V(hi[0], lo[1], lo[2]), v010 = V(lo[0], hi[1], lo[2]);
    float v110 = V(hi[0], hi[1], lo[2]), v001 = V(lo[0], lo[1], hi[2]), v101 = V(hi[0], lo[1], hi[2]);
    float v011 = V(lo[0], hi[1], hi[2]), v111 = V(hi[0], hi[1], hi[2]);
#undef V
    const float tx = t[0], ty = t[1], tz = t[2];
    f3 r;
    float s = (1.0f - ty) * (1.0f - tz) * (v100 - v000);
    s = s + ty * (1.0f - tz) * (v110 - v010);
    s = s + (1.0f - ty) * tz * (v101 - v001);
    s = s + ty * tz * (v111 - v011);
    r.x = s / g->hx;
    s = (1.0f - tx) * (1.0f - tz) * (v010 - v000);
    s = s + tx * (1.0f - tz) * (v110 - v100);
    s = s + (1.0f - tx) * tz * (v011 - v001);
    s = s + tx * tz * (v111 - v101);
    r.y = s / g->hy;
    s = (1.0f - tx) * (1.0f - ty) * (v001 - v000);
    s = s + tx * (1.0f - ty) * (v101 - v100);
    s = s + (1.0f - tx) * ty * (v011 - v010);
    s = s + tx * ty * (v111 - v110);
    r.z = s / g->hz;
    return r;
}

/* projectAndApplyFriction (grid_blocked_boundary_condition_solver3.js:30-44) */
static f3 friction(f3 vel, f3 n, float mu) {
    float vn = vel.x * n.x + vel.y * n.y + vel.z * n.z;
    f3 vt = {vel.x - n.x * vn, vel.y - n.y * vn, vel.z - n.z * vn};
    float tl = sqrtf(vt.x * vt.x + vt.y * vt.y + vt.z * vt.z);
    if (tl > 0.0f) {
        float veln = fmaxf(-vn, 0.0f);
        float scale = fmaxf(1.0f - veln * mu / tl, 0.0f);
        vt.x = vt.x * scale;
        vt.y = vt.y * scale;
        vt.z = vt.z * scale;
    }
    return vt;
}

static void extrapolate(float *val, const int32_t *marker, int sx, int sy, int sz, int depth) {
    const int64_t n = (int64_t)sx * sy * sz;
    int32_t *va = (int32_t *)malloc(sizeof(int32_t) * n), *vb = (int32_t *)malloc(sizeof(int32_t) * n);
    float *scratch = (float *)malloc(sizeof(float) * n);
    memcpy(va, marker, sizeof(int32_t) * n);
    float *src = val, *dst = scratch;
    int32_t *vs = va, *vd = vb;
    for (int it = 0; it < depth; ++it) {
        for (int64_t c = 0; c < n; ++c) {
            int i = (int)(c % sx), j = (int)((c / sx) % sy), k = (int)(c / ((int64_t)sx * sy));
            if (vs[c] != 0) {
                dst[c] = src[c];
                vd[c] = 1;
                continue;
            }
            float total = 0.0f;
            int count = 0;
            const int64_t sy_ = sx, sz_ = (int64_t)sx * sy;
            if (i + 1 < sx && vs[c + 1]) { total = total + src[c + 1]; count++; }
            if (i > 0 && vs[c - 1]) { total = total + src[c - 1]; count++; }
            if (j + 1 < sy && vs[c + sy_]) { total = total + src[c + sy_]; count++; }
            if (j > 0 && vs[c - sy_]) { total = total + src[c - sy_]; count++; }
            if (k + 1 < sz && vs[c + sz_]) { total = total + src[c + sz_]; count++; }
            if (k > 0 && vs[c - sz_]) { total = total + src[c - sz_]; count++; }
            if (count > 0) {
                dst[c] = total / (float)count;
                vd[c] = 1;
            } else {
                dst[c] = src[c];
                vd[c] = 0;
            }
        }
        float *tf = src; src = dst; dst = tf;
        int32_t *ti = vs; vs = vd; vd = ti;
    }
    if (src != val) memcpy(val, src, sizeof(float) * n);
    free(va);
    free(vb);
    free(scratch);
}

static inline float clamp_component(float v) {
    if (isnan(v) || isinf(v)) return 0.0f;
    return fminf(fmaxf(v, -100.0f), 100.0f);
}

/* constrainVelocity(depth) on (u, v, w) in place.  phi: collider SDF (cell
 * centred, NULL = no collider); cw*: collider face weights (NULL = decide
 * by sampling phi); closed: DIRECTION_* bits; inflows: n_in cell-centred
 * SDFs (phis, n_in * ncell floats) with velocities (3 per inflow) and modes
 * (0 set, 1 add). */
void orc_constrain_velocity(const int *res, const float *h, const float *o, float *u, float *v, float *w,
                            const float *phi, const float *cwu, const float *cwv, const float *cww, int closed,
                            int n_in, const float *in_phis, const float *in_vel, const int *in_mode, int depth) {
    og_field F = make_field(res, h, o, u, v, w, phi);
    const og_geom *g = &F.g;
    float *data[3] = {u, v, w};
    const float *cw[3] = {cwu, cwv, cww};
    const int nx = g->nx, ny = g->ny, nz = g->nz;
    if (phi) {
        int32_t *marker[3];
        float *temp[3];
        for (int a = 0; a < 3; ++a) {
            int sx, sy, sz;
            comp_shape(g, a, &sx, &sy, &sz);
            const int64_t n = (int64_t)sx * sy * sz;
            marker[a] = (int32_t *)malloc(sizeof(int32_t) * n);
            temp[a] = (float *)malloc(sizeof(float) * n);
            f3 oa = comp_origin(g, a);
            for (int64_t f = 0; f < n; ++f) {
                int i = (int)(f % sx), j = (int)((f / sx) % sy), k = (int)(f / ((int64_t)sx * sy));
                f3 pt = index_pos(g, oa, i, j, k);
                float open;
                if (cw[a]) {
                    open = cw[a][f];
                } else {
                    f3 off = {a == 0 ? g->hx * 0.5f : 0.0f, a == 1 ? g->hy * 0.5f : 0.0f, a == 2 ? g->hz * 0.5f : 0.0f};
                    f3 pm = {pt.x - off.x, pt.y - off.y, pt.z - off.z}, pp = {pt.x + off.x, pt.y + off.y, pt.z + off.z};
                    float fr = frac_inside_sdf(sample_phi(&F, pm), sample_phi(&F, pp));
                    open = 1.0f - fminf(fmaxf(fr, 0.0f), 1.0f);
                }
                if (open > 0.0f) {
                    marker[a][f] = 1;
                } else {
                    data[a][f] = 0.0f;   /* static collider: velocityAt = 0 */
                    marker[a][f] = 0;
                }
            }
        }
        for (int a = 0; a < 3; ++a) {
            int sx, sy, sz;
            comp_shape(g, a, &sx, &sy, &sz);
            extrapolate(data[a], marker[a], sx, sy, sz, depth);
        }
        const f3 oc = comp_origin(g, 3);
        for (int a = 0; a < 3; ++a) {
            int sx, sy, sz;
            comp_shape(g, a, &sx, &sy, &sz);
            const int64_t n = (int64_t)sx * sy * sz;
            f3 oa = comp_origin(g, a);
            for (int64_t f = 0; f < n; ++f) {
                int i = (int)(f % sx), j = (int)((f / sx) % sy), k = (int)(f / ((int64_t)sx * sy));
                f3 pt = index_pos(g, oa, i, j, k);
                int blocked = cw[a] ? (cw[a][f] <= 0.0f) : (sample_phi(&F, pt) < 0.0f);
                if (!blocked) {
                    temp[a][f] = data[a][f];
                    continue;
                }
                f3 vel = sample_vel(&F, pt);
                f3 gr = trilinear_gradient(phi, g, oc, pt);
                float gl = sqrtf(gr.x * gr.x + gr.y * gr.y + gr.z * gr.z);
                if (gl > 0.0f) {
                    f3 nn = {gr.x / gl, gr.y / gl, gr.z / gl};
                    f3 vt = friction(vel, nn, 0.5f);
                    temp[a][f] = a == 0 ? vt.x : (a == 1 ? vt.y : vt.z);
                } else {
                    temp[a][f] = 0.0f;
                }
            }
        }
        for (int a = 0; a < 3; ++a) {
            int sx, sy, sz;
            comp_shape(g, a, &sx, &sy, &sz);
            memcpy(data[a], temp[a], sizeof(float) * (int64_t)sx * sy * sz);
            free(temp[a]);
            free(marker[a]);
        }
        /* blockedBoundary: a collider cell's faces toward fluid cells */
        for (int k = 0; k < nz; ++k)
            for (int j = 0; j < ny; ++j)
                for (int i = 0; i < nx; ++i) {
                    const int64_t c = i + (int64_t)nx * (j + (int64_t)ny * k);
#define SOLID(ii, jj, kk) (phi[(ii) + (int64_t)nx * ((jj) + (int64_t)ny * (kk))] < 0.0f)
                    if (!SOLID(i, j, k)) continue;
                    (void)c;
                    if (i > 0 && !SOLID(i - 1, j, k)) u[i + (int64_t)(nx + 1) * (j + (int64_t)ny * k)] = 0.0f;
                    if (i < nx - 1 && !SOLID(i + 1, j, k)) u[i + 1 + (int64_t)(nx + 1) * (j + (int64_t)ny * k)] = 0.0f;
                    if (j > 0 && !SOLID(i, j - 1, k)) v[i + (int64_t)nx * (j + (int64_t)(ny + 1) * k)] = 0.0f;
                    if (j < ny - 1 && !SOLID(i, j + 1, k)) v[i + (int64_t)nx * (j + 1 + (int64_t)(ny + 1) * k)] = 0.0f;
                    if (k > 0 && !SOLID(i, j, k - 1)) w[i + (int64_t)nx * (j + (int64_t)ny * k)] = 0.0f;
                    if (k < nz - 1 && !SOLID(i, j, k + 1)) w[i + (int64_t)nx * (j + (int64_t)ny * (k + 1))] = 0.0f;
#undef SOLID
                }
    }
    /* closed domain walls (DIRECTION_* of constant.js:24-38) */
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j) {
            if (closed & 1) u[0 + (int64_t)(nx + 1) * (j + (int64_t)ny * k)] = 0.0f;
            if (closed & 2) u[nx + (int64_t)(nx + 1) * (j + (int64_t)ny * k)] = 0.0f;
        }
    for (int k = 0; k < nz; ++k)
        for (int i = 0; i < nx; ++i) {
            if (closed & 4) v[i + (int64_t)nx * (0 + (int64_t)(ny + 1) * k)] = 0.0f;
            if (closed & 8) v[i + (int64_t)nx * (ny + (int64_t)(ny + 1) * k)] = 0.0f;
        }
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            if (closed & 16) w[i + (int64_t)nx * (j + (int64_t)ny * 0)] = 0.0f;
            if (closed & 32) w[i + (int64_t)nx * (j + (int64_t)ny * nz)] = 0.0f;
        }
    /* inflows: faces inside the inflow's SDF get (or gain) its velocity */
    const int64_t ncell = (int64_t)nx * ny * nz;
    for (int q = 0; q < n_in; ++q) {
        og_field Fi = F;
        Fi.phi = in_phis + ncell * q;
        for (int a = 0; a < 3; ++a) {
            int sx, sy, sz;
            comp_shape(g, a, &sx, &sy, &sz);
            f3 oa = comp_origin(g, a);
            const int64_t n = (int64_t)sx * sy * sz;
            for (int64_t f = 0; f < n; ++f) {
                int i = (int)(f % sx), j = (int)((f / sx) % sy), k = (int)(f / ((int64_t)sx * sy));
                f3 pt = index_pos(g, oa, i, j, k);
                if (sample_phi(&Fi, pt) < 0.0f) {
                    float val = in_vel[3 * q + a];
                    data[a][f] = in_mode[q] ? data[a][f] + val : val;
                }
            }
        }
    }
    for (int a = 0; a < 3; ++a) {
        int sx, sy, sz;
        comp_shape(g, a, &sx, &sy, &sz);
        const int64_t n = (int64_t)sx * sy * sz;
        for (int64_t f = 0; f < n; ++f) data[a][f] = clamp_component(data[a][f]);
    }
}

/* explicit viscosity: out = in + (dt nu) lap(in) on faces strictly inside
 * the component's own axis range; neighbours past an array end read the
 * face itself (Neumann); faces on the component's boundary planes copy. */
void orc_viscosity(const int *res, const float *h, const float *u, const float *v, const float *w, float nu,
                   float dt, float *uo, float *vo, float *wo) {
    og_geom g = {res[0], res[1], res[2], h[0], h[1], h[2], 0, 0, 0};
    const float *in[3] = {u, v, w};
    float *out[3] = {uo, vo, wo};
    const float ih[3] = {1.0f / (h[0] * h[0]), 1.0f / (h[1] * h[1]), 1.0f / (h[2] * h[2])};
    const float c = dt * nu;
    for (int a = 0; a < 3; ++a) {
        int s[3];
        comp_shape(&g, a, &s[0], &s[1], &s[2]);
        const float *d = in[a];
        for (int k = 0; k < s[2]; ++k)
            for (int j = 0; j < s[1]; ++j)
                for (int i = 0; i < s[0]; ++i) {
                    const int idx[3] = {i, j, k};
                    const int64_t f = i + (int64_t)s[0] * (j + (int64_t)s[1] * k);
                    const float x = d[f];
                    if (idx[a] == 0 || idx[a] == s[a] - 1) {
                        out[a][f] = x;
                        continue;
                    }
                    const int64_t st[3] = {1, s[0], (int64_t)s[0] * s[1]};
                    float lap = 0.0f;
                    for (int b = 0; b < 3; ++b) {
                        float up = idx[b] + 1 < s[b] ? d[f + st[b]] : x;
                        float dn = idx[b] > 0 ? d[f - st[b]] : x;
                        lap = lap + ((up - x) + (dn - x)) * ih[b];
                    }
                    out[a][f] = x + c * lap;
                }
    }
}

/* ---- outflow (grid_outflow_solver3.js:79-210) --------------------------
 * Each outflow is a cell-centred SDF on its own grid (geometry pres/ph/po,
 * three entries per outflow; the SDFs concatenated in phi_all); inside is
 * phi < 0 (level_set_utils.js:5-9), sampled trilinearly (sdf_collider3.js:33-45). */
static og_geom outflow_geom(const int *pres, const float *ph, const float *po, int q) {
    og_geom G = {pres[3 * q], pres[3 * q + 1], pres[3 * q + 2], ph[3 * q],     ph[3 * q + 1],
                 ph[3 * q + 2], po[3 * q], po[3 * q + 1], po[3 * q + 2]};
    return G;
}
static const float *outflow_phi(const float *phi_all, const int *pres, int q) {
    const float *p = phi_all;
    for (int r = 0; r < q; ++r) p += (int64_t)pres[3 * r] * pres[3 * r + 1] * pres[3 * r + 2];
    return p;
}
static float outflow_sample(const float *phi, const og_geom *G, f3 pt) {
    return trilinear(phi, G->nx, G->ny, G->nz, G, comp_origin(G, 3), pt);
}

/* applyOutflowVelocityBC (:98-170): per outflow, per component (u, v, w in
 * turn, each written back before the next is computed), a face inside the
 * outflow with a non-zero SDF gradient relaxes toward the velocity sampled
 * one spacing upstream, pt + n h, n = grad / |grad|, by the Courant number
 * clamp(max(0, U . -n) dt / h, 0, 1) of the bulk velocity U at the face,
 * then clamps to +-1e3; a face with a zero gradient keeps its value. */
void orc_outflow_velocity(const int *res, const float *h, const float *o, float *u, float *v, float *w, float dt,
                          int n_out, const float *phi_all, const int *pres, const float *ph, const float *po) {
    og_field F = make_field(res, h, o, u, v, w, NULL);
    float *data[3] = {u, v, w};
    const float hs[3] = {h[0], h[1], h[2]};
    for (int q = 0; q < n_out; ++q) {
        og_geom G = outflow_geom(pres, ph, po, q);
        const float *phi = outflow_phi(phi_all, pres, q);
        for (int a = 0; a < 3; ++a) {
            int sx, sy, sz;
            comp_shape(&F.g, a, &sx, &sy, &sz);
            const int64_t n = (int64_t)sx * sy * sz;
            float *dst = (float *)malloc(sizeof(float) * (size_t)n);
            unsigned char *in = (unsigned char *)calloc((size_t)n, 1);
            const f3 oa = comp_origin(&F.g, a);
            for (int k = 0; k < sz; ++k)
                for (int j = 0; j < sy; ++j)
                    for (int i = 0; i < sx; ++i) {
                        const int64_t c = i + (int64_t)sx * (j + (int64_t)sy * k);
                        const f3 pt = index_pos(&F.g, oa, i, j, k);
                        if (!(outflow_sample(phi, &G, pt) < 0.0f)) continue;
                        in[c] = 1;
                        const float cur = data[a][c];
                        const f3 gr = trilinear_gradient(phi, &G, comp_origin(&G, 3), pt);
                        const float gl = sqrtf(gr.x * gr.x + gr.y * gr.y + gr.z * gr.z);
                        if (!(gl > 0.0f)) {
                            dst[c] = cur;
                            continue;
                        }
                        const f3 nn = {gr.x / gl, gr.y / gl, gr.z / gl};
                        const f3 up = {pt.x + nn.x * hs[a], pt.y + nn.y * hs[a], pt.z + nn.z * hs[a]};
                        const f3 bulk = sample_vel(&F, pt);
                        float dot = bulk.x * -nn.x;
                        dot = dot + bulk.y * -nn.y;
                        dot = dot + bulk.z * -nn.z;
                        const float speed = fmaxf(0.0f, dot);
                        const float courant = fminf(fmaxf(speed * dt / hs[a], 0.0f), 1.0f);
                        const f3 uv = sample_vel(&F, up);
                        const float upc = a == 0 ? uv.x : (a == 1 ? uv.y : uv.z);
                        const float relaxed = cur + (upc - cur) * courant;
                        dst[c] = fminf(fmaxf(relaxed, -1.0e3f), 1.0e3f);
                    }
            for (int64_t c = 0; c < n; ++c)
                if (in[c]) data[a][c] = dst[c];
            free(dst);
            free(in);
        }
    }
}

/* clearOutflowScalarField (:174-196): cells of a cell-centred scalar grid
 * (geometry sres/sh/so) inside any outflow become 0 */
void orc_outflow_clear_scalar(const int *sres, const float *sh, const float *so, float *data, int n_out,
                              const float *phi_all, const int *pres, const float *ph, const float *po) {
    og_geom S = {sres[0], sres[1], sres[2], sh[0], sh[1], sh[2], so[0], so[1], so[2]};
    const f3 oc = comp_origin(&S, 3);
    for (int q = 0; q < n_out; ++q) {
        og_geom G = outflow_geom(pres, ph, po, q);
        const float *phi = outflow_phi(phi_all, pres, q);
        for (int k = 0; k < S.nz; ++k)
            for (int j = 0; j < S.ny; ++j)
                for (int i = 0; i < S.nx; ++i)
                    if (outflow_sample(phi, &G, index_pos(&S, oc, i, j, k)) < 0.0f)
                        data[i + (int64_t)S.nx * (j + (int64_t)S.ny * k)] = 0.0f;
    }
}

/* createOutflowPressureDirichlet3 (sdf_inflow_outflow3.js:44-64) at the
 * cell centres of the pressure grid (geometry sres/sh/so): active where any
 * outflow holds the centre, target everywhere */
void orc_outflow_dirichlet(const int *sres, const float *sh, const float *so, float target, int n_out,
                           const float *phi_all, const int *pres, const float *ph, const float *po,
                           uint8_t *active, float *tgt) {
    og_geom S = {sres[0], sres[1], sres[2], sh[0], sh[1], sh[2], so[0], so[1], so[2]};
    const f3 oc = comp_origin(&S, 3);
    for (int k = 0; k < S.nz; ++k)
        for (int j = 0; j < S.ny; ++j)
            for (int i = 0; i < S.nx; ++i) {
                const int64_t c = i + (int64_t)S.nx * (j + (int64_t)S.ny * k);
                const f3 pt = index_pos(&S, oc, i, j, k);
                int in = 0;
                for (int q = 0; q < n_out; ++q) {
                    og_geom G = outflow_geom(pres, ph, po, q);
                    in |= outflow_sample(outflow_phi(phi_all, pres, q), &G, pt) < 0.0f;
                }
                active[c] = (uint8_t)in;
                tgt[c] = target;
            }
}
