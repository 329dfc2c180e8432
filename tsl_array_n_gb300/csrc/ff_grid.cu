// Grid-velocity kernels around the projection: semi-Lagrangian advection of
// the MAC velocity and of cell scalars (fluxflow src/grid/advection_solver3.js),
// the blocked-boundary velocity constraint
// (src/grid/grid_blocked_boundary_condition_solver3.js) and explicit viscosity
// (no reference counterpart; src/grid/grid_solver3.js:104 leaves it a no-op).
//
// Arithmetic is FP32 as in the reference's WGSL, one IEEE operation at a
// time: this file is compiled with -fmad=false so no multiply-add is fused,
// and every expression keeps the reference's evaluation order.  That makes
// the results reproducible operation for operation on any IEEE FP32 machine.
//
// All kernels are HBM/L2-bound gathers (a tricubic sample reads 64 taps of
// one component, mostly L1/L2 hits); one thread per face or cell.
#include "ff_grid.cuh"
#include <algorithm>
#include <cmath>
#include <utility>

namespace {
using namespace ffg;

// makeMarkAndProject (grid_blocked_boundary_condition_solver3.js:196-249):
// open faces are fluid (marker 1); closed faces take the collider's
// velocity (a static collider: 0) and marker 0
__global__ void __launch_bounds__(256, 6) k_mark(VelField F, int a, const float *__restrict__ cw, float *__restrict__ data,
                       int *__restrict__ marker) {
    int sx, sy, sz;
    comp_shape(F.g, a, sx, sy, sz);
    const long long n = (long long)sx * sy * sz;
    const F3 o = comp_origin(F.g, a);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(f, sx, sy, i, j, k);
        float open;
        if (cw) {
            open = cw[f];
        } else {
            const F3 pt = index_pos(F.g, o, i, j, k);
            const F3 off{a == 0 ? F.g.hx * 0.5f : 0.0f, a == 1 ? F.g.hy * 0.5f : 0.0f, a == 2 ? F.g.hz * 0.5f : 0.0f};
            const float fr = frac_inside_sdf(sample_phi(F, F.phi, F3{pt.x - off.x, pt.y - off.y, pt.z - off.z}),
                                             sample_phi(F, F.phi, F3{pt.x + off.x, pt.y + off.y, pt.z + off.z}));
            open = 1.0f - fminf(fmaxf(fr, 0.0f), 1.0f);
        }
        if (open > 0.0f) {
            marker[f] = 1;
        } else {
            data[f] = 0.0f;
            marker[f] = 0;
        }
    }
}

// Advection stages on one component (a = 0..2 faces, 3 cell scalar):
//   0 order 1: out = cubic(src @ trace(+1)) where the position is open
//   1 MacCormack forward:  aux = open ? cubic(src @ trace(+1)) : src
//   2 MacCormack backward: aux = open ? cubic(fwd @ trace(-1)) : fwd
//   3 MacCormack correct:  out = clamp(fwd + (src - bwd)/2) where open
// (one kernel per stage: a smaller body for the instruction cache)
template <int stage>
__global__ void k_advect(VelField F, int a, const float *__restrict__ src, const float *__restrict__ fwd,
                         const float *__restrict__ bwd, float *__restrict__ out, float dt, int max_substeps) {
    int sx, sy, sz;
    if (a < 3) comp_shape(F.g, a, sx, sy, sz);
    else sx = F.g.nx, sy = F.g.ny, sz = F.g.nz;
    const long long n = (long long)sx * sy * sz;
    const F3 o = comp_origin(F.g, a);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(f, sx, sy, i, j, k);
        const F3 pos = index_pos(F.g, o, i, j, k);
        const bool open = sample_phi(F, F.phi, pos) > 0.0f;
        if constexpr (stage == 0) {
            if (open) out[f] = tricubic(src, sx, sy, sz, F.g, o, back_trace(F, pos, dt, 1.0f, max_substeps));
        } else if constexpr (stage == 1) {
            out[f] = open ? tricubic(src, sx, sy, sz, F.g, o, back_trace(F, pos, dt, 1.0f, max_substeps)) : src[f];
        } else if constexpr (stage == 2) {
            out[f] = open ? tricubic(fwd, sx, sy, sz, F.g, o, back_trace(F, pos, dt, -1.0f, max_substeps)) : fwd[f];
        } else if (open) {
            // clampCorrection (stage 3): min/max over the 8 trilinear corners of the
            // traced point whose own positions are open
            const F3 tr = back_trace(F, pos, dt, 1.0f, max_substeps);
            const float fv = fwd[f];
            const float corr = fv + (src[f] - bwd[f]) * 0.5f;
            const float gx = gclamp((tr.x - o.x) / F.g.hx), gy = gclamp((tr.y - o.y) / F.g.hy),
                        gz = gclamp((tr.z - o.z) / F.g.hz);
            const int i0 = (int)floorf(gx), j0 = (int)floorf(gy), k0 = (int)floorf(gz);
            const int ic[2] = {iclamp(i0, 0, sx - 1), iclamp(i0 + 1, 0, sx - 1)};
            const int jc[2] = {iclamp(j0, 0, sy - 1), iclamp(j0 + 1, 0, sy - 1)};
            const int kc[2] = {iclamp(k0, 0, sz - 1), iclamp(k0 + 1, 0, sz - 1)};
            float mn = 1e30f, mx = -1e30f;
            bool have = false;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int ni = ic[c & 1], nj = jc[(c >> 1) & 1], nk = kc[(c >> 2) & 1];
                const bool valid = sample_phi(F, F.phi, index_pos(F.g, o, ni, nj, nk)) > 0.0f;
                const float val = src[ni + (long long)sx * (nj + (long long)sy * nk)];
                if (valid) {
                    mn = fminf(mn, val);
                    mx = fmaxf(mx, val);
                    have = true;
                }
            }
            out[f] = (have && corr >= mn && corr <= mx) ? corr : fv;
        }
    }
}

// trace(start, direction) of a list of points (float3 per point)
__global__ void k_trace(VelField F, long long n, const float *__restrict__ pin, float *__restrict__ pout, float dt,
                        float dirn, int max_substeps) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const F3 r = back_trace(F, F3{pin[3 * q], pin[3 * q + 1], pin[3 * q + 2]}, dt, dirn, max_substeps);
        pout[3 * q] = r.x;
        pout[3 * q + 1] = r.y;
        pout[3 * q + 2] = r.z;
    }
}

// makeNoFluxProjection (:251-286) with projectAndApplyFriction (:30-44):
// a closed face takes the tangential part of the sampled velocity,
// reduced by Coulomb friction (coefficient 0.5, sdf_collider3.js:16)
__global__ void __launch_bounds__(256, 6) k_noflux(VelField F, int a, const float *__restrict__ cw, const float *__restrict__ data,
                         float *__restrict__ temp) {
    int sx, sy, sz;
    comp_shape(F.g, a, sx, sy, sz);
    const long long n = (long long)sx * sy * sz;
    const F3 o = comp_origin(F.g, a), oc = comp_origin(F.g, 3);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(f, sx, sy, i, j, k);
        const F3 pt = index_pos(F.g, o, i, j, k);
        const bool blocked = cw ? (cw[f] <= 0.0f) : (sample_phi(F, F.phi, pt) < 0.0f);
        if (!blocked) {
            temp[f] = data[f];
            continue;
        }
        const F3 vel = sample_vel(F, pt);
        const F3 gr = trilinear_gradient(F.phi, F.g, oc, pt);
        const float gl = sqrtf(gr.x * gr.x + gr.y * gr.y + gr.z * gr.z);
        if (gl > 0.0f) {
            const F3 nn{gr.x / gl, gr.y / gl, gr.z / gl};
            const float vn = vel.x * nn.x + vel.y * nn.y + vel.z * nn.z;
            F3 vt{vel.x - nn.x * vn, vel.y - nn.y * vn, vel.z - nn.z * vn};
            const float tl = sqrtf(vt.x * vt.x + vt.y * vt.y + vt.z * vt.z);
            if (tl > 0.0f) {
                const float veln = fmaxf(-vn, 0.0f);
                const float scale = fmaxf(1.0f - veln * 0.5f / tl, 0.0f);
                vt = F3{vt.x * scale, vt.y * scale, vt.z * scale};
            }
            temp[f] = a == 0 ? vt.x : (a == 1 ? vt.y : vt.z);
        } else {
            temp[f] = 0.0f;
        }
    }
}

// blockedBoundary (:288-330): a collider cell's faces toward fluid cells
// take the collider velocity (0)
__global__ void k_blocked(G3 g, const float *__restrict__ phi, float *u, float *v, float *w) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(c, g.nx, g.ny, i, j, k);
        auto solid = [&](int ii, int jj, int kk) { return phi[ii + (long long)g.nx * (jj + (long long)g.ny * kk)] < 0.0f; };
        if (!solid(i, j, k)) continue;
        const int nx = g.nx, ny = g.ny, nz = g.nz;
        if (i > 0 && !solid(i - 1, j, k)) u[i + (long long)(nx + 1) * (j + (long long)ny * k)] = 0.0f;
        if (i < nx - 1 && !solid(i + 1, j, k)) u[i + 1 + (long long)(nx + 1) * (j + (long long)ny * k)] = 0.0f;
        if (j > 0 && !solid(i, j - 1, k)) v[i + (long long)nx * (j + (long long)(ny + 1) * k)] = 0.0f;
        if (j < ny - 1 && !solid(i, j + 1, k)) v[i + (long long)nx * (j + 1 + (long long)(ny + 1) * k)] = 0.0f;
        if (k > 0 && !solid(i, j, k - 1)) w[i + (long long)nx * (j + (long long)ny * k)] = 0.0f;
        if (k < nz - 1 && !solid(i, j, k + 1)) w[i + (long long)nx * (j + (long long)ny * (k + 1))] = 0.0f;
    }
}

// walls (zeroULeft .. zeroWFront), inflows (buildInflowKernels) and the
// final clamp (clampComponent, |v| <= 100, non-finite -> 0), per component
__global__ void __launch_bounds__(256, 6) k_walls_inflow_clamp(G3 g, int a, float *__restrict__ data, int closed, int n_in,
                                     const float *const *__restrict__ in_phi, const float *__restrict__ in_vel,
                                     const int *__restrict__ in_mode) {
    int sx, sy, sz;
    comp_shape(g, a, sx, sy, sz);
    const long long n = (long long)sx * sy * sz;
    const F3 o = comp_origin(g, a);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(f, sx, sy, i, j, k);
        float val = data[f];
        const int idx = a == 0 ? i : (a == 1 ? j : k), last = (a == 0 ? sx : (a == 1 ? sy : sz)) - 1;
        if (((closed >> (2 * a)) & 1) && idx == 0) val = 0.0f;
        if (((closed >> (2 * a + 1)) & 1) && idx == last) val = 0.0f;
        if (n_in) {
            const F3 pt = index_pos(g, o, i, j, k);
            VelField F{g, nullptr, nullptr, nullptr, nullptr};
            for (int q = 0; q < n_in; ++q) {
                if (sample_phi(F, in_phi[q], pt) < 0.0f) {
                    const float add = in_vel[3 * q + a];
                    val = in_mode[q] ? val + add : add;
                }
            }
        }
        data[f] = (isnan(val) || isinf(val)) ? 0.0f : fminf(fmaxf(val, -100.0f), 100.0f);
    }
}

// explicit viscosity: out = in + (dt nu) lap(in) inside the component's own
// axis range, Neumann past the array ends; the component's boundary planes
// copy through
__global__ void k_viscosity(G3 g, int a, const float *__restrict__ in, float *__restrict__ out, float c, float ihx,
                            float ihy, float ihz) {
    int s[3];
    comp_shape(g, a, s[0], s[1], s[2]);
    const long long n = (long long)s[0] * s[1] * s[2];
    const long long st[3] = {1, s[0], (long long)s[0] * s[1]};
    const float ih[3] = {ihx, ihy, ihz};
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        int idx[3];
        unflatten(f, s[0], s[1], idx[0], idx[1], idx[2]);
        const float x = in[f];
        if (idx[a] == 0 || idx[a] == s[a] - 1) {
            out[f] = x;
            continue;
        }
        float lap = 0.0f;
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            const float up = idx[b] + 1 < s[b] ? in[f + st[b]] : x;
            const float dn = idx[b] > 0 ? in[f - st[b]] : x;
            lap = lap + ((up - x) + (dn - x)) * ih[b];
        }
        out[f] = x + c * lap;
    }
}

int launch_blocks(long long n) { return (int)std::min<long long>((n + 255) / 256, 152LL * 16); }

int post(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return ff_set_error(FF_E_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
    return FF_OK;
}

G3 geom_of(const int *res, const double *h, const double *o) {
    G3 g;
    g.nx = res[0];
    g.ny = res[1];
    g.nz = res[2];
    g.hx = (float)h[0];
    g.hy = (float)h[1];
    g.hz = (float)h[2];
    g.ox = o ? (float)o[0] : 0.0f;
    g.oy = o ? (float)o[1] : 0.0f;
    g.oz = o ? (float)o[2] : 0.0f;
    return g;
}

long long comp_count(const G3 &g, int a) {
    int sx, sy, sz;
    if (a == 3) return (long long)g.nx * g.ny * g.nz;
    comp_shape(g, a, sx, sy, sz);
    return (long long)sx * sy * sz;
}

bool field_is(ff_field f, long long count) { return f && f->dtype == FF_FLOAT && f->count == count; }

}  // namespace

// ----------------------------------------------------------------- advect --
struct ff_advect_s {
    ff_ctx ctx = nullptr;
    ff_advect_desc desc{};
    G3 g{};
    ff_field phi = nullptr;           // borrowed
    float *fwd[4] = {}, *bwd[4] = {};  // order-2 scratch per component (3 = scalar)
};

extern "C" int ff_advect3_create(ff_ctx ctx, const ff_advect_desc *d, ff_advect *out) {
    FF_CHECK(ctx && d && out, FF_E_ARG, "ff_advect3_create: NULL argument");
    FF_CHECK(d->resolution[0] > 0 && d->resolution[1] > 0 && d->resolution[2] > 0, FF_E_ARG,
             "createSemiLagrangianAdvectionSolver3: resolution must be positive");
    FF_CHECK(d->order == 1 || d->order == 2, FF_E_ARG, "createSemiLagrangianAdvectionSolver3: order must be 1 or 2");
    FF_CHECK(d->max_substeps > 0, FF_E_ARG, "createSemiLagrangianAdvectionSolver3: maxSubsteps must be positive");
    FF_TRY(check_grid32(d->resolution, "createSemiLagrangianAdvectionSolver3"));
    *out = nullptr;
    cudaSetDevice(ctx->device);
    ff_advect a = new ff_advect_s();
    a->ctx = ctx;
    a->desc = *d;
    a->g = geom_of(d->resolution, d->grid_spacing, d->origin);
    if (d->order == 2) {
        for (int c = 0; c < 4; ++c) {
            size_t bytes = (size_t)comp_count(a->g, c) * 4;
            int st = ff_dev_alloc((void **)&a->fwd[c], bytes, ctx->stream);
            if (st == FF_OK) st = ff_dev_alloc((void **)&a->bwd[c], bytes, ctx->stream);
            if (st != FF_OK) {
                ff_advect3_destroy(a);
                return st;
            }
        }
    }
    *out = a;
    return FF_OK;
}

extern "C" int ff_advect3_destroy(ff_advect a) {
    if (!a) return FF_OK;
    cudaStreamSynchronize(a->ctx->stream);
    for (int c = 0; c < 4; ++c) {
        ff_dev_free(a->fwd[c]);
        ff_dev_free(a->bwd[c]);
    }
    delete a;
    return FF_OK;
}

extern "C" int ff_advect3_set_dt(ff_advect a, double dt) {
    FF_CHECK(a, FF_E_ARG, "NULL advection solver");
    a->desc.dt = dt;
    return FF_OK;
}

extern "C" int ff_advect3_set_collider(ff_advect a, ff_field phi) {
    FF_CHECK(a, FF_E_ARG, "NULL advection solver");
    FF_CHECK(!phi || field_is(phi, comp_count(a->g, 3)), FF_E_ARG, "collider SDF must be a float cell field");
    a->phi = phi;
    return FF_OK;
}

static int advect_component(ff_advect a, const VelField &F, int c, const float *src, float *out) {
    cudaStream_t s = a->ctx->stream;
    const long long n = comp_count(a->g, c);
    const int nb = launch_blocks(n);
    const float dt = (float)a->desc.dt;
    const int ms = a->desc.max_substeps;
    if (a->desc.order == 1) {
        k_advect<0><<<nb, 256, 0, s>>>(F, c, src, nullptr, nullptr, out, dt, ms);
        return post("advect");
    }
    k_advect<1><<<nb, 256, 0, s>>>(F, c, src, nullptr, nullptr, a->fwd[c], dt, ms);
    k_advect<2><<<nb, 256, 0, s>>>(F, c, src, a->fwd[c], nullptr, a->bwd[c], dt, ms);
    k_advect<3><<<nb, 256, 0, s>>>(F, c, src, a->fwd[c], a->bwd[c], out, dt, ms);
    return post("advect (MacCormack)");
}

extern "C" int ff_advect3_faces(ff_advect a, ff_field vu, ff_field vv, ff_field vw, ff_field iu, ff_field iv,
                                ff_field iw, ff_field ou, ff_field ov, ff_field ow) {
    FF_CHECK(a, FF_E_ARG, "NULL advection solver");
    ff_field vel[3] = {vu, vv, vw}, in[3] = {iu, iv, iw}, out[3] = {ou, ov, ow};
    for (int c = 0; c < 3; ++c)
        FF_CHECK(field_is(vel[c], comp_count(a->g, c)) && field_is(in[c], comp_count(a->g, c)) &&
                     field_is(out[c], comp_count(a->g, c)),
                 FF_E_ARG, "advectFaceCentered3: face field %d has the wrong shape or type", c);
    for (int c = 0; c < 3; ++c)
        FF_CHECK(out[c]->d != in[c]->d && out[c]->d != vel[c]->d, FF_E_ARG,
                 "advectFaceCentered3: output must not alias the input or the velocity");
    cudaSetDevice(a->ctx->device);
    VelField F{a->g, (const float *)vu->d, (const float *)vv->d, (const float *)vw->d,
               a->phi ? (const float *)a->phi->d : nullptr};
    for (int c = 0; c < 3; ++c) FF_TRY(advect_component(a, F, c, (const float *)in[c]->d, (float *)out[c]->d));
    return FF_OK;
}

extern "C" int ff_advect3_scalar(ff_advect a, ff_field vu, ff_field vv, ff_field vw, ff_field s_in, ff_field s_out) {
    FF_CHECK(a, FF_E_ARG, "NULL advection solver");
    for (int c = 0; c < 3; ++c)
        FF_CHECK(field_is(c == 0 ? vu : (c == 1 ? vv : vw), comp_count(a->g, c)), FF_E_ARG,
                 "advectScalar3: velocity component %d has the wrong shape", c);
    FF_CHECK(field_is(s_in, comp_count(a->g, 3)) && field_is(s_out, comp_count(a->g, 3)) && s_in->d != s_out->d,
             FF_E_ARG, "advectScalar3: scalar fields must be distinct float cell fields");
    cudaSetDevice(a->ctx->device);
    VelField F{a->g, (const float *)vu->d, (const float *)vv->d, (const float *)vw->d,
               a->phi ? (const float *)a->phi->d : nullptr};
    return advect_component(a, F, 3, (const float *)s_in->d, (float *)s_out->d);
}

extern "C" int ff_advect3_trace(ff_advect a, ff_field vu, ff_field vv, ff_field vw, ff_field p_in, ff_field p_out,
                                int direction) {
    FF_CHECK(a && p_in && p_out, FF_E_ARG, "NULL argument");
    for (int c = 0; c < 3; ++c)
        FF_CHECK(field_is(c == 0 ? vu : (c == 1 ? vv : vw), comp_count(a->g, c)), FF_E_ARG,
                 "trace: velocity component %d has the wrong shape", c);
    FF_CHECK(p_in->dtype == FF_VEC3 && p_out->dtype == FF_VEC3 && p_in->count == p_out->count, FF_E_ARG,
             "trace: points must be vec3 fields of equal length");
    FF_CHECK(direction == 1 || direction == -1, FF_E_ARG, "trace: direction must be 1 or -1");
    cudaSetDevice(a->ctx->device);
    VelField F{a->g, (const float *)vu->d, (const float *)vv->d, (const float *)vw->d,
               a->phi ? (const float *)a->phi->d : nullptr};
    const long long n = p_in->count;
    if (n == 0) return FF_OK;
    k_trace<<<launch_blocks(n), 256, 0, a->ctx->stream>>>(F, n, (const float *)p_in->d, (float *)p_out->d,
                                                          (float)a->desc.dt, (float)direction, a->desc.max_substeps);
    return post("trace");
}

// --------------------------------------------------------------------- bc --
struct ff_bc_s {
    ff_ctx ctx = nullptr;
    G3 g{};
    int closed = 63;                       // DIRECTION_ALL_3D
    ff_field phi = nullptr, cw[3] = {};    // borrowed
    int *marker[3] = {}, *valid[2][3] = {};
    float *temp[3] = {}, *scratch[3] = {};
    int n_in = 0;
    const float **in_phi = nullptr;        // device array of n_in pointers
    float *in_vel = nullptr;
    int *in_mode = nullptr;
};

extern "C" int ff_bc3_create(ff_ctx ctx, const int *res, const double *h, const double *origin, ff_bc *out) {
    FF_CHECK(ctx && res && h && out, FF_E_ARG, "ff_bc3_create: NULL argument");
    FF_CHECK(res[0] > 0 && res[1] > 0 && res[2] > 0, FF_E_ARG, "createGridBlockedBoundaryConditionSolver3: bad resolution");
    FF_TRY(check_grid32(res, "createGridBlockedBoundaryConditionSolver3"));
    *out = nullptr;
    cudaSetDevice(ctx->device);
    ff_bc b = new ff_bc_s();
    b->ctx = ctx;
    b->g = geom_of(res, h, origin);
    int st = FF_OK;
    for (int a = 0; a < 3 && st == FF_OK; ++a) {
        const size_t n = (size_t)comp_count(b->g, a);
        st = ff_dev_alloc((void **)&b->marker[a], n * 4, ctx->stream);
        if (st == FF_OK) st = ff_dev_alloc((void **)&b->valid[0][a], n * 4, ctx->stream);
        if (st == FF_OK) st = ff_dev_alloc((void **)&b->valid[1][a], n * 4, ctx->stream);
        if (st == FF_OK) st = ff_dev_alloc((void **)&b->temp[a], n * 4, ctx->stream);
        if (st == FF_OK) st = ff_dev_alloc((void **)&b->scratch[a], n * 4, ctx->stream);
    }
    if (st != FF_OK) {
        ff_bc3_destroy(b);
        return st;
    }
    *out = b;
    return FF_OK;
}

extern "C" int ff_bc3_destroy(ff_bc b) {
    if (!b) return FF_OK;
    cudaStreamSynchronize(b->ctx->stream);
    for (int a = 0; a < 3; ++a) {
        ff_dev_free(b->marker[a]);
        ff_dev_free(b->valid[0][a]);
        ff_dev_free(b->valid[1][a]);
        ff_dev_free(b->temp[a]);
        ff_dev_free(b->scratch[a]);
    }
    ff_dev_free((void *)b->in_phi);
    ff_dev_free(b->in_vel);
    ff_dev_free(b->in_mode);
    delete b;
    return FF_OK;
}

extern "C" int ff_bc3_set_collider(ff_bc b, ff_field phi, ff_field wu, ff_field wv, ff_field ww) {
    FF_CHECK(b, FF_E_ARG, "NULL boundary solver");
    FF_CHECK(!phi || field_is(phi, comp_count(b->g, 3)), FF_E_ARG, "setCollider: SDF must be a float cell field");
    ff_field w[3] = {wu, wv, ww};
    FF_CHECK((!wu && !wv && !ww) || (wu && wv && ww), FF_E_ARG, "setCollider: give all three face weights or none");
    for (int a = 0; a < 3; ++a)
        FF_CHECK(!w[a] || field_is(w[a], comp_count(b->g, a)), FF_E_ARG, "setCollider: face weight %d shape", a);
    b->phi = phi;
    for (int a = 0; a < 3; ++a) b->cw[a] = phi ? w[a] : nullptr;
    return FF_OK;
}

extern "C" int ff_bc3_set_closed(ff_bc b, int flags) {
    FF_CHECK(b, FF_E_ARG, "NULL boundary solver");
    FF_CHECK(flags >= 0 && flags <= 63, FF_E_ARG, "closedDomainBoundaryFlag must be a DIRECTION_* mask");
    b->closed = flags;
    return FF_OK;
}

extern "C" int ff_bc3_set_inflows(ff_bc b, int n, const ff_field *phis, const double *velocities, const int *modes) {
    FF_CHECK(b && n >= 0 && (n == 0 || (phis && velocities && modes)), FF_E_ARG, "setInflows: bad arguments");
    FF_CHECK(n <= 64, FF_E_LIMIT, "setInflows: at most 64 inflows");
    std::vector<const float *> hp(n);
    std::vector<float> hv(3 * n);
    std::vector<int> hm(n);
    for (int q = 0; q < n; ++q) {
        FF_CHECK(field_is(phis[q], comp_count(b->g, 3)), FF_E_ARG, "setInflows: inflow %d SDF must be a float cell field", q);
        FF_CHECK(modes[q] == 0 || modes[q] == 1, FF_E_ARG, "setInflows: mode must be 0 (set) or 1 (add)");
        hp[q] = (const float *)phis[q]->d;
        for (int c = 0; c < 3; ++c) hv[3 * q + c] = (float)velocities[3 * q + c];
        hm[q] = modes[q];
    }
    cudaStream_t s = b->ctx->stream;
    FF_CUDA(cudaStreamSynchronize(s));
    ff_dev_free((void *)b->in_phi);
    ff_dev_free(b->in_vel);
    ff_dev_free(b->in_mode);
    b->in_phi = nullptr;
    b->in_vel = nullptr;
    b->in_mode = nullptr;
    b->n_in = 0;
    if (n == 0) return FF_OK;
    FF_TRY(ff_dev_alloc((void **)&b->in_phi, sizeof(float *) * n, s));
    FF_TRY(ff_dev_alloc((void **)&b->in_vel, sizeof(float) * 3 * n, s));
    FF_TRY(ff_dev_alloc((void **)&b->in_mode, sizeof(int) * n, s));
    FF_CUDA(cudaMemcpyAsync((void *)b->in_phi, hp.data(), sizeof(float *) * n, cudaMemcpyHostToDevice, s));
    FF_CUDA(cudaMemcpyAsync(b->in_vel, hv.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
    FF_CUDA(cudaMemcpyAsync(b->in_mode, hm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    FF_CUDA(cudaStreamSynchronize(s));
    b->n_in = n;
    return FF_OK;
}

// constrainVelocity(extrapolationDepth) (:427-477), in place on (u, v, w)
extern "C" int ff_bc3_constrain(ff_bc b, ff_field u, ff_field v, ff_field w, int depth) {
    FF_CHECK(b, FF_E_ARG, "NULL boundary solver");
    FF_CHECK(depth >= 0, FF_E_ARG, "constrainVelocity: depth must be >= 0");
    ff_field fs[3] = {u, v, w};
    for (int a = 0; a < 3; ++a)
        FF_CHECK(field_is(fs[a], comp_count(b->g, a)), FF_E_ARG, "constrainVelocity: velocity component %d shape", a);
    cudaSetDevice(b->ctx->device);
    cudaStream_t s = b->ctx->stream;
    float *d[3] = {(float *)u->d, (float *)v->d, (float *)w->d};
    VelField F{b->g, d[0], d[1], d[2], b->phi ? (const float *)b->phi->d : nullptr};
    if (b->phi) {
        for (int a = 0; a < 3; ++a) {
            const long long n = comp_count(b->g, a);
            k_mark<<<launch_blocks(n), 256, 0, s>>>(F, a, b->cw[a] ? (const float *)b->cw[a]->d : nullptr, d[a],
                                                    b->marker[a]);
        }
        for (int a = 0; a < 3; ++a) {
            const long long n = comp_count(b->g, a);
            int sx, sy, sz;
            comp_shape(b->g, a, sx, sy, sz);
            FF_CUDA(cudaMemcpyAsync(b->valid[0][a], b->marker[a], n * 4, cudaMemcpyDeviceToDevice, s));
            float *src = d[a], *dst = b->scratch[a];
            int *vs = b->valid[0][a], *vd = b->valid[1][a];
            for (int it = 0; it < depth; ++it) {
                k_extrapolate<<<launch_blocks(n), 256, 0, s>>>(sx, sy, sz, src, dst, vs, vd);
                std::swap(src, dst);
                std::swap(vs, vd);
            }
            if (src != d[a]) FF_CUDA(cudaMemcpyAsync(d[a], src, n * 4, cudaMemcpyDeviceToDevice, s));
        }
        for (int a = 0; a < 3; ++a) {
            const long long n = comp_count(b->g, a);
            k_noflux<<<launch_blocks(n), 256, 0, s>>>(F, a, b->cw[a] ? (const float *)b->cw[a]->d : nullptr, d[a],
                                                      b->temp[a]);
        }
        for (int a = 0; a < 3; ++a)
            FF_CUDA(cudaMemcpyAsync(d[a], b->temp[a], comp_count(b->g, a) * 4, cudaMemcpyDeviceToDevice, s));
        k_blocked<<<launch_blocks(comp_count(b->g, 3)), 256, 0, s>>>(b->g, F.phi, d[0], d[1], d[2]);
    }
    for (int a = 0; a < 3; ++a) {
        const long long n = comp_count(b->g, a);
        k_walls_inflow_clamp<<<launch_blocks(n), 256, 0, s>>>(b->g, a, d[a], b->closed, b->n_in, b->in_phi, b->in_vel,
                                                              b->in_mode);
    }
    return post("constrainVelocity");
}

// ------------------------------------------------------------ forces --
namespace {
__global__ void k_add_const(long long n, float *__restrict__ d, float fdt) {
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x)
        d[f] = d[f] + fdt;
}
}  // namespace

// createExternalForceSolver3 (external_force_solver3.js:7-29) with a
// uniform force: u += f.x dt on every face of each component
extern "C" int ff_velocity3_add_force(ff_ctx ctx, const int *res, ff_field u, ff_field v, ff_field w, double fx,
                                      double fy, double fz, double dt) {
    FF_CHECK(ctx && res, FF_E_ARG, "ff_velocity3_add_force: NULL argument");
    const double unit[3] = {1.0, 1.0, 1.0};   // spacing does not enter
    const G3 g = geom_of(res, unit, nullptr);
    ff_field fs[3] = {u, v, w};
    const float fdt[3] = {(float)fx * (float)dt, (float)fy * (float)dt, (float)fz * (float)dt};
    cudaSetDevice(ctx->device);
    for (int a = 0; a < 3; ++a) {
        FF_CHECK(field_is(fs[a], comp_count(g, a)), FF_E_ARG, "add_force: component %d shape", a);
        k_add_const<<<launch_blocks(comp_count(g, a)), 256, 0, ctx->stream>>>(comp_count(g, a), (float *)fs[a]->d,
                                                                             fdt[a]);
    }
    return post("add_force");
}

// -------------------------------------------------------------- viscosity --
extern "C" int ff_viscosity3_apply(ff_ctx ctx, const int *res, const double *h, ff_field u, ff_field v, ff_field w,
                                   double nu, double dt, ff_field uo, ff_field vo, ff_field wo) {
    FF_CHECK(ctx && res && h, FF_E_ARG, "ff_viscosity3_apply: NULL argument");
    FF_TRY(check_grid32(res, "ff_viscosity3_apply"));
    const G3 g = geom_of(res, h, nullptr);
    ff_field in[3] = {u, v, w}, out[3] = {uo, vo, wo};
    for (int a = 0; a < 3; ++a)
        FF_CHECK(field_is(in[a], comp_count(g, a)) && field_is(out[a], comp_count(g, a)) && in[a]->d != out[a]->d,
                 FF_E_ARG, "viscosity: component %d must be distinct float face fields of the grid's shape", a);
    cudaSetDevice(ctx->device);
    const float ihx = 1.0f / ((float)h[0] * (float)h[0]), ihy = 1.0f / ((float)h[1] * (float)h[1]),
                ihz = 1.0f / ((float)h[2] * (float)h[2]);
    const float c = (float)dt * (float)nu;
    for (int a = 0; a < 3; ++a) {
        const long long n = comp_count(g, a);
        k_viscosity<<<launch_blocks(n), 256, 0, ctx->stream>>>(g, a, (const float *)in[a]->d, (float *)out[a]->d, c,
                                                               ihx, ihy, ihz);
    }
    return post("viscosity");
}

// ---------------------------------------------------------------- outflow --
// createGridOutflowSolver3 (src/grid/grid_outflow_solver3.js:79-210).  Each
// outflow is a cell-centred SDF on its own grid, inside where phi < 0
// (level_set_utils.js:5-9), sampled trilinearly (sdf_collider3.js:33-45).
namespace {

// extrapolate kernel of applyOutflowVelocityBC (:98-133) for one outflow and
// one component: faces inside the outflow relax toward the velocity one
// spacing upstream (pt + n h, n the unit SDF gradient) by the Courant number
// of the outward bulk speed, clamped to +-1e3; a zero gradient keeps the
// face.  Faces outside are not written (the copy kernel skips them too).
__global__ void k_outflow_relax(VelField F, int a, G3 pg, const float *__restrict__ phi, float dt,
                                float *__restrict__ dst) {
    int sx, sy, sz;
    comp_shape(F.g, a, sx, sy, sz);
    const long long n = (long long)sx * sy * sz;
    const F3 o = comp_origin(F.g, a), po = comp_origin(pg, 3);
    const float h = a == 0 ? F.g.hx : (a == 1 ? F.g.hy : F.g.hz);
    const float *cur_d = a == 0 ? F.u : (a == 1 ? F.v : F.w);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(f, sx, sy, i, j, k);
        const F3 pt = index_pos(F.g, o, i, j, k);
        if (!(trilinear(phi, pg.nx, pg.ny, pg.nz, pg, po, pt) < 0.0f)) continue;
        const float cur = cur_d[f];
        const F3 gr = trilinear_gradient(phi, pg, po, pt);
        const float gl = sqrtf(gr.x * gr.x + gr.y * gr.y + gr.z * gr.z);
        if (!(gl > 0.0f)) {
            dst[f] = cur;
            continue;
        }
        const F3 nn{gr.x / gl, gr.y / gl, gr.z / gl};
        const F3 up{pt.x + nn.x * h, pt.y + nn.y * h, pt.z + nn.z * h};
        const F3 bulk = sample_vel(F, pt);
        float dot = bulk.x * -nn.x;
        dot = dot + bulk.y * -nn.y;
        dot = dot + bulk.z * -nn.z;
        const float courant = fminf(fmaxf(fmaxf(0.0f, dot) * dt / h, 0.0f), 1.0f);
        const F3 uv = sample_vel(F, up);
        const float upc = a == 0 ? uv.x : (a == 1 ? uv.y : uv.z);
        const float relaxed = cur + (upc - cur) * courant;
        dst[f] = fminf(fmaxf(relaxed, -1.0e3f), 1.0e3f);
    }
}

// copy kernel (:137-150): faces inside the outflow take the relaxed value;
// also clearOutflowScalarField (:174-196) with src == nullptr (a = 3, the
// cells of a scalar grid, set to 0)
__global__ void k_outflow_copy(G3 g, int a, G3 pg, const float *__restrict__ phi, const float *__restrict__ src,
                               float *__restrict__ data) {
    int sx, sy, sz;
    if (a == 3) {
        sx = g.nx;
        sy = g.ny;
        sz = g.nz;
    } else {
        comp_shape(g, a, sx, sy, sz);
    }
    const long long n = (long long)sx * sy * sz;
    const F3 o = comp_origin(g, a), po = comp_origin(pg, 3);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(f, sx, sy, i, j, k);
        if (trilinear(phi, pg.nx, pg.ny, pg.nz, pg, po, index_pos(g, o, i, j, k)) < 0.0f)
            data[f] = src ? src[f] : 0.0f;
    }
}

// createOutflowPressureDirichlet3 (sdf_inflow_outflow3.js:44-64) at the cell
// centres of grid g (dataPosition, grid_data3.js:10-18): active where any
// outflow holds the centre; the target everywhere
__global__ void k_outflow_dirichlet(G3 g, int n_out, const float *const *__restrict__ phis,
                                    const G3 *__restrict__ pgs, float target, uint8_t *__restrict__ active,
                                    float *__restrict__ tgt) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    const F3 o = comp_origin(g, 3);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(c, g.nx, g.ny, i, j, k);
        const F3 pt = index_pos(g, o, i, j, k);
        bool in = false;
        for (int q = 0; q < n_out; ++q) {
            const G3 pg = pgs[q];
            in |= trilinear(phis[q], pg.nx, pg.ny, pg.nz, pg, comp_origin(pg, 3), pt) < 0.0f;
        }
        active[c] = in ? 1 : 0;
        tgt[c] = target;
    }
}

}  // namespace

struct ff_outflow_s {
    ff_ctx ctx = nullptr;
    G3 g{};
    float dt = 0.0f;
    int apply = 1;
    std::vector<ff_field> phi;   // borrowed
    std::vector<G3> pg;
    float *dst[3] = {};
    const float **d_phi = nullptr;   // device copies for the Dirichlet kernel
    G3 *d_pg = nullptr;
};

extern "C" int ff_outflow3_destroy(ff_outflow o) {
    if (!o) return FF_OK;
    cudaStreamSynchronize(o->ctx->stream);
    for (int a = 0; a < 3; ++a) ff_dev_free(o->dst[a]);
    ff_dev_free((void *)o->d_phi);
    ff_dev_free(o->d_pg);
    delete o;
    return FF_OK;
}

extern "C" int ff_outflow3_create(ff_ctx ctx, const int *res, const double *h, const double *origin, int n,
                                  const ff_field *phis, const int *phi_res, const double *phi_h,
                                  const double *phi_origin, double dt, int apply_velocity_bc, ff_outflow *out) {
    FF_CHECK(ctx && res && h && out && n >= 0 && (n == 0 || (phis && phi_res && phi_h)), FF_E_ARG,
             "ff_outflow3_create: bad arguments");
    FF_CHECK(res[0] > 0 && res[1] > 0 && res[2] > 0, FF_E_ARG, "createGridOutflowSolver3: bad resolution");
    FF_CHECK(n <= 64, FF_E_LIMIT, "createGridOutflowSolver3: at most 64 outflows");
    FF_TRY(check_grid32(res, "createGridOutflowSolver3"));
    for (int q = 0; q < n; ++q) FF_TRY(check_grid32(phi_res + 3 * q, "createGridOutflowSolver3"));
    *out = nullptr;
    std::vector<G3> pg(n);
    for (int q = 0; q < n; ++q) {
        pg[q] = geom_of(phi_res + 3 * q, phi_h + 3 * q, phi_origin ? phi_origin + 3 * q : nullptr);
        FF_CHECK(pg[q].nx > 0 && pg[q].ny > 0 && pg[q].nz > 0 && field_is(phis[q], comp_count(pg[q], 3)), FF_E_ARG,
                 "createGridOutflowSolver3: outflow %d must be a float cell SDF of its grid's shape", q);
    }
    cudaSetDevice(ctx->device);
    ff_outflow o = new ff_outflow_s();
    o->ctx = ctx;
    o->g = geom_of(res, h, origin);
    o->dt = (float)dt;
    o->apply = apply_velocity_bc != 0;
    o->phi.assign(phis, phis + n);
    o->pg = pg;
    int st = FF_OK;
    for (int a = 0; a < 3 && st == FF_OK; ++a)
        st = ff_dev_alloc((void **)&o->dst[a], (size_t)comp_count(o->g, a) * 4, ctx->stream);
    if (st == FF_OK) st = ff_dev_alloc((void **)&o->d_phi, sizeof(float *) * std::max(1, n), ctx->stream);
    if (st == FF_OK) st = ff_dev_alloc((void **)&o->d_pg, sizeof(G3) * std::max(1, n), ctx->stream);
    if (st == FF_OK && n) {
        std::vector<const float *> hp(n);
        for (int q = 0; q < n; ++q) hp[q] = (const float *)phis[q]->d;
        if (cudaMemcpy(o->d_phi, hp.data(), sizeof(float *) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(o->d_pg, pg.data(), sizeof(G3) * n, cudaMemcpyHostToDevice) != cudaSuccess)
            st = ff_set_error(FF_E_CUDA, "createGridOutflowSolver3: upload");
    }
    if (st != FF_OK) {
        ff_outflow3_destroy(o);
        return st;
    }
    *out = o;
    return FF_OK;
}

extern "C" int ff_outflow3_set_dt(ff_outflow o, double dt) {
    FF_CHECK(o, FF_E_ARG, "NULL outflow solver");
    o->dt = (float)dt;
    return FF_OK;
}

extern "C" int ff_outflow3_apply_velocity_bc(ff_outflow o, ff_field u, ff_field v, ff_field w) {
    FF_CHECK(o, FF_E_ARG, "NULL outflow solver");
    ff_field fs[3] = {u, v, w};
    for (int a = 0; a < 3; ++a)
        FF_CHECK(field_is(fs[a], comp_count(o->g, a)), FF_E_ARG, "applyOutflowVelocityBC: component %d shape", a);
    if (!o->apply) return FF_OK;
    cudaSetDevice(o->ctx->device);
    cudaStream_t s = o->ctx->stream;
    VelField F{o->g, (const float *)u->d, (const float *)v->d, (const float *)w->d, nullptr};
    for (size_t q = 0; q < o->phi.size(); ++q)
        for (int a = 0; a < 3; ++a) {
            const long long n = comp_count(o->g, a);
            const float *phi = (const float *)o->phi[q]->d;
            k_outflow_relax<<<launch_blocks(n), 256, 0, s>>>(F, a, o->pg[q], phi, o->dt, o->dst[a]);
            k_outflow_copy<<<launch_blocks(n), 256, 0, s>>>(o->g, a, o->pg[q], phi, o->dst[a], (float *)fs[a]->d);
        }
    return post("applyOutflowVelocityBC");
}

extern "C" int ff_outflow3_clear_scalar(ff_outflow o, ff_field scalar, const int *res, const double *h,
                                        const double *origin) {
    FF_CHECK(o && res && h, FF_E_ARG, "clearOutflowScalarField: NULL argument");
    const G3 sg = geom_of(res, h, origin);
    FF_CHECK(field_is(scalar, comp_count(sg, 3)), FF_E_ARG, "clearOutflowScalarField: float cell field expected");
    cudaSetDevice(o->ctx->device);
    const long long n = comp_count(sg, 3);
    for (size_t q = 0; q < o->phi.size(); ++q)
        k_outflow_copy<<<launch_blocks(n), 256, 0, o->ctx->stream>>>(sg, 3, o->pg[q], (const float *)o->phi[q]->d,
                                                                    nullptr, (float *)scalar->d);
    return post("clearOutflowScalarField");
}

extern "C" int ff_outflow3_dirichlet(ff_outflow o, const int *res, const double *h, const double *origin,
                                     double target, ff_field active, ff_field target_field) {
    FF_CHECK(o && res && h, FF_E_ARG, "outflow dirichlet: NULL argument");
    const G3 cg = geom_of(res, h, origin);
    const long long n = comp_count(cg, 3);
    FF_CHECK(active && active->dtype == FF_UINT8 && active->count == n && field_is(target_field, n), FF_E_ARG,
             "outflow dirichlet: active must be a uint8 and target a float cell field");
    cudaSetDevice(o->ctx->device);
    k_outflow_dirichlet<<<launch_blocks(n), 256, 0, o->ctx->stream>>>(cg, (int)o->phi.size(), o->d_phi, o->d_pg,
                                                                      (float)target, (uint8_t *)active->d,
                                                                      (float *)target_field->d);
    return post("outflow dirichlet");
}
