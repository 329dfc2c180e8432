// FP32 grid sampling, trace and extrapolation helpers shared by the
// grid-velocity (ff_grid.cu) and FLIP (ff_flip.cu) kernels.  Both files are
// compiled with -fmad=false: every operation rounds on its own, in the
// evaluation order of the reference's expressions (fluxflow
// src/grid/grid_math3.js, advection_solver3.js, array_utils3.js).
#pragma once
#include "ff_internal.h"

// private to each translation unit that includes it
namespace {
namespace ffg {

struct G3 {
    int nx, ny, nz;
    float hx, hy, hz, ox, oy, oz;
};
struct F3 {
    float x, y, z;
};

__device__ __forceinline__ int iclamp(int v, int lo, int hi) { return max(lo, min(v, hi)); }
// keeps the float->int conversion defined for absurd or non-finite positions
__device__ __forceinline__ float gclamp(float g) { return fminf(fmaxf(g, -1.0e8f), 1.0e8f); }

__host__ __device__ __forceinline__ void comp_shape(const G3 &g, int a, int &sx, int &sy, int &sz) {
    sx = g.nx + (a == 0);
    sy = g.ny + (a == 1);
    sz = g.nz + (a == 2);
}
// dataOriginU/V/W (grid_data3.js:131-133); a == 3: cell centres (:208)
__device__ __forceinline__ F3 comp_origin(const G3 &g, int a) {
    F3 o;
    o.x = g.ox + (a == 0 ? 0.0f : g.hx * 0.5f);
    o.y = g.oy + (a == 1 ? 0.0f : g.hy * 0.5f);
    o.z = g.oz + (a == 2 ? 0.0f : g.hz * 0.5f);
    return o;
}
__device__ __forceinline__ F3 index_pos(const G3 &g, F3 o, int i, int j, int k) {
    return F3{o.x + g.hx * (float)i, o.y + g.hy * (float)j, o.z + g.hz * (float)k};
}

// collocatedValueAtPosition3 (grid_math3.js:61-117): clamped corners,
// weights (1-f) products in x, y, z order, summed corner by corner
__device__ float trilinear(const float *__restrict__ d, int sx, int sy, int sz, const G3 &g, F3 o, F3 p) {
    const float gx = gclamp((p.x - o.x) / g.hx), gy = gclamp((p.y - o.y) / g.hy), gz = gclamp((p.z - o.z) / g.hz);
    const int i0 = (int)floorf(gx), j0 = (int)floorf(gy), k0 = (int)floorf(gz);
    const float fx = gx - (float)i0, fy = gy - (float)j0, fz = gz - (float)k0;
    const int i0c = iclamp(i0, 0, sx - 1), i1c = iclamp(i0 + 1, 0, sx - 1);
    const int j0c = iclamp(j0, 0, sy - 1), j1c = iclamp(j0 + 1, 0, sy - 1);
    const int k0c = iclamp(k0, 0, sz - 1), k1c = iclamp(k0 + 1, 0, sz - 1);
    const float ux = 1.0f - fx, uy = 1.0f - fy, uz = 1.0f - fz;
    // 32-bit offsets: the entry points keep every array below 2^31 elements
    const int r00 = sx * (j0c + sy * k0c), r10 = sx * (j1c + sy * k0c);
    const int r01 = sx * (j0c + sy * k1c), r11 = sx * (j1c + sy * k1c);
    float s = __ldg(d + r00 + i0c) * (ux * uy * uz);
    s = s + __ldg(d + r00 + i1c) * (fx * uy * uz);
    s = s + __ldg(d + r10 + i0c) * (ux * fy * uz);
    s = s + __ldg(d + r10 + i1c) * (fx * fy * uz);
    s = s + __ldg(d + r01 + i0c) * (ux * uy * fz);
    s = s + __ldg(d + r01 + i1c) * (fx * uy * fz);
    s = s + __ldg(d + r11 + i0c) * (ux * fy * fz);
    s = s + __ldg(d + r11 + i1c) * (fx * fy * fz);
    return s;
}

// monotonicCubic1d3 (grid_math3.js:137-160)
__device__ __forceinline__ float mono_cubic(float f0, float f1, float f2, float f3, float f) {
    const float D1 = f2 - f1;
    const float rawD1 = (f2 - f0) * 0.5f, rawD2 = (f3 - f1) * 0.5f;
    const bool flat = fabsf(D1) < 1e-12f;
    const float d1 = (flat || rawD1 * D1 < 0.0f) ? 0.0f : rawD1;
    const float d2 = (flat || rawD2 * D1 < 0.0f) ? 0.0f : rawD2;
    const float a3 = (d1 + d2) - D1 * 2.0f;
    const float a2 = (D1 * 3.0f - d1 * 2.0f) - d2;
    float t = a3 * f * f * f;
    t = t + a2 * f * f;
    t = t + d1 * f;
    return t + f1;
}

__device__ __forceinline__ void cubic_idx(float coord, int n, int idx[4], float &f) {
    const int i0 = (int)floorf(coord);
    f = coord - (float)i0;
    idx[0] = iclamp(i0 - 1, 0, n - 1);
    idx[1] = iclamp(i0, 0, n - 1);
    idx[2] = iclamp(i0 + 1, 0, n - 1);
    idx[3] = iclamp(i0 + 2, 0, n - 1);
}

// collocatedCubicValueAtPosition3 (grid_math3.js:174-199): cubic in x for
// each (y, z) tap, then y per z tap, then z
__device__ float tricubic(const float *__restrict__ d, int sx, int sy, int sz, const G3 &g, F3 o, F3 p) {
    const float gx = gclamp((p.x - o.x) / g.hx), gy = gclamp((p.y - o.y) / g.hy), gz = gclamp((p.z - o.z) / g.hz);
    int xi[4], yi[4], zi[4];
    float fx, fy, fz;
    cubic_idx(gx, sx, xi, fx);
    cubic_idx(gy, sy, yi, fy);
    cubic_idx(gz, sz, zi, fz);
    float zv[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float row[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const float *r = d + sx * (yi[b] + sy * zi[c]);
            row[b] = mono_cubic(__ldg(r + xi[0]), __ldg(r + xi[1]), __ldg(r + xi[2]), __ldg(r + xi[3]), fx);
        }
        zv[c] = mono_cubic(row[0], row[1], row[2], row[3], fy);
    }
    return mono_cubic(zv[0], zv[1], zv[2], zv[3], fz);
}

struct VelField {
    G3 g;
    const float *u, *v, *w;   // velocity the trace follows
    const float *phi;         // collider SDF (cell centred) or null
};

__device__ __forceinline__ F3 sample_vel(const VelField &F, F3 p) {
    int sx, sy, sz;
    F3 r;
    comp_shape(F.g, 0, sx, sy, sz);
    r.x = trilinear(F.u, sx, sy, sz, F.g, comp_origin(F.g, 0), p);
    comp_shape(F.g, 1, sx, sy, sz);
    r.y = trilinear(F.v, sx, sy, sz, F.g, comp_origin(F.g, 1), p);
    comp_shape(F.g, 2, sx, sy, sz);
    r.z = trilinear(F.w, sx, sy, sz, F.g, comp_origin(F.g, 2), p);
    return r;
}
__device__ __forceinline__ float sample_phi(const VelField &F, const float *phi, F3 p) {
    if (!phi) return 1.0f;
    return trilinear(phi, F.g.nx, F.g.ny, F.g.nz, F.g, comp_origin(F.g, 3), p);
}

// backTrace (advection_solver3.js:20-62): RK2 midpoint substeps of at most
// one cell, stopping on the collider with a linear blend of the last step
__device__ F3 back_trace(const VelField &F, F3 pos, float dt, float dirn, int max_substeps) {
    const float h = fminf(F.g.hx, fminf(F.g.hy, F.g.hz));
    F3 pt = pos;
    float T = dt;
    for (int s = 0; s < max_substeps; ++s) {
        if (T <= 1e-6f) break;
        const F3 v0 = sample_vel(F, pt);
        const float len = sqrtf(v0.x * v0.x + v0.y * v0.y + v0.z * v0.z);
        const float nsub = fmaxf(ceilf(len * T / h), 1.0f);
        const float sdt = T / nsub;
        const float hs = sdt * 0.5f;
        const F3 mid{pt.x - v0.x * hs * dirn, pt.y - v0.y * hs * dirn, pt.z - v0.z * hs * dirn};
        const F3 mv = sample_vel(F, mid);
        const F3 nxt{pt.x - mv.x * sdt * dirn, pt.y - mv.y * sdt * dirn, pt.z - mv.z * sdt * dirn};
        const float phi0 = sample_phi(F, F.phi, pt), phi1 = sample_phi(F, F.phi, nxt);
        if (phi1 <= 0.0f) {
            const float w = fabsf(phi1) / (fabsf(phi0) + fabsf(phi1));
            const float wm = 1.0f - w;
            pt = F3{pt.x * w + nxt.x * wm, pt.y * w + nxt.y * wm, pt.z * w + nxt.z * wm};
            break;
        }
        T = T - sdt;
        pt = nxt;
    }
    return pt;
}

// (i, j, k) of a flat index; below 2^31 in 32-bit unsigned arithmetic (a
// 64-bit division is a long software sequence on the GPU)
__device__ __forceinline__ void unflatten(long long f, int sx, int sy, int &i, int &j, int &k) {
    if (f < 0x7fffffffLL) {
        const unsigned u = (unsigned)f, r = u / (unsigned)sx, q = r / (unsigned)sy;
        i = (int)(u - r * (unsigned)sx);
        j = (int)(r - q * (unsigned)sy);
        k = (int)q;
        return;
    }
    i = (int)(f % sx);
    long long r = f / sx;
    j = (int)(r % sy);
    k = (int)(r / sy);
}

// ---------------------------------------------------- velocity constraint --
// fractionInsideSdf (level_set_utils.js:24-40)
__device__ __forceinline__ float frac_inside_sdf(float p0, float p1) {
    const bool a = p0 < 0.0f, b = p1 < 0.0f;
    if (a && b) return 1.0f;
    if (a) return p0 / (p0 - p1);
    if (b) return p1 / (p1 - p0);
    return 0.0f;
}

// one Jacobi step of createExtrapolateToRegion3 (array_utils3.js:88-150)
__global__ void __launch_bounds__(256, 8) k_extrapolate(int sx, int sy, int sz, const float *__restrict__ src, float *__restrict__ dst,
                              const int *__restrict__ vs, int *__restrict__ vd) {
    const long long n = (long long)sx * sy * sz, sy_ = sx, sz_ = (long long)sx * sy;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(c, sx, sy, i, j, k);
        if (vs[c] != 0) {
            dst[c] = src[c];
            vd[c] = 1;
            continue;
        }
        float total = 0.0f;
        int count = 0;
        if (i + 1 < sx && vs[c + 1]) { total = total + src[c + 1]; ++count; }
        if (i > 0 && vs[c - 1]) { total = total + src[c - 1]; ++count; }
        if (j + 1 < sy && vs[c + sy_]) { total = total + src[c + sy_]; ++count; }
        if (j > 0 && vs[c - sy_]) { total = total + src[c - sy_]; ++count; }
        if (k + 1 < sz && vs[c + sz_]) { total = total + src[c + sz_]; ++count; }
        if (k > 0 && vs[c - sz_]) { total = total + src[c - sz_]; ++count; }
        if (count > 0) {
            dst[c] = total / (float)count;
            vd[c] = 1;
        } else {
            dst[c] = src[c];
            vd[c] = 0;
        }
    }
}

// trilinearGradientAtPosition3 (grid_math3.js:295-352)
__device__ F3 trilinear_gradient(const float *__restrict__ d, const G3 &g, F3 o, F3 pos) {
    const int n[3] = {g.nx, g.ny, g.nz};
    const float coord[3] = {gclamp((pos.x - o.x) / g.hx), gclamp((pos.y - o.y) / g.hy), gclamp((pos.z - o.z) / g.hz)};
    int lo[3], hi[3];
    float t[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int idx = (int)floorf(coord[a]);
        lo[a] = max(0, min(idx, n[a] - 2));
        hi[a] = min(lo[a] + 1, n[a] - 1);
        t[a] = fminf(fmaxf(coord[a] - (float)lo[a], 0.0f), 1.0f);
    }
    auto V = [&](int i, int j, int k) { return __ldg(d + i + g.nx * (j + g.ny * k)); };
    const float v000 = V(lo[0], lo[1], lo[2]), v100 = V(hi[0], lo[1], lo[2]), v010 = V(lo[0], hi[1], lo[2]);
    const float v110 = V(hi[0], hi[1], lo[2]), v001 = V(lo[0], lo[1], hi[2]), v101 = V(hi[0], lo[1], hi[2]);
    const float v011 = V(lo[0], hi[1], hi[2]), v111 = V(hi[0], hi[1], hi[2]);
    const float tx = t[0], ty = t[1], tz = t[2];
    F3 r;
    float s = (1.0f - ty) * (1.0f - tz) * (v100 - v000);
    s = s + ty * (1.0f - tz) * (v110 - v010);
    s = s + (1.0f - ty) * tz * (v101 - v001);
    s = s + ty * tz * (v111 - v011);
    r.x = s / g.hx;
    s = (1.0f - tx) * (1.0f - tz) * (v010 - v000);
    s = s + tx * (1.0f - tz) * (v110 - v100);
    s = s + (1.0f - tx) * tz * (v011 - v001);
    s = s + tx * tz * (v111 - v101);
    r.y = s / g.hy;
    s = (1.0f - tx) * (1.0f - ty) * (v001 - v000);
    s = s + tx * (1.0f - ty) * (v101 - v100);
    s = s + (1.0f - tx) * ty * (v011 - v010);
    s = s + tx * ty * (v111 - v110);
    r.z = s / g.hz;
    return r;
}


}  // namespace ffg
}  // namespace
