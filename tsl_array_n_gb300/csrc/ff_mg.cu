// Multigrid V-cycle kernels (fluxflow src/linalg/multigrid.js:626-1184):
// red-black relax, residual, full-weighting restriction, trilinear
// prolongation, coarsest-level solve, and the per-level coarsening of masks
// and face weights.  Arrays are FP32 or BF16 (storage only; arithmetic is
// FP32 throughout).
#include "ff_device.cuh"

using namespace ffd;

namespace {

struct C3 {
    int i, j, k;
    long long c;
    bool ok;
};
__device__ __forceinline__ C3 cell(const Dims &d) {
    C3 q;
    q.i = blockIdx.x * blockDim.x + threadIdx.x;
    q.j = blockIdx.y * blockDim.y + threadIdx.y;
    q.k = blockIdx.z;
    q.ok = q.i < d.nx && q.j < d.ny;
    q.c = (long long)q.i + (long long)d.nx * ((long long)q.j + (long long)d.ny * q.k);
    return q;
}

// (A x)_c and the diagonal at a cell, difference form (see Level in
// ff_internal.h).  X(n) reads the operand.
template <bool C16, class XF>
__device__ __forceinline__ float op_and_diag(const Dims &d, int i, int j, int k, long long c,
                                             const float4 *c32, const uint2 *c16, float xc,
                                             XF X, float &D) {
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    float4 kc = ldcoef<C16>(c32, c16, c);
    float s = -kc.w * xc;
    D = -(kc.w + kc.x + kc.y + kc.z);
    if (i > 0) s += kc.x * (X(c - 1) - xc);
    if (i < d.nx - 1) { float k1 = ldkx<C16>(c32, c16, c + 1); s += k1 * (X(c + 1) - xc); D -= k1; }
    if (j > 0) s += kc.y * (X(c - sy) - xc);
    if (j < d.ny - 1) { float k1 = ldky<C16>(c32, c16, c + sy); s += k1 * (X(c + sy) - xc); D -= k1; }
    if (k > 0) s += kc.z * (X(c - sz) - xc);
    if (k < d.nz - 1) { float k1 = ldkz<C16>(c32, c16, c + sz); s += k1 * (X(c + sz) - xc); D -= k1; }
    return s;
}

template <bool C16>
__device__ __forceinline__ float diag_at(const Dims &d, int i, int j, int k, long long c,
                                         const float4 *c32, const uint2 *c16) {
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    float4 kc = ldcoef<C16>(c32, c16, c);
    float D = -(kc.w + kc.x + kc.y + kc.z);
    if (i < d.nx - 1) D -= ldkx<C16>(c32, c16, c + 1);
    if (j < d.ny - 1) D -= ldky<C16>(c32, c16, c + sy);
    if (k < d.nz - 1) D -= ldkz<C16>(c32, c16, c + sz);
    return D;
}

// buildRelaxKernel (multigrid.js:626-640): x += sor (b - Ax) / diag on one
// colour ((i+j+k) mod 2, :442-448).  `first` treats x as all zeros, which
// folds the V-cycle's zeroX into the first pass.
template <class XT, class BT, bool C16>
__global__ void k_relax(Dims d, XT *x, const BT *__restrict__ b, const float4 *c32,
                        const uint2 *c16, int colour, float sor, int first, const PcgState *st) {
    if (st && st->stop) return;
    C3 q = cell(d);
    if (!q.ok) return;
    const bool mine = ((q.i + q.j + q.k) & 1) == colour;
    if (first) {
        if (mine) {
            float D = diag_at<C16>(d, q.i, q.j, q.k, q.c, c32, c16);
            ffd::st(x, q.c, (ld(b, q.c) / D) * sor);
        } else {
            ffd::st(x, q.c, 0.f);
        }
        return;
    }
    if (!mine) return;
    float xc = ldw(x, q.c);
    float D;
    float ax = op_and_diag<C16>(d, q.i, q.j, q.k, q.c, c32, c16, xc,
                                [&](long long n) { return ldw(x, n); }, D);
    ffd::st(x, q.c, xc + ((ld(b, q.c) - ax) / D) * sor);
}

// buildResidualKernel (multigrid.js:741-749): buf = b - A x
template <class XT, class BT, class RT, bool C16>
__global__ void k_residual(Dims d, const XT *__restrict__ x, const BT *__restrict__ b,
                           RT *__restrict__ buf, const float4 *c32, const uint2 *c16,
                           const PcgState *st) {
    if (st && st->stop) return;
    C3 q = cell(d);
    if (!q.ok) return;
    float xc = ld(x, q.c), D;
    float ax = op_and_diag<C16>(d, q.i, q.j, q.k, q.c, c32, c16, xc,
                                [&](long long n) { return ld(x, n); }, D);
    ffd::st(buf, q.c, ld(b, q.c) - ax);
}

// restrictionTapsForAxis (multigrid.js:847-864)
__device__ __forceinline__ void rtaps(int c, int nc, int *idx) {
    idx[0] = c > 0 ? 2 * c - 1 : 2 * c;
    idx[1] = 2 * c;
    idx[2] = 2 * c + 1;
    idx[3] = c + 1 < nc ? 2 * c + 2 : 2 * c + 1;
}
__constant__ float kRW[4] = {0.125f, 0.375f, 0.375f, 0.125f};

// buildRestrictKernel (multigrid.js:866-914): 64-tap full weighting (16 in
// 2D), fine-masked values read as 0, coarse-masked results 0; optionally
// clears the coarse x (foldClearIntoRestrict).
template <class FT, class CT>
__global__ void k_restrict(Dims fd, Dims cd, int dims, const FT *__restrict__ fine,
                           const uint8_t *fmask, const uint8_t *cmask, CT *coarse, CT *cx,
                           const PcgState *st) {
    if (st && st->stop) return;
    C3 q = cell(cd);
    if (!q.ok) return;
    int ii[4], jj[4], kk[4];
    rtaps(q.i, cd.nx, ii);
    rtaps(q.j, cd.ny, jj);
    int nk = 4;
    if (dims == 3) rtaps(q.k, cd.nz, kk); else { kk[0] = 0; nk = 1; }
    float s = 0.f;
    for (int a = 0; a < 4; ++a) {
        for (int bq = 0; bq < 4; ++bq) {
            for (int g = 0; g < nk; ++g) {
                float w = kRW[a] * kRW[bq] * (dims == 3 ? kRW[g] : 1.f);
                long long f = ii[a] + (long long)fd.nx * (jj[bq] + (long long)fd.ny * kk[g]);
                float v = (fmask && fmask[f]) ? 0.f : ld(fine, f);
                s += v * w;
            }
        }
    }
    ffd::st(coarse, q.c, (cmask && cmask[q.c]) ? 0.f : s);
    if (cx) ffd::st(cx, q.c, 0.f);
}

// correctionTapsForAxis (multigrid.js:924-938)
__device__ __forceinline__ void ptaps(int f, int nc, int *idx, float *w) {
    int ci = f >> 1;
    bool even = (f & 1) == 0;
    int lo = ci > 0 ? ci - 1 : ci, hi = ci < nc - 1 ? ci + 1 : ci;
    if (even) { idx[0] = lo; w[0] = 0.25f; idx[1] = ci; w[1] = 0.75f; }
    else { idx[0] = ci; w[0] = 0.75f; idx[1] = hi; w[1] = 0.25f; }
}

// buildCorrectKernel (multigrid.js:990-1040): fine += P coarse, not on
// fine-masked cells.
template <class CT, class FT>
__global__ void k_prolong(Dims fd, Dims cd, int dims, const CT *__restrict__ coarse,
                          const uint8_t *fmask, FT *fine, const PcgState *st) {
    if (st && st->stop) return;
    C3 q = cell(fd);
    if (!q.ok) return;
    if (fmask && fmask[q.c]) return;
    int ii[2], jj[2], kk[2];
    float wi[2], wj[2], wk[2];
    ptaps(q.i, cd.nx, ii, wi);
    ptaps(q.j, cd.ny, jj, wj);
    int nk = 2;
    if (dims == 3) ptaps(q.k, cd.nz, kk, wk); else { kk[0] = 0; wk[0] = 1.f; nk = 1; }
    float s = 0.f;
    for (int a = 0; a < 2; ++a)
        for (int bq = 0; bq < 2; ++bq)
            for (int g = 0; g < nk; ++g) {
                long long c = ii[a] + (long long)cd.nx * (jj[bq] + (long long)cd.ny * kk[g]);
                s += ld(coarse, c) * (wi[a] * wj[bq] * wk[g]);
            }
    ffd::st(fine, q.c, ldw(fine, q.c) + s);
}

// buildCoarseSweepKernel (multigrid.js:679-737): every coarsest sweep in one
// CTA, colour 0 then colour 1, a barrier between the halves.
template <class XT, class BT, bool C16>
__global__ void k_coarse_sweeps(Dims d, XT *x, const BT *__restrict__ b, const float4 *c32,
                                const uint2 *c16, int sweeps, float sor, const PcgState *st) {
    if (st && st->stop) return;
    const long long n = d.n();
    for (int s = 0; s < sweeps; ++s) {
        for (int colour = 0; colour < 2; ++colour) {
            for (long long c = threadIdx.x; c < n; c += blockDim.x) {
                int i = (int)(c % d.nx);
                long long t = c / d.nx;
                int j = (int)(t % d.ny);
                int k = (int)(t / d.ny);
                if (((i + j + k) & 1) != colour) continue;
                float xc = ldw(x, c), D;
                float ax = op_and_diag<C16>(d, i, j, k, c, c32, c16, xc,
                                            [&](long long m) { return ldw(x, m); }, D);
                ffd::st(x, c, xc + ((ld(b, c) - ax) / D) * sor);
            }
            __syncthreads();
        }
    }
}

// FP64 direct coarsest solve: x = G b with G the generalised inverse built
// on the host (ff_coarse.cpp).  One warp per row.
template <class XT, class BT>
__global__ void k_coarse_direct(int n, const double *__restrict__ G, const BT *__restrict__ b,
                                XT *x, const PcgState *st) {
    if (st && st->stop) return;
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const double *row = G + (size_t)warp * n;
    double s = 0.0;
    for (int j = lane; j < n; j += 32) s += __ldg(row + j) * (double)ld(b, j);
    s = warp_sum(s);
    if (lane == 0) ffd::st(x, warp, (float)s);
}

// ------------------------------------------------------------ coefficients --
__global__ void k_build_coef(Dims d, int dims, const float *wu, const float *wv, const float *ww,
                             const uint8_t *mask, float hx2, float hy2, float hz2, float4 *coef,
                             uint2 *coef16) {
    C3 q = cell(d);
    if (!q.ok) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    const bool pc = mask && mask[q.c];
    long long fu = q.i + (long long)(d.nx + 1) * (q.j + (long long)d.ny * q.k);
    long long fv = q.i + (long long)d.nx * (q.j + (long long)(d.ny + 1) * q.k);
    long long fw = q.c;
    auto W = [](const float *w, long long f) { return w ? w[f] : 1.f; };
    auto P = [&](long long n) { return mask ? mask[n] != 0 : false; };
    float kx = 0.f, ky = 0.f, kz = 0.f, e = 0.f;
    if (q.i > 0) { if (!pc && !P(q.c - 1)) kx = W(wu, fu) * hx2; else if (!pc) e += W(wu, fu) * hx2; }
    if (q.i < d.nx - 1 && !pc && P(q.c + 1)) e += W(wu, fu + 1) * hx2;
    if (q.j > 0) { if (!pc && !P(q.c - sy)) ky = W(wv, fv) * hy2; else if (!pc) e += W(wv, fv) * hy2; }
    if (q.j < d.ny - 1 && !pc && P(q.c + sy)) e += W(wv, fv + d.nx) * hy2;
    if (dims == 3) {
        if (q.k > 0) { if (!pc && !P(q.c - sz)) kz = W(ww, fw) * hz2; else if (!pc) e += W(ww, fw) * hz2; }
        if (q.k < d.nz - 1 && !pc && P(q.c + sz)) e += W(ww, fw + sz) * hz2;
    }
    if (pc) e = 1.f;
    coef[q.c] = make_float4(kx, ky, kz, e);
    if (coef16) {
        auto b16 = [](float v) { return (unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(v)); };
        coef16[q.c] = make_uint2(b16(kx) | (b16(ky) << 16), b16(kz) | (b16(e) << 16));
    }
}

// buildFaceWeightCoarsenKernel (multigrid.js:1138-1184)
__global__ void k_coarsen_weights(Dims fd, Dims cd, int dims, int axis, const float *fw,
                                  float *cw) {
    int cx = cd.nx + (axis == 0), cy = cd.ny + (axis == 1), cz = cd.nz + (axis == 2);
    int fx = fd.nx + (axis == 0), fy = fd.ny + (axis == 1);
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y * blockDim.y + threadIdx.y;
    int k = blockIdx.z;
    if (i >= cx || j >= cy || k >= cz) return;
    int ni = axis == 0 ? 1 : 2, nj = axis == 1 ? 1 : 2;
    int nk = dims == 2 ? 1 : (axis == 2 ? 1 : 2);
    float s = 0.f;
    int cnt = 0;
    for (int dk = 0; dk < nk; ++dk)
        for (int dj = 0; dj < nj; ++dj)
            for (int di = 0; di < ni; ++di) {
                int fi = 2 * i + di, fj = 2 * j + dj, fk = dims == 2 ? 0 : 2 * k + dk;
                s += fw[fi + (long long)fx * (fj + (long long)fy * fk)];
                cnt++;
            }
    cw[i + (long long)cx * (j + (long long)cy * k)] = s / (float)cnt;
}

// buildMaskCoarsenKernel (multigrid.js:1066-1122)
__global__ void k_coarsen_mask(Dims fd, Dims cd, int dims, const uint8_t *src, const float *wu,
                               const float *wv, const float *ww, uint8_t *cmask) {
    C3 q = cell(cd);
    if (!q.ok) return;
    int masked = -1;
    if (src) {
        int all = 1;
        int nk = dims == 2 ? 1 : 2;
        for (int dk = 0; dk < nk; ++dk)
            for (int dj = 0; dj < 2; ++dj)
                for (int di = 0; di < 2; ++di) {
                    int fk = dims == 2 ? 0 : 2 * q.k + dk;
                    long long f = 2 * q.i + di + (long long)fd.nx * (2 * q.j + dj + (long long)fd.ny * fk);
                    if (!src[f]) all = 0;
                }
        masked = all;
    }
    if (wu) {
        long long fu = q.i + (long long)(cd.nx + 1) * (q.j + (long long)cd.ny * q.k);
        long long fv = q.i + (long long)cd.nx * (q.j + (long long)(cd.ny + 1) * q.k);
        float t = wu[fu] + wu[fu + 1] + wv[fv] + wv[fv + cd.nx];
        if (dims == 3) t += ww[q.c] + ww[q.c + (long long)cd.nx * cd.ny];
        int enclosed = t < 1e-6f;
        masked = masked < 0 ? enclosed : (masked || enclosed);
    }
    cmask[q.c] = masked > 0 ? 1 : 0;
}

}  // namespace

namespace ffk {

static int post(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return ff_set_error(FF_E_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
    return FF_OK;
}

#define DISPATCH_XB(xbf, bbf, ...)                                                   \
    do {                                                                              \
        if (xbf && bbf) { using XT = __nv_bfloat16; using BT = __nv_bfloat16; __VA_ARGS__; } \
        else if (xbf) { using XT = __nv_bfloat16; using BT = float; __VA_ARGS__; }          \
        else if (bbf) { using XT = float; using BT = __nv_bfloat16; __VA_ARGS__; }          \
        else { using XT = float; using BT = float; __VA_ARGS__; }                           \
    } while (0)

int mg_relax(const Level &L, int dims, int colour, float sor, int first, int xbf, int bbf,
             int coef16, const PcgState *st, cudaStream_t s) {
    (void)dims;
    auto g = launch3(L.d.nx, L.d.ny, L.d.nz);
    DISPATCH_XB(xbf, bbf, {
        if (coef16)
            k_relax<XT, BT, true><<<g.grid, g.block, 0, s>>>(L.d, (XT *)L.x, (const BT *)L.b, L.coef, L.coef16, colour, sor, first, st);
        else
            k_relax<XT, BT, false><<<g.grid, g.block, 0, s>>>(L.d, (XT *)L.x, (const BT *)L.b, L.coef, L.coef16, colour, sor, first, st);
    });
    return post("relax");
}

int mg_residual(const Level &L, int dims, int xbf, int bbf, int rbf, int coef16, const PcgState *st,
                cudaStream_t s) {
    (void)dims;
    auto g = launch3(L.d.nx, L.d.ny, L.d.nz);
    DISPATCH_XB(xbf, bbf, {
        if (rbf) {
            using RT = __nv_bfloat16;
            if (coef16)
                k_residual<XT, BT, RT, true><<<g.grid, g.block, 0, s>>>(L.d, (const XT *)L.x, (const BT *)L.b, (RT *)L.buf, L.coef, L.coef16, st);
            else
                k_residual<XT, BT, RT, false><<<g.grid, g.block, 0, s>>>(L.d, (const XT *)L.x, (const BT *)L.b, (RT *)L.buf, L.coef, L.coef16, st);
        } else {
            using RT = float;
            if (coef16)
                k_residual<XT, BT, RT, true><<<g.grid, g.block, 0, s>>>(L.d, (const XT *)L.x, (const BT *)L.b, (RT *)L.buf, L.coef, L.coef16, st);
            else
                k_residual<XT, BT, RT, false><<<g.grid, g.block, 0, s>>>(L.d, (const XT *)L.x, (const BT *)L.b, (RT *)L.buf, L.coef, L.coef16, st);
        }
    });
    return post("residual");
}

int mg_restrict(const Level &f, Level &c, int dims, int fbf, int cbf, int zero_x,
                const PcgState *st, cudaStream_t s) {
    auto g = launch3(c.d.nx, c.d.ny, c.d.nz);
    DISPATCH_XB(fbf, cbf, {
        k_restrict<XT, BT><<<g.grid, g.block, 0, s>>>(f.d, c.d, dims, (const XT *)f.buf, f.mask, c.mask,
                                                      (BT *)c.b, zero_x ? (BT *)c.x : (BT *)nullptr, st);
    });
    return post("restrict");
}

int mg_prolong(const Level &c, Level &f, int dims, int cbf, int fbf, const PcgState *st,
               cudaStream_t s) {
    auto g = launch3(f.d.nx, f.d.ny, f.d.nz);
    DISPATCH_XB(cbf, fbf, {
        k_prolong<XT, BT><<<g.grid, g.block, 0, s>>>(f.d, c.d, dims, (const XT *)c.x, f.mask, (BT *)f.x, st);
    });
    return post("prolong");
}

int mg_coarse_sweeps(const Level &L, int dims, int sweeps, float sor, int xbf, int bbf,
                     int coef16, const PcgState *st, cudaStream_t s) {
    (void)dims;
    DISPATCH_XB(xbf, bbf, {
        if (coef16)
            k_coarse_sweeps<XT, BT, true><<<1, 1024, 0, s>>>(L.d, (XT *)L.x, (const BT *)L.b, L.coef, L.coef16, sweeps, sor, st);
        else
            k_coarse_sweeps<XT, BT, false><<<1, 1024, 0, s>>>(L.d, (XT *)L.x, (const BT *)L.b, L.coef, L.coef16, sweeps, sor, st);
    });
    return post("coarse_sweeps");
}

int mg_coarse_direct(const Level &L, const double *G, int n, int xbf, int bbf,
                     const PcgState *st, cudaStream_t s) {
    int threads = 256;
    int blocks = (n * 32 + threads - 1) / threads;
    DISPATCH_XB(xbf, bbf, {
        k_coarse_direct<XT, BT><<<blocks, threads, 0, s>>>(n, G, (const BT *)L.b, (XT *)L.x, st);
    });
    return post("coarse_direct");
}

int build_coef(const Level &L, int dims, int want16, cudaStream_t s) {
    auto g = launch3(L.d.nx, L.d.ny, L.d.nz);
    k_build_coef<<<g.grid, g.block, 0, s>>>(L.d, dims, L.w[0], L.w[1], L.w[2], L.mask, L.h2inv[0],
                                             L.h2inv[1], L.h2inv[2], L.coef, want16 ? L.coef16 : nullptr);
    return post("build_coef");
}

int coarsen_weights(const Level &f, Level &c, int dims, cudaStream_t s) {
    for (int a = 0; a < dims; ++a) {
        auto g = launch3(c.d.nx + (a == 0), c.d.ny + (a == 1), c.d.nz + (a == 2));
        k_coarsen_weights<<<g.grid, g.block, 0, s>>>(f.d, c.d, dims, a, f.w[a], c.w[a]);
    }
    return post("coarsen_weights");
}

int coarsen_mask(const Level &f, const uint8_t *src, Level &c, int dims, cudaStream_t s) {
    auto g = launch3(c.d.nx, c.d.ny, c.d.nz);
    k_coarsen_mask<<<g.grid, g.block, 0, s>>>(f.d, c.d, dims, src, c.w[0], c.w[1], c.w[2], c.mask);
    return post("coarsen_mask");
}

int mg_restrict_f32(Dims fd, int dims, const float *fine, const uint8_t *fmask,
                    const uint8_t *cmask, float *coarse, cudaStream_t s) {
    Dims cd{fd.nx / 2, fd.ny / 2, dims == 3 ? fd.nz / 2 : 1};
    auto g = launch3(cd.nx, cd.ny, cd.nz);
    k_restrict<float, float><<<g.grid, g.block, 0, s>>>(fd, cd, dims, fine, fmask, cmask, coarse, nullptr, nullptr);
    return post("restrict_f32");
}

int mg_prolong_f32(Dims fd, int dims, const float *coarse, const uint8_t *fmask, float *fine,
                   cudaStream_t s) {
    Dims cd{fd.nx / 2, fd.ny / 2, dims == 3 ? fd.nz / 2 : 1};
    auto g = launch3(fd.nx, fd.ny, fd.nz);
    k_prolong<float, float><<<g.grid, g.block, 0, s>>>(fd, cd, dims, coarse, fmask, fine, nullptr);
    return post("prolong_f32");
}

}  // namespace ffk
