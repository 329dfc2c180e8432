// Fused, bandwidth-first kernels for the level-by-level hot loop.
//
//  * k_sweep: one full red-black Gauss-Seidel sweep (both colours) in a
//    single pass over the level, out of place (x_in -> x_out).  A block owns
//    a 32 x 16 column tile and marches along z as a wavefront: at step m it
//    relaxes the first colour on plane m+1 over the tile plus a one-cell
//    halo ring, then the second colour on plane m over the tile, then writes
//    plane m.  Each cell sees exactly the neighbour values the reference's
//    two colour dispatches give it (fluxflow src/linalg/multigrid.js:626-640),
//    so a sweep equals colour pass + colour pass.  Optional fusions: x_in
//    treated as zero (the V-cycle's zeroX) and r.z with the beta update of
//    linalg.js:1201-1240 accumulated from the final values.
//  * k_res_restrict: buildResidualKernel + buildRestrictKernel in one pass;
//    the fine residual lives only in shared memory.
//  * k_p_pap / k_x_residual: the two CG kernels; the operand (p = z + beta p,
//    or x + alpha p) is formed once per cell in shared memory.
//  * Every thread owns an x-adjacent pair of cells, so each colour pass keeps
//    every lane busy (one cell of each colour per thread).
//  * Planes are staged into shared-memory rings with cp.async (16-byte
//    chunks, zero-filled outside the domain) several z-steps ahead of use.
//  * Cells of a "regular" brick (every coefficient the plain unweighted,
//    unmasked value) that are not on the domain boundary take a short path:
//    no coefficient memory, no branches, a reciprocal instead of a divide.
// Requires nx % 4 == 0 (16-byte rows); other levels use the per-colour path.
#include "ff_device.cuh"
#include <algorithm>

using namespace ffd;

namespace {

constexpr int TX = 32, TY = 16;   // tile (cells)
constexpr int PX = TX / 2;        // threads per tile row (one x-pair each)
constexpr int NT = PX * TY;       // 256 threads
constexpr int BZ = 8;             // brick depth (bricks are TX x TY x BZ)
constexpr int RW = TX + 8;        // staged row width: [i0-4, i0+TX+4), 16-byte aligned
constexpr int CPR = RW / 4;       // 16-byte chunks per staged row
constexpr double MAX_BETA_MAGNITUDE = 10.0;
constexpr double MAX_ALPHA_MAGNITUDE = 1e6;
constexpr double MAX_PAP_GROWTH_FACTOR = 1e8;
constexpr double PAP_BASELINE_FLOOR = 1e-12;
constexpr double MAX_RESIDUAL_GROWTH = 100.0;

struct Geo {
    Dims d;
    float h2x, h2y, h2z;
    float dreg;          // diagonal of a regular interior cell: -2(h2x+h2y+h2z)
    long long sy, sz;
    int bnx, bny;        // bricks per row / column
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool valid) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    int sz = valid ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// One thread's share of staging a plane region: chunk `q` of a region of
// `rows` rows starting at global row j_start, columns [i0-4, i0+TX+4).
struct Chunk {
    int soff;          // offset in the staged plane (floats), or -1 if none
    long long goff;    // global offset within a plane
    bool dom;          // chunk inside the domain in (i, j)
};
__device__ __forceinline__ Chunk make_chunk(const Geo &g, int q, int i0, int j_start, int rows) {
    Chunk c;
    if (q >= rows * CPR) { c.soff = -1; c.goff = 0; c.dom = false; return c; }
    int row = q / CPR, cc = q - row * CPR;
    int gi = i0 - 4 + 4 * cc, gj = j_start + row;
    c.soff = row * RW + 4 * cc;
    c.dom = gi >= 0 && gi < g.d.nx && gj >= 0 && gj < g.d.ny;
    c.goff = c.dom ? gi + g.sy * gj : 0;
    return c;
}
__device__ __forceinline__ void stage1(float *plane, const Chunk &c, const float *src, const Geo &g, int k) {
    if (c.soff < 0) return;
    bool valid = c.dom && k >= 0 && k < g.d.nz;
    cp_async16(plane + c.soff, valid ? src + c.goff + g.sz * k : src, valid);
}

__device__ __forceinline__ bool brick_regular(const Geo &g, const uint8_t *bricks, int k) {
    if (!bricks) return false;
    int bz = k / BZ;
    return bricks[blockIdx.x + (long long)g.bnx * (blockIdx.y + (long long)g.bny * bz)] != 0;
}

struct Coef {
    float kx, ky, kz, e, ux, uy, uz;
};
__device__ __forceinline__ Coef coef_at(const Geo &g, const float4 *coef, bool regular, int i, int j,
                                        int k, long long c) {
    Coef q;
    if (regular) {
        q.kx = i > 0 ? g.h2x : 0.f;
        q.ky = j > 0 ? g.h2y : 0.f;
        q.kz = k > 0 ? g.h2z : 0.f;
        q.e = 0.f;
        q.ux = i < g.d.nx - 1 ? g.h2x : 0.f;
        q.uy = j < g.d.ny - 1 ? g.h2y : 0.f;
        q.uz = k < g.d.nz - 1 ? g.h2z : 0.f;
    } else {
        float4 a = __ldg(coef + c);
        q.kx = i > 0 ? a.x : 0.f;
        q.ky = j > 0 ? a.y : 0.f;
        q.kz = k > 0 ? a.z : 0.f;
        q.e = a.w;
        q.ux = i < g.d.nx - 1 ? __ldg(&coef[c + 1].x) : 0.f;
        q.uy = j < g.d.ny - 1 ? __ldg(&coef[c + g.sy].y) : 0.f;
        q.uz = k < g.d.nz - 1 ? __ldg(&coef[c + g.sz].z) : 0.f;
    }
    return q;
}

// (A v)_c, difference form; absent faces carry zero coefficients and their
// staged neighbour values are zero-filled (finite).
__device__ __forceinline__ float apply_q(const Coef &q, float vc, float xm, float xp, float ym, float yp,
                                         float zm, float zp) {
    float s = -q.e * vc;
    s += q.kx * (xm - vc);
    s += q.ux * (xp - vc);
    s += q.ky * (ym - vc);
    s += q.uy * (yp - vc);
    s += q.kz * (zm - vc);
    s += q.uz * (zp - vc);
    return s;
}
__device__ __forceinline__ float diag_q(const Coef &q) {
    return -(q.e + q.kx + q.ux + q.ky + q.uy + q.kz + q.uz);
}
// regular interior cell: second differences per axis
__device__ __forceinline__ float apply_reg(const Geo &g, float vc, float xm, float xp, float ym, float yp,
                                           float zm, float zp) {
    float s = g.h2x * ((xm - vc) + (xp - vc));
    s = __fmaf_rn(g.h2y, (ym - vc) + (yp - vc), s);
    s = __fmaf_rn(g.h2z, (zm - vc) + (zp - vc), s);
    return s;
}
__device__ __forceinline__ bool interior(const Geo &g, int i, int j, int k) {
    return i > 0 && i < g.d.nx - 1 && j > 0 && j < g.d.ny - 1 && k > 0 && k < g.d.nz - 1;
}

// compensated (TwoSum) FP32 accumulation, folded into FP64 once
struct Acc {
    float s = 0.f, e = 0.f;
    __device__ __forceinline__ void add(float v) {
        float t, err;
        two_sum(s, v, t, err);
        s = t;
        e = __fadd_rn(e, err);
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)e; }
};

// ----------------------------------------------------------------- sweep --
struct SweepArgs {
    Geo g;
    const float *x_in;      // ignored when FIRST (staged as zeros)
    float *x_out;
    const float *b;
    const float4 *coef;
    const uint8_t *bricks;
    float sor;
    float rdreg_sor;        // sor / dreg
    int colour_a;           // colour relaxed first (0 forward, 1 reversed)
    int zc;                 // planes per block
    PcgState *st;
    double *partials;
    int rz_mode;            // 0 none, 1 iteration (beta), 2 setup (seed)
};

constexpr int SDIST = 4;                   // sweep prefetch distance (z-steps)
constexpr int XR = TY + 4;                 // x rows staged: j0-2 .. j0+TY+1
constexpr int BR = TY + 2;                 // b rows staged: j0-1 .. j0+TY
constexpr int XSLOTS = 4 + SDIST;          // planes m-1..m+2 in use, SDIST in flight
constexpr int BSLOTS = 2 + SDIST;
constexpr int XPLANE = XR * RW, BPLANE = BR * RW;
constexpr int RING = 2 * (TX / 2 + 1) + 2 * (TY / 2);   // first-colour cells of the halo ring
static_assert(XR * CPR <= NT && BR * CPR <= NT, "one staging chunk per thread");
static_assert(RING <= NT, "one ring cell per thread");
constexpr size_t sweep_smem() { return sizeof(float) * ((size_t)XSLOTS * XPLANE + (size_t)BSLOTS * BPLANE); }

// spread the ring cells over the warps (every 5th thread) so no warp carries
// two relaxations while the others wait at the barrier
__device__ __forceinline__ int ring_slot(int tid) { return (tid % 5 == 0) ? tid / 5 : -1; }

template <bool FIRST, bool RZ>
__global__ void __launch_bounds__(NT, 4) k_sweep(SweepArgs a) {
    if (a.st && a.rz_mode != 2 && a.st->stop) return;
    extern __shared__ __align__(16) float dyn[];
    float *xs = dyn, *bs = dyn + XSLOTS * XPLANE;
    const Geo &g = a.g;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + PX * ty;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int k0 = blockIdx.z * a.zc, k1 = min(k0 + a.zc, g.d.nz);
    const Chunk cx = make_chunk(g, tid, i0, j0 - 2, XR);
    const Chunk cb = make_chunk(g, tid, i0, j0 - 1, BR);
    const float *xsrc = FIRST ? a.b : a.x_in;
    Acc acc;
    auto xslot = [&](int k) { return xs + ((k + 64) % XSLOTS) * XPLANE; };
    auto bslot = [&](int k) { return bs + ((k + 64) % BSLOTS) * BPLANE; };
    auto issue = [&](int m) {   // step m needs x(m+2), b(m+1)
        if (m < k1) {
            stage1(xslot(m + 2), cx, xsrc, g, FIRST ? -1 : m + 2);
            stage1(bslot(m + 1), cb, a.b, g, m + 1);
        }
        cp_commit();
    };
    stage1(xslot(k0 - 2), cx, xsrc, g, FIRST ? -1 : k0 - 2);
    stage1(xslot(k0 - 1), cx, xsrc, g, FIRST ? -1 : k0 - 1);
    cp_commit();
    for (int s = 0; s < SDIST; ++s) issue(k0 - 2 + s);
    cp_wait<SDIST - 1>();
    __syncthreads();

    const int ca = a.colour_a, cbl = 1 - a.colour_a;
    const int base = i0 + j0;   // parity helper (i0 is even)
    // the ring cell this thread relaxes, as (side, index)
    const int rs = ring_slot(tid);

    // relax the cell at tile-local (lx, ly); X planes k-1, k, k+1; B plane k
    auto relax = [&](int lx, int ly, int k, bool reg, float *P, const float *Pm, const float *Pp,
                     const float *B) {
        const int gi = i0 + lx, gj = j0 + ly;
        if (gi < 0 || gi >= g.d.nx || gj < 0 || gj >= g.d.ny) return;
        const int o = (ly + 2) * RW + lx + 4;
        const float xc = P[o];
        const float bval = B[(ly + 1) * RW + lx + 4];
        if (reg && interior(g, gi, gj, k)) {
            float ax = apply_reg(g, xc, P[o - 1], P[o + 1], P[o - RW], P[o + RW], Pm[o], Pp[o]);
            P[o] = __fmaf_rn(bval - ax, a.rdreg_sor, xc);
        } else {
            const long long c = gi + g.sy * gj + g.sz * k;
            Coef q = coef_at(g, a.coef, reg, gi, gj, k, c);
            float ax = apply_q(q, xc, P[o - 1], P[o + 1], P[o - RW], P[o + RW], Pm[o], Pp[o]);
            P[o] = xc + ((bval - ax) / diag_q(q)) * a.sor;
        }
    };

    for (int m = k0 - 2; m < k1; ++m) {
        float *Xm1 = xslot(m - 1), *X0 = xslot(m), *Xp1 = xslot(m + 1), *Xp2 = xslot(m + 2);
        const float *B0 = bslot(m), *Bp1 = bslot(m + 1);
        const int ka = m + 1;
        if (ka >= 0 && ka < g.d.nz) {
            const bool reg = brick_regular(g, a.bricks, ka);
            // tile: the first-colour cell of this thread's pair
            relax(2 * tx + ((ca - (base + ty + ka)) & 1), ty, ka, reg, Xp1, X0, Xp2, Bp1);
            // halo ring, first colour only
            if (rs >= 0 && rs < RING) {
                int lx, ly, t = rs;
                if (t < TX / 2 + 1) {
                    ly = -1;
                    lx = -1 + 2 * t + ((ca - (base - 2 + ka)) & 1);
                } else if ((t -= TX / 2 + 1) < TX / 2 + 1) {
                    ly = TY;
                    lx = -1 + 2 * t + ((ca - (base - 1 + TY + ka)) & 1);
                } else if ((t -= TX / 2 + 1) < TY / 2) {
                    lx = -1;
                    ly = 2 * t + ((ca - (base - 1 + ka)) & 1);
                } else {
                    t -= TY / 2;
                    lx = TX;
                    ly = 2 * t + ((ca - (base + TX + ka)) & 1);
                }
                relax(lx, ly, ka, reg, Xp1, X0, Xp2, Bp1);
            }
        }
        __syncthreads();
        if (m >= k0) {
            const int k = m;
            relax(2 * tx + ((cbl - (base + ty + k)) & 1), ty, k, brick_regular(g, a.bricks, k), X0, Xm1, Xp1, B0);
            const int gi = i0 + 2 * tx, gj = j0 + ty;
            if (gi < g.d.nx && gj < g.d.ny) {
                const int o = (ty + 2) * RW + 2 * tx + 4;
                float2 v = make_float2(X0[o], X0[o + 1]);
                *reinterpret_cast<float2 *>(a.x_out + gi + g.sy * gj + g.sz * k) = v;
                if (RZ) {
                    const float *Bq = B0 + (ty + 1) * RW + 2 * tx + 4;
                    acc.add(Bq[0] * v.x);
                    acc.add(Bq[1] * v.y);
                }
            }
        }
        // the slot of plane m-2 and b(m-1) are free: prefetch, then wait for
        // the next step's data
        issue(m + SDIST);
        cp_wait<SDIST - 1>();
        __syncthreads();
    }
    cp_wait<0>();
    if (RZ) {
        double v[1] = {acc.value()};
        double tot[1];
        if (grid_reduce<1>(v, a.partials, &a.st->ticket[3], tot)) {
            if (tid == 0) {
                PcgState *st = a.st;
                double rz = tot[0];
                st->rz = rz;
                if (a.rz_mode == 2) {
                    // seedScalarsKernel (linalg.js:1259-1267)
                    st->rz_old = rz;
                    st->pap_baseline = fmax(fabs(st->rr), PAP_BASELINE_FLOOR);
                    st->stop = 0;
                    st->iter = 0;
                    st->stop_iter = 0;
                    st->first = 1;
                    st->best_rr = -1.0;
                } else {
                    // betaKernel (linalg.js:1201-1240)
                    double rz_old = st->rz_old;
                    double value = rz / rz_old;
                    bool degenerate = nonfinite_d(rz_old) || rz_old == 0.0;
                    bool restart = (rz_old * rz < 0.0) || nonfinite_or_above(value, MAX_BETA_MAGNITUDE);
                    bool already = st->stop != 0;
                    st->beta = (already || restart) ? 0.0 : value;
                    if (degenerate && st->stop == 0) st->stop = FF_STOP_DEGENERATE_OLD_RZ;
                    st->rz_old = rz;
                }
            }
        }
    }
}

// ------------------------------------------------------------------ CG ----
struct CgArgs {
    Geo g;
    const float4 *coef;
    const uint8_t *bricks;
    const float *z;
    float *p0, *p1;
    const float *b;
    float *xh0, *xl0, *xh1, *xl1;
    float *r;
    PcgState *st;
    double *partials;
    int zc;
};

constexpr int CR = TY + 2;          // rows staged: j0-1 .. j0+TY
constexpr int CPLANE = CR * RW;
constexpr int TCOLS = TX + 2;       // columns the operand transform covers: i0-1 .. i0+TX
constexpr int TCELLS = CR * TCOLS;  // 612
constexpr int TPER = (TCELLS + NT - 1) / NT;   // transform elements per thread (3)
static_assert(CR * CPR <= NT, "one staging chunk per thread");
constexpr int PDIST = 4;
constexpr int PSLOTS = 3 + PDIST;   // planes k-1..k+1 in use, PDIST in flight
constexpr size_t p_pap_smem() { return sizeof(float) * (size_t)2 * PSLOTS * CPLANE; }

// p = z + beta p (linalg.js:954-988 updateP), A p, p.Ap, then alphaKernel
__global__ void __launch_bounds__(NT, 4) k_p_pap(CgArgs a) {
    PcgState *st = a.st;
    if (st->stop) return;
    extern __shared__ __align__(16) float dyn[];
    float *zs = dyn;                       // PSLOTS planes
    float *ps = dyn + PSLOTS * CPLANE;     // PSLOTS planes
    const Geo &g = a.g;
    const int pc = st->p_cur;
    const float *pold = pc ? a.p1 : a.p0;
    float *pnew = pc ? a.p0 : a.p1;
    const float beta = (float)st->beta;
    const bool first = st->first != 0;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + PX * ty;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int k0 = blockIdx.z * a.zc, k1 = min(k0 + a.zc, g.d.nz);
    const Chunk ch = make_chunk(g, tid, i0, j0 - 1, CR);
    int toff[TPER];
#pragma unroll
    for (int t = 0; t < TPER; ++t) {
        int q = tid + t * NT;
        toff[t] = q < TCELLS ? (q / TCOLS) * RW + (q % TCOLS) + 3 : -1;
    }
    auto slot = [&](int k) { return ((k + 64) % PSLOTS) * CPLANE; };
    auto issue = [&](int k) {   // plane k of z and p
        if (k <= k1) {
            stage1(zs + slot(k), ch, a.z, g, k);
            if (!first) stage1(ps + slot(k), ch, pold, g, k);
        }
        cp_commit();
    };
    // operand transform of plane k in place: p <- first ? z : z + beta p
    auto transform = [&](int k) {
        float *P = ps + slot(k);
        const float *Z = zs + slot(k);
#pragma unroll
        for (int t = 0; t < TPER; ++t) {
            int q = toff[t];
            if (q >= 0) P[q] = first ? Z[q] : __fmaf_rn(beta, P[q], Z[q]);
        }
    };
    for (int s = -1; s <= PDIST; ++s) issue(k0 + s);     // planes k0-1 .. k0+PDIST
    cp_wait<PDIST - 1>();                                 // k0-1, k0, k0+1 landed
    __syncthreads();
    transform(k0 - 1);
    transform(k0);
    transform(k0 + 1);
    __syncthreads();
    Acc acc;
    const int gi = i0 + 2 * tx, gj = j0 + ty;
    const bool in = gi < g.d.nx && gj < g.d.ny;
    const int o = (ty + 1) * RW + 2 * tx + 4;
    for (int k = k0; k < k1; ++k) {
        if (in) {
            const bool reg = brick_regular(g, a.bricks, k);
            const float *P = ps + slot(k), *Pm = ps + slot(k - 1), *Pp = ps + slot(k + 1);
            const long long c = gi + g.sy * gj + g.sz * k;
            float2 out;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int oo = o + h;
                float vc = P[oo];
                float ap;
                if (reg && interior(g, gi + h, gj, k)) {
                    ap = apply_reg(g, vc, P[oo - 1], P[oo + 1], P[oo - RW], P[oo + RW], Pm[oo], Pp[oo]);
                } else {
                    Coef q = coef_at(g, a.coef, reg, gi + h, gj, k, c + h);
                    ap = apply_q(q, vc, P[oo - 1], P[oo + 1], P[oo - RW], P[oo + RW], Pm[oo], Pp[oo]);
                }
                acc.add(vc * ap);
                if (h == 0) out.x = vc; else out.y = vc;
            }
            *reinterpret_cast<float2 *>(pnew + c) = out;
        }
        issue(k + PDIST + 1);
        cp_wait<PDIST - 1>();     // plane k+2 landed
        __syncthreads();
        transform(k + 2);
        __syncthreads();
    }
    cp_wait<0>();
    double v[1] = {acc.value()};
    double tot[1];
    if (grid_reduce<1>(v, a.partials, &st->ticket[1], tot)) {
        if (tid == 0) {
            // alphaKernel (linalg.js:1147-1199)
            double pAp = tot[0];
            double value = st->rz_old / pAp;
            int code = 0;
            if (nonfinite_d(pAp) || pAp == 0.0) code = FF_STOP_DEGENERATE_PAP;
            else if (fabs(pAp) > st->pap_baseline * MAX_PAP_GROWTH_FACTOR) code = FF_STOP_PAP_GROWTH;
            else if (nonfinite_or_above(value, MAX_ALPHA_MAGNITUDE)) code = FF_STOP_ALPHA_MAGNITUDE;
            st->pAp = pAp;
            st->alpha = (st->stop != 0 || code != 0) ? 0.0 : value;
            if (st->stop == 0) st->stop = code;
            st->p_cur = pc ^ 1;
            st->first = 0;
        }
    }
}

// x += alpha p; r = b - A x; r.r; convergence test (linalg.js:1283-1311).
// SETUP: the current x as is, plus b.b.  DS: x is a hi+lo pair.  In a
// regular interior cell the residual is formed from second differences of
// hi and of lo separately: each difference of neighbouring hi values is
// exact (or rounded relative to its own small size), so the residual keeps
// FP32 accuracy relative to b rather than to the much larger A-terms.
// Elsewhere every flux term is carried as an unevaluated pair (TwoProd /
// TwoSum).  Dynamic shared memory: hs, ls, qs: XSL planes each (x hi, x lo,
// p), bs: XBSL tile planes.
constexpr int XD = 3;
constexpr int XSL = 3 + XD;
constexpr int XBSL = 1 + XD;

template <bool SETUP, bool DS>
constexpr size_t xres_smem() {
    return sizeof(float) * ((size_t)XSL * CPLANE * (1 + (DS ? 1 : 0) + (SETUP ? 0 : 1)) +
                            (size_t)XBSL * TY * RW);
}

template <bool SETUP, bool DS>
__global__ void __launch_bounds__(NT, 3) k_x_residual(CgArgs a) {
    PcgState *st = a.st;
    if (!SETUP && st->stop) return;
    extern __shared__ __align__(16) float dyn[];
    float *hs = dyn;
    float *ls = hs + XSL * CPLANE;
    float *qs = ls + (DS ? XSL * CPLANE : 0);
    float *bs = qs + (SETUP ? 0 : XSL * CPLANE);
    const Geo &g = a.g;
    const int xc = SETUP ? 0 : st->x_cur;
    const float *p = st->p_cur ? a.p1 : a.p0;
    const float *xh = xc ? a.xh1 : a.xh0;
    const float *xl = xc ? a.xl1 : a.xl0;
    float *oh = xc ? a.xh0 : a.xh1;
    float *ol = xc ? a.xl0 : a.xl1;
    const double alpha = SETUP ? 0.0 : st->alpha;
    const float ahi = (float)alpha, alo = (float)(alpha - (double)ahi);
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + PX * ty;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int k0 = blockIdx.z * a.zc, k1 = min(k0 + a.zc, g.d.nz);
    const Chunk ch = make_chunk(g, tid, i0, j0 - 1, CR);
    const Chunk cbk = make_chunk(g, tid, i0, j0, TY);
    int toff[TPER];
#pragma unroll
    for (int t = 0; t < TPER; ++t) {
        int q = tid + t * NT;
        toff[t] = q < TCELLS ? (q / TCOLS) * RW + (q % TCOLS) + 3 : -1;
    }
    auto slot = [&](int k) { return ((k + 64) % XSL) * CPLANE; };
    auto bslot = [&](int k) { return bs + ((k + 64) % XBSL) * (TY * RW); };
    auto issue = [&](int k) {   // plane k of x (and p), and b of plane k-1
        if (k <= k1) {
            stage1(hs + slot(k), ch, xh, g, k);
            if (DS) stage1(ls + slot(k), ch, xl, g, k);
            if (!SETUP) stage1(qs + slot(k), ch, p, g, k);
        }
        if (k - 1 >= k0 && k - 1 < k1) stage1(bslot(k - 1), cbk, a.b, g, k - 1);
        cp_commit();
    };
    auto transform = [&](int k) {
        if (SETUP) return;
        float *H = hs + slot(k), *L = ls + slot(k);
        const float *Q = qs + slot(k);
#pragma unroll
        for (int t = 0; t < TPER; ++t) {
            int q = toff[t];
            if (q < 0) continue;
            if (DS) {
                float h, l;
                ds_axpy(H[q], L[q], ahi, alo, Q[q], h, l);
                H[q] = h;
                L[q] = l;
            } else {
                H[q] = __fmaf_rn(ahi, Q[q], H[q]);
            }
        }
    };
    for (int s = -1; s <= XD; ++s) issue(k0 + s);   // planes k0-1 .. k0+XD (b: k0 .. k0+XD-1)
    cp_wait<XD - 1>();                               // planes k0-1..k0+1, b(k0) landed
    __syncthreads();
    transform(k0 - 1);
    transform(k0);
    transform(k0 + 1);
    __syncthreads();
    Acc acc_rr, acc_bb;
    const int gi = i0 + 2 * tx, gj = j0 + ty;
    const bool in = gi < g.d.nx && gj < g.d.ny;
    const int o = (ty + 1) * RW + 2 * tx + 4;
    for (int k = k0; k < k1; ++k) {
        if (in) {
            const bool reg = brick_regular(g, a.bricks, k);
            const long long c = gi + g.sy * gj + g.sz * k;
            const float *H = hs + slot(k), *Hm = hs + slot(k - 1), *Hp = hs + slot(k + 1);
            const float *L = ls + slot(k), *Lm = ls + slot(k - 1), *Lp = ls + slot(k + 1);
            const float *B = bslot(k) + ty * RW + 2 * tx + 4;
            float2 rout, hout, lout;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int oo = o + h;
                const float bc = B[h];
                const float chv = H[oo];
                const float clv = DS ? L[oo] : 0.f;
                float rc;
                if (reg && interior(g, gi + h, gj, k)) {
                    float ax = apply_reg(g, chv, H[oo - 1], H[oo + 1], H[oo - RW], H[oo + RW], Hm[oo], Hp[oo]);
                    if (DS) ax += apply_reg(g, clv, L[oo - 1], L[oo + 1], L[oo - RW], L[oo + RW], Lm[oo], Lp[oo]);
                    rc = bc - ax;
                } else if (DS) {
                    Coef q = coef_at(g, a.coef, reg, gi + h, gj, k, c + h);
                    float S = 0.f, Se = 0.f;
                    auto term = [&](float K, float hn, float ln) {
                        float dh, de;
                        two_sum(hn, -chv, dh, de);
                        de = __fadd_rn(de, __fsub_rn(ln, clv));
                        float pr, pe;
                        two_prod(K, dh, pr, pe);
                        pe = __fmaf_rn(K, de, pe);
                        float s2, e2;
                        two_sum(S, pr, s2, e2);
                        S = s2;
                        Se = __fadd_rn(Se, __fadd_rn(e2, pe));
                    };
                    term(q.kx, H[oo - 1], L[oo - 1]);
                    term(q.ux, H[oo + 1], L[oo + 1]);
                    term(q.ky, H[oo - RW], L[oo - RW]);
                    term(q.uy, H[oo + RW], L[oo + RW]);
                    term(q.kz, Hm[oo], Lm[oo]);
                    term(q.uz, Hp[oo], Lp[oo]);
                    {
                        float pr, pe;
                        two_prod(-q.e, chv, pr, pe);
                        pe = __fmaf_rn(-q.e, clv, pe);
                        float s2, e2;
                        two_sum(S, pr, s2, e2);
                        S = s2;
                        Se = __fadd_rn(Se, __fadd_rn(e2, pe));
                    }
                    float r0, e0;
                    two_sum(bc, -S, r0, e0);
                    rc = __fadd_rn(r0, __fsub_rn(e0, Se));
                } else {
                    Coef q = coef_at(g, a.coef, reg, gi + h, gj, k, c + h);
                    rc = bc - apply_q(q, chv, H[oo - 1], H[oo + 1], H[oo - RW], H[oo + RW], Hm[oo], Hp[oo]);
                }
                acc_rr.add(rc * rc);
                if (SETUP) acc_bb.add(bc * bc);
                if (h == 0) { rout.x = rc; hout.x = chv; lout.x = clv; }
                else { rout.y = rc; hout.y = chv; lout.y = clv; }
            }
            if (!SETUP) {
                *reinterpret_cast<float2 *>(oh + c) = hout;
                if (DS) *reinterpret_cast<float2 *>(ol + c) = lout;
            }
            *reinterpret_cast<float2 *>(a.r + c) = rout;
        }
        issue(k + XD + 1);
        cp_wait<XD - 1>();        // plane k+2 (and b(k+1)) landed
        __syncthreads();
        transform(k + 2);
        __syncthreads();
    }
    cp_wait<0>();
    if (SETUP) {
        double v[2] = {acc_rr.value(), acc_bb.value()};
        double tot[2];
        if (grid_reduce<2>(v, a.partials, &st->ticket[0], tot)) {
            if (tid == 0) {
                st->rr = tot[0];
                st->bb = tot[1];
                double nb = sqrt(fabs(tot[1]));
                st->thr = st->relative ? fmax(st->tol * nb, st->tol) : st->tol;
            }
        }
    } else {
        double v[1] = {acc_rr.value()};
        double tot[1];
        if (grid_reduce<1>(v, a.partials, &st->ticket[2], tot)) {
            if (tid == 0) {
                double rr = tot[0];
                st->rr = rr;
                st->x_cur = xc ^ 1;
                st->iter += 1;
                if (!nonfinite_d(rr)) {
                    if (st->best_rr < 0.0 || fabs(rr) < st->best_rr) st->best_rr = fabs(rr);
                    else if (st->best_rr > 0.0 && fabs(rr) > st->best_rr * MAX_RESIDUAL_GROWTH && st->stop == 0)
                        st->growth_stop = 1;
                }
                double res = sqrt(fabs(rr));
                bool conv = !nonfinite_or_above(res, st->thr);
                if (conv && st->stop == 0) {
                    st->stop = FF_STOP_CONVERGED;
                    st->stop_iter = st->iter;
                } else if (st->growth_stop && st->stop == 0) {
                    st->stop = FF_STOP_RESIDUAL_GROWING;
                }
            }
        }
    }
}

// ------------------------------------------------- residual + restriction --
// buildResidualKernel (multigrid.js:741-749) fused with buildRestrictKernel
// (:866-914): the fine residual b - A x is formed in shared memory, plane
// by plane, over the tile plus a one-cell ring (fine-masked cells read as
// 0), restricted in-plane with the 1/8, 3/8, 3/8, 1/8 taps, and accumulated
// along z into the coarse planes it feeds; coarse-masked results are 0.
// The fine residual never goes to memory.
struct RrArgs {
    Geo g;                 // fine level
    const float *x, *b;
    const float4 *coef;
    const uint8_t *bricks;
    const uint8_t *fmask, *cmask;
    float *cb;             // coarse b
    Dims cd;
    int dims;
    int zc;                // fine planes per block (even)
    const PcgState *st;
};

constexpr int RRING = 2 * (TX + 2) + 2 * TY;   // ring cells around the tile
constexpr int RDIST = 4;
constexpr int RXSLOTS = 3 + RDIST;             // x planes kf-1..kf+1 in use
constexpr int RBSLOTS = 1 + RDIST;
constexpr size_t rr_smem() {
    return sizeof(float) * ((size_t)RXSLOTS * XPLANE + (size_t)RBSLOTS * BPLANE + (size_t)(TY + 2) * (TX + 2));
}

__device__ __forceinline__ void rtap4(int c, int nc, int *idx) {
    idx[0] = c > 0 ? 2 * c - 1 : 2 * c;
    idx[1] = 2 * c;
    idx[2] = 2 * c + 1;
    idx[3] = c + 1 < nc ? 2 * c + 2 : 2 * c + 1;
}

__global__ void __launch_bounds__(NT, 4) k_res_restrict(RrArgs a) {
    if (a.st && a.st->stop) return;
    extern __shared__ __align__(16) float dyn[];
    float *xs = dyn, *bs = dyn + RXSLOTS * XPLANE;
    float(*rs)[TX + 2] = reinterpret_cast<float(*)[TX + 2]>(bs + RBSLOTS * BPLANE);
    const Geo &g = a.g;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + PX * ty;
    const int i0 = blockIdx.x * TX, j0 = blockIdx.y * TY;
    const int k0 = blockIdx.z * a.zc, k1 = min(k0 + a.zc, g.d.nz);
    const int kf_lo = max(0, k0 - 1), kf_hi = min(g.d.nz, k1 + 1);   // fine planes touched
    const Chunk cx = make_chunk(g, tid, i0, j0 - 2, XR);
    const Chunk cbk = make_chunk(g, tid, i0, j0 - 1, BR);
    auto xslot = [&](int k) { return xs + ((k + 64) % RXSLOTS) * XPLANE; };
    auto bslot = [&](int k) { return bs + ((k + 64) % RBSLOTS) * BPLANE; };
    auto issue = [&](int kf) {   // step kf needs x(kf-1..kf+1) and b(kf)
        if (kf < kf_hi) {
            stage1(xslot(kf + 1), cx, a.x, g, kf + 1);
            stage1(bslot(kf), cbk, a.b, g, kf);
        }
        cp_commit();
    };
    stage1(xslot(kf_lo - 1), cx, a.x, g, kf_lo - 1);
    stage1(xslot(kf_lo), cx, a.x, g, kf_lo);
    cp_commit();
    for (int s = 0; s < RDIST; ++s) issue(kf_lo + s);
    cp_wait<RDIST - 1>();
    __syncthreads();
    // this thread's coarse cell (threads < TX/2 * TY/2)
    const bool has_c = tid < (TX / 2) * (TY / 2);
    const int ccx = tid % (TX / 2), ccy = tid / (TX / 2);
    const int ci = i0 / 2 + ccx, cj = j0 / 2 + ccy;
    const bool c_in = has_c && ci < a.cd.nx && cj < a.cd.ny;
    int ix[4], iy[4];
    rtap4(ci, a.cd.nx, ix);
    rtap4(cj, a.cd.ny, iy);
    const float w4[4] = {0.125f, 0.375f, 0.375f, 0.125f};
    float acc3[3] = {0.f, 0.f, 0.f};   // coarse planes, by c mod 3
    const int c_first = k0 / 2, c_last = (k1 + 1) / 2;   // owned coarse planes [c_first, c_last)

    // residual of the cell at tile-local (lx, ly), plane kf, into rs
    auto res_cell = [&](int lx, int ly, int kf, bool reg, const float *P, const float *Pm, const float *Pp,
                        const float *B) {
        const int gi = i0 + lx, gj = j0 + ly;
        float v = 0.f;
        if (gi >= 0 && gi < g.d.nx && gj >= 0 && gj < g.d.ny) {
            const int o = (ly + 2) * RW + lx + 4;
            if (reg && interior(g, gi, gj, kf)) {
                v = B[(ly + 1) * RW + lx + 4] - apply_reg(g, P[o], P[o - 1], P[o + 1], P[o - RW], P[o + RW], Pm[o], Pp[o]);
            } else {
                const long long c = gi + g.sy * gj + g.sz * kf;
                if (!(a.fmask && a.fmask[c])) {
                    Coef q = coef_at(g, a.coef, reg, gi, gj, kf, c);
                    v = B[(ly + 1) * RW + lx + 4] - apply_q(q, P[o], P[o - 1], P[o + 1], P[o - RW], P[o + RW], Pm[o], Pp[o]);
                }
            }
        }
        rs[ly + 1][lx + 1] = v;
    };

    for (int kf = kf_lo; kf < kf_hi; ++kf) {
        const float *P = xslot(kf), *Pm = xslot(kf - 1), *Pp = xslot(kf + 1), *B = bslot(kf);
        const bool reg = brick_regular(g, a.bricks, kf);
        res_cell(2 * tx, ty, kf, reg, P, Pm, Pp, B);
        res_cell(2 * tx + 1, ty, kf, reg, P, Pm, Pp, B);
        if (tid < RRING) {
            int t = tid, lx, ly;
            if (t < TX + 2) { ly = -1; lx = t - 1; }
            else if ((t -= TX + 2) < TX + 2) { ly = TY; lx = t - 1; }
            else if ((t -= TX + 2) < TY) { lx = -1; ly = t; }
            else { lx = TX; ly = t - TY; }
            res_cell(lx, ly, kf, reg, P, Pm, Pp, B);
        }
        __syncthreads();
        if (c_in) {
            // in-plane restriction of this plane
            float part = 0.f;
#pragma unroll
            for (int b2 = 0; b2 < 4; ++b2)
#pragma unroll
                for (int a2 = 0; a2 < 4; ++a2)
                    part += rs[iy[b2] - j0 + 1][ix[a2] - i0 + 1] * (w4[a2] * w4[b2]);
            if (a.dims == 2) {
                const long long co = ci + (long long)a.cd.nx * cj;
                a.cb[co] = (a.cmask && a.cmask[co]) ? 0.f : part;
            } else {
                // coarse planes this fine plane feeds, with their z weight;
                // flush a coarse plane once its last tap has been added
#pragma unroll
                for (int dc = -1; dc <= 1; ++dc) {
                    int c = (kf >> 1) + dc;
                    if (c < c_first || c >= c_last || c < 0 || c >= a.cd.nz) continue;
                    int iz[4];
                    rtap4(c, a.cd.nz, iz);
                    float wz = 0.f;
#pragma unroll
                    for (int q = 0; q < 4; ++q) wz += iz[q] == kf ? w4[q] : 0.f;
                    acc3[c % 3] += part * wz;
                    if (iz[3] == kf) {
                        const long long co = ci + (long long)a.cd.nx * (cj + (long long)a.cd.ny * c);
                        a.cb[co] = (a.cmask && a.cmask[co]) ? 0.f : acc3[c % 3];
                        acc3[c % 3] = 0.f;
                    }
                }
            }
        }
        issue(kf + RDIST);
        cp_wait<RDIST - 1>();
        __syncthreads();
    }
    cp_wait<0>();
}

// ------------------------------------------------------------ brick flags --
// A brick is regular when every cell of it, extended by two cells on each
// side, carries the plain coefficients (h^-2 on interior faces, E = 0).
__global__ void k_brick_flags(Geo g, const float4 *coef, uint8_t *bricks) {
    const int bx = blockIdx.x, by = blockIdx.y, bz = blockIdx.z;
    const int ia = max(0, bx * TX - 2), ib = min(g.d.nx, bx * TX + TX + 2);
    const int ja = max(0, by * TY - 2), jb = min(g.d.ny, by * TY + TY + 2);
    const int ka = max(0, bz * BZ - 2), kb = min(g.d.nz, bz * BZ + BZ + 2);
    const int w = ib - ia, hgt = jb - ja, dep = kb - ka;
    const int total = w * hgt * dep;
    int ok = 1;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int i = ia + t % w, r = t / w, j = ja + r % hgt, k = ka + r / hgt;
        float4 c = coef[i + g.sy * j + g.sz * k];
        float ex = i > 0 ? g.h2x : 0.f, ey = j > 0 ? g.h2y : 0.f, ez = k > 0 ? g.h2z : 0.f;
        if (!(c.x == ex && c.y == ey && c.z == ez && c.w == 0.f)) ok = 0;
    }
    ok = __syncthreads_and(ok);
    if (threadIdx.x == 0) bricks[bx + (long long)g.bnx * (by + (long long)g.bny * bz)] = (uint8_t)ok;
}

Geo make_geo(const Level &L) {
    Geo g;
    g.d = L.d;
    g.h2x = L.h2inv[0];
    g.h2y = L.h2inv[1];
    g.h2z = L.d.nz > 1 ? L.h2inv[2] : 0.f;
    g.dreg = -2.f * (g.h2x + g.h2y + g.h2z);
    g.sy = L.d.nx;
    g.sz = (long long)L.d.nx * L.d.ny;
    g.bnx = (L.d.nx + TX - 1) / TX;
    g.bny = (L.d.ny + TY - 1) / TY;
    return g;
}

int zchunk(const Dims &d, int sm_count, int blocks_per_sm) {
    // as many z-chunks as fit one wave of resident blocks, at least 8
    // planes per block
    long long cols = (long long)((d.nx + TX - 1) / TX) * ((d.ny + TY - 1) / TY);
    long long want = (long long)blocks_per_sm * sm_count;
    int chunks = (int)std::max(1LL, std::min((long long)d.nz, want / cols));
    int zc = (d.nz + chunks - 1) / chunks;
    if (zc < 8) zc = std::min(8, d.nz);
    return zc;
}

}  // namespace

namespace ffk {

static int post(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return ff_set_error(FF_E_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
    return FF_OK;
}

bool fused_ok(const Dims &d) { return d.nx % 4 == 0; }

size_t brick_count(const Dims &d) {
    return (size_t)((d.nx + TX - 1) / TX) * ((d.ny + TY - 1) / TY) * ((d.nz + BZ - 1) / BZ);
}

int brick_flags(const Level &L, uint8_t *bricks, cudaStream_t s) {
    Geo g = make_geo(L);
    dim3 grid(g.bnx, g.bny, (L.d.nz + BZ - 1) / BZ);
    k_brick_flags<<<grid, 256, 0, s>>>(g, L.coef, bricks);
    return post("brick_flags");
}

size_t fused_blocks(const Dims &d, int sm_count) {
    int zc = std::min(zchunk(d, sm_count, 4), zchunk(d, sm_count, 3));
    return (size_t)((d.nx + TX - 1) / TX) * ((d.ny + TY - 1) / TY) * ((d.nz + zc - 1) / zc);
}

int sweep(const Level &L, const uint8_t *bricks, const float *x_in, float *x_out, int colour_a, float sor,
          int first, const Level *coarse, int dims, PcgState *st, double *partials, int rz_mode,
          int sm_count, cudaStream_t s) {
    (void)coarse;
    (void)dims;
    SweepArgs a;
    a.g = make_geo(L);
    a.x_in = x_in;
    a.x_out = x_out;
    a.b = (const float *)L.b;
    a.coef = L.coef;
    a.bricks = bricks;
    a.sor = sor;
    a.rdreg_sor = sor / a.g.dreg;
    a.colour_a = colour_a;
    a.zc = zchunk(L.d, sm_count, 4);
    a.st = st;
    a.partials = partials;
    a.rz_mode = rz_mode;
    dim3 grid(a.g.bnx, a.g.bny, (L.d.nz + a.zc - 1) / a.zc), block(PX, TY, 1);
    const bool rz = rz_mode != 0;
    const size_t smem = sweep_smem();
    if (first) {
        if (rz) k_sweep<true, true><<<grid, block, smem, s>>>(a);
        else k_sweep<true, false><<<grid, block, smem, s>>>(a);
    } else {
        if (rz) k_sweep<false, true><<<grid, block, smem, s>>>(a);
        else k_sweep<false, false><<<grid, block, smem, s>>>(a);
    }
    return post("sweep");
}

int res_restrict(const Level &f, const uint8_t *bricks, const float *x, Level &c, int dims,
                 const PcgState *st, int sm_count, cudaStream_t s) {
    RrArgs a;
    a.g = make_geo(f);
    a.x = x;
    a.b = (const float *)f.b;
    a.coef = f.coef;
    a.bricks = bricks;
    a.fmask = f.mask;
    a.cmask = c.mask;
    a.cb = (float *)c.b;
    a.cd = c.d;
    a.dims = dims;
    int zc = zchunk(f.d, sm_count, 4);
    if (dims == 3 && (zc & 1)) zc += 1;
    a.zc = zc;
    a.st = st;
    dim3 grid(a.g.bnx, a.g.bny, (f.d.nz + zc - 1) / zc), block(PX, TY, 1);
    k_res_restrict<<<grid, block, rr_smem(), s>>>(a);
    return post("res_restrict");
}

static CgArgs cg_args(const Level &L0, const uint8_t *bricks, const float *z, float *p0, float *p1,
                      const float *b, float *xh0, float *xl0, float *xh1, float *xl1, float *r,
                      PcgState *st, double *partials, int sm_count, int blocks_per_sm) {
    CgArgs a;
    a.g = make_geo(L0);
    a.coef = L0.coef;
    a.bricks = bricks;
    a.z = z;
    a.p0 = p0;
    a.p1 = p1;
    a.b = b;
    a.xh0 = xh0;
    a.xl0 = xl0;
    a.xh1 = xh1;
    a.xl1 = xl1;
    a.r = r;
    a.st = st;
    a.partials = partials;
    a.zc = zchunk(L0.d, sm_count, blocks_per_sm);
    return a;
}

int fused_p_pap(const Level &L0, const uint8_t *bricks, const float *z, float *p0, float *p1,
                PcgState *st, double *partials, int sm_count, cudaStream_t s) {
    CgArgs a = cg_args(L0, bricks, z, p0, p1, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, st,
                       partials, sm_count, 4);
    dim3 grid(a.g.bnx, a.g.bny, (L0.d.nz + a.zc - 1) / a.zc), block(PX, TY, 1);
    k_p_pap<<<grid, block, p_pap_smem(), s>>>(a);
    return post("p_pap");
}

template <bool SETUP, bool DS>
static int launch_xres(const CgArgs &a, dim3 grid, dim3 block, cudaStream_t s) {
    constexpr size_t smem = xres_smem<SETUP, DS>();
    k_x_residual<SETUP, DS><<<grid, block, smem, s>>>(a);
    return FF_OK;
}

// opt in to the dynamic shared memory the fused kernels use (once per
// process, before any stream capture)
int fused_configure() {
    FF_CUDA(cudaFuncSetAttribute(k_sweep<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_smem()));
    FF_CUDA(cudaFuncSetAttribute(k_sweep<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_smem()));
    FF_CUDA(cudaFuncSetAttribute(k_sweep<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_smem()));
    FF_CUDA(cudaFuncSetAttribute(k_sweep<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_smem()));
    FF_CUDA(cudaFuncSetAttribute(k_res_restrict, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rr_smem()));
    FF_CUDA(cudaFuncSetAttribute(k_p_pap, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p_pap_smem()));
    FF_CUDA(cudaFuncSetAttribute(k_x_residual<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)xres_smem<true, true>()));
    FF_CUDA(cudaFuncSetAttribute(k_x_residual<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)xres_smem<true, false>()));
    FF_CUDA(cudaFuncSetAttribute(k_x_residual<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)xres_smem<false, true>()));
    FF_CUDA(cudaFuncSetAttribute(k_x_residual<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)xres_smem<false, false>()));
    return FF_OK;
}

int fused_x_residual(const Level &L0, const uint8_t *bricks, const float *p0, const float *p1,
                     const float *b, float *xh0, float *xl0, float *xh1, float *xl1, float *r,
                     PcgState *st, double *partials, int ds, int setup, int sm_count, cudaStream_t s) {
    CgArgs a = cg_args(L0, bricks, nullptr, (float *)p0, (float *)p1, b, xh0, xl0, xh1, xl1, r, st,
                       partials, sm_count, 3);
    dim3 grid(a.g.bnx, a.g.bny, (L0.d.nz + a.zc - 1) / a.zc), block(PX, TY, 1);
    int rc;
    if (setup) rc = ds ? launch_xres<true, true>(a, grid, block, s) : launch_xres<true, false>(a, grid, block, s);
    else rc = ds ? launch_xres<false, true>(a, grid, block, s) : launch_xres<false, false>(a, grid, block, s);
    FF_TRY(rc);
    return post("x_residual");
}

}  // namespace ffk
