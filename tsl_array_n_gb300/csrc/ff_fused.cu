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
#include <cudaTypedefs.h>
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
                    if (st->stop != FF_STOP_CONVERGED) {
                        st->stop = 0;
                        st->stop_iter = 0;
                    }
                    st->iter = 0;
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

// ------------------------------------------------------- TMA-staged sweep --
// The red-black sweep as a z-marching wavefront on a 64 x 16 tile, one
// barrier per plane: step m relaxes the second colour on plane m and the
// first colour on plane m+2 (plus the tile's one-cell halo ring on m+2) in
// one phase.  The two touch disjoint cells: the second colour on m reads
// first-colour values of planes m-1..m+1 (final since steps m-3..m-1), the
// first colour on m+2 reads second-colour values of planes m+1..m+3 (not
// yet relaxed), so every cell sees exactly the neighbour values of the
// reference's two colour dispatches (fluxflow src/linalg/multigrid.js:626-640).
// Plane regions of x (rows j0-2 .. j0+17) and b (rows j0-1 .. j0+16),
// columns i0-4 .. i0+67, come into shared-memory rings through
// cp.async.bulk.tensor copies issued by one thread, completing on one
// mbarrier per stage; the tensor map zero-fills everything outside the
// domain.  Each thread owns an x-quad and keeps it in registers for planes
// m-1..m+3 as the wavefront marches in z: z-neighbours come from registers,
// x-neighbours from the next lane by shuffle (the tile's edge columns from
// shared memory), y-neighbours from shared memory, where each thread leaves
// its quad after the first colour.  A warp holds two rows of the same
// parity, so the colour offset inside a quad is uniform across the warp.
// Waits are bounded in time: a block that gives up records bit 0 of
// PcgState::err and stops (the host then reports the solve as failed).
namespace tq {
constexpr int TX = 64, TY = 16, QX = TX / 4, NT = QX * TY;   // 16 x 16 threads
constexpr int RW = TX + 8;                  // staged columns i0-4 .. i0+TX+3
constexpr int XR = TY + 4, BR = TY + 2;     // staged rows of x and of b
constexpr int SD = 3;                       // stages in flight
constexpr int XS = SD + 3, BS = SD;         // ring slots: x planes m..m+3+SD-1, b planes m+2..m+2+SD-1
constexpr int XPL = XR * RW;                // 1440 floats, 45 x 128 B
constexpr int BPL = ((BR * RW * 4 + 127) / 128) * 32;   // b slot padded to 128 B (1312 floats)
constexpr unsigned XBYTES = XR * RW * 4, BBYTES = BR * RW * 4;
constexpr int CW = 48, CR = TY + 2;         // staged class bytes: quads i0/4-16 .. i0/4+31, rows j0-1 ..
constexpr int CPL = ((CW * CR + 127) / 128) * 128;      // class slot padded to 128 B (896)
constexpr unsigned CBYTES = CW * CR;
constexpr int MAXZC = 256;                  // planes per block
constexpr int CS = SD + 1;                  // class slots: plane k0-1, then planes m+3..m+3+SD-1
constexpr size_t SMEM = 128 + sizeof(float) * ((size_t)XS * XPL + (size_t)BS * BPL) + (size_t)CS * CPL + 8 * SD;
static_assert((XPL * 4) % 128 == 0 && (BPL * 4) % 128 == 0, "TMA destinations stay 128-byte aligned");
}  // namespace tq

struct TqArgs {
    Geo g;
    float *x_out;
    const float4 *coef;
    const uint8_t *bricks;
    const float4 *gco;             // class-3 upper couplings and 1 / diagonal
    const int *order;              // work item of each block (tile column + z-chunk)
    int gx, gy;                    // tiles along x and y
    float sor, rdreg_sor, omsor;   // sor, sor / dreg, 1 - sor
    int colour_a, zc;
    PcgState *st;
    double *partials;
    int rz_mode;
};

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
// Kernels launched with programmatic stream serialization may start while
// the previous kernel drains; this waits until it has completed and its
// writes are visible (a no-op for an ordinary launch).  Every such kernel
// calls it before its first global-memory access.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Wait for the phase with the given parity to complete; false after 0.5 s.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity) {
    if (mbar_test(bar, parity)) return true;
    const unsigned long long t0 = globaltimer_ns();
    while (!mbar_test(bar, parity))
        if (globaltimer_ns() - t0 > 500000000ull) return false;
    return true;
}
__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap *map, int x, int y, int z,
                                            unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One relaxation of a cell with the plain couplings (class 0 or 2).  With
// S the h^-2-weighted sum of the six neighbours (the tensor maps zero-fill
// those across the domain edge, which drops the absent faces from S) and
// d = dreg + corr the cell's diagonal (corr = h^-2 summed over the absent
// faces), the row is (A v) = S + d v and the relaxation
// v + sor (b - A v) / d = (1 - sor) v + (b - S) rd, rd = sor / d.
__device__ __forceinline__ float relax_plain(const Geo &g, float omsor, float vc, float xm, float xp, float ym,
                                             float yp, float zm, float zp, float bval, float rd) {
    const float s = __fmaf_rn(g.h2z, zm + zp, __fmaf_rn(g.h2y, ym + yp, g.h2x * (xm + xp)));
    return __fmaf_rn(bval - s, rd, omsor * vc);
}

// One relaxation by cell class (see SweepMaps), all in the form
// (1 - sor) v + (b - S) rd with S the coupling-weighted neighbour sum:
// classes 0 and 2 with the plain couplings (rd given), class 1 (a Dirichlet
// row, A x = -x) with no coupling and rd = -sor, class 3 with its stored
// couplings (lower faces from coef, upper faces and 1 / diagonal from gco).
// Neighbours across the domain edge are zero-filled, so the lower-face
// couplings need no masking there.
__device__ __forceinline__ float relax_any(const Geo &g, const TqArgs &a, unsigned cls, long long c, float vc,
                                           float xm, float xp, float ym, float yp, float zm, float zp, float bval,
                                           float rd) {
    float kx = g.h2x, ux = g.h2x, ky = g.h2y, uy = g.h2y, kz = g.h2z, uz = g.h2z;
    if (cls == 1u) {
        kx = ux = ky = uy = kz = uz = 0.f;
        rd = -a.sor;
    } else if (cls == 3u) {
        const float4 lo = __ldg(a.coef + c), hi = __ldg(a.gco + c);
        kx = lo.x;
        ky = lo.y;
        kz = lo.z;
        ux = hi.x;
        uy = hi.y;
        uz = hi.z;
        rd = a.sor * hi.w;
    }
    float s = kx * xm;
    s = __fmaf_rn(ux, xp, s);
    s = __fmaf_rn(ky, ym, s);
    s = __fmaf_rn(uy, yp, s);
    s = __fmaf_rn(kz, zm, s);
    s = __fmaf_rn(uz, zp, s);
    return __fmaf_rn(bval - s, rd, a.omsor * vc);
}

// Scales (sor over the diagonal) of a quad's plain cells on one plane:
// cells 0, 1-2 and 3 differ only in the x faces.
struct QuadScale {
    float r0, r12, r3;
};

// Relax the two cells of colour offset P (cells P and P+2) of quad q in
// registers: s is the x-neighbour outside the quad (cell -1 for P = 0, cell
// 4 for P = 1), ym/yp/zm/zp the neighbouring quads, bq the right-hand side,
// cq the class byte.
template <int P>
__device__ __forceinline__ void relax_pair(const Geo &g, const TqArgs &a, float4 &q, float s, const float4 &ym,
                                           const float4 &yp, const float4 &zm, const float4 &zp, const float4 &bq,
                                           unsigned cq, const QuadScale &e, int gi, int gj, int k) {
    const float v0 = P ? q.y : q.x, l0 = P ? q.x : s, r0 = P ? q.z : q.y;
    const float v1 = P ? q.w : q.z, l1 = P ? q.z : q.y, r1 = P ? s : q.w;
    const float ym0 = P ? ym.y : ym.x, ym1 = P ? ym.w : ym.z, yp0 = P ? yp.y : yp.x, yp1 = P ? yp.w : yp.z;
    const float zm0 = P ? zm.y : zm.x, zm1 = P ? zm.w : zm.z, zp0 = P ? zp.y : zp.x, zp1 = P ? zp.w : zp.z;
    const float b0 = P ? bq.y : bq.x, b1 = P ? bq.w : bq.z;
    const float ra = P ? e.r12 : e.r0, rb = P ? e.r3 : e.r12;
    float n0, n1;
    if (!(cq & (0x11u << (2 * P)))) {
        n0 = relax_plain(g, a.omsor, v0, l0, r0, ym0, yp0, zm0, zp0, b0, ra);
        n1 = relax_plain(g, a.omsor, v1, l1, r1, ym1, yp1, zm1, zp1, b1, rb);
    } else {
        const long long c = gi + P + g.sy * gj + g.sz * k;
        n0 = relax_any(g, a, (cq >> (2 * P)) & 3u, c, v0, l0, r0, ym0, yp0, zm0, zp0, b0, ra);
        n1 = relax_any(g, a, (cq >> (2 * P + 4)) & 3u, c + 2, v1, l1, r1, ym1, yp1, zm1, zp1, b1, rb);
    }
    if (P) {
        q.y = n0;
        q.w = n1;
    } else {
        q.x = n0;
        q.z = n1;
    }
}

// relax_pair with the colour offset P chosen at run time (selects instead of
// a branch): the two rows of the halo ring, whose colours differ, share one
// warp without diverging.
__device__ __forceinline__ void relax_pair_rt(const Geo &g, const TqArgs &a, float4 &q, float s, const float4 &ym,
                                              const float4 &yp, const float4 &zm, const float4 &zp, const float4 &bq,
                                              unsigned cq, const QuadScale &e, int gi, int gj, int k, int P) {
    const bool p1 = P != 0;
    const float v0 = p1 ? q.y : q.x, l0 = p1 ? q.x : s, r0 = p1 ? q.z : q.y;
    const float v1 = p1 ? q.w : q.z, l1 = p1 ? q.z : q.y, r1 = p1 ? s : q.w;
    const float ym0 = p1 ? ym.y : ym.x, ym1 = p1 ? ym.w : ym.z, yp0 = p1 ? yp.y : yp.x, yp1 = p1 ? yp.w : yp.z;
    const float zm0 = p1 ? zm.y : zm.x, zm1 = p1 ? zm.w : zm.z, zp0 = p1 ? zp.y : zp.x, zp1 = p1 ? zp.w : zp.z;
    const float b0 = p1 ? bq.y : bq.x, b1 = p1 ? bq.w : bq.z;
    const float ra = p1 ? e.r12 : e.r0, rb = p1 ? e.r3 : e.r12;
    float n0, n1;
    if (!(cq & (0x11u << (2 * P)))) {
        n0 = relax_plain(g, a.omsor, v0, l0, r0, ym0, yp0, zm0, zp0, b0, ra);
        n1 = relax_plain(g, a.omsor, v1, l1, r1, ym1, yp1, zm1, zp1, b1, rb);
    } else {
        const long long c = gi + P + g.sy * gj + g.sz * k;
        n0 = relax_any(g, a, (cq >> (2 * P)) & 3u, c, v0, l0, r0, ym0, yp0, zm0, zp0, b0, ra);
        n1 = relax_any(g, a, (cq >> (2 * P + 4)) & 3u, c + 2, v1, l1, r1, ym1, yp1, zm1, zp1, b1, rb);
    }
    q.x = p1 ? q.x : n0;
    q.y = p1 ? n0 : q.y;
    q.z = p1 ? q.z : n1;
    q.w = p1 ? n1 : q.w;
}

// The first colour of a sweep from x = 0: every neighbour and the cell
// itself are zero, so the coupling sum S is +0 and (1 - sor) v + (b - S) rd
// is fma(b, rd, (1 - sor) 0), bit for bit what relax_plain and relax_any
// give, with rd by class (-sor for a Dirichlet row, sor / diagonal for
// class 3).  P: the colour offset of the pair (cells P and P + 2) in the
// quad, whose staged values are zero and stay so at the other offset.
__device__ __forceinline__ float first_scale(const TqArgs &a, unsigned cls, long long c, float rd) {
    if (cls == 1u) return -a.sor;
    if (cls == 3u) return a.sor * __ldg(&a.gco[c].w);
    return rd;
}
__device__ __forceinline__ void relax_pair_first(const Geo &g, const TqArgs &a, float4 &q, const float4 &bq,
                                                 unsigned cq, const QuadScale &e, int gi, int gj, int k, int P) {
    const bool p1 = P != 0;
    const float b0 = p1 ? bq.y : bq.x, b1 = p1 ? bq.w : bq.z;
    float r0 = p1 ? e.r12 : e.r0, r1 = p1 ? e.r3 : e.r12;
    if (cq & (0x11u << (2 * P))) {
        const long long c = gi + P + g.sy * gj + g.sz * k;
        r0 = first_scale(a, (cq >> (2 * P)) & 3u, c, r0);
        r1 = first_scale(a, (cq >> (2 * P + 4)) & 3u, c + 2, r1);
    }
    const float z = a.omsor * 0.f;
    const float n0 = __fmaf_rn(b0, r0, z), n1 = __fmaf_rn(b1, r1, z);
    q.x = p1 ? q.x : n0;
    q.y = p1 ? n0 : q.y;
    q.z = p1 ? q.z : n1;
    q.w = p1 ? n1 : q.w;
}

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void prefetch_l1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
// any cell of class 3 among the four 2-bit fields of a class byte
__device__ __forceinline__ bool any_general(unsigned c) { return (c & (c >> 1) & 0x55u) != 0; }

template <bool FIRST, bool RZ>
__global__ void __launch_bounds__(tq::NT, 4)
    k_sweep_tma(TqArgs a, const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap bmap,
                const __grid_constant__ CUtensorMap cmap) {
    constexpr int TX = tq::TX, TY = tq::TY, QX = tq::QX, RW = tq::RW, SD = tq::SD, XS = tq::XS, BS = tq::BS;
    constexpr int XPL = tq::XPL, BPL = tq::BPL;
    constexpr unsigned XBYTES = tq::XBYTES, BBYTES = tq::BBYTES, CBYTES = tq::CBYTES;
    constexpr int CW = tq::CW, CPL = tq::CPL, CS = tq::CS;
    constexpr unsigned FULL = 0xffffffffu;
    pdl_wait();
    if (a.st && a.rz_mode != 2 && (a.st->stop || a.st->err)) return;
    extern __shared__ __align__(16) unsigned char dyn_raw[];
    // 128-byte alignment by pointer arithmetic on the shared array (keeps the
    // shared address space visible to the compiler: LDS/STS, not generic)
    float *xs = reinterpret_cast<float *>(dyn_raw + ((128u - (smem_u32(dyn_raw) & 127u)) & 127u));
    float *bs = xs + XS * XPL;
    uint8_t *cs = reinterpret_cast<uint8_t *>(bs + BS * BPL);
    const unsigned bar0 = smem_u32(cs + CS * CPL);
    const Geo &g = a.g;
    // warp w holds rows r and r+2 (same colour parity), r = 4(w/2) + w%2
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int qx = lane & (QX - 1), ty = 4 * (warp >> 1) + (warp & 1) + 2 * (lane >> 4);
    // the TMA issuer is the last thread, which has no ring cell
    constexpr int ISSUER = tq::NT - 1;
    static_assert(ISSUER / 32 >= 3, "issuer carries no ring cell");
    // one block per work item (a tile column and a z-chunk of it), in the
    // order the work list gives
    const int item = a.order ? a.order[blockIdx.x] : (int)blockIdx.x;
    const int i0 = (item % a.gx) * TX, j0 = ((item / a.gx) % a.gy) * TY;
    const int k0 = (item / (a.gx * a.gy)) * a.zc, k1 = min(k0 + a.zc, g.d.nz);
    // steps k0-3 .. k1-1; step m's stage brings x(m+3), b(m+2) and the
    // class bytes of plane m+3
    const int mstart = k0 - 3;
    // x planes are read at z = -64 (entirely outside: zero fill) when the
    // input is identically zero
    auto xz = [&](int p) { return FIRST ? -64 : p; };
    __shared__ float rdt[27];
    if (tid < 27) {
        const int mx = tid % 3, myy = (tid / 3) % 3, mz = tid / 9;
        const float corr = g.h2x * (float)mx + g.h2y * (float)myy + g.h2z * (float)mz;
        rdt[tid] = corr == 0.f ? a.rdreg_sor : a.sor / (g.dreg + corr);
    }
    if (tid == ISSUER) {
        asm volatile("prefetch.tensormap [%0];" ::"l"(&xmap) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(&bmap) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(&cmap) : "memory");
        for (int q = 0; q < SD; ++q) mbar_init(bar0 + 8 * q, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // x plane p lives in slot (p - k0 + 3) mod XS, b plane p in slot
        // (p - k0 + 1) mod BS, class plane p >= k0 in slot 1 + (p - k0) mod
        // SD (slot 0 holds class plane k0-1).  Stage of step mstart: x(k0-2),
        // x(k0-1), x(k0), b(k0-1), class(k0-1), class(k0); stage of step
        // mstart+q: x(k0+q), b(k0-1+q), class(k0+q).
        mbar_expect_tx(bar0, 3 * XBYTES + BBYTES + 2 * CBYTES);
        for (int q = 0; q < 3; ++q) tma_load_3d(smem_u32(xs + (1 + q) * XPL), &xmap, i0 - 4, j0 - 2, xz(k0 - 2 + q), bar0);
        tma_load_3d(smem_u32(bs), &bmap, i0 - 4, j0 - 1, k0 - 1, bar0);
        tma_load_3d(smem_u32(cs), &cmap, i0 / 4 - 16, j0 - 1, k0 - 1, bar0);
        tma_load_3d(smem_u32(cs + CPL), &cmap, i0 / 4 - 16, j0 - 1, k0, bar0);
        for (int q = 1; q < SD && mstart + q < k1; ++q) {
            mbar_expect_tx(bar0 + 8 * q, XBYTES + BBYTES + CBYTES);
            tma_load_3d(smem_u32(xs + (3 + q) * XPL), &xmap, i0 - 4, j0 - 2, xz(k0 + q), bar0 + 8 * q);
            tma_load_3d(smem_u32(bs + q * BPL), &bmap, i0 - 4, j0 - 1, k0 - 1 + q, bar0 + 8 * q);
            tma_load_3d(smem_u32(cs + (1 + q) * CPL), &cmap, i0 / 4 - 16, j0 - 1, k0 + q, bar0 + 8 * q);
        }
    }
    __syncthreads();

    // slot of x plane m (planes m+1..m+3 follow, mod XS) and of b plane m+2;
    // the class plane m+3 sits in slot 1 + bi
    int sx = 0, sb = 0, bi = 0;
    unsigned ph = 0;
    const int ca = a.colour_a, cb = 1 - ca;
    const int lx = 4 * qx, gi = i0 + lx, gj = j0 + ty;
    const bool quad_in = gi < g.d.nx && gj < g.d.ny;
    const int o = (ty + 2) * RW + 4 + lx, bo = (ty + 1) * RW + 4 + lx;
    const int co = (ty + 1) * CW + 16 + qx;   // this quad's class byte in a class plane
    const long long qoff = gi + g.sy * gj;
    // h^-2 of the absent faces in y and in x (cells 0 and 3); planes strictly
    // inside in z use `inner`, the first and last plane add h^-2 in z (a
    // block-uniform branch)
    // rdt[mx + 3 my + 9 mz] (written before the first barrier): sor over the
    // diagonal of a plain cell with mx, my, mz faces across the domain edge
    const int my = (gj == 0) + (gj == g.d.ny - 1);
    const int mx0 = gi == 0, mx3 = gi + 3 == g.d.nx - 1;
    const int mze = g.d.nz == 1 ? 2 : 1;   // faces across the edge on the first and last plane
    QuadScale inner;
    // the scales, from the table written before the first barrier; the first
    // and last plane (a block-uniform branch) read theirs when they come
    inner.r0 = rdt[mx0 + 3 * my];
    inner.r12 = rdt[3 * my];
    inner.r3 = rdt[mx3 + 3 * my];
    const int tix = mx0 | (my << 1) | (mx3 << 3);   // table indices, packed
    auto scale_at = [&](int k) {
        if (k != 0 && k != g.d.nz - 1) return inner;
        const int m0 = tix & 1, myy = (tix >> 1) & 3, m3 = tix >> 3, mz = 9 * mze;
        QuadScale e;
        e.r0 = rdt[m0 + 3 * myy + mz];
        e.r12 = rdt[3 * myy + mz];
        e.r3 = rdt[m3 + 3 * myy + mz];
        return e;
    };
    // The tile's halo ring on plane m+2 (its first colour, which the second
    // colour on that plane reads two steps later): warp 0 the rows above
    // (lanes 0..15) and below (lanes 16..31) the tile, as quads; lanes 0..15
    // of warp 1 the cells left (lanes 0..7) and right (8..15) of the tile,
    // one pair of rows each.
    // (the ring's per-thread positions are recomputed inside its branches,
    // so they take no registers across the z-march)
    const int rrole = warp == 0 ? 0 : ((warp == 1 && lane < 16) ? 2 : -1);   // 0 rows; 2 columns
    // The thread's quad on planes m-1 .. m+2: q0 (plane m) and q1 carry the
    // first colour relaxed, q2 the values as staged; b of planes m and m+1;
    // the class bytes of planes m .. m+3 (bits 0-7 .. 24-31).
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 qm1 = zero4, q0 = zero4, q1 = zero4, q2 = zero4, bb0 = zero4, bb1 = zero4;
    unsigned cpipe = 0;
    unsigned rcls = 0;   // class byte of this thread's ring quad or cell on plane m+2
    Acc acc;
    bool failed = false;
    for (int m = mstart; m < k1; ++m) {
        const bool got = mbar_wait_bounded(bar0 + 8 * bi, ph);
        const int s1 = sx + 1 == XS ? 0 : sx + 1, s2 = s1 + 1 == XS ? 0 : s1 + 1, s3 = s2 + 1 == XS ? 0 : s2 + 1;
        float *X0 = xs + sx * XPL, *X1 = xs + s1 * XPL, *X2 = xs + s2 * XPL, *X3 = xs + s3 * XPL;
        const float *Bn = bs + sb * BPL;
        const uint8_t *C3 = cs + (1 + bi) * CPL;
        if (got) {
            if (m == mstart) {
                q1 = lds4(X1 + o);
                q2 = lds4(X2 + o);
                cpipe = (unsigned)cs[co] << 16;
            }
            const float4 q3 = lds4(X3 + o);
            const float4 bb2 = lds4(Bn + bo);
            const unsigned c3 = C3[co];
            cpipe |= c3 << 24;
            // coefficient lines of this quad's class-3 cells on plane m+3 go
            // to L1 ahead of their first use in step m+1
            const int kp = m + 3;
            if (quad_in && any_general(c3) && kp < g.d.nz) {
                const long long off = qoff + g.sz * kp;
                prefetch_l1(a.coef + off);
                prefetch_l1(a.gco + off);
            }
            const int ka = m + 2;
            if (ka >= 0 && ka <= k1 && ka < g.d.nz) {
                // first colour on plane m+2 (its neighbours carry the second
                // colour: values as staged)
                if (FIRST) {
                    const QuadScale e = scale_at(ka);
                    const unsigned c2 = (cpipe >> 16) & 0xffu;
                    if (quad_in) relax_pair_first(g, a, q2, bb2, c2, e, gi, gj, ka, (ca ^ gj ^ ka) & 1);
                } else {
                    const float4 ym = lds4(X2 + o - RW), yp = lds4(X2 + o + RW);
                    const QuadScale e = scale_at(ka);
                    const unsigned c2 = (cpipe >> 16) & 0xffu;
                    if ((ca ^ gj ^ ka) & 1) {
                        float s = __shfl_down_sync(FULL, q2.x, 1);
                        if (qx == QX - 1) s = X2[o + 4];
                        if (quad_in) relax_pair<1>(g, a, q2, s, ym, yp, q1, q3, bb2, c2, e, gi, gj, ka);
                    } else {
                        float s = __shfl_up_sync(FULL, q2.w, 1);
                        if (qx == 0) s = X2[o - 1];
                        if (quad_in) relax_pair<0>(g, a, q2, s, ym, yp, q1, q3, bb2, c2, e, gi, gj, ka);
                    }
                }
                if (quad_in) *reinterpret_cast<float4 *>(X2 + o) = q2;
            }
            if (m >= k0) {
                // second colour on plane m (its neighbours carry the first
                // colour: relaxed in steps m-3..m-1), then plane m is final
                const float4 ym = lds4(X0 + o - RW), yp = lds4(X0 + o + RW);
                const QuadScale e = scale_at(m);
                const unsigned c0 = cpipe & 0xffu;
                if ((cb ^ gj ^ m) & 1) {
                    float s = __shfl_down_sync(FULL, q0.x, 1);
                    if (qx == QX - 1) s = X0[o + 4];
                    if (quad_in) relax_pair<1>(g, a, q0, s, ym, yp, qm1, q1, bb0, c0, e, gi, gj, m);
                } else {
                    float s = __shfl_up_sync(FULL, q0.w, 1);
                    if (qx == 0) s = X0[o - 1];
                    if (quad_in) relax_pair<0>(g, a, q0, s, ym, yp, qm1, q1, bb0, c0, e, gi, gj, m);
                }
                if (quad_in) {
                    *reinterpret_cast<float4 *>(a.x_out + qoff + g.sz * m) = q0;
                    if (RZ) {
                        acc.add(bb0.x * q0.x);
                        acc.add(bb0.y * q0.y);
                        acc.add(bb0.z * q0.z);
                        acc.add(bb0.w * q0.w);
                    }
                }
            }
            qm1 = q0; q0 = q1; q1 = q2; q2 = q3;
            bb0 = bb1; bb1 = bb2;
            cpipe >>= 8;
            // the halo ring on plane m+2 last: the quads' transients are dead
            if (rrole == 0) {
                // ring row quad: its class byte on plane m+3 (kept for the
                // next step; class-3 lines go to L1), then the first colour
                // on plane m+2.  The two half-warps are the two rows; their
                // x-neighbours come by shuffles within 16-lane segments, taken
                // by the whole warp before the rows' own conditions.
                const int rl = lane & (QX - 1);
                const int rlrow = lane < QX ? -1 : TY;   // staged-row offset
                const int rgi = i0 + 4 * rl, rgj = j0 + rlrow;
                const bool rquad_in = rgj >= 0 && rgj < g.d.ny && rgi < g.d.nx;
                const int ro4 = (rlrow + 2) * RW + 4 + 4 * rl, rbo = (rlrow + 1) * RW + 4 + 4 * rl;
                const int rco = (rlrow + 1) * CW + 16 + rl;
                if (m == mstart) rcls = cs[rco];
                const unsigned rnext = C3[rco];
                if (rquad_in && any_general(rnext) && kp < g.d.nz) {
                    const long long off = rgi + g.sy * rgj + g.sz * kp;
                    prefetch_l1(a.coef + off);
                    prefetch_l1(a.gco + off);
                }
                if (FIRST && ka >= 0 && ka <= k1 && ka < g.d.nz) {
                    if (rquad_in) {
                        float4 rq = lds4(X2 + ro4);
                        const float4 rbq = lds4(Bn + rbo);
                        const int mz = (ka == 0 || ka == g.d.nz - 1) ? 9 * mze : 0;
                        const int rmy = (rgj == 0) + (rgj == g.d.ny - 1);
                        QuadScale re;
                        re.r0 = rdt[(rgi == 0) + 3 * rmy + mz];
                        re.r12 = rdt[3 * rmy + mz];
                        re.r3 = rdt[(rgi + 3 == g.d.nx - 1) + 3 * rmy + mz];
                        relax_pair_first(g, a, rq, rbq, rcls, re, rgi, rgj, ka, (ca ^ rgj ^ ka) & 1);
                        *reinterpret_cast<float4 *>(X2 + ro4) = rq;
                    }
                } else if (ka >= 0 && ka <= k1 && ka < g.d.nz) {
                    float4 rq = lds4(X2 + ro4);
                    float sd = __shfl_down_sync(FULL, rq.x, 1, QX), su = __shfl_up_sync(FULL, rq.w, 1, QX);
                    if (rl == QX - 1) sd = X2[ro4 + 4];
                    if (rl == 0) su = X2[ro4 - 1];
                    if (rquad_in) {
                        const float4 rym = lds4(X2 + ro4 - RW), ryp = lds4(X2 + ro4 + RW);
                        const float4 rzm = lds4(X1 + ro4), rzp = lds4(X3 + ro4), rbq = lds4(Bn + rbo);
                        const int mz = (ka == 0 || ka == g.d.nz - 1) ? 9 * mze : 0;
                        const int rmy = (rgj == 0) + (rgj == g.d.ny - 1);
                        QuadScale re;
                        re.r0 = rdt[(rgi == 0) + 3 * rmy + mz];
                        re.r12 = rdt[3 * rmy + mz];
                        re.r3 = rdt[(rgi + 3 == g.d.nx - 1) + 3 * rmy + mz];
                        const int P = (ca ^ rgj ^ ka) & 1;
                        relax_pair_rt(g, a, rq, P ? sd : su, rym, ryp, rzm, rzp, rbq, rcls, re, rgi, rgj, ka, P);
                        *reinterpret_cast<float4 *>(X2 + ro4) = rq;
                    }
                }
                rcls = rnext;
            } else if (rrole == 2) {
                // ring column cell: rows crow, crow+1, the first colour's one
                const int clx = (lane & 8) ? TX : -1, crow = 2 * (lane & 7);
                const int cgi = i0 + clx;
                const int sh0 = (ca + j0 + ka + clx + crow) & 1, sh1 = (ca + j0 + kp + clx + crow) & 1;
                const int ly0 = crow + sh0, ly1 = crow + sh1;
                const int byt = (clx >> 2) + 16, bit = 2 * (clx & 3);
                if (m == mstart) rcls = (cs[(ly0 + 1) * CW + byt] >> bit) & 3u;
                const unsigned rnext = (C3[(ly1 + 1) * CW + byt] >> bit) & 3u;
                const bool col_in = cgi >= 0 && cgi < g.d.nx;
                if (rnext == 3u && col_in && j0 + ly1 < g.d.ny && kp < g.d.nz) {
                    const long long off = cgi + g.sy * (j0 + ly1) + g.sz * kp;
                    prefetch_l1(a.coef + off);
                    prefetch_l1(a.gco + off);
                }
                const int rj = j0 + ly0;
                if (ka >= 0 && ka <= k1 && ka < g.d.nz && col_in && rj < g.d.ny) {
                    const int ro = (ly0 + 2) * RW + clx + 4;
                    const int mz = (ka == 0 || ka == g.d.nz - 1) ? 9 * mze : 0;
                    const float rd = rdt[(cgi == 0) + (cgi == g.d.nx - 1) + 3 * ((rj == 0) + (rj == g.d.ny - 1)) + mz];
                    const long long rc = cgi + g.sy * rj + g.sz * ka;
                    if (FIRST)
                        X2[ro] = __fmaf_rn(Bn[(ly0 + 1) * RW + clx + 4], first_scale(a, rcls, rc, rd), a.omsor * 0.f);
                    else
                        X2[ro] = relax_any(g, a, rcls, rc, X2[ro], X2[ro - 1], X2[ro + 1], X2[ro - RW], X2[ro + RW],
                                           X1[ro], X3[ro], Bn[(ly0 + 1) * RW + clx + 4], rd);
                }
                rcls = rnext;
            }
        }
        // x plane m, b plane m+2 and class plane m+3 are dead: refill them
        // with step m+SD's data
        fence_proxy_async_smem();
        if (__syncthreads_or(!got)) {
            failed = true;
            break;
        }
        if (tid == ISSUER && m + SD < k1) {
            const int mn = m + SD;
            mbar_expect_tx(bar0 + 8 * bi, XBYTES + BBYTES + CBYTES);
            tma_load_3d(smem_u32(X0), &xmap, i0 - 4, j0 - 2, xz(mn + 3), bar0 + 8 * bi);
            tma_load_3d(smem_u32(bs + sb * BPL), &bmap, i0 - 4, j0 - 1, mn + 2, bar0 + 8 * bi);
            tma_load_3d(smem_u32(C3), &cmap, i0 / 4 - 16, j0 - 1, mn + 3, bar0 + 8 * bi);
        }
        sx = s1;
        sb = sb + 1 == BS ? 0 : sb + 1;
        if (++bi == SD) { bi = 0; ph ^= 1; }
    }
    if (failed) {
        // record the failure, then wait (bounded) for the copies still in
        // flight to this block's shared memory before leaving
        if (tid == ISSUER) {
            if (a.st) atomicOr(&a.st->err, 1);
            for (int q = 0; q < SD; ++q) {
                const int b2 = (bi + q) % SD;
                const unsigned p2 = ph ^ (unsigned)((bi + q) / SD);
                mbar_wait_bounded(bar0 + 8 * b2, p2);
            }
        }
        __syncthreads();
        return;
    }
    if (RZ) {
        double v[1] = {acc.value()};
        double tot[1];
        if (grid_reduce<1>(v, a.partials, &a.st->ticket[3], tot, item)) {
            if (tid == 0) {
                PcgState *st = a.st;
                double rz = tot[0];
                st->rz = rz;
                if (a.rz_mode == 2) {
                    // seedScalarsKernel (linalg.js:1259-1267)
                    st->rz_old = rz;
                    st->pap_baseline = fmax(fabs(st->rr), PAP_BASELINE_FLOOR);
                    if (st->stop != FF_STOP_CONVERGED) {
                        st->stop = 0;
                        st->stop_iter = 0;
                    }
                    st->iter = 0;
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

// ------------------------------------------------------ CG on TMA levels --
// The two CG kernels of level 0 in the layout of the TMA sweep: 64 x 16
// tiles in the sweep's work order, one x-quad per thread, a z-march with
// one barrier per plane.  Step k brings plane k+1 of the operands (rows
// j0-1 .. j0+16, columns i0-4 .. i0+67) through cp.async.bulk.tensor, forms
// the operand there (p = z + beta p, or x + alpha p in double-single) for
// the thread's quad, the halo rows and the halo columns, keeps the quad in
// registers and leaves the plane in shared memory, then applies A to plane
// k: z-neighbours from registers, x-neighbours by shuffle, y-neighbours from
// the shared plane.  Cells by class: the plain second differences (class 0),
// plus h^-2 v for each face across the domain edge (class 2, whose
// zero-filled neighbour entered as 0 - v), -v for a Dirichlet row (class 1),
// the stored couplings otherwise (class 3).
namespace tcg {
constexpr int TX = 64, TY = 16, QX = TX / 4, NT = QX * TY;
constexpr int RW = TX + 8, PR = TY + 2;   // staged columns i0-4 .. i0+TX+3, rows j0-1 .. j0+TY
constexpr int PPL = ((PR * RW * 4 + 127) / 128) * 32;   // plane slot (1312 floats)
constexpr int BPL = TY * RW;                            // b: rows j0 .. j0+TY-1 (1152 floats)
constexpr unsigned PBYTES = PR * RW * 4, BBYTES = TY * RW * 4;
constexpr int CW = 48, CPL = 896;
constexpr unsigned CBYTES = CW * PR;
constexpr int PSD = 3, XSD = 3;           // stages in flight
constexpr size_t PAP_SMEM = 128 + 4 * ((size_t)PSD * 2 * PPL + 2 * PPL) + (size_t)PSD * CPL + 8 * PSD;
constexpr size_t XR_SMEM =
    128 + 4 * ((size_t)XSD * (3 * PPL + BPL) + 4 * PPL) + (size_t)XSD * CPL + 8 * XSD;
static_assert((BPL * 4) % 128 == 0, "TMA destinations stay 128-byte aligned");
}  // namespace tcg

struct TcgArgs {
    Geo g;
    const float4 *coef, *gco;
    const int *order;
    int gx, gy, zc;
    float *p0, *p1;
    float *xh0, *xl0, *xh1, *xl1, *r;
    PcgState *st;
    double *partials;
};

__device__ __forceinline__ float4 fma4(float s, const float4 &a, const float4 &b) {
    return make_float4(__fmaf_rn(s, a.x, b.x), __fmaf_rn(s, a.y, b.y), __fmaf_rn(s, a.z, b.z),
                       __fmaf_rn(s, a.w, b.w));
}
__device__ __forceinline__ void st4(float *p, const float4 &v) { *reinterpret_cast<float4 *>(p) = v; }

// A neighbour across the domain edge stands in as the cell itself, so the
// absent face's difference is an exact zero.  (Adding h^-2 v back to a
// zero-filled neighbour's -h^-2 v cancels to within a rounding of h^-2 |v|:
// near a wall under a hydrostatic pressure that is far above the residual
// the solve has to reach.)
__device__ __forceinline__ void edge_self(const Geo &g, int i, int j, int k, float vc, float &xm, float &xp,
                                          float &ym, float &yp, float &zm, float &zp) {
    if (i == 0) xm = vc;
    if (i == g.d.nx - 1) xp = vc;
    if (j == 0) ym = vc;
    if (j == g.d.ny - 1) yp = vc;
    if (k == 0) zm = vc;
    if (k == g.d.nz - 1) zp = vc;
}

// (A v)_c of one cell by class; ci its index.
__device__ __forceinline__ float ap_cell(const Geo &g, const float4 *coef, const float4 *gco, unsigned c, int i,
                                         int j, int k, long long ci, float vc, float xm, float xp, float ym, float yp,
                                         float zm, float zp) {
    if (c == 2u) edge_self(g, i, j, k, vc, xm, xp, ym, yp, zm, zp);
    const float ar = apply_reg(g, vc, xm, xp, ym, yp, zm, zp);
    if (c == 0u || c == 2u) return ar;
    if (c == 1u) return -vc;
    const float4 lo = __ldg(coef + ci), hi = __ldg(gco + ci);
    Coef q;
    q.kx = i > 0 ? lo.x : 0.f;
    q.ky = j > 0 ? lo.y : 0.f;
    q.kz = k > 0 ? lo.z : 0.f;
    q.e = lo.w;
    q.ux = hi.x;
    q.uy = hi.y;
    q.uz = hi.z;
    return apply_q(q, vc, xm, xp, ym, yp, zm, zp);
}

__global__ void __launch_bounds__(tcg::NT, 4)
    k_p_pap_tma(TcgArgs a, const __grid_constant__ CUtensorMap zmap, const __grid_constant__ CUtensorMap p0map,
                const __grid_constant__ CUtensorMap p1map, const __grid_constant__ CUtensorMap cmap) {
    constexpr int TX = tcg::TX, TY = tcg::TY, QX = tcg::QX, RW = tcg::RW, PPL = tcg::PPL, CW = tcg::CW;
    constexpr int CPL = tcg::CPL, SD = tcg::PSD;
    constexpr unsigned PBYTES = tcg::PBYTES, CBYTES = tcg::CBYTES, FULL = 0xffffffffu;
    pdl_wait();
    PcgState *st = a.st;
    if (st->stop || st->err) return;
    extern __shared__ __align__(16) unsigned char dyn_raw[];
    float *zs = reinterpret_cast<float *>(dyn_raw + ((128u - (smem_u32(dyn_raw) & 127u)) & 127u));
    float *pos = zs + SD * PPL;   // old p, one plane per stage
    float *pn = pos + SD * PPL;   // new p of plane k in slot k & 1
    uint8_t *cs = reinterpret_cast<uint8_t *>(pn + 2 * PPL);
    const unsigned bar0 = smem_u32(cs + SD * CPL);
    const Geo &g = a.g;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int qx = lane & (QX - 1), ty = 4 * (warp >> 1) + (warp & 1) + 2 * (lane >> 4);
    constexpr int ISSUER = tcg::NT - 1;
    const int pc = st->p_cur;
    const bool first = st->first != 0;
    const float beta = (float)st->beta;
    const CUtensorMap *pm = pc ? &p1map : &p0map;
    float *pnew = pc ? a.p0 : a.p1;
    const int item = a.order ? a.order[blockIdx.x] : (int)blockIdx.x;
    const int i0 = (item % a.gx) * TX, j0 = ((item / a.gx) % a.gy) * TY;
    const int k0 = (item / (a.gx * a.gy)) * a.zc, k1 = min(k0 + a.zc, g.d.nz);
    // steps k0-2 .. k1-1: step k brings plane k+1 of z, the old p and the
    // classes, forms the new p there and applies A to plane k
    const int mstart = k0 - 2;
    const unsigned stage_bytes = (first ? 1u : 2u) * PBYTES + CBYTES;
    if (tid == ISSUER) {
        asm volatile("prefetch.tensormap [%0];" ::"l"(&zmap) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(pm) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(&cmap) : "memory");
        for (int q = 0; q < SD; ++q) mbar_init(bar0 + 8 * q, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int q = 0; q < SD && mstart + q < k1; ++q) {
            const int pl = mstart + q + 1;
            mbar_expect_tx(bar0 + 8 * q, stage_bytes);
            tma_load_3d(smem_u32(zs + q * PPL), &zmap, i0 - 4, j0 - 1, pl, bar0 + 8 * q);
            if (!first) tma_load_3d(smem_u32(pos + q * PPL), pm, i0 - 4, j0 - 1, pl, bar0 + 8 * q);
            tma_load_3d(smem_u32(cs + q * CPL), &cmap, i0 / 4 - 16, j0 - 1, pl, bar0 + 8 * q);
        }
    }
    __syncthreads();
    const int lx = 4 * qx, gi = i0 + lx, gj = j0 + ty;
    const bool quad_in = gi < g.d.nx && gj < g.d.ny;
    const int o = (ty + 1) * RW + 4 + lx;
    const int co = (ty + 1) * CW + 16 + qx;
    const long long qoff = gi + g.sy * gj;
    // halo quads of the new p: rows j0-1 and j0+TY on lanes 0..15 of warps 0 and 1
    const bool halo = warp < 2 && lane < QX;   // warp 0: row j0-1, warp 1: row j0+TY (16 quads each)
    const int ho = (warp == 0 ? 0 : tcg::PR - 1) * RW + 4 + 4 * (lane & (QX - 1));
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float4 pm1 = zero4, p0 = zero4;   // new p on planes k-1 and k
    unsigned ck = 0;                  // class byte of plane k
    Acc acc;
    int bi = 0;
    unsigned ph = 0;
    bool failed = false;
    for (int k = mstart; k < k1; ++k) {
        const bool got = mbar_wait_bounded(bar0 + 8 * bi, ph);
        const float *Z = zs + bi * PPL, *Po = pos + bi * PPL;
        float *N1 = pn + ((k + 1) & 1) * PPL;
        const float *N0 = pn + (k & 1) * PPL;
        float4 p1 = zero4;
        unsigned cnext = 0;
        if (got) {
            // the new p on plane k+1: this quad, the halo rows, the halo columns
            const int kn = k + 1;
            const float4 zq = lds4(Z + o);
            p1 = first ? zq : fma4(beta, lds4(Po + o), zq);
            st4(N1 + o, p1);
            if (halo) {
                const float4 zh = lds4(Z + ho);
                st4(N1 + ho, first ? zh : fma4(beta, lds4(Po + ho), zh));
            }
            if (qx == 0) N1[o - 1] = first ? Z[o - 1] : __fmaf_rn(beta, Po[o - 1], Z[o - 1]);
            if (qx == QX - 1) N1[o + 4] = first ? Z[o + 4] : __fmaf_rn(beta, Po[o + 4], Z[o + 4]);
            if (quad_in && kn >= k0 && kn < k1) st4(pnew + qoff + g.sz * kn, p1);
            cnext = cs[bi * CPL + co];
            if (quad_in && any_general(cnext) && kn < g.d.nz) {
                prefetch_l1(a.coef + qoff + g.sz * kn);
                prefetch_l1(a.gco + qoff + g.sz * kn);
            }
            if (k >= k0) {
                // A on plane k
                const float4 ym = lds4(N0 + o - RW), yp = lds4(N0 + o + RW);
                float xl = __shfl_up_sync(FULL, p0.w, 1), xr = __shfl_down_sync(FULL, p0.x, 1);
                if (qx == 0) xl = N0[o - 1];
                if (qx == QX - 1) xr = N0[o + 4];
                if (quad_in) {
                    float a0, a1, a2, a3;
                    if (ck == 0u) {
                        a0 = apply_reg(g, p0.x, xl, p0.y, ym.x, yp.x, pm1.x, p1.x);
                        a1 = apply_reg(g, p0.y, p0.x, p0.z, ym.y, yp.y, pm1.y, p1.y);
                        a2 = apply_reg(g, p0.z, p0.y, p0.w, ym.z, yp.z, pm1.z, p1.z);
                        a3 = apply_reg(g, p0.w, p0.z, xr, ym.w, yp.w, pm1.w, p1.w);
                    } else {
                        const long long ci = qoff + g.sz * k;
                        a0 = ap_cell(g, a.coef, a.gco, ck & 3u, gi, gj, k, ci, p0.x, xl, p0.y, ym.x, yp.x, pm1.x,
                                     p1.x);
                        a1 = ap_cell(g, a.coef, a.gco, (ck >> 2) & 3u, gi + 1, gj, k, ci + 1, p0.y, p0.x, p0.z,
                                     ym.y, yp.y, pm1.y, p1.y);
                        a2 = ap_cell(g, a.coef, a.gco, (ck >> 4) & 3u, gi + 2, gj, k, ci + 2, p0.z, p0.y, p0.w,
                                     ym.z, yp.z, pm1.z, p1.z);
                        a3 = ap_cell(g, a.coef, a.gco, ck >> 6, gi + 3, gj, k, ci + 3, p0.w, p0.z, xr, ym.w, yp.w,
                                     pm1.w, p1.w);
                    }
                    acc.add(p0.x * a0);
                    acc.add(p0.y * a1);
                    acc.add(p0.z * a2);
                    acc.add(p0.w * a3);
                }
            }
        }
        pm1 = p0;
        p0 = p1;
        ck = cnext;
        // plane k+1's stage is consumed: refill it with plane k+1+SD
        fence_proxy_async_smem();
        if (__syncthreads_or(!got)) {
            failed = true;
            break;
        }
        if (tid == ISSUER && k + SD < k1) {
            const int pl = k + SD + 1;
            mbar_expect_tx(bar0 + 8 * bi, stage_bytes);
            tma_load_3d(smem_u32(zs + bi * PPL), &zmap, i0 - 4, j0 - 1, pl, bar0 + 8 * bi);
            if (!first) tma_load_3d(smem_u32(pos + bi * PPL), pm, i0 - 4, j0 - 1, pl, bar0 + 8 * bi);
            tma_load_3d(smem_u32(cs + bi * CPL), &cmap, i0 / 4 - 16, j0 - 1, pl, bar0 + 8 * bi);
        }
        if (++bi == SD) { bi = 0; ph ^= 1; }
    }
    if (failed) {
        if (tid == ISSUER) {
            atomicOr(&st->err, 1);
            for (int q = 0; q < SD; ++q) mbar_wait_bounded(bar0 + 8 * ((bi + q) % SD), ph ^ (unsigned)((bi + q) / SD));
        }
        __syncthreads();
        return;
    }
    double v[1] = {acc.value()};
    double tot[1];
    if (grid_reduce<1>(v, a.partials, &st->ticket[1], tot, item)) {
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

// r = b - A x in double-single for one cell of class 1 or 3: each coupling
// term K (x_n - x_c) formed from (hi, lo) with an error-free difference and
// product, summed with TwoSum (the general path of the cp.async kernel).
__device__ __forceinline__ float resid_ds_general(const Coef &q, float bc, float chv, float clv, float xmh,
                                                  float xml, float xph, float xpl, float ymh, float yml, float yph,
                                                  float ypl, float zmh, float zml, float zph, float zpl) {
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
    term(q.kx, xmh, xml);
    term(q.ux, xph, xpl);
    term(q.ky, ymh, yml);
    term(q.uy, yph, ypl);
    term(q.kz, zmh, zml);
    term(q.uz, zph, zpl);
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
    return __fadd_rn(r0, __fsub_rn(e0, Se));
}

// One cell's residual by class (hi/lo of the cell and its six neighbours).
template <bool DS>
__device__ __forceinline__ float resid_cell(const Geo &g, const float4 *coef, const float4 *gco, unsigned c, int i,
                                            int j, int k, long long ci, float bc, float ch, float cl, float xmh,
                                            float xml, float xph, float xpl, float ymh, float yml, float yph,
                                            float ypl, float zmh, float zml, float zph, float zpl) {
    if (!(c & 1u)) {
        if (c == 2u) {
            edge_self(g, i, j, k, ch, xmh, xph, ymh, yph, zmh, zph);
            if (DS) edge_self(g, i, j, k, cl, xml, xpl, yml, ypl, zml, zpl);
        }
        float ax = apply_reg(g, ch, xmh, xph, ymh, yph, zmh, zph);
        if (DS) ax += apply_reg(g, cl, xml, xpl, yml, ypl, zml, zpl);
        return bc - ax;
    }
    Coef q;
    if (c == 1u) {
        q.kx = q.ky = q.kz = q.ux = q.uy = q.uz = 0.f;
        q.e = 1.f;
    } else {
        const float4 lo = __ldg(coef + ci), hi = __ldg(gco + ci);
        q.kx = i > 0 ? lo.x : 0.f;
        q.ky = j > 0 ? lo.y : 0.f;
        q.kz = k > 0 ? lo.z : 0.f;
        q.e = lo.w;
        q.ux = hi.x;
        q.uy = hi.y;
        q.uz = hi.z;
    }
    if (DS)
        return resid_ds_general(q, bc, ch, cl, xmh, xml, xph, xpl, ymh, yml, yph, ypl, zmh, zml, zph, zpl);
    return bc - apply_q(q, ch, xmh, xph, ymh, yph, zmh, zph);
}

template <bool SETUP, bool DS>
__global__ void __launch_bounds__(tcg::NT, 2)
    k_x_residual_tma(TcgArgs a, const __grid_constant__ CUtensorMap h0map, const __grid_constant__ CUtensorMap h1map,
                     const __grid_constant__ CUtensorMap l0map, const __grid_constant__ CUtensorMap l1map,
                     const __grid_constant__ CUtensorMap p0map, const __grid_constant__ CUtensorMap p1map,
                     const __grid_constant__ CUtensorMap bmap, const __grid_constant__ CUtensorMap cmap) {
    constexpr int TX = tcg::TX, TY = tcg::TY, QX = tcg::QX, RW = tcg::RW, PPL = tcg::PPL, BPL = tcg::BPL;
    constexpr int CW = tcg::CW, CPL = tcg::CPL, SD = tcg::XSD;
    constexpr unsigned PBYTES = tcg::PBYTES, BBYTES = tcg::BBYTES, CBYTES = tcg::CBYTES, FULL = 0xffffffffu;
    pdl_wait();
    PcgState *st = a.st;
    if (!SETUP && (st->stop || st->err)) return;
    extern __shared__ __align__(16) unsigned char dyn_raw[];
    float *hs = reinterpret_cast<float *>(dyn_raw + ((128u - (smem_u32(dyn_raw) & 127u)) & 127u));
    float *ls = hs + SD * PPL;    // x lo per stage
    float *qs = ls + SD * PPL;    // p per stage
    float *bs = qs + SD * PPL;    // b per stage
    float *nh = bs + SD * BPL;    // new x hi of plane k in slot k & 1
    float *nl = nh + 2 * PPL;     // new x lo
    uint8_t *cs = reinterpret_cast<uint8_t *>(nl + 2 * PPL);
    const unsigned bar0 = smem_u32(cs + SD * CPL);
    const Geo &g = a.g;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int qx = lane & (QX - 1), ty = 4 * (warp >> 1) + (warp & 1) + 2 * (lane >> 4);
    constexpr int ISSUER = tcg::NT - 1;
    const int xc = SETUP ? 0 : st->x_cur;
    const CUtensorMap *hm = xc ? &h1map : &h0map, *lm = xc ? &l1map : &l0map;
    const CUtensorMap *qm = st->p_cur ? &p1map : &p0map;
    float *oh = xc ? a.xh0 : a.xh1, *ol = xc ? a.xl0 : a.xl1;
    const double alpha = SETUP ? 0.0 : st->alpha;
    const float ahi = (float)alpha, alo = (float)(alpha - (double)ahi);
    const int item = a.order ? a.order[blockIdx.x] : (int)blockIdx.x;
    const int i0 = (item % a.gx) * TX, j0 = ((item / a.gx) % a.gy) * TY;
    const int k0 = (item / (a.gx * a.gy)) * a.zc, k1 = min(k0 + a.zc, g.d.nz);
    // steps k0-2 .. k1-1: step k brings plane k+1 of x (hi, lo), p, b and
    // the classes, forms x + alpha p there and forms r on plane k
    const int mstart = k0 - 2;
    constexpr unsigned stage_bytes = (1u + (DS ? 1u : 0u) + (SETUP ? 0u : 1u)) * PBYTES + BBYTES + CBYTES;
    if (tid == ISSUER) {
        for (int q = 0; q < SD; ++q) mbar_init(bar0 + 8 * q, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int q = 0; q < SD && mstart + q < k1; ++q) {
            const int pl = mstart + q + 1;
            const unsigned bar = bar0 + 8 * q;
            mbar_expect_tx(bar, stage_bytes);
            tma_load_3d(smem_u32(hs + q * PPL), hm, i0 - 4, j0 - 1, pl, bar);
            if (DS) tma_load_3d(smem_u32(ls + q * PPL), lm, i0 - 4, j0 - 1, pl, bar);
            if (!SETUP) tma_load_3d(smem_u32(qs + q * PPL), qm, i0 - 4, j0 - 1, pl, bar);
            tma_load_3d(smem_u32(bs + q * BPL), &bmap, i0 - 4, j0, pl, bar);
            tma_load_3d(smem_u32(cs + q * CPL), &cmap, i0 / 4 - 16, j0 - 1, pl, bar);
        }
    }
    __syncthreads();
    const int lx = 4 * qx, gi = i0 + lx, gj = j0 + ty;
    const bool quad_in = gi < g.d.nx && gj < g.d.ny;
    const int o = (ty + 1) * RW + 4 + lx, bo = ty * RW + 4 + lx;
    const int co = (ty + 1) * CW + 16 + qx;
    const long long qoff = gi + g.sy * gj;
    const bool halo = warp < 2 && lane < QX;   // warp 0: row j0-1, warp 1: row j0+TY (16 quads each)
    const int ho = (warp == 0 ? 0 : tcg::PR - 1) * RW + 4 + 4 * (lane & (QX - 1));
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    // x (hi, lo) on planes k-1 and k, b on plane k
    float4 hm1 = zero4, lm1 = zero4, h0 = zero4, l0 = zero4, b0 = zero4;
    unsigned ck = 0;
    Acc acc_rr, acc_bb;
    int bi = 0;
    unsigned ph = 0;
    bool failed = false;
    // x + alpha p of one staged value
    auto form1 = [&](const float *H, const float *L, const float *Q, int off, float &oh1, float &ol1) {
        const float hv = H[off], lv = DS ? L[off] : 0.f;
        if (SETUP) {
            oh1 = hv;
            ol1 = lv;
        } else if (DS) {
            ds_axpy(hv, lv, ahi, alo, Q[off], oh1, ol1);
        } else {
            oh1 = __fmaf_rn(ahi, Q[off], hv);
            ol1 = 0.f;
        }
    };
    auto form4 = [&](const float *H, const float *L, const float *Q, int off, float4 &oh4, float4 &ol4) {
        const float4 hv = lds4(H + off), lv = DS ? lds4(L + off) : zero4;
        if (SETUP) {
            oh4 = hv;
            ol4 = lv;
        } else {
            const float4 qv = lds4(Q + off);
            if (DS) {
                ds_axpy(hv.x, lv.x, ahi, alo, qv.x, oh4.x, ol4.x);
                ds_axpy(hv.y, lv.y, ahi, alo, qv.y, oh4.y, ol4.y);
                ds_axpy(hv.z, lv.z, ahi, alo, qv.z, oh4.z, ol4.z);
                ds_axpy(hv.w, lv.w, ahi, alo, qv.w, oh4.w, ol4.w);
            } else {
                oh4 = fma4(ahi, qv, hv);
                ol4 = zero4;
            }
        }
    };
    for (int k = mstart; k < k1; ++k) {
        const bool got = mbar_wait_bounded(bar0 + 8 * bi, ph);
        const float *H = hs + bi * PPL, *L = ls + bi * PPL, *Q = qs + bi * PPL, *B = bs + bi * BPL;
        float *NH1 = nh + ((k + 1) & 1) * PPL, *NL1 = nl + ((k + 1) & 1) * PPL;
        const float *NH0 = nh + (k & 1) * PPL, *NL0 = nl + (k & 1) * PPL;
        float4 h1 = zero4, l1 = zero4, b1 = zero4;
        unsigned cnext = 0;
        if (got) {
            const int kn = k + 1;
            // x + alpha p on plane k+1: this quad, the halo rows, the halo columns
            form4(H, L, Q, o, h1, l1);
            st4(NH1 + o, h1);
            if (DS) st4(NL1 + o, l1);
            if (halo) {
                float4 hh, hl;
                form4(H, L, Q, ho, hh, hl);
                st4(NH1 + ho, hh);
                if (DS) st4(NL1 + ho, hl);
            }
            if (qx == 0 || qx == QX - 1) {
                const int eo = qx == 0 ? o - 1 : o + 4;
                float eh, el;
                form1(H, L, Q, eo, eh, el);
                NH1[eo] = eh;
                if (DS) NL1[eo] = el;
            }
            if (!SETUP && quad_in && kn >= k0 && kn < k1) {
                st4(oh + qoff + g.sz * kn, h1);
                if (DS) st4(ol + qoff + g.sz * kn, l1);
            }
            b1 = lds4(B + bo);
            cnext = cs[bi * CPL + co];
            if (quad_in && any_general(cnext) && kn < g.d.nz) {
                prefetch_l1(a.coef + qoff + g.sz * kn);
                prefetch_l1(a.gco + qoff + g.sz * kn);
            }
            if (k >= k0) {
                // r = b - A x on plane k
                const float4 ymh = lds4(NH0 + o - RW), yph = lds4(NH0 + o + RW);
                const float4 yml = DS ? lds4(NL0 + o - RW) : zero4, ypl = DS ? lds4(NL0 + o + RW) : zero4;
                float xlh = __shfl_up_sync(FULL, h0.w, 1), xrh = __shfl_down_sync(FULL, h0.x, 1);
                float xll = DS ? __shfl_up_sync(FULL, l0.w, 1) : 0.f, xrl = DS ? __shfl_down_sync(FULL, l0.x, 1) : 0.f;
                if (qx == 0) {
                    xlh = NH0[o - 1];
                    if (DS) xll = NL0[o - 1];
                }
                if (qx == QX - 1) {
                    xrh = NH0[o + 4];
                    if (DS) xrl = NL0[o + 4];
                }
                if (quad_in) {
                    float4 rq;
                    if (ck == 0u) {
                        float ax0 = apply_reg(g, h0.x, xlh, h0.y, ymh.x, yph.x, hm1.x, h1.x);
                        float ax1 = apply_reg(g, h0.y, h0.x, h0.z, ymh.y, yph.y, hm1.y, h1.y);
                        float ax2 = apply_reg(g, h0.z, h0.y, h0.w, ymh.z, yph.z, hm1.z, h1.z);
                        float ax3 = apply_reg(g, h0.w, h0.z, xrh, ymh.w, yph.w, hm1.w, h1.w);
                        if (DS) {
                            ax0 += apply_reg(g, l0.x, xll, l0.y, yml.x, ypl.x, lm1.x, l1.x);
                            ax1 += apply_reg(g, l0.y, l0.x, l0.z, yml.y, ypl.y, lm1.y, l1.y);
                            ax2 += apply_reg(g, l0.z, l0.y, l0.w, yml.z, ypl.z, lm1.z, l1.z);
                            ax3 += apply_reg(g, l0.w, l0.z, xrl, yml.w, ypl.w, lm1.w, l1.w);
                        }
                        rq = make_float4(b0.x - ax0, b0.y - ax1, b0.z - ax2, b0.w - ax3);
                    } else {
                        const long long ci = qoff + g.sz * k;
                        rq.x = resid_cell<DS>(g, a.coef, a.gco, ck & 3u, gi, gj, k, ci, b0.x, h0.x, l0.x, xlh, xll,
                                              h0.y, l0.y, ymh.x, yml.x, yph.x, ypl.x, hm1.x, lm1.x, h1.x, l1.x);
                        rq.y = resid_cell<DS>(g, a.coef, a.gco, (ck >> 2) & 3u, gi + 1, gj, k, ci + 1, b0.y, h0.y,
                                              l0.y, h0.x, l0.x, h0.z, l0.z, ymh.y, yml.y, yph.y, ypl.y, hm1.y, lm1.y,
                                              h1.y, l1.y);
                        rq.z = resid_cell<DS>(g, a.coef, a.gco, (ck >> 4) & 3u, gi + 2, gj, k, ci + 2, b0.z, h0.z,
                                              l0.z, h0.y, l0.y, h0.w, l0.w, ymh.z, yml.z, yph.z, ypl.z, hm1.z, lm1.z,
                                              h1.z, l1.z);
                        rq.w = resid_cell<DS>(g, a.coef, a.gco, ck >> 6, gi + 3, gj, k, ci + 3, b0.w, h0.w, l0.w,
                                              h0.z, l0.z, xrh, xrl, ymh.w, yml.w, yph.w, ypl.w, hm1.w, lm1.w, h1.w,
                                              l1.w);
                    }
                    st4(a.r + qoff + g.sz * k, rq);
                    acc_rr.add(rq.x * rq.x);
                    acc_rr.add(rq.y * rq.y);
                    acc_rr.add(rq.z * rq.z);
                    acc_rr.add(rq.w * rq.w);
                    if (SETUP) {
                        acc_bb.add(b0.x * b0.x);
                        acc_bb.add(b0.y * b0.y);
                        acc_bb.add(b0.z * b0.z);
                        acc_bb.add(b0.w * b0.w);
                    }
                }
            }
        }
        hm1 = h0;
        lm1 = l0;
        h0 = h1;
        l0 = l1;
        b0 = b1;
        ck = cnext;
        fence_proxy_async_smem();
        if (__syncthreads_or(!got)) {
            failed = true;
            break;
        }
        if (tid == ISSUER && k + SD < k1) {
            const int pl = k + SD + 1;
            const unsigned bar = bar0 + 8 * bi;
            mbar_expect_tx(bar, stage_bytes);
            tma_load_3d(smem_u32(hs + bi * PPL), hm, i0 - 4, j0 - 1, pl, bar);
            if (DS) tma_load_3d(smem_u32(ls + bi * PPL), lm, i0 - 4, j0 - 1, pl, bar);
            if (!SETUP) tma_load_3d(smem_u32(qs + bi * PPL), qm, i0 - 4, j0 - 1, pl, bar);
            tma_load_3d(smem_u32(bs + bi * BPL), &bmap, i0 - 4, j0, pl, bar);
            tma_load_3d(smem_u32(cs + bi * CPL), &cmap, i0 / 4 - 16, j0 - 1, pl, bar);
        }
        if (++bi == SD) { bi = 0; ph ^= 1; }
    }
    if (failed) {
        if (tid == ISSUER) {
            atomicOr(&st->err, 1);
            for (int q = 0; q < SD; ++q) mbar_wait_bounded(bar0 + 8 * ((bi + q) % SD), ph ^ (unsigned)((bi + q) / SD));
        }
        __syncthreads();
        return;
    }
    if (SETUP) {
        double v[2] = {acc_rr.value(), acc_bb.value()};
        double tot[2];
        if (grid_reduce<2>(v, a.partials, &st->ticket[0], tot, item)) {
            if (tid == 0) {
                st->rr = tot[0];
                st->bb = tot[1];
                double nb = sqrt(fabs(tot[1]));
                st->thr = st->relative ? fmax(st->tol * nb, st->tol) : st->tol;
                // the start already meets the tolerance (linalg.js:1695-1699)
                if (sqrt(fabs(tot[0])) < st->thr) {
                    st->stop = FF_STOP_CONVERGED;
                    st->stop_iter = 0;
                }
            }
        }
    } else {
        double v[1] = {acc_rr.value()};
        double tot[1];
        if (grid_reduce<1>(v, a.partials, &st->ticket[2], tot, item)) {
            if (tid == 0) {
                double rr = tot[0];
                st->rr = rr;
                st->x_cur = xc ^ 1;
                st->iter += 1;
                // residual-growing, sampled where the reference's host reads
                // the residual: at its chunk ends
                if (!nonfinite_d(rr) && st->iter >= st->guard_next) {
                    st->guard_next += GROWTH_SAMPLE;
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
                // the start already meets the tolerance (linalg.js:1695-1699)
                if (sqrt(fabs(tot[0])) < st->thr) {
                    st->stop = FF_STOP_CONVERGED;
                    st->stop_iter = 0;
                }
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
                // residual-growing, sampled where the reference's host reads
                // the residual: at its chunk ends
                if (!nonfinite_d(rr) && st->iter >= st->guard_next) {
                    st->guard_next += GROWTH_SAMPLE;
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

// --------------------------------------------- residual and restriction --
// buildResidualKernel (multigrid.js:741-749) + buildRestrictKernel
// (:866-914) as two streaming passes on levels with cell classes:
//  k_resid_rx: r = b - A x per cell (class dispatch as the sweep; zero on a
//   Dirichlet cell), then the x-direction restriction taps (1/8, 3/8, 3/8,
//   1/8 at fine 2I-1 .. 2I+2, clamped) into rx (nx/2 x ny x nz);
//  k_restrict_yz: the y and z taps of rx into the coarse b, zero on coarse
//   Dirichlet cells.
__device__ __forceinline__ float resid_cls(const Geo &g, const float4 *coef, unsigned cls, int i, int j, int k,
                                           float bval, float vc, float xm, float xp, float ym, float yp, float zm,
                                           float zp) {
    if (cls == 0) return bval - apply_reg(g, vc, xm, xp, ym, yp, zm, zp);
    if (cls == 1) return 0.0f;   // Dirichlet cell (the fine-mask zero)
    const long long c = i + g.sy * j + g.sz * k;
    Coef q = coef_at(g, coef, cls == 2, i, j, k, c);
    return bval - apply_q(q, vc, xm, xp, ym, yp, zm, zp);
}

// residual of the fine cell i of row `row` with scalar loads (used for the
// cells next to a quad that another warp owns)
__device__ __forceinline__ float resid_scalar(const Geo &g, const float *__restrict__ x, const float *__restrict__ b,
                                              const float4 *__restrict__ coef, const uint8_t *crow, long long row,
                                              long long rym, long long ryp, long long rzm, long long rzp, int i, int j,
                                              int k) {
    const unsigned cb = (crow[i >> 2] >> (2 * (i & 3))) & 3u;
    const float xm = __ldg(x + row + (i > 0 ? i - 1 : i));
    const float xp = __ldg(x + row + (i < g.d.nx - 1 ? i + 1 : i));
    return resid_cls(g, coef, cb, i, j, k, __ldg(b + row + i), __ldg(x + row + i), xm, xp, __ldg(x + rym + i),
                     __ldg(x + ryp + i), __ldg(x + rzm + i), __ldg(x + rzp + i));
}

// One thread per fine x-quad: float4 loads of the quad's row, its y and z
// neighbours and b; the residual at the cells just outside the quad comes
// from the neighbouring lanes (same row), computed directly at warp edges.
// Block (32, 8): a warp holds 32 consecutive quads of one row; grid (quads
// / 32, rows / 8, planes) so no index needs a division.
__global__ void __launch_bounds__(256, 4) k_resid_rx(Geo g, const float *__restrict__ x, const float *__restrict__ b,
                                                  const float4 *__restrict__ coef, const uint8_t *__restrict__ cls,
                                                  int cpitch, float *__restrict__ rx, const PcgState *st) {
    pdl_wait();
    if (st && st->stop) return;
    const int nq = g.d.nx >> 2, cnx = g.d.nx >> 1;
    const int j = blockIdx.y * 8 + threadIdx.y, k = blockIdx.z;
    if (j >= g.d.ny) return;   // whole warps (a warp is one row segment)
    const int qraw = blockIdx.x * 32 + threadIdx.x;
    const bool valid = qraw < nq;
    const int qx = valid ? qraw : nq - 1;
    const int i0 = 4 * qx;
    const long long row = g.sy * j + g.sz * k;
    const long long rym = row + (j > 0 ? -g.sy : 0), ryp = row + (j < g.d.ny - 1 ? g.sy : 0);
    const long long rzm = row + (k > 0 ? -g.sz : 0), rzp = row + (k < g.d.nz - 1 ? g.sz : 0);
    const uint8_t *crow = cls + (long long)cpitch * (j + (long long)g.d.ny * k);
    const int lane = threadIdx.x;
    const float4 c = __ldg(reinterpret_cast<const float4 *>(x + row + i0));
    const float xl = i0 > 0 ? __ldg(x + row + i0 - 1) : c.x;
    const float xr = i0 + 4 < g.d.nx ? __ldg(x + row + i0 + 4) : c.w;
    const float4 ym = __ldg(reinterpret_cast<const float4 *>(x + rym + i0));
    const float4 yp = __ldg(reinterpret_cast<const float4 *>(x + ryp + i0));
    const float4 zm = __ldg(reinterpret_cast<const float4 *>(x + rzm + i0));
    const float4 zp = __ldg(reinterpret_cast<const float4 *>(x + rzp + i0));
    const float4 bq = __ldg(reinterpret_cast<const float4 *>(b + row + i0));
    const unsigned cq = crow[qx];
    float r0, r1, r2, r3;
    if (cq == 0) {
        r0 = bq.x - apply_reg(g, c.x, xl, c.y, ym.x, yp.x, zm.x, zp.x);
        r1 = bq.y - apply_reg(g, c.y, c.x, c.z, ym.y, yp.y, zm.y, zp.y);
        r2 = bq.z - apply_reg(g, c.z, c.y, c.w, ym.z, yp.z, zm.z, zp.z);
        r3 = bq.w - apply_reg(g, c.w, c.z, xr, ym.w, yp.w, zm.w, zp.w);
    } else {
        r0 = resid_cls(g, coef, cq & 3u, i0, j, k, bq.x, c.x, xl, c.y, ym.x, yp.x, zm.x, zp.x);
        r1 = resid_cls(g, coef, (cq >> 2) & 3u, i0 + 1, j, k, bq.y, c.y, c.x, c.z, ym.y, yp.y, zm.y, zp.y);
        r2 = resid_cls(g, coef, (cq >> 4) & 3u, i0 + 2, j, k, bq.z, c.z, c.y, c.w, ym.z, yp.z, zm.z, zp.z);
        r3 = resid_cls(g, coef, (cq >> 6) & 3u, i0 + 3, j, k, bq.w, c.w, c.z, xr, ym.w, yp.w, zm.w, zp.w);
    }
    // r at i0-1 (left neighbour's r3) and i0+4 (right neighbour's r0)
    float rl = __shfl_up_sync(0xffffffffu, r3, 1);
    float rh = __shfl_down_sync(0xffffffffu, r0, 1);
    if (!valid) return;
    if (qx == 0) rl = r0;                                   // fine 2I-1 clamps to 2I at I = 0
    else if (lane == 0) rl = resid_scalar(g, x, b, coef, crow, row, rym, ryp, rzm, rzp, i0 - 1, j, k);
    if (2 * qx + 1 >= cnx - 1) rh = r3;                     // fine 2I+2 clamps to 2I+1 at the end
    else if (lane == 31) rh = resid_scalar(g, x, b, coef, crow, row, rym, ryp, rzm, rzp, i0 + 4, j, k);
    float2 out;
    out.x = 0.125f * rl + 0.375f * r0 + 0.375f * r1 + 0.125f * r2;
    out.y = 0.125f * r1 + 0.375f * r2 + 0.375f * r3 + 0.125f * rh;
    *reinterpret_cast<float2 *>(rx + (long long)cnx * (j + (long long)g.d.ny * k) + 2 * qx) = out;
}

// k_resid_rx with whole rows of quads in the block (blockDim.x = nx / 4,
// which divides 256): the residuals at i0 - 1 and i0 + 4 are the row
// neighbours' r3 and r0, exchanged through shared memory, so no lane
// recomputes a residual at a warp's edge
__global__ void __launch_bounds__(256, 5) k_resid_rx_rows(Geo g, const float *__restrict__ x,
                                                       const float *__restrict__ b, const float4 *__restrict__ coef,
                                                       const uint8_t *__restrict__ cls, int cpitch,
                                                       float *__restrict__ rx, const PcgState *st) {
    __shared__ float s_r0[256], s_r3[256];
    pdl_wait();
    if (st && st->stop) return;
    const int nq = g.d.nx >> 2, cnx = g.d.nx >> 1;
    const int qx = threadIdx.x;
    const int jr = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const bool valid = jr < g.d.ny;
    const int j = valid ? jr : g.d.ny - 1;   // rows past the end compute a copy of the last and store nothing
    const int i0 = 4 * qx;
    const long long row = g.sy * j + g.sz * k;
    const long long rym = row + (j > 0 ? -g.sy : 0), ryp = row + (j < g.d.ny - 1 ? g.sy : 0);
    const long long rzm = row + (k > 0 ? -g.sz : 0), rzp = row + (k < g.d.nz - 1 ? g.sz : 0);
    const uint8_t *crow = cls + (long long)cpitch * (j + (long long)g.d.ny * k);
    const float4 c = __ldg(reinterpret_cast<const float4 *>(x + row + i0));
    const float xl = i0 > 0 ? __ldg(x + row + i0 - 1) : c.x;
    const float xr = i0 + 4 < g.d.nx ? __ldg(x + row + i0 + 4) : c.w;
    const float4 ym = __ldg(reinterpret_cast<const float4 *>(x + rym + i0));
    const float4 yp = __ldg(reinterpret_cast<const float4 *>(x + ryp + i0));
    const float4 zm = __ldg(reinterpret_cast<const float4 *>(x + rzm + i0));
    const float4 zp = __ldg(reinterpret_cast<const float4 *>(x + rzp + i0));
    const float4 bq = __ldg(reinterpret_cast<const float4 *>(b + row + i0));
    const unsigned cq = crow[qx];
    float r0, r1, r2, r3;
    if (cq == 0) {
        r0 = bq.x - apply_reg(g, c.x, xl, c.y, ym.x, yp.x, zm.x, zp.x);
        r1 = bq.y - apply_reg(g, c.y, c.x, c.z, ym.y, yp.y, zm.y, zp.y);
        r2 = bq.z - apply_reg(g, c.z, c.y, c.w, ym.z, yp.z, zm.z, zp.z);
        r3 = bq.w - apply_reg(g, c.w, c.z, xr, ym.w, yp.w, zm.w, zp.w);
    } else {
        r0 = resid_cls(g, coef, cq & 3u, i0, j, k, bq.x, c.x, xl, c.y, ym.x, yp.x, zm.x, zp.x);
        r1 = resid_cls(g, coef, (cq >> 2) & 3u, i0 + 1, j, k, bq.y, c.y, c.x, c.z, ym.y, yp.y, zm.y, zp.y);
        r2 = resid_cls(g, coef, (cq >> 4) & 3u, i0 + 2, j, k, bq.z, c.z, c.y, c.w, ym.z, yp.z, zm.z, zp.z);
        r3 = resid_cls(g, coef, (cq >> 6) & 3u, i0 + 3, j, k, bq.w, c.w, c.z, xr, ym.w, yp.w, zm.w, zp.w);
    }
    const int t = threadIdx.y * blockDim.x + qx;
    s_r0[t] = r0;
    s_r3[t] = r3;
    __syncthreads();
    // fine 2I-1 clamps to 2I at I = 0, fine 2I+2 to 2I+1 at the row's end
    const float rl = qx == 0 ? r0 : s_r3[t - 1];
    const float rh = qx == nq - 1 ? r3 : s_r0[t + 1];
    if (!valid) return;
    float2 out;
    out.x = 0.125f * rl + 0.375f * r0 + 0.375f * r1 + 0.125f * r2;
    out.y = 0.125f * r1 + 0.375f * r2 + 0.375f * r3 + 0.125f * rh;
    *reinterpret_cast<float2 *>(rx + (long long)cnx * (j + (long long)g.d.ny * k) + 2 * qx) = out;
}

__global__ void k_restrict_yz(Dims fd, Dims cd, int dims, const float *__restrict__ rx,
                              const uint8_t *__restrict__ cmask, float *__restrict__ cb, const PcgState *st) {
    if (st && st->stop) return;
    const long long n = cd.n();
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const int I = (int)(c % cd.nx);
        const long long rr = c / cd.nx;
        const int J = (int)(rr % cd.ny), K = (int)(rr / cd.ny);
        if (cmask && cmask[c]) {
            cb[c] = 0.0f;
            continue;
        }
        int jy[4], kz[4];
        rtap4(J, cd.ny, jy);
        const float w4[4] = {0.125f, 0.375f, 0.375f, 0.125f};
        int nzt = 4;
        if (dims == 3) rtap4(K, cd.nz, kz);
        else { kz[0] = K; nzt = 1; }
        float s = 0.0f;
        for (int q = 0; q < nzt; ++q) {
            const float wz = dims == 3 ? w4[q] : 1.0f;
            float part = 0.0f;
#pragma unroll
            for (int p = 0; p < 4; ++p)
                part += __ldg(rx + I + (long long)cd.nx * (jy[p] + (long long)fd.ny * kz[q])) * w4[p];
            s += part * wz;
        }
        cb[c] = s;
    }
}

// The y and z taps for four consecutive coarse cells per thread (float4 rows
// of rx and of the coarse b; needs the coarse nx % 4 == 0).  Block (32, 8),
// grid (coarse nx / 128, coarse ny / 8, coarse nz).
__global__ void __launch_bounds__(256) k_restrict_yz4(Dims fd, Dims cd, int dims, const float *__restrict__ rx,
                                                      const uint8_t *__restrict__ cmask, float *__restrict__ cb,
                                                      const PcgState *st) {
    pdl_wait();
    if (st && st->stop) return;
    const int I = 4 * (blockIdx.x * 32 + threadIdx.x), J = blockIdx.y * 8 + threadIdx.y, K = blockIdx.z;
    if (I >= cd.nx || J >= cd.ny) return;
    int jy[4], kz[4];
    rtap4(J, cd.ny, jy);
    const float w4[4] = {0.125f, 0.375f, 0.375f, 0.125f};
    int nzt = 4;
    if (dims == 3) rtap4(K, cd.nz, kz);
    else { kz[0] = K; nzt = 1; }
    float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int q = 0; q < nzt; ++q) {
        const float wz = dims == 3 ? w4[q] : 1.0f;
        float4 part = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const float4 v =
                __ldg(reinterpret_cast<const float4 *>(rx + I + (long long)cd.nx * (jy[p] + (long long)fd.ny * kz[q])));
            part.x += v.x * w4[p];
            part.y += v.y * w4[p];
            part.z += v.z * w4[p];
            part.w += v.w * w4[p];
        }
        s.x += part.x * wz;
        s.y += part.y * wz;
        s.z += part.z * wz;
        s.w += part.w * wz;
    }
    const long long c = I + (long long)cd.nx * (J + (long long)cd.ny * K);
    if (cmask) {
        const uchar4 m = *reinterpret_cast<const uchar4 *>(cmask + c);
        if (m.x) s.x = 0.f;
        if (m.y) s.y = 0.f;
        if (m.z) s.z = 0.f;
        if (m.w) s.w = 0.f;
    }
    *reinterpret_cast<float4 *>(cb + c) = s;
}

// ------------------------------------------------------------ prolongation --
// buildCorrectKernel (multigrid.js:990-1040) on FP32 levels with nx % 4 == 0:
// x_f += P x_c, skipped on fine Dirichlet cells.  A thread owns an x-quad
// of fine cells; along x the quad's four cells take (1/4, 3/4), (3/4, 1/4),
// (1/4, 3/4), (3/4, 1/4) of the coarse cells 2q-1 .. 2q+2 (clamped), along
// y and z the correctionTapsForAxis pair of its row and plane.
__device__ __forceinline__ void ptaps2(int f, int nc, int *idx, float *w) {
    const int ci = f >> 1;
    if ((f & 1) == 0) {
        idx[0] = ci > 0 ? ci - 1 : ci; w[0] = 0.25f;
        idx[1] = ci; w[1] = 0.75f;
    } else {
        idx[0] = ci; w[0] = 0.75f;
        idx[1] = ci < nc - 1 ? ci + 1 : ci; w[1] = 0.25f;
    }
}

// Block (32, 8), grid (quads / 32, rows / 8, planes / PL): one quad per
// thread on PL consecutive planes (2 in 3D: the planes 2c and 2c + 1 share
// the coarse plane c, and each thread keeps two quads' loads in flight).
template <int PL>
__global__ void __launch_bounds__(256) k_prolong4(Dims fd, Dims cd, int dims, const float *__restrict__ coarse,
                                                  const uint8_t *__restrict__ fmask, float *__restrict__ fine,
                                                  const PcgState *st) {
    pdl_wait();
    if (st && st->stop) return;
    const int nq = fd.nx >> 2;
    const int qx = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    if (qx >= nq || j >= fd.ny) return;
    const int c1 = 2 * qx, c2 = 2 * qx + 1;
    const int c0 = c1 > 0 ? c1 - 1 : c1, c3 = c2 < cd.nx - 1 ? c2 + 1 : c2;
    int jj[2];
    float wj[2];
    ptaps2(j, cd.ny, jj, wj);
    float4 x[PL];
    uchar4 m[PL];
    float a[PL][4];
#pragma unroll
    for (int p = 0; p < PL; ++p) {
        const int k = blockIdx.z * PL + p;
        const long long f0 = 4LL * (qx + (long long)nq * (j + (long long)fd.ny * k));
        x[p] = *reinterpret_cast<const float4 *>(fine + f0);
        m[p] = fmask ? *reinterpret_cast<const uchar4 *>(fmask + f0) : make_uchar4(0, 0, 0, 0);
    }
#pragma unroll
    for (int p = 0; p < PL; ++p) {
        const int k = blockIdx.z * PL + p;
        int kk[2];
        float wk[2];
        int nk = 2;
        if (dims == 3) ptaps2(k, cd.nz, kk, wk);
        else { kk[0] = 0; wk[0] = 1.f; nk = 1; }
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
        for (int b = 0; b < 2; ++b)
            for (int g = 0; g < nk; ++g) {
                const float *row = coarse + (long long)cd.nx * (jj[b] + (long long)cd.ny * kk[g]);
                const float w = wj[b] * wk[g];
                const float v0 = __ldg(row + c0), v1 = __ldg(row + c1), v2 = __ldg(row + c2), v3 = __ldg(row + c3);
                a0 += (0.25f * v0 + 0.75f * v1) * w;
                a1 += (0.75f * v1 + 0.25f * v2) * w;
                a2 += (0.25f * v1 + 0.75f * v2) * w;
                a3 += (0.75f * v2 + 0.25f * v3) * w;
            }
        a[p][0] = a0;
        a[p][1] = a1;
        a[p][2] = a2;
        a[p][3] = a3;
    }
#pragma unroll
    for (int p = 0; p < PL; ++p) {
        const int k = blockIdx.z * PL + p;
        const long long f0 = 4LL * (qx + (long long)nq * (j + (long long)fd.ny * k));
        float4 v = x[p];
        if (!m[p].x) v.x += a[p][0];
        if (!m[p].y) v.y += a[p][1];
        if (!m[p].z) v.z += a[p][2];
        if (!m[p].w) v.w += a[p][3];
        *reinterpret_cast<float4 *>(fine + f0) = v;
    }
}

// ------------------------------------------------- coarse-level V-cycle --
// The V-cycle below a level (its pre-smoothing, residual and restriction,
// every coarser level, the direct coarsest solve, the prolongations and the
// post-smoothing) in one cooperative launch: phases over all cells of one
// level separated by grid-wide barriers.  Tail levels hold at most 2^18
// cells (the host picks them so), so cell indices are 32-bit.  The coarse levels are too small
// to fill the GPU, so one launch per sweep would cost more in launch and
// pipeline latency than in work.  Colour passes run in place (a colour
// reads only the other colour); the first pass on a level writes every cell,
// the level starting from x = 0.  Values written inside the launch are read
// through L2 (ld.global.cg), never from a possibly stale L1 line.  Per cell the arithmetic is that of the
// level kernels: the TMA sweep's relaxation by class, k_resid_rx's residual
// and x-taps followed by k_restrict_yz's y and z taps, k_coarse_direct's
// row products, k_prolong4's correction.
constexpr int TAIL_MAXL = 8;
constexpr int TAIL_NT = 1024;
// Levels up to this many cells run in one block (measured: a 64 x 64 level
// gains, a 16^3 level, with its 64-tap restriction and 7-point colours,
// loses against the grid barriers it saves).
constexpr int TAIL_ONE_BLOCK_2D = 8192;
constexpr int TAIL_ONE_BLOCK_3D = 512;
// the coarsest level's sweeps (7-point colours, no restriction) in 2D and 3D
constexpr int TAIL_ONE_BLOCK_COARSE = 8192;
struct TailLevel {
    Geo g;
    float *x, *b, *r;              // r: residual scratch of the level
    // block-0 levels held in shared memory: offset (floats) of the level's
    // x, b and r there (n floats each), -1 for a level in global memory
    int smo;
    // t / hx, t / nx and t / ny as (t m) >> 40 with m = ceil(2^40 / divisor)
    // (exact for every t below 2^22 and divisor below 2^18)
    unsigned long long mhx, mnx, mny;
    const float4 *coef, *gco;
    const uint8_t *cls, *mask;     // class bytes (cpitch bytes per row), Dirichlet mask (may be null)
    int cpitch;
    float rdreg_sor;               // sor / dreg
};
struct TailArgs {
    TailLevel lv[TAIL_MAXL];
    int nl;                        // levels, the last one the coarsest
    int down, up, dims;
    float sor, omsor;
    const double *G;               // coarsest inverse, nG x nG, row-major (direct mode)
    int nG;
    int coarse_sweeps;             // > 0: that many sweeps on the coarsest level instead of G b
    PcgState *st;                  // may be null
    unsigned *bar;                 // grid barrier: arrivals, generation, abort
    int cxo;                       // the coarsest x's copy in shared memory (floats; -1: none)
};

// Grid-wide barrier of the cooperative launch over three words: a count of
// arrivals that only grows within a launch (barrier k completes when it
// reaches k x blocks), the number of blocks done with the launch (the last
// one clears both counts, once no block polls them), and an abort flag.  A
// block that waits more than 0.5 s raises the abort flag, which releases
// every waiting block; all then return false.
__device__ bool tail_sync(unsigned *bar, unsigned &passed) {
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned *vb = bar;
        if (vb[2]) {
            ok = 0;
        } else {
            const unsigned target = (passed + 1) * gridDim.x;
            __threadfence();
            atomicAdd(&bar[0], 1u);
            const unsigned long long t0 = globaltimer_ns();
            while (vb[0] < target) {
                if (vb[2]) { ok = 0; break; }
                if (globaltimer_ns() - t0 > 500000000ull) {
                    atomicExch(&bar[2], 1u);
                    ok = 0;
                    break;
                }
            }
            __threadfence();
        }
        ok_s = ok;
    }
    __syncthreads();
    ++passed;
    return ok_s != 0;
}

// after a block's last barrier: the last block to get here clears the counts
__device__ void tail_done(unsigned *bar) {
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&bar[1], 1u) == gridDim.x - 1) {
            atomicExch(&bar[0], 0u);
            atomicExch(&bar[1], 0u);
        }
    }
}

__device__ __forceinline__ unsigned tail_class(const TailLevel &L, int i, int j, int k) {
    return (__ldg(L.cls + L.cpitch * (j + L.g.d.ny * k) + (i >> 2)) >> (2 * (i & 3))) & 3u;
}

// the relaxation of one cell by class (the TMA sweep's arithmetic)
__device__ __forceinline__ float tail_relax(const TailArgs &a, const TailLevel &L, unsigned cl, long long c, int i,
                                           int j, int k, float vc, float xm, float xp, float ym, float yp, float zm,
                                           float zp, float bval) {
    const Geo &g = L.g;
    if (!(cl & 1u)) {
        const float corr = g.h2x * (float)((i == 0) + (i == g.d.nx - 1)) +
                           g.h2y * (float)((j == 0) + (j == g.d.ny - 1)) +
                           g.h2z * (float)((k == 0) + (k == g.d.nz - 1));
        const float rd = corr == 0.f ? L.rdreg_sor : a.sor / (g.dreg + corr);
        return relax_plain(g, a.omsor, vc, xm, xp, ym, yp, zm, zp, bval, rd);
    }
    if (cl == 1u) return __fmaf_rn(bval, -a.sor, a.omsor * vc);
    const float4 lo = __ldg(L.coef + c), hi = __ldg(L.gco + c);
    float s = lo.x * xm;
    s = __fmaf_rn(hi.x, xp, s);
    s = __fmaf_rn(lo.y, ym, s);
    s = __fmaf_rn(hi.y, yp, s);
    s = __fmaf_rn(lo.z, zm, s);
    s = __fmaf_rn(hi.z, zp, s);
    return __fmaf_rn(bval - s, a.sor * hi.w, a.omsor * vc);
}

// A 2D level of at most TAIL_SMEM_CELLS cells (and every coarser one but the
// coarsest) lives in block 0's shared memory while the launch runs: block 0
// alone runs its phases, so they need no grid barrier and no L2 round
// trip.  Its b arrives there by the restriction into it (or, for the
// launch's first level, by a copy from global memory) and its x leaves for
// global memory after its last pass when the next finer level is a
// grid-wide one.  SM: the level's arrays are there (plain loads); otherwise
// loads bypass L1, which other blocks' writes in this launch leave stale.
constexpr int TAIL_SMEM_CELLS = 8192;
constexpr int TAIL_SMEM_BYTES = 3 * 4 * 8192 + 3 * 4 * 1024;   // 3 arrays of a 8192- and a 1024-cell level
__device__ __forceinline__ int tdiv(int t, unsigned long long m) {
    return (int)(((unsigned long long)(unsigned)t * m) >> 40);
}
template <bool SM>
__device__ __forceinline__ float tld(const float *p) {
    if constexpr (SM) return *p;
    else return __ldcg(p);
}
struct TailArr {
    float *x, *b, *r;
};
template <bool SM>
__device__ __forceinline__ TailArr tail_arrays(const TailLevel &L) {
    if constexpr (SM) {
        extern __shared__ __align__(16) float tail_sm[];
        const int n = (int)L.g.d.n();
        float *x = tail_sm + L.smo;
        return TailArr{x, x + n, x + 2 * n};
    } else {
        return TailArr{L.x, L.b, L.r};
    }
}

// one colour pass (colour col = (i + j + k) & 1) in place, one thread per
// cell of the colour (nx is even: nx / 2 of them per row); `first`: x is 0
// on entry and the thread also writes 0 to the row neighbour of the other
// colour
template <bool SM>
__device__ void tail_colour(const TailArgs &a, const TailLevel &L, int col, bool first, long long t0,
                            long long stride) {
    const Geo &g = L.g;
    const int nx = g.d.nx, ny = g.d.ny, nz = g.d.nz, hx = nx >> 1;
    const int n = hx * ny * nz;
    const TailArr A = tail_arrays<SM>(L);
    float *x = A.x;
    for (int t = (int)t0; t < n; t += (int)stride) {
        const int rr = tdiv(t, L.mhx);
        const int m = t - rr * hx;
        const int k = tdiv(rr, L.mny);
        const int j = rr - k * ny;
        const int par = (j + k + col) & 1;
        const int i = 2 * m + par;
        const int c = i + (int)g.sy * j + (int)g.sz * k;
        float vc = 0.f, xm = 0.f, xp = 0.f, ym = 0.f, yp = 0.f, zm = 0.f, zp = 0.f;
        if (first) {
            x[c + (par ? -1 : 1)] = 0.f;
        } else {
            vc = tld<SM>(x + c);
            if (i > 0) xm = tld<SM>(x + c - 1);
            if (i < nx - 1) xp = tld<SM>(x + c + 1);
            if (j > 0) ym = tld<SM>(x + c - g.sy);
            if (j < ny - 1) yp = tld<SM>(x + c + g.sy);
            if (k > 0) zm = tld<SM>(x + c - g.sz);
            if (k < nz - 1) zp = tld<SM>(x + c + g.sz);
        }
        x[c] = tail_relax(a, L, tail_class(L, i, j, k), c, i, j, k, vc, xm, xp, ym, yp, zm, zp, tld<SM>(A.b + c));
    }
}

// r = b - A x (0 on Dirichlet cells); xzero: x is taken as 0 and cleared
template <bool SM>
__device__ void tail_residual(const TailLevel &L, bool xzero, long long t0, long long stride) {
    const Geo &g = L.g;
    const int nx = g.d.nx, ny = g.d.ny, nz = g.d.nz;
    const int n = nx * ny * nz;
    const TailArr A = tail_arrays<SM>(L);
    const float *x = A.x;
    for (int c = (int)t0; c < n; c += (int)stride) {
        const int rr = tdiv(c, L.mnx);
        const int i = c - rr * nx;
        const int k = tdiv(rr, L.mny);
        const int j = rr - k * ny;
        const unsigned cl = tail_class(L, i, j, k);
        if (xzero) {
            A.r[c] = cl == 1u ? 0.f : tld<SM>(A.b + c);
            A.x[c] = 0.f;
            continue;
        }
        const float vc = tld<SM>(x + c);
        const float xm = i > 0 ? tld<SM>(x + c - 1) : vc, xp = i < nx - 1 ? tld<SM>(x + c + 1) : vc;
        const float ym = j > 0 ? tld<SM>(x + c - g.sy) : vc, yp = j < ny - 1 ? tld<SM>(x + c + g.sy) : vc;
        const float zm = k > 0 ? tld<SM>(x + c - g.sz) : vc, zp = k < nz - 1 ? tld<SM>(x + c + g.sz) : vc;
        A.r[c] = resid_cls(g, L.coef, cl, i, j, k, tld<SM>(A.b + c), vc, xm, xp, ym, yp, zm, zp);
    }
}

// coarse b = R r (the 1/8, 3/8, 3/8, 1/8 taps per axis), 0 on coarse
// Dirichlet cells; relax0: also the coarse level's first colour-0 pass
// (from x = 0 a cell needs only its own b; colour-1 cells get 0)
template <bool FSM, bool CSM>
__device__ void tail_restrict(const TailArgs &a, const TailLevel &F, const TailLevel &C, bool relax0, long long t0,
                              long long stride) {
    const Dims fd = F.g.d, cd = C.g.d;
    const TailArr FA = tail_arrays<FSM>(F), CA = tail_arrays<CSM>(C);
    const int n = cd.nx * cd.ny * cd.nz;
    const float w4[4] = {0.125f, 0.375f, 0.375f, 0.125f};
    for (int c = (int)t0; c < n; c += (int)stride) {
        const int rr = tdiv(c, C.mnx);
        const int I = c - rr * cd.nx;
        const int K = tdiv(rr, C.mny);
        const int J = rr - K * cd.ny;
        if (C.mask && __ldg(C.mask + c)) {
            CA.b[c] = 0.f;
            if (relax0)
                CA.x[c] = ((I + J + K) & 1) ? 0.f
                                           : tail_relax(a, C, tail_class(C, I, J, K), c, I, J, K, 0.f, 0.f, 0.f, 0.f,
                                                        0.f, 0.f, 0.f, 0.f);
            continue;
        }
        int ix[4], jy[4], kz[4];
        rtap4(I, cd.nx, ix);
        rtap4(J, cd.ny, jy);
        int nzt = 4;
        if (a.dims == 3) rtap4(K, cd.nz, kz);
        else { kz[0] = K; nzt = 1; }
        float s = 0.f;
        for (int q = 0; q < nzt; ++q) {
            const float wz = a.dims == 3 ? w4[q] : 1.0f;
            float part = 0.f;
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const float *row = FA.r + fd.nx * (jy[p] + fd.ny * kz[q]);
                const float rx = 0.125f * tld<FSM>(row + ix[0]) + 0.375f * tld<FSM>(row + ix[1]) +
                                 0.375f * tld<FSM>(row + ix[2]) + 0.125f * tld<FSM>(row + ix[3]);
                part += rx * w4[p];
            }
            s += part * wz;
        }
        CA.b[c] = s;
        if (relax0)
            CA.x[c] = ((I + J + K) & 1) ? 0.f
                                       : tail_relax(a, C, tail_class(C, I, J, K), c, I, J, K, 0.f, 0.f, 0.f, 0.f, 0.f,
                                                    0.f, 0.f, s);
    }
}

// coarsest x = G b, one warp per row (FP64)
__device__ void tail_direct(const TailArgs &a, const TailLevel &C) {
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (long long row = warp; row < a.nG; row += nwarps) {
        const double *gr = a.G + row * a.nG;
        double s = 0.0;
        for (int j = lane; j < a.nG; j += 32) s += __ldg(gr + j) * (double)__ldcg(C.b + j);
        s = warp_sum(s);
        if (lane == 0) C.x[row] = (float)s;
    }
}

// fine x += P coarse x, skipped on fine Dirichlet cells
template <bool CSM, bool FSM>
__device__ void tail_prolong(const TailArgs &a, const TailLevel &C, const TailLevel &F, long long t0,
                             long long stride) {
    const Dims fd = F.g.d, cd = C.g.d;
    const TailArr CA = tail_arrays<CSM>(C), FA = tail_arrays<FSM>(F);
    const int n = fd.nx * fd.ny * fd.nz;
    for (int c = (int)t0; c < n; c += (int)stride) {
        if (F.mask && __ldg(F.mask + c)) continue;
        const int rr = tdiv(c, F.mnx);
        const int i = c - rr * fd.nx;
        const int k = tdiv(rr, F.mny);
        const int j = rr - k * fd.ny;
        int ii[2], jj[2], kk[2];
        float wi[2], wj[2], wk[2];
        ptaps2(i, cd.nx, ii, wi);
        ptaps2(j, cd.ny, jj, wj);
        int nk = 2;
        if (a.dims == 3) ptaps2(k, cd.nz, kk, wk);
        else { kk[0] = 0; wk[0] = 1.f; nk = 1; }
        float acc = 0.f;
        for (int b = 0; b < 2; ++b)
            for (int q = 0; q < nk; ++q) {
                const float *row = CA.x + cd.nx * (jj[b] + cd.ny * kk[q]);
                const float w = wj[b] * wk[q];
                acc += (wi[0] * tld<CSM>(row + ii[0]) + wi[1] * tld<CSM>(row + ii[1])) * w;
            }
        FA.x[c] = tld<FSM>(FA.x + c) + acc;
    }
}

// one colour pass on the coarsest level from the stored coefficients
// (k_coarse_sweeps' arithmetic: x += sor (b - A x) / diag)
__device__ void tail_coarse_colour(const TailArgs &a, const TailLevel &C, int col, long long t0, long long stride) {
    const Dims d = C.g.d;
    const int sy = d.nx, sz = d.nx * d.ny, n = (int)d.n();
    float *x = C.x;
    for (int c = (int)t0; c < n; c += (int)stride) {
        const int rr = tdiv(c, C.mnx);
        const int i = c - rr * d.nx;
        const int k = tdiv(rr, C.mny);
        const int j = rr - k * d.ny;
        if (((i + j + k) & 1) != col) continue;
        const float xc = __ldcg(x + c);
        const float4 kc = __ldg(C.coef + c);
        float s = -kc.w * xc;
        float D = -(kc.w + kc.x + kc.y + kc.z);
        if (i > 0) s += kc.x * (__ldcg(x + c - 1) - xc);
        if (i < d.nx - 1) { const float k1 = __ldg(&C.coef[c + 1].x); s += k1 * (__ldcg(x + c + 1) - xc); D -= k1; }
        if (j > 0) s += kc.y * (__ldcg(x + c - sy) - xc);
        if (j < d.ny - 1) { const float k1 = __ldg(&C.coef[c + sy].y); s += k1 * (__ldcg(x + c + sy) - xc); D -= k1; }
        if (k > 0) s += kc.z * (__ldcg(x + c - sz) - xc);
        if (k < d.nz - 1) { const float k1 = __ldg(&C.coef[c + sz].z); s += k1 * (__ldcg(x + c + sz) - xc); D -= k1; }
        x[c] = xc + ((__ldcg(C.b + c) - s) / D) * a.sor;
    }
}

// HELD: some levels are held in block 0's shared memory (the instance
// without them carries none of their dispatch)
template <bool HELD>
__global__ void __launch_bounds__(TAIL_NT, 1) k_vcycle_tail(TailArgs a) {
    PcgState *st = a.st;
    if (st && (st->stop || st->err)) return;
    unsigned *bar = a.bar;
    unsigned passed = 0;
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    // A phase over a level of at most one_block cells, or held in block 0's
    // shared memory, runs in block 0 alone, with a block barrier after it; a
    // phase over a larger level runs on every block with a grid barrier
    // after it, and one more grid barrier first when block-0 phases precede
    // it.  Every block takes the same sequence of grid barriers (the choice
    // depends only on level sizes).
    bool solo_prev = false;
    const int one_block = a.dims == 3 ? TAIL_ONE_BLOCK_3D : TAIL_ONE_BLOCK_2D;
    auto held = [&](int l) { return HELD && a.lv[l].smo >= 0; };
    auto small = [&](int l) { return held(l) || a.lv[l].g.d.n() <= one_block; };
    auto phase = [&](bool solo, bool sync_after, auto &&work) -> bool {
        if (solo) {
            if (blockIdx.x == 0) {
                work((long long)threadIdx.x, (long long)blockDim.x);
                __syncthreads();
            }
            solo_prev = true;
            return true;
        }
        if (solo_prev) {
            solo_prev = false;
            if (!tail_sync(bar, passed)) return false;
        }
        work(t0, stride);
        return sync_after ? tail_sync(bar, passed) : true;
    };
    // a held level's x to global memory, or its b and x from there (block 0)
    auto copy_x_out = [&](int l) {
        if constexpr (!HELD) return;
        const TailArr A = tail_arrays<true>(a.lv[l]);
        const int n = (int)a.lv[l].g.d.n();
        for (int c = threadIdx.x; c < n; c += blockDim.x) a.lv[l].x[c] = A.x[c];
    };
    auto copy_in = [&](int l) {
        if constexpr (!HELD) return;
        const TailArr A = tail_arrays<true>(a.lv[l]);
        const int n = (int)a.lv[l].g.d.n();
        for (int c = threadIdx.x; c < n; c += blockDim.x) {
            A.b[c] = __ldcg(a.lv[l].b + c);
            A.x[c] = __ldcg(a.lv[l].x + c);
        }
    };
    bool ok = true;
    if (held(0))
        ok = phase(true, true, [&](long long q0, long long qs) {
            const TailArr A = tail_arrays<true>(a.lv[0]);
            for (long long c = q0; c < a.lv[0].g.d.n(); c += qs) A.b[c] = __ldcg(a.lv[0].b + c);
        });
    // the coarse level's first colour-0 pass rides on the restriction into it
    // (not into the coarsest level, which is solved directly or swept)
    for (int l = 0; l < a.nl - 1 && ok; ++l) {
        const TailLevel &L = a.lv[l];
        const bool fused0 = l > 0 && a.down > 0, sl = small(l), hl = held(l);
        for (int it = 0; it < a.down && ok; ++it) {
            if (!(fused0 && it == 0))
                ok = phase(sl, true, [&](long long q0, long long qs) {
                    if (hl) tail_colour<true>(a, L, 0, it == 0, q0, qs);
                    else tail_colour<false>(a, L, 0, it == 0, q0, qs);
                });
            if (ok) ok = phase(sl, true, [&](long long q0, long long qs) {
                if (hl) tail_colour<true>(a, L, 1, false, q0, qs);
                else tail_colour<false>(a, L, 1, false, q0, qs);
            });
        }
        if (!ok) break;
        ok = phase(sl, true, [&](long long q0, long long qs) {
            if (hl) tail_residual<true>(L, a.down == 0, q0, qs);
            else tail_residual<false>(L, a.down == 0, q0, qs);
        });
        if (!ok) break;
        // the restriction runs over the coarse level's cells; into a held
        // level from a grid-wide one it runs grid-wide into the level's global
        // arrays, which block 0 then takes into shared memory
        const bool relax0 = l + 1 < a.nl - 1 && a.down > 0, hc = held(l + 1);
        if (!HELD) {
            ok = phase(small(l + 1), true, [&](long long q0, long long qs) {
                tail_restrict<false, false>(a, L, a.lv[l + 1], relax0, q0, qs);
            });
        } else if (hc && !hl) {
            ok = phase(false, true, [&](long long q0, long long qs) {
                tail_restrict<false, false>(a, L, a.lv[l + 1], relax0, q0, qs);
            });
            if (ok) ok = phase(true, true, [&](long long, long long) { copy_in(l + 1); });
        } else {
            ok = phase(small(l + 1), true, [&](long long q0, long long qs) {
                if (hl && hc) tail_restrict<true, true>(a, L, a.lv[l + 1], relax0, q0, qs);
                else if (hl) tail_restrict<true, false>(a, L, a.lv[l + 1], relax0, q0, qs);
                else tail_restrict<false, false>(a, L, a.lv[l + 1], relax0, q0, qs);
            });
        }
    }
    if (ok) {
        const TailLevel &C = a.lv[a.nl - 1];
        if (a.coarse_sweeps > 0) {
            const bool sc = a.lv[a.nl - 1].g.d.n() <= TAIL_ONE_BLOCK_COARSE;
            ok = phase(sc, true, [&](long long q0, long long qs) {
                for (long long c = q0; c < C.g.d.n(); c += qs) C.x[c] = 0.f;
            });
            for (int it = 0; it < a.coarse_sweeps && ok; ++it)
                for (int col = 0; col < 2 && ok; ++col)
                    ok = phase(sc, true, [&](long long q0, long long qs) { tail_coarse_colour(a, C, col, q0, qs); });
        } else {
            // G b as one FP64 matvec over every block's warps
            ok = phase(false, true, [&](long long, long long) { tail_direct(a, C); });
        }
    }
    for (int l = a.nl - 2; l >= 0 && ok; --l) {
        const TailLevel &L = a.lv[l];
        const bool sl = small(l), hl = held(l);
        // a held coarse level is read from shared memory only by a held fine
        // level's phase (block 0); a grid-wide phase reads its global copy
        const bool hc = hl && held(l + 1);
        const bool out = hl && (l == 0 || !held(l - 1));
        ok = phase(sl, true, [&](long long q0, long long qs) {
            if (hl && hc) {
                tail_prolong<true, true>(a, a.lv[l + 1], L, q0, qs);
            } else if (hl && l + 1 == a.nl - 1 && a.cxo >= 0) {
                // the coarsest x (global, written grid-wide) into shared memory first
                extern __shared__ __align__(16) float tail_sm[];
                const TailLevel &C = a.lv[l + 1];
                for (long long c = q0; c < C.g.d.n(); c += qs) tail_sm[a.cxo + c] = __ldcg(C.x + c);
                __syncthreads();
                TailLevel Cs = C;
                Cs.smo = a.cxo;
                tail_prolong<true, true>(a, Cs, L, q0, qs);
            } else if (hl) {
                tail_prolong<false, true>(a, a.lv[l + 1], L, q0, qs);
            } else {
                tail_prolong<false, false>(a, a.lv[l + 1], L, q0, qs);
            }
            if (out && a.up == 0) {
                __syncthreads();
                copy_x_out(l);
            }
        });
        for (int it = 0; it < a.up && ok; ++it) {
            ok = phase(sl, true, [&](long long q0, long long qs) {
                if (hl) tail_colour<true>(a, L, 1, false, q0, qs);
                else tail_colour<false>(a, L, 1, false, q0, qs);
            });
            // the kernel's end orders the last pass before the next launch
            if (ok) ok = phase(sl, !(l == 0 && it == a.up - 1), [&](long long q0, long long qs) {
                if (hl) tail_colour<true>(a, L, 0, false, q0, qs);
                else tail_colour<false>(a, L, 0, false, q0, qs);
                if (out && it == a.up - 1) {
                    __syncthreads();
                    copy_x_out(l);
                }
            });
        }
    }
    if (ok) tail_done(bar);
    else if (threadIdx.x == 0 && st) atomicOr(&st->err, 2);
}

// ----------------------------------------------------------- cell classes --
// Two bits per cell, one byte per x-quad (rows `pitch` bytes apart): 0 an
// interior cell whose six couplings are the plain h^-2 and E = 0; 1 a
// Dirichlet cell (E = 1, no coupling); 2 a domain-edge cell with the plain
// couplings (zero across the edge); 3 anything else, which also stores gco =
// (upper x, y, z couplings, 1 / diagonal).
//
// The level's coefficients (k_build_coef's formulas, from the weights and
// the Dirichlet mask) and its classes in one pass: the upper couplings a
// class needs are the lower couplings of the next cells, computed here from
// the same faces instead of read back from the coefficient array.
__global__ void k_coef_classes(Geo g, int dims, const float *__restrict__ wu, const float *__restrict__ wv,
                               const float *__restrict__ ww, const uint8_t *__restrict__ mask, float hx2, float hy2,
                               float hz2, float4 *__restrict__ coef, uint2 *__restrict__ coef16,
                               uint8_t *__restrict__ cls, int pitch, float4 *__restrict__ gco) {
    // one thread per cell (coalesced coefficient stores); the four lanes of
    // an x-quad (nx % 4 == 0, blockDim.x a multiple of 32) merge their
    // classes into the quad's byte with shuffles
    const Dims d = g.d;
    const int ir = blockIdx.x * blockDim.x + threadIdx.x;
    const int jr = blockIdx.y * blockDim.y + threadIdx.y, k = blockIdx.z;
    const bool in = ir < d.nx && jr < d.ny;   // whole quads are in or out
    const int i = in ? ir : 0, j = in ? jr : 0;
    auto W = [](const float *w, long long f) { return w ? w[f] : 1.f; };
    auto P = [&](long long n) { return mask ? mask[n] != 0 : false; };
    const long long c = i + g.sy * j + g.sz * k;
    const long long fu = i + (long long)(d.nx + 1) * (j + (long long)d.ny * k);
    const long long fv = i + (long long)d.nx * (j + (long long)(d.ny + 1) * k);
    const bool pc = P(c);
    float kx = 0.f, ky = 0.f, kz = 0.f, e = 0.f;
    if (i > 0) { if (!pc && !P(c - 1)) kx = W(wu, fu) * hx2; else if (!pc) e += W(wu, fu) * hx2; }
    if (i < d.nx - 1 && !pc && P(c + 1)) e += W(wu, fu + 1) * hx2;
    if (j > 0) { if (!pc && !P(c - g.sy)) ky = W(wv, fv) * hy2; else if (!pc) e += W(wv, fv) * hy2; }
    if (j < d.ny - 1 && !pc && P(c + g.sy)) e += W(wv, fv + d.nx) * hy2;
    if (dims == 3) {
        if (k > 0) { if (!pc && !P(c - g.sz)) kz = W(ww, c) * hz2; else if (!pc) e += W(ww, c) * hz2; }
        if (k < d.nz - 1 && !pc && P(c + g.sz)) e += W(ww, c + g.sz) * hz2;
    }
    if (pc) e = 1.f;
    // the next cells' lower couplings (their k_build_coef x, y, z)
    const float ux = (i < d.nx - 1 && !P(c + 1) && !pc) ? W(wu, fu + 1) * hx2 : 0.f;
    const float uy = (j < d.ny - 1 && !P(c + g.sy) && !pc) ? W(wv, fv + d.nx) * hy2 : 0.f;
    const float uz = (dims == 3 && k < d.nz - 1 && !P(c + g.sz) && !pc) ? W(ww, c + g.sz) * hz2 : 0.f;
    const bool plain = kx == (i > 0 ? g.h2x : 0.f) && ux == (i < d.nx - 1 ? g.h2x : 0.f) &&
                       ky == (j > 0 ? g.h2y : 0.f) && uy == (j < d.ny - 1 ? g.h2y : 0.f) &&
                       kz == (k > 0 ? g.h2z : 0.f) && uz == (k < d.nz - 1 ? g.h2z : 0.f) && e == 0.f;
    const bool pinned = e == 1.f && kx == 0.f && ky == 0.f && kz == 0.f && ux == 0.f && uy == 0.f && uz == 0.f;
    const bool inner = i > 0 && i < d.nx - 1 && j > 0 && j < d.ny - 1 && k > 0 && k < d.nz - 1;
    const unsigned cl = plain ? (inner ? 0u : 2u) : (pinned ? 1u : 3u);
    unsigned byte = cl << (2 * (ir & 3));
    byte |= __shfl_xor_sync(0xffffffffu, byte, 1);
    byte |= __shfl_xor_sync(0xffffffffu, byte, 2);
    if (!in) return;
    coef[c] = make_float4(kx, ky, kz, e);
    if (coef16) {
        auto b16 = [](float v) { return (unsigned)__bfloat16_as_ushort(__float2bfloat16_rn(v)); };
        coef16[c] = make_uint2(b16(kx) | (b16(ky) << 16), b16(kz) | (b16(e) << 16));
    }
    if (cl == 3u) {
        const float diag = -(e + kx + ux + ky + uy + kz + uz);
        gco[c] = make_float4(ux, uy, uz, 1.f / diag);
    }
    if ((i & 3) == 0) cls[(i >> 2) + (long long)pitch * (j + (long long)d.ny * k)] = (uint8_t)byte;
}

// Brick flags from the classes: a brick is regular when every cell of it,
// extended by two cells on each side, is of class 0 or 2.  A plain class
// also checks the cell's upper couplings, so this marks a subset of the
// bricks the coefficient test (k_brick_flags) marks: every brick flagged
// regular here is regular by that test too.
__global__ void k_brick_flags_cls(Geo g, const uint8_t *__restrict__ cls, int pitch, uint8_t *bricks) {
    const int bx = blockIdx.x, by = blockIdx.y, bz = blockIdx.z;
    const int ia = max(0, bx * TX - 2), ib = min(g.d.nx, bx * TX + TX + 2);
    const int ja = max(0, by * TY - 2), jb = min(g.d.ny, by * TY + TY + 2);
    const int ka = max(0, bz * BZ - 2), kb = min(g.d.nz, bz * BZ + BZ + 2);
    // whole class bytes (x-quads) covering [ia, ib), cells outside masked off
    const int qa = ia >> 2, qb = (ib - 1) >> 2;
    const int wq = qb - qa + 1, hgt = jb - ja, dep = kb - ka;
    const int total = wq * hgt * dep;
    int ok = 1;
    for (int t = threadIdx.x; t < total && ok; t += blockDim.x) {
        const int q = qa + t % wq, r = t / wq, j = ja + r % hgt, k = ka + r / hgt;
        unsigned m = 0;
#pragma unroll
        for (int dd = 0; dd < 4; ++dd) {
            const int i = 4 * q + dd;
            if (i >= ia && i < ib) m |= 1u << (2 * dd);   // the odd classes (1, 3) have the low bit set
        }
        if (cls[(long long)pitch * (j + (long long)g.d.ny * k) + q] & m) ok = 0;
    }
    ok = __syncthreads_and(ok);
    if (threadIdx.x == 0) bricks[bx + (long long)g.bnx * (by + (long long)g.bny * bz)] = (uint8_t)ok;
}

// ------------------------------------------------------- sweep work order --
// The TMA sweep's work items (tile columns x z-chunks) in launch order: the
// items whose bricks hold a non-plain cell (solid faces, Dirichlet cells)
// first, then the rest, each group by item index (a stable partition, so
// the order is deterministic).  One block of 1024 threads; each thread
// takes a contiguous run of at most 32 items.
__global__ void __launch_bounds__(1024) k_sweep_order(Geo g, const uint8_t *__restrict__ bricks, int gx, int gy,
                                                      int gz, int zc, int tby, int *order) {
    __shared__ int wsum[32];
    __shared__ int total;
    const int n = gx * gy * gz;
    const int per = (n + (int)blockDim.x - 1) / (int)blockDim.x;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int lo = min(n, t * per), hi = min(n, lo + per);
    unsigned mask = 0;
    int cnt = 0;
    for (int it = lo; it < hi; ++it) {
        bool heavy = false;
        if (bricks) {
            const int tx = it % gx, ty = (it / gx) % gy, tz = it / (gx * gy);
            const int k0 = tz * zc, k1 = min(k0 + zc, g.d.nz);
            const int bz0 = max(0, k0 - 1) / BZ, bz1 = min(g.d.nz - 1, k1) / BZ;
            const int bx1 = min(2 * tx + 2, g.bnx), by1 = min(tby * ty + tby, g.bny);
            for (int bz = bz0; bz <= bz1 && !heavy; ++bz)
                for (int by = tby * ty; by < by1 && !heavy; ++by)
                    for (int bx = 2 * tx; bx < bx1 && !heavy; ++bx)
                        heavy = bricks[bx + (long long)g.bnx * (by + (long long)g.bny * bz)] == 0;
        }
        if (heavy) {
            mask |= 1u << (it - lo);
            ++cnt;
        }
    }
    // exclusive scan of the heavy counts over the threads
    int inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int nw = (int)blockDim.x >> 5;
        int w = lane < nw ? wsum[lane] : 0;
        int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += v;
        }
        if (lane < nw) wsum[lane] = wi - w;
        if (lane == 31) total = wi;
    }
    __syncthreads();
    int hpos = wsum[warp] + inc - cnt;       // heavy items before this thread's run
    int lpos = total + (lo - hpos);          // light items go after all heavy ones
    for (int it = lo; it < hi; ++it) {
        if ((mask >> (it - lo)) & 1u) order[hpos++] = it;
        else order[lpos++] = it;
    }
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

// launch with programmatic stream serialization (the kernel calls pdl_wait
// before touching memory)
template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

int res_restrict2(const Level &f, const SweepMaps &m, const float *x, float *rx, Level &c, int dims,
                  const PcgState *st, cudaStream_t s) {
    FF_CHECK(m.ok && m.cls_ptr && f.d.nx % 4 == 0, FF_E_STATE, "res_restrict2 needs cell classes and nx %% 4 == 0");
    Geo g = make_geo(f);
    const long long nq = (long long)(f.d.nx / 4) * f.d.ny * f.d.nz;
    (void)nq;
    const int nqr = f.d.nx / 4;
    if (nqr <= 256 && 256 % nqr == 0)
        FF_CUDA(launch_pdl(k_resid_rx_rows, dim3(1, (f.d.ny + 256 / nqr - 1) / (256 / nqr), f.d.nz),
                           dim3(nqr, 256 / nqr), 0, s, g, x, (const float *)f.b, f.coef, m.cls_ptr, m.cls_pitch, rx,
                           st));
    else
        FF_CUDA(launch_pdl(k_resid_rx, dim3((f.d.nx / 4 + 31) / 32, (f.d.ny + 7) / 8, f.d.nz), dim3(32, 8), 0, s,
                           g, x, (const float *)f.b, f.coef, m.cls_ptr, m.cls_pitch, rx, st));
    const long long nc = c.d.n();
    if (c.d.nx % 4 == 0 && c.d.nx == f.d.nx / 2)
        FF_CUDA(launch_pdl(k_restrict_yz4, dim3((c.d.nx / 4 + 31) / 32, (c.d.ny + 7) / 8, c.d.nz), dim3(32, 8), 0,
                           s, f.d, c.d, dims, (const float *)rx, (const uint8_t *)c.mask, (float *)c.b,
                           (const PcgState *)st));
    else
        k_restrict_yz<<<(int)std::min<long long>((nc + 255) / 256, 152LL * 16), 256, 0, s>>>(f.d, c.d, dims, rx,
                                                                                              c.mask, (float *)c.b, st);
    return post("res_restrict2");
}

int prolong4(const Level &c, const Level &f, int dims, float *fine_x, const PcgState *st, cudaStream_t s) {
    FF_CHECK(f.d.nx % 4 == 0, FF_E_ARG, "prolong4 needs nx %% 4 == 0");
    // two planes a thread in 3D (every level above the coarsest has an even nz)
    if (dims == 3 && f.d.nz % 2 == 0)
        FF_CUDA(launch_pdl(k_prolong4<2>, dim3((f.d.nx / 4 + 31) / 32, (f.d.ny + 7) / 8, f.d.nz / 2), dim3(32, 8), 0,
                           s, f.d, c.d, dims, (const float *)c.x, (const uint8_t *)f.mask, fine_x, st));
    else
        FF_CUDA(launch_pdl(k_prolong4<1>, dim3((f.d.nx / 4 + 31) / 32, (f.d.ny + 7) / 8, f.d.nz), dim3(32, 8), 0, s,
                           f.d, c.d, dims, (const float *)c.x, (const uint8_t *)f.mask, fine_x, st));
    return post("prolong4");
}

// ---- TMA sweep
bool sweep_tma_ok(const Dims &d) { return d.nx % 4 == 0 && d.nx >= 32; }

static int tma_zchunk_bps(const Dims &d, int sm_count, int bps, int tx, int ty) {
    // About two waves of resident blocks (bps per SM) when the z-chunks stay
    // at 12 planes or more (the work order then starts the expensive items
    // first and the cheap ones fill in behind them), else one wave; at
    // least 4 planes.
    long long cols = (long long)((d.nx + tx - 1) / tx) * ((d.ny + ty - 1) / ty);
    long long wave = (long long)bps * sm_count;
    int c2 = (int)std::max(1LL, std::min((long long)d.nz, 2 * wave / cols));
    int zc = (d.nz + c2 - 1) / c2;
    if (zc < 12) {
        int c1 = (int)std::max(1LL, std::min((long long)d.nz, wave / cols));
        zc = (d.nz + c1 - 1) / c1;
    }
    return std::min(std::max(zc, std::min(4, d.nz)), tq::MAXZC);
}
// the sweep: four blocks per SM (64 registers), its own tiles
static int tma_zchunk(const Dims &d, int sm_count) { return tma_zchunk_bps(d, sm_count, 4, tq::TX, tq::TY); }
// the CG kernels: p.Ap four blocks per SM, x + alpha p with b - A x two
static int cg_bps(int which) { return which == 0 ? 4 : 2; }

size_t cg_tma_items(const Dims &d, int sm_count, int which) {
    const int zc = tma_zchunk_bps(d, sm_count, cg_bps(which), tcg::TX, tcg::TY);
    return (size_t)((d.nx + tcg::TX - 1) / tcg::TX) * ((d.ny + tcg::TY - 1) / tcg::TY) * ((d.nz + zc - 1) / zc);
}

size_t sweep_tma_blocks(const Dims &d, int sm_count) {
    int zc = tma_zchunk(d, sm_count);
    return (size_t)((d.nx + tq::TX - 1) / tq::TX) * ((d.ny + tq::TY - 1) / tq::TY) * ((d.nz + zc - 1) / zc);
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

static int encode_planes(CUtensorMap *m, const float *base, const Dims &d, int rows) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    FF_CHECK(enc, FF_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    cuuint64_t dims[3] = {(cuuint64_t)d.nx, (cuuint64_t)d.ny, (cuuint64_t)d.nz};
    cuuint64_t strides[2] = {(cuuint64_t)d.nx * 4, (cuuint64_t)d.nx * d.ny * 4};
    cuuint32_t box[3] = {(cuuint32_t)tq::RW, (cuuint32_t)rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void *)base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    FF_CHECK(r == CUDA_SUCCESS, FF_E_CUDA, "cuTensorMapEncodeTiled failed (%d) for a %dx%dx%d level", (int)r,
             d.nx, d.ny, d.nz);
    return FF_OK;
}

static int cls_pitch(const Dims &d) { return ((d.nx / 4 + 15) / 16) * 16; }

size_t sweep_tma_cls_bytes(const Dims &d) { return (size_t)cls_pitch(d) * d.ny * d.nz; }

int sweep_tma_maps(const Level &L, const float *x0, const float *x1, uint8_t *cls, SweepMaps &m) {
    m.ok = false;
    FF_CHECK(sweep_tma_ok(L.d), FF_E_ARG, "TMA sweep needs nx %% 4 == 0 and nx >= 32");
    // TMA global addresses must be 16-byte aligned (the allocator gives 256)
    FF_CHECK(((uintptr_t)x0 | (uintptr_t)x1 | (uintptr_t)L.b | (uintptr_t)cls) % 16 == 0, FF_E_ARG,
             "TMA operand misaligned");
    FF_TRY(encode_planes(&m.x[0], x0, L.d, tq::XR));
    FF_TRY(encode_planes(&m.x[1], x1, L.d, tq::XR));
    FF_TRY(encode_planes(&m.b, (const float *)L.b, L.d, tq::BR));
    // class bytes: (nx/4, ny, nz) uint8 with 16-byte row pitch; box (48, TY+2, 1)
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    FF_CHECK(enc, FF_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    const int pitch = cls_pitch(L.d);
    cuuint64_t dims[3] = {(cuuint64_t)(L.d.nx / 4), (cuuint64_t)L.d.ny, (cuuint64_t)L.d.nz};
    cuuint64_t strides[2] = {(cuuint64_t)pitch, (cuuint64_t)pitch * L.d.ny};
    cuuint32_t box[3] = {(cuuint32_t)tq::CW, (cuuint32_t)tq::CR, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(&m.cls, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, (void *)cls, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    FF_CHECK(r == CUDA_SUCCESS, FF_E_CUDA, "cuTensorMapEncodeTiled (classes) failed (%d)", (int)r);
    // the CG kernels stage the same bytes in boxes of their own tiles, so
    // the sweep's tile can change without their slots overflowing
    cuuint32_t box_cg[3] = {(cuuint32_t)tcg::CW, (cuuint32_t)tcg::PR, 1};
    r = enc(&m.cls_cg, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, (void *)cls, dims, strides, box_cg, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    FF_CHECK(r == CUDA_SUCCESS, FF_E_CUDA, "cuTensorMapEncodeTiled (CG classes) failed (%d)", (int)r);
    m.xp[0] = x0;
    m.xp[1] = x1;
    m.cls_ptr = cls;
    m.cls_pitch = pitch;
    m.ok = true;
    return FF_OK;
}

static int work_orders(const Level &L, const SweepMaps &m, const uint8_t *bricks, int sm_count, cudaStream_t s);

int coef_classes(const Level &L, const SweepMaps &m, uint8_t *bricks, int dims, int want16, int sm_count,
                 cudaStream_t s) {
    FF_CHECK(m.cls_ptr && m.cls_pitch > 0 && m.gco, FF_E_STATE, "cell classes: class arrays not allocated");
    Geo g = make_geo(L);
    // one thread per cell, blocks of (a row rounded up to a warp, at most
    // 128 cells) x rows
    const int bx = std::min(128, (L.d.nx + 31) / 32 * 32), by = 256 / bx;
    dim3 grid((L.d.nx + bx - 1) / bx, (L.d.ny + by - 1) / by, L.d.nz);
    FF_CHECK(L.d.nx % 4 == 0, FF_E_STATE, "cell classes need nx %% 4 == 0");
    k_coef_classes<<<grid, dim3(bx, by), 0, s>>>(g, dims, L.w[0], L.w[1], L.w[2], L.mask, L.h2inv[0], L.h2inv[1],
                                                  L.h2inv[2], L.coef, want16 ? L.coef16 : nullptr, m.cls_ptr,
                                                  m.cls_pitch, m.gco);
    FF_TRY(post("coef_classes"));
    if (bricks) {
        dim3 bg(g.bnx, g.bny, (L.d.nz + BZ - 1) / BZ);
        k_brick_flags_cls<<<bg, 256, 0, s>>>(g, m.cls_ptr, m.cls_pitch, bricks);
        FF_TRY(post("brick_flags_cls"));
    }
    return work_orders(L, m, bricks, sm_count, s);
}

static int work_orders(const Level &L, const SweepMaps &m, const uint8_t *bricks, int sm_count, cudaStream_t s) {
    Geo g = make_geo(L);
    // work orders: the sweep's, and on level 0 those of the two CG kernels
    // (their own z-chunks for their own blocks per SM)
    for (int w = 0; w < 3; ++w) {
        int *order = w == 0 ? m.order : w == 1 ? m.order_pap : m.order_xr;
        if (!order) continue;
        // each kernel's own tiles (16-row bricks: one or more per tile row)
        const int tx = w == 0 ? tq::TX : tcg::TX, ty = w == 0 ? tq::TY : tcg::TY;
        const int zc = w == 0 ? tma_zchunk(L.d, sm_count) : tma_zchunk_bps(L.d, sm_count, cg_bps(w - 1), tx, ty);
        const int gx = (L.d.nx + tx - 1) / tx, gy = (L.d.ny + ty - 1) / ty;
        const int gz = (L.d.nz + zc - 1) / zc;
        FF_CHECK((long long)gx * gy * gz <= 1024LL * 32, FF_E_ARG, "sweep work order: too many items");
        k_sweep_order<<<1, 1024, 0, s>>>(g, bricks, gx, gy, gz, zc, ty / 16, order);
        FF_TRY(post("sweep_order"));
    }
    return FF_OK;
}

int sweep_tma(const Level &L, const SweepMaps &m, const uint8_t *bricks, int in, int colour_a, float sor,
              PcgState *st, double *partials, int rz_mode, int sm_count, cudaStream_t s) {
    FF_CHECK(m.ok, FF_E_STATE, "TMA sweep maps not built");
    const int out = in == 0 ? 1 : 0;
    TqArgs a;
    a.g = make_geo(L);
    a.x_out = const_cast<float *>(m.xp[out]);
    a.coef = L.coef;
    a.bricks = bricks;
    a.sor = sor;
    a.rdreg_sor = sor / a.g.dreg;
    a.omsor = 1.f - sor;
    a.gco = m.gco;
    a.order = m.order;
    a.colour_a = colour_a;
    a.zc = tma_zchunk(L.d, sm_count);
    a.st = st;
    a.partials = partials;
    a.rz_mode = rz_mode;
    a.gx = (L.d.nx + tq::TX - 1) / tq::TX;
    a.gy = (L.d.ny + tq::TY - 1) / tq::TY;
    dim3 grid(a.gx * a.gy * ((L.d.nz + a.zc - 1) / a.zc));
    const CUtensorMap &xm = m.x[in < 0 ? out : in];
    const bool rz = rz_mode != 0;
    if (in < 0) {
        if (rz) FF_CUDA(launch_pdl(k_sweep_tma<true, true>, grid, dim3(tq::NT), tq::SMEM, s, a, xm, m.b, m.cls));
        else FF_CUDA(launch_pdl(k_sweep_tma<true, false>, grid, dim3(tq::NT), tq::SMEM, s, a, xm, m.b, m.cls));
    } else {
        if (rz) FF_CUDA(launch_pdl(k_sweep_tma<false, true>, grid, dim3(tq::NT), tq::SMEM, s, a, xm, m.b, m.cls));
        else FF_CUDA(launch_pdl(k_sweep_tma<false, false>, grid, dim3(tq::NT), tq::SMEM, s, a, xm, m.b, m.cls));
    }
    return post("sweep_tma");
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
    FF_CUDA(cudaFuncSetAttribute(k_sweep_tma<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tq::SMEM));
    FF_CUDA(cudaFuncSetAttribute(k_sweep_tma<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tq::SMEM));
    FF_CUDA(cudaFuncSetAttribute(k_sweep_tma<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tq::SMEM));
    FF_CUDA(cudaFuncSetAttribute(k_sweep_tma<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tq::SMEM));
    FF_CUDA(cudaFuncSetAttribute(k_res_restrict, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rr_smem()));
    FF_CUDA(cudaFuncSetAttribute(k_p_pap, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p_pap_smem()));
    FF_CUDA(cudaFuncSetAttribute(k_p_pap_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tcg::PAP_SMEM));
    FF_CUDA(cudaFuncSetAttribute(k_x_residual_tma<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tcg::XR_SMEM));
    FF_CUDA(cudaFuncSetAttribute(k_x_residual_tma<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tcg::XR_SMEM));
    FF_CUDA(cudaFuncSetAttribute(k_x_residual_tma<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tcg::XR_SMEM));
    FF_CUDA(cudaFuncSetAttribute(k_x_residual_tma<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tcg::XR_SMEM));
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


int cg_tma_maps(const Level &L0, const float *z0, const float *z1, const float *p0, const float *p1,
                const float *xh0, const float *xl0, const float *xh1, const float *xl1, const float *b, bool ds,
                CgMaps &m) {
    m.ok = false;
    FF_CHECK(sweep_tma_ok(L0.d), FF_E_ARG, "TMA CG kernels need nx %% 4 == 0 and nx >= 32");
    uintptr_t any = (uintptr_t)z0 | (uintptr_t)z1 | (uintptr_t)p0 | (uintptr_t)p1 | (uintptr_t)xh0 |
                    (uintptr_t)xh1 | (uintptr_t)b;
    if (ds) any |= (uintptr_t)xl0 | (uintptr_t)xl1;
    FF_CHECK(any % 16 == 0, FF_E_ARG, "TMA operand misaligned");
    FF_TRY(encode_planes(&m.z[0], z0, L0.d, tcg::PR));
    FF_TRY(encode_planes(&m.z[1], z1, L0.d, tcg::PR));
    FF_TRY(encode_planes(&m.p[0], p0, L0.d, tcg::PR));
    FF_TRY(encode_planes(&m.p[1], p1, L0.d, tcg::PR));
    FF_TRY(encode_planes(&m.xh[0], xh0, L0.d, tcg::PR));
    FF_TRY(encode_planes(&m.xh[1], xh1, L0.d, tcg::PR));
    if (ds) {
        FF_TRY(encode_planes(&m.xl[0], xl0, L0.d, tcg::PR));
        FF_TRY(encode_planes(&m.xl[1], xl1, L0.d, tcg::PR));
    } else {
        m.xl[0] = m.xh[0];
        m.xl[1] = m.xh[1];
    }
    FF_TRY(encode_planes(&m.b, b, L0.d, tcg::TY));
    m.zp[0] = z0;
    m.zp[1] = z1;
    m.ds = ds;
    m.ok = true;
    return FF_OK;
}

// which: 0 p.Ap, 1 x + alpha p with b - A x
static TcgArgs tcg_args(const Level &L0, const SweepMaps &sm, int sm_count, int which) {
    TcgArgs a;
    a.g = make_geo(L0);
    a.coef = L0.coef;
    a.gco = sm.gco;
    a.order = which == 0 ? sm.order_pap : sm.order_xr;
    a.gx = (L0.d.nx + tcg::TX - 1) / tcg::TX;
    a.gy = (L0.d.ny + tcg::TY - 1) / tcg::TY;
    a.zc = tma_zchunk_bps(L0.d, sm_count, cg_bps(which), tcg::TX, tcg::TY);
    return a;
}

int p_pap_tma(const Level &L0, const SweepMaps &sm, const CgMaps &m, const float *z, float *p0, float *p1,
              PcgState *st, double *partials, int sm_count, cudaStream_t s) {
    FF_CHECK(sm.ok && m.ok, FF_E_STATE, "TMA CG maps not built");
    const int zi = z == m.zp[0] ? 0 : z == m.zp[1] ? 1 : -1;
    FF_CHECK(zi >= 0, FF_E_STATE, "p.Ap: z is in neither sweep buffer");
    TcgArgs a = tcg_args(L0, sm, sm_count, 0);
    a.p0 = p0;
    a.p1 = p1;
    a.st = st;
    a.partials = partials;
    dim3 grid(a.gx * a.gy * ((L0.d.nz + a.zc - 1) / a.zc));
    FF_CUDA(launch_pdl(k_p_pap_tma, grid, dim3(tcg::NT), tcg::PAP_SMEM, s, a, m.z[zi], m.p[0], m.p[1], sm.cls_cg));
    return post("p_pap_tma");
}

int x_residual_tma(const Level &L0, const SweepMaps &sm, const CgMaps &m, float *xh0, float *xl0, float *xh1,
                   float *xl1, float *r, PcgState *st, double *partials, int setup, int sm_count, cudaStream_t s) {
    FF_CHECK(sm.ok && m.ok, FF_E_STATE, "TMA CG maps not built");
    TcgArgs a = tcg_args(L0, sm, sm_count, 1);
    a.xh0 = xh0;
    a.xl0 = xl0;
    a.xh1 = xh1;
    a.xl1 = xl1;
    a.r = r;
    a.st = st;
    a.partials = partials;
    dim3 grid(a.gx * a.gy * ((L0.d.nz + a.zc - 1) / a.zc));
    const size_t sh = tcg::XR_SMEM;
    if (setup) {
        if (m.ds) FF_CUDA(launch_pdl(k_x_residual_tma<true, true>, grid, dim3(tcg::NT), sh, s, a, m.xh[0], m.xh[1], m.xl[0], m.xl[1], m.p[0], m.p[1], m.b, sm.cls_cg));
        else FF_CUDA(launch_pdl(k_x_residual_tma<true, false>, grid, dim3(tcg::NT), sh, s, a, m.xh[0], m.xh[1], m.xl[0], m.xl[1], m.p[0], m.p[1], m.b, sm.cls_cg));
    } else {
        if (m.ds) FF_CUDA(launch_pdl(k_x_residual_tma<false, true>, grid, dim3(tcg::NT), sh, s, a, m.xh[0], m.xh[1], m.xl[0], m.xl[1], m.p[0], m.p[1], m.b, sm.cls_cg));
        else FF_CUDA(launch_pdl(k_x_residual_tma<false, false>, grid, dim3(tcg::NT), sh, s, a, m.xh[0], m.xh[1], m.xl[0], m.xl[1], m.p[0], m.p[1], m.b, sm.cls_cg));
    }
    return post("x_residual_tma");
}


size_t cls_row_pitch(const Dims &d) { return (size_t)cls_pitch(d); }

int vcycle_tail(const Level *lv, const SweepMaps *sm, int nl, int dims, int down, int up, float sor,
                const double *G, int nG, int coarse_sweeps, PcgState *st, unsigned *bar, int sm_count,
                cudaStream_t s) {
    FF_CHECK(nl >= 2 && nl <= TAIL_MAXL, FF_E_ARG, "coarse V-cycle: %d levels (2..%d)", nl, TAIL_MAXL);
    FF_CHECK(bar, FF_E_ARG, "coarse V-cycle: no barrier words");
    FF_CHECK(coarse_sweeps > 0 || (G && nG == lv[nl - 1].d.n()), FF_E_STATE, "coarse V-cycle: no coarsest inverse");
    TailArgs a;
    for (int l = 0; l < nl; ++l) {
        TailLevel &t = a.lv[l];
        const Level &L = lv[l];
        t.g = make_geo(L);
        t.x = (float *)L.x;
        t.b = (float *)L.b;
        t.r = (float *)L.buf;
        t.coef = L.coef;
        t.mask = L.mask;
        t.rdreg_sor = sor / t.g.dreg;
        t.smo = -1;
        auto magic = [](long long d) { return ((1ULL << 40) + (unsigned long long)d - 1) / (unsigned long long)d; };
        t.mhx = magic(std::max(1, L.d.nx / 2));
        t.mnx = magic(L.d.nx);
        t.mny = magic(L.d.ny);
        if (l < nl - 1) {
            FF_CHECK(sm[l].cls_ptr && sm[l].gco && L.buf, FF_E_STATE, "coarse V-cycle: level %d lacks classes", l);
            t.cls = sm[l].cls_ptr;
            t.cpitch = sm[l].cls_pitch;
            t.gco = sm[l].gco;
        } else {
            t.cls = nullptr;
            t.cpitch = 0;
            t.gco = nullptr;
        }
    }
    a.nl = nl;
    a.down = down;
    a.up = up;
    a.dims = dims;
    a.sor = sor;
    a.omsor = 1.f - sor;
    a.G = G;
    a.nG = nG;
    a.coarse_sweeps = coarse_sweeps;
    a.st = st;
    a.bar = bar;
    // levels held in block 0's shared memory (2D): from the last but one
    // upward while they have at most TAIL_SMEM_CELLS cells and fit the budget
    // (and, beside the last but one, a copy of the coarsest x).  In 3D the
    // 16^3 level held there made the 256^3 V-cycle slower (0.587 -> 0.596
    // ms: its block-0 phases cost more than the grid barriers they saved), so
    // 3D levels stay grid-wide.
    int smem = 0;
    const long long nc = lv[nl - 1].d.n();
    for (int l = nl - 2; l >= 0 && dims == 2; --l) {
        const long long n = lv[l].d.n();
        if (n > TAIL_SMEM_CELLS || smem + 12 * n + (l == nl - 2 ? 4 * nc : 0) > TAIL_SMEM_BYTES) break;
        a.lv[l].smo = smem / 4;
        smem += (int)(12 * n);
    }
    a.cxo = -1;
    if (a.lv[nl - 2].smo >= 0) {
        a.cxo = smem / 4;
        smem += (int)(4 * nc);
    }
    static int per_sm = -1, per_sm_held = -1;
    if (per_sm < 0) {
        FF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vcycle_tail<false>, TAIL_NT, 0));
        FF_CUDA(cudaFuncSetAttribute(k_vcycle_tail<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     TAIL_SMEM_BYTES));
        FF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_held, k_vcycle_tail<true>, TAIL_NT,
                                                              TAIL_SMEM_BYTES));
    }
    FF_CHECK(per_sm >= 1 && per_sm_held >= 1 && smem <= TAIL_SMEM_BYTES, FF_E_CUDA,
             "coarse V-cycle kernel does not fit an SM");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)sm_count);
    cfg.blockDim = dim3(TAIL_NT);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (smem > 0) FF_CUDA(cudaLaunchKernelEx(&cfg, k_vcycle_tail<true>, a));
    else FF_CUDA(cudaLaunchKernelEx(&cfg, k_vcycle_tail<false>, a));
    return post("vcycle_tail");
}

}  // namespace ffk
