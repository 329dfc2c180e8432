// 3D FLIP particle-grid transfer (fluxflow src/grid/grid_flip_solver3.js):
// particle advection through the grid velocity, fixed-point P2G with int32
// atomics, fluid marking and the reduced-pressure Dirichlet condition of
// air cells, the variable-density beta faces and reduced gravity, G2P with
// the FLIP/PIC blend, and the per-step orchestration (onAdvanceTimeStep).
//
// FP32 arithmetic rounds one operation at a time (-fmad=false), in the
// reference's evaluation order; P2G accumulates round(v w S) and round(w S)
// as int32 (wrapping like the reference's i32 atomics), so its result does
// not depend on the order particles arrive in.  Host-side seeding
// (computeFlipBoxSeed3, mulberry32) is computed in doubles as JavaScript
// does (-ffp-contract=off on the host compiler).
#include "ff_grid.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {
using namespace ffg;

constexpr float MAX_PARTICLE_VELOCITY = 500.0f;   // grid_flip_solver3.js:176 (via the 2D file)
constexpr float MIN_DENSITY = 1e-4f;              // :182
constexpr double PRESSURE_BOUND_HEADROOM = 8.0;   // :175

__device__ __forceinline__ bool nonfinite(float v) { return isnan(v) || isinf(v); }

// cellIndexOf (:227-235)
__device__ __forceinline__ long long cell_of(const G3 &g, const float *p) {
    const float cx = gclamp((p[0] - g.ox) / g.hx), cy = gclamp((p[1] - g.oy) / g.hy), cz = gclamp((p[2] - g.oz) / g.hz);
    const int i = iclamp((int)floorf(cx), 0, g.nx - 1), j = iclamp((int)floorf(cy), 0, g.ny - 1),
              k = iclamp((int)floorf(cz), 0, g.nz - 1);
    return i + (long long)g.nx * (j + (long long)g.ny * k);
}

// advectParticles (:925-933) then pushOutOfCollider (:939-951).  keep_z:
// particles of a one-cell-thick grid standing in for a 2D one stay on their
// plane (the trace leaves z alone there anyway, except for the rounding of
// the collider-crossing blend)
__global__ void k_flip_advect(VelField F, long long n, float *__restrict__ pos, float dt, int max_substeps, F3 mn,
                              F3 mx, float push_thresh, float push_shift, int keep_z) {
    const F3 oc = comp_origin(F.g, 3);
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const F3 prev{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]};
        const F3 tr = back_trace(F, prev, dt, -1.0f, max_substeps);
        const bool bad = nonfinite(tr.x) || nonfinite(tr.y) || nonfinite(tr.z);
        F3 q{fminf(fmaxf(bad ? prev.x : tr.x, mn.x), mx.x), fminf(fmaxf(bad ? prev.y : tr.y, mn.y), mx.y),
             fminf(fmaxf(bad ? prev.z : tr.z, mn.z), mx.z)};
        if (F.phi) {
            const float val = trilinear(F.phi, F.g.nx, F.g.ny, F.g.nz, F.g, oc, q);
            if (val < push_thresh) {
                const F3 gr = trilinear_gradient(F.phi, F.g, oc, q);
                const float gl = sqrtf(gr.x * gr.x + gr.y * gr.y + gr.z * gr.z);
                if (gl > 0.0f) {
                    const float shift = (push_thresh - val) + push_shift;
                    q = F3{q.x + gr.x / gl * shift, q.y + gr.y / gl * shift, q.z + gr.z / gl * shift};
                }
            }
        }
        pos[3 * p] = q.x;
        pos[3 * p + 1] = q.y;
        pos[3 * p + 2] = keep_z ? prev.z : q.z;
    }
}

// markFluidCellsKernel (:241-245), after a cleared mask
__global__ void k_flip_mark(G3 g, long long n, const float *__restrict__ pos, float *__restrict__ mask) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        mask[cell_of(g, pos + 3 * p)] = 1.0f;
}

// buildScatter (:508-530): each particle adds round(v w S) and round(w S)
// to the 8 faces around it, per component (the first ncomp components)
__global__ void k_flip_scatter(G3 g, long long n, const float *__restrict__ pos, const float *__restrict__ vel,
                               float scale, int *__restrict__ nu, int *__restrict__ du, int *__restrict__ nv,
                               int *__restrict__ dv, int *__restrict__ nw, int *__restrict__ dw, int ncomp) {
    int *num[3] = {nu, nv, nw}, *den[3] = {du, dv, dw};
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const F3 q{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            if (a >= ncomp) break;
            int sx, sy, sz;
            comp_shape(g, a, sx, sy, sz);
            const F3 o = comp_origin(g, a);
            const float value = vel[3 * p + a];
            const float gx = gclamp((q.x - o.x) / g.hx), gy = gclamp((q.y - o.y) / g.hy), gz = gclamp((q.z - o.z) / g.hz);
            const int i0 = (int)floorf(gx), j0 = (int)floorf(gy), k0 = (int)floorf(gz);
            const float fx = gx - (float)i0, fy = gy - (float)j0, fz = gz - (float)k0;
            const int ic[2] = {iclamp(i0, 0, sx - 1), iclamp(i0 + 1, 0, sx - 1)};
            const int jc[2] = {iclamp(j0, 0, sy - 1), iclamp(j0 + 1, 0, sy - 1)};
            const int kc[2] = {iclamp(k0, 0, sz - 1), iclamp(k0 + 1, 0, sz - 1)};
            const float ux = 1.0f - fx, uy = 1.0f - fy, uz = 1.0f - fz;
            const float w[8] = {ux * uy * uz, fx * uy * uz, ux * fy * uz, fx * fy * uz,
                                ux * uy * fz, fx * uy * fz, ux * fy * fz, fx * fy * fz};
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const long long f = ic[c & 1] + (long long)sx * (jc[(c >> 1) & 1] + (long long)sy * kc[(c >> 2) & 1]);
                atomicAdd(num[a] + f, __float2int_rn(value * w[c] * scale));
                atomicAdd(den[a] + f, __float2int_rn(w[c] * scale));
            }
        }
    }
}

// buildFinalize (:532-550)
__global__ void k_flip_finalize(long long n, const int *__restrict__ num, const int *__restrict__ den, float scale,
                                float eps, float *__restrict__ data, int *__restrict__ valid) {
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        const float numer = (float)num[f] / scale;
        const float denom = (float)den[f] / scale;
        if (denom > eps) {
            data[f] = numer / denom;
            valid[f] = 1;
        } else {
            data[f] = 0.0f;
            valid[f] = 0;
        }
    }
}

// computeU/V/WFluidAdjacent (:586-618)
__global__ void k_flip_adjacent(G3 g, int a, const float *__restrict__ mask, int *__restrict__ adj) {
    int s[3];
    comp_shape(g, a, s[0], s[1], s[2]);
    const long long n = (long long)s[0] * s[1] * s[2];
    const int nn = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        int idx[3];
        unflatten(f, s[0], s[1], idx[0], idx[1], idx[2]);
        int lo[3] = {idx[0], idx[1], idx[2]}, hi[3] = {idx[0], idx[1], idx[2]};
        lo[a] = iclamp(idx[a] - 1, 0, nn - 1);
        hi[a] = iclamp(idx[a], 0, nn - 1);
        const float ml = mask[lo[0] + (long long)g.nx * (lo[1] + (long long)g.ny * lo[2])];
        const float mh = mask[hi[0] + (long long)g.nx * (hi[1] + (long long)g.ny * hi[2])];
        adj[f] = (ml > 0.5f || mh > 0.5f) ? 1 : 0;
    }
}

// dirichlet(pos) evaluated at the cell centres (:252-259)
__global__ void k_flip_dirichlet(G3 g, const float *__restrict__ mask, F3 grav, float dt, int reduced,
                                 uint8_t *__restrict__ active, float *__restrict__ target) {
    const long long n = (long long)g.nx * g.ny * g.nz;
    const F3 oc = comp_origin(g, 3);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        unflatten(c, g.nx, g.ny, i, j, k);
        const F3 p = index_pos(g, oc, i, j, k);
        const float m = trilinear(mask, g.nx, g.ny, g.nz, g, oc, p);
        active[c] = m < 0.5f;
        target[c] = reduced ? -((grav.x * p.x + grav.y * p.y + grav.z * p.z) * dt) : 0.0f;
    }
}

// accumulateConcentration (:999-1004)
__global__ void k_flip_conc_accum(G3 g, long long n, const float *__restrict__ pos, const float *__restrict__ conc,
                                  float cscale, int *__restrict__ cnt, int *__restrict__ acc) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const long long c = cell_of(g, pos + 3 * p);
        atomicAdd(cnt + c, 1);
        atomicAdd(acc + c, __float2int_rn(fminf(fmaxf(conc[p], 0.0f), 1.0f) * cscale));
    }
}

// resolveCellConcentration (:1006-1015)
__global__ void k_flip_conc_resolve(long long nc, const int *__restrict__ cnt, const int *__restrict__ acc, float cscale,
                                    int density, float r0, float r1, float *__restrict__ cell_conc,
                                    float *__restrict__ cell_rho) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
        const float total = (float)cnt[c];
        const float sum = (float)acc[c] / cscale;
        const float mean = sum / fmaxf(total, 1.0f);
        const float cv = total > 0.5f ? fminf(fmaxf(mean, 0.0f), 1.0f) : 0.0f;
        cell_conc[c] = cv;
        if (density) cell_rho[c] = r0 + (r1 - r0) * cv;
    }
}

// computeBetaU/V/W with faceDensity (:315-345); mask == nullptr: every
// cell is fluid, the face density is the mean of its two cells
// (grid_two_phase_flip_solver2.js:750-762)
__global__ void k_flip_beta(G3 g, int a, const float *__restrict__ rho, const float *__restrict__ mask, float rref,
                            float *__restrict__ beta) {
    int s[3];
    comp_shape(g, a, s[0], s[1], s[2]);
    const long long n = (long long)s[0] * s[1] * s[2];
    const int nn = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        int idx[3];
        unflatten(f, s[0], s[1], idx[0], idx[1], idx[2]);
        int A[3] = {idx[0], idx[1], idx[2]}, B[3] = {idx[0], idx[1], idx[2]};
        A[a] = iclamp(idx[a] - 1, 0, nn - 1);
        B[a] = iclamp(idx[a], 0, nn - 1);
        const long long ca = A[0] + (long long)g.nx * (A[1] + (long long)g.ny * A[2]);
        const long long cb = B[0] + (long long)g.nx * (B[1] + (long long)g.ny * B[2]);
        const float ra = rho[ca], rb = rho[cb];
        const bool fa = !mask || mask[ca] > 0.5f, fb = !mask || mask[cb] > 0.5f;
        const float rf = (fa && fb) ? (ra + rb) * 0.5f : ((fa || fb) ? (fa ? ra : rb) : rref);
        beta[f] = rref / fmaxf(rf, MIN_DENSITY);
    }
}

// applyReducedGravityU/V/W (:848-884); plain gravity (:821-831) when beta is null
__global__ void k_flip_gravity(G3 g, int a, const float *__restrict__ rho, const float *__restrict__ beta, F3 grav,
                               float dt, float rref, float *__restrict__ data) {
    int s[3];
    comp_shape(g, a, s[0], s[1], s[2]);
    const long long n = (long long)s[0] * s[1] * s[2];
    const int nn = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
    const float ga = a == 0 ? grav.x : (a == 1 ? grav.y : grav.z);
    const float ha = a == 0 ? g.hx : (a == 1 ? g.hy : g.hz);
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n; f += (long long)gridDim.x * blockDim.x) {
        if (!beta) {
            data[f] = data[f] + ga * dt;
            continue;
        }
        int idx[3];
        unflatten(f, s[0], s[1], idx[0], idx[1], idx[2]);
        const float px = g.ox + (a == 0 ? (float)idx[0] * g.hx : ((float)idx[0] + 0.5f) * g.hx);
        const float py = g.oy + (a == 1 ? (float)idx[1] * g.hy : ((float)idx[1] + 0.5f) * g.hy);
        const float pz = g.oz + (a == 2 ? (float)idx[2] * g.hz : ((float)idx[2] + 0.5f) * g.hz);
        int A[3] = {idx[0], idx[1], idx[2]}, B[3] = {idx[0], idx[1], idx[2]};
        B[a] = iclamp(idx[a], 0, nn - 1);
        A[a] = iclamp(idx[a] - 1, 0, nn - 1);
        const float rb = rho[B[0] + (long long)g.nx * (B[1] + (long long)g.ny * B[2])];
        const float ra = rho[A[0] + (long long)g.nx * (A[1] + (long long)g.ny * A[2])];
        const float drho = (rb - ra) / ha;
        const float gp = grav.x * px + grav.y * py + grav.z * pz;
        const float term = beta[f] * dt / rref * gp * drho;
        data[f] = data[f] - term;
    }
}

// g2pUpdate (:909-922).  conc != nullptr: the per-particle blend of the
// two-phase solver, gas_ratio + (ratio - gas_ratio) clamp(c, 0, 1)
// (grid_two_phase_flip_solver2.js:966-992)
__global__ void k_flip_g2p(G3 g, long long n, const float *__restrict__ pos, float *__restrict__ vel,
                           const float *__restrict__ u, const float *__restrict__ v, const float *__restrict__ w,
                           const float *__restrict__ uo, const float *__restrict__ vo, const float *__restrict__ wo,
                           float flip_ratio, float damp, const float *__restrict__ conc, float gas_ratio) {
    const float *nw[3] = {u, v, w}, *od[3] = {uo, vo, wo};
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const F3 q{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]};
        const float ratio =
            conc ? gas_ratio + (flip_ratio - gas_ratio) * fminf(fmaxf(conc[p], 0.0f), 1.0f) : flip_ratio;
        float out[3];
        bool bad = false;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            int sx, sy, sz;
            comp_shape(g, a, sx, sy, sz);
            const F3 o = comp_origin(g, a);
            const float nv = trilinear(nw[a], sx, sy, sz, g, o, q);
            const float ov = trilinear(od[a], sx, sy, sz, g, o, q);
            const float delta = nv - ov;
            const float flipv = vel[3 * p + a] + delta;
            const float blended = flipv * ratio + nv * (1.0f - ratio);
            out[a] = blended * (1.0f - damp);
            bad |= nonfinite(out[a]);
        }
#pragma unroll
        for (int a = 0; a < 3; ++a)
            vel[3 * p + a] = bad ? 0.0f : fminf(fmaxf(out[a], -MAX_PARTICLE_VELOCITY), MAX_PARTICLE_VELOCITY);
    }
}

// mixAndFade (:1022-1029)
__global__ void k_flip_mix_fade(G3 g, long long n, const float *__restrict__ pos, const float *__restrict__ cell_conc,
                                float mixing, float fade, float *__restrict__ conc) {
    const F3 oc = comp_origin(g, 3);
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
        const F3 q{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]};
        const float sampled = trilinear(cell_conc, g.nx, g.ny, g.nz, g, oc, q);
        const float c = fminf(fmaxf(conc[p], 0.0f), 1.0f);
        const float local = nonfinite(sampled) ? c : sampled;
        const float blended = c + (local - c) * mixing;
        conc[p] = fminf(fmaxf(blended * (1.0f - fade), 0.0f), 1.0f);
    }
}

// ---- resamplePass (:621-820) ------------------------------------------
// Donor ranks and claim slots are prefix sums in index order -- particle
// order for donors, flat cell order (i fastest) for claims -- so which
// particle lands where does not depend on scheduling.  A block owns
// RS_CHUNK consecutive items, each warp RS_WARP_ITEMS of them in rounds of
// 32 (coalesced); a warp ranks its items by ballot (donors) or a shuffle
// scan (needs), and the scanned block totals place the blocks.
constexpr int RS_ROUNDS = 16, RS_WARP_ITEMS = RS_ROUNDS * 32, RS_CHUNK = 8 * RS_WARP_ITEMS;

// markDonorsKernel (:686-693): every particle of a cell above max_pc
__device__ __forceinline__ bool rs_donor(const G3 &g, const float *__restrict__ pos, long long p,
                                         const int *__restrict__ cnt, int max_pc) {
    return cnt[cell_of(g, pos + 3 * p)] > max_pc;
}

// markNeedKernel (:716-724) with neighborFluidCount (:700-713): min_pc -
// count for a cell below min_pc with at least 3 of its 6 face neighbours
// (indices clamped to the grid) at min_pc or more
__device__ __forceinline__ int rs_need(const G3 &g, const int *__restrict__ cnt, long long c, int min_pc) {
    const int count = cnt[c];
    if (count >= min_pc) return 0;
    const long long plane = (long long)g.nx * g.ny;
    const int k = (int)(c / plane), rem = (int)(c - k * plane), j = rem / g.nx, i = rem - j * g.nx;
    const int nb = (cnt[i > 0 ? c - 1 : c] >= min_pc) + (cnt[i < g.nx - 1 ? c + 1 : c] >= min_pc) +
                   (cnt[j > 0 ? c - g.nx : c] >= min_pc) + (cnt[j < g.ny - 1 ? c + g.nx : c] >= min_pc) +
                   (cnt[k > 0 ? c - plane : c] >= min_pc) + (cnt[k < g.nz - 1 ? c + plane : c] >= min_pc);
    return nb >= 3 ? min_pc - count : 0;
}

__device__ __forceinline__ long long rs_warp_sum(long long v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// the exclusive offset of this warp's total inside the block (every lane
// passes the same warp total); *total: the block's sum
__device__ __forceinline__ long long rs_warp_offset(long long mine, long long *total) {
    __shared__ long long wsum[8];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) wsum[w] = mine;
    __syncthreads();
    long long off = 0, tot = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        off += q < w ? wsum[q] : 0;
        tot += wsum[q];
    }
    *total = tot;
    return off;
}

// countPerCellKernel (:674-679)
__global__ void k_rs_count(G3 g, long long n, const float *__restrict__ pos, int *__restrict__ cnt) {
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x)
        atomicAdd(cnt + cell_of(g, pos + 3 * p), 1);
}

// per-block donor totals (blocks [0, nbp)) and need totals (the rest)
__global__ void __launch_bounds__(256) k_rs_sums(G3 g, long long n, const float *__restrict__ pos,
                                                 const int *__restrict__ cnt, int min_pc, int max_pc, int nbp,
                                                 long long *__restrict__ bsum_p, long long *__restrict__ bsum_c) {
    const bool parts = (int)blockIdx.x < nbp;
    const long long b = parts ? blockIdx.x : blockIdx.x - nbp;
    const long long first = b * RS_CHUNK + (threadIdx.x >> 5) * RS_WARP_ITEMS + (threadIdx.x & 31);
    const long long nc = (long long)g.nx * g.ny * g.nz;
    long long mine = 0;
#pragma unroll 4
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const long long x = first + 32 * r;
        if (parts)
            mine += (x < n && rs_donor(g, pos, x, cnt, max_pc)) ? 1 : 0;
        else
            mine += x < nc ? rs_need(g, cnt, x, min_pc) : 0;
    }
    long long total;
    rs_warp_offset(rs_warp_sum(mine), &total);
    if (threadIdx.x == 0) (parts ? bsum_p : bsum_c)[b] = total;
}

// the inclusive scans of donorFlag and cellNeed (:650-651) at block
// granularity: both block-total arrays become exclusive offsets in place;
// tot[0] = donors (donorScan's last entry), tot[1] = cells' total need
__global__ void __launch_bounds__(1024) k_rs_scan(long long *__restrict__ a, int na, long long *__restrict__ c, int nc,
                                                  long long *__restrict__ tot) {
    __shared__ long long ws[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int which = 0; which < 2; ++which) {
        long long *x = which ? c : a;
        const int m = which ? nc : na;
        long long carry = 0;
        for (int base = 0; base < m; base += 1024) {
            const int i = base + threadIdx.x;
            const long long v = i < m ? x[i] : 0;
            long long s = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long t = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += t;
            }
            if (lane == 31) ws[w] = s;
            __syncthreads();
            if (w == 0) {
                long long t = ws[lane];
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const long long u = __shfl_up_sync(0xffffffffu, t, o);
                    if (lane >= o) t += u;
                }
                ws[lane] = t;
            }
            __syncthreads();
            if (i < m) x[i] = carry + (w ? ws[w - 1] : 0) + s - v;
            carry += ws[31];
            __syncthreads();
        }
        if (threadIdx.x == 0) tot[which] = carry;
    }
}

// scatterDonorsKernel (:697-704): donorPool[rank] = p, rank = the number
// of donors before p in particle order
__global__ void __launch_bounds__(256) k_rs_scatter(G3 g, long long n, const float *__restrict__ pos,
                                                    const int *__restrict__ cnt, int max_pc,
                                                    const long long *__restrict__ bsum_p, int *__restrict__ pool) {
    const int lane = threadIdx.x & 31;
    const long long first = blockIdx.x * (long long)RS_CHUNK + (threadIdx.x >> 5) * RS_WARP_ITEMS;
    unsigned bal[RS_ROUNDS];
    long long mine = 0;
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const long long x = first + 32 * r + lane;
        bal[r] = __ballot_sync(0xffffffffu, x < n && rs_donor(g, pos, x, cnt, max_pc));
        mine += __popc(bal[r]);
    }
    long long total;
    long long run = bsum_p[blockIdx.x] + rs_warp_offset(mine, &total);
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        if ((bal[r] >> lane) & 1u) pool[run + __popc(bal[r] & below)] = (int)(first + 32 * r + lane);
        run += __popc(bal[r]);
    }
}

// claimDonorsKernel (:726-790): the cell's slots start at the need of the
// cells before it; while a slot is below the donor total, that donor moves
// to the cell centre with the face-centred velocity sampled there
__global__ void __launch_bounds__(256) k_rs_claim(G3 g, const int *__restrict__ cnt, int min_pc,
                                                  const long long *__restrict__ bsum_c,
                                                  const long long *__restrict__ tot, const int *__restrict__ pool,
                                                  const float *__restrict__ u, const float *__restrict__ v,
                                                  const float *__restrict__ w, float *__restrict__ pos,
                                                  float *__restrict__ vel) {
    const int lane = threadIdx.x & 31;
    const long long nc = (long long)g.nx * g.ny * g.nz;
    const long long first = blockIdx.x * (long long)RS_CHUNK + (threadIdx.x >> 5) * RS_WARP_ITEMS + lane;
    int need[RS_ROUNDS];
    long long mine = 0;
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const long long x = first + 32 * r;
        need[r] = x < nc ? rs_need(g, cnt, x, min_pc) : 0;
        mine += need[r];
    }
    long long total;
    long long run = bsum_c[blockIdx.x] + rs_warp_offset(rs_warp_sum(mine), &total);
    if (total == 0) return;
    const long long donors = tot[0];
    const float *comp[3] = {u, v, w};
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        long long s = need[r];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        const long long slot0 = run + s - need[r];
        run += __shfl_sync(0xffffffffu, s, 31);
        if (need[r] > 0 && slot0 < donors) {
            const long long c = first + 32 * r, plane = (long long)g.nx * g.ny;
            const int k = (int)(c / plane), rem = (int)(c - k * plane), j = rem / g.nx, i = rem - j * g.nx;
            const F3 q = index_pos(g, comp_origin(g, 3), i, j, k);
            float vq[3];
            for (int a = 0; a < 3; ++a) {
                int sx, sy, sz;
                comp_shape(g, a, sx, sy, sz);
                vq[a] = trilinear(comp[a], sx, sy, sz, g, comp_origin(g, a), q);
            }
            for (int m = 0; m < need[r] && slot0 + m < donors; ++m) {
                const long long d = pool[slot0 + m];
                pos[3 * d] = q.x;
                pos[3 * d + 1] = q.y;
                pos[3 * d + 2] = q.z;
                vel[3 * d] = vq[0];
                vel[3 * d + 1] = vq[1];
                vel[3 * d + 2] = vq[2];
            }
        }
    }
}

// ---- per-phase resampling of the two-phase solvers
// (grid_two_phase_flip_solver2.js:1226-1500), on the one-cell-thick grid of
// the 2D solver or the full grid of the 3D one.
// Two donor pools share one buffer: liquid donors (phase > 0.5) rank
// upward from 0, gas donors downward from the top, each capped at
// pool_half; a cell's need is signed (+ liquid, - gas) and each phase's
// cells claim from that phase's pool in flat cell order.

// computeRecipientNeedKernel (:1298-1310): eligible below min_pc with at
// least 2 of the 4 clamped neighbours at min_pc or more; the phase is the
// cell's own majority, or its neighbours' when it is empty
// (recipientWantsLiquid, :1270-1296).  On a 3D grid (nz > 1) the neighbours
// are the 6 clamped face neighbours and at least 3 must be full, the rule of
// the 3D single-phase pass (grid_flip_solver3.js:700-724).
__global__ void k_tp_need(G3 g, const int *__restrict__ cnt, const int *__restrict__ acc, float cscale, int min_pc,
                          int *__restrict__ need) {
    const long long plane = (long long)g.nx * g.ny, nc = plane * g.nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < nc; c += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(c / plane);
        const long long rem = c - (long long)k * plane;
        const int j = (int)(rem / g.nx), i = (int)(rem - (long long)j * g.nx);
        const long long l = i > 0 ? c - 1 : c, r = i < g.nx - 1 ? c + 1 : c;
        const long long d = j > 0 ? c - g.nx : c, u = j < g.ny - 1 ? c + g.nx : c;
        const int count = cnt[c];
        int nb = (cnt[l] >= min_pc) + (cnt[r] >= min_pc) + (cnt[d] >= min_pc) + (cnt[u] >= min_pc);
        int ctot = cnt[l] + cnt[r] + cnt[d] + cnt[u], atot = acc[l] + acc[r] + acc[d] + acc[u];
        int min_nb = 2;
        if (g.nz > 1) {
            const long long b = k > 0 ? c - plane : c, f = k < g.nz - 1 ? c + plane : c;
            nb += (cnt[b] >= min_pc) + (cnt[f] >= min_pc);
            ctot += cnt[b] + cnt[f];
            atot += acc[b] + acc[f];
            min_nb = 3;
        }
        const bool eligible = count < min_pc && nb >= min_nb;
        const float total = (float)count, sum = (float)acc[c] / cscale;
        const float ntot = (float)ctot;
        const float nsum = (float)atot / cscale;
        const float own = sum / fmaxf(total, 1.0f), around = nsum / fmaxf(ntot, 1.0f);
        const bool liquid = total > 0.5f ? own > 0.5f : around > 0.5f;
        const int needed = min_pc - count;
        need[c] = eligible ? (liquid ? needed : -needed) : 0;
    }
}

// offsets of this warp's two totals inside the block, and the block's sums
__device__ __forceinline__ void rs_warp_offset2(long long a, long long b, long long &oa, long long &ob, long long &ta,
                                                long long &tb) {
    __shared__ long long ws[2][8];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        ws[0][w] = a;
        ws[1][w] = b;
    }
    __syncthreads();
    oa = ob = ta = tb = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        oa += q < w ? ws[0][q] : 0;
        ob += q < w ? ws[1][q] : 0;
        ta += ws[0][q];
        tb += ws[1][q];
    }
}

__device__ __forceinline__ bool tp_over(const G3 &g, const float *__restrict__ pos, long long p,
                                        const int *__restrict__ cnt, int max_pc) {
    return cnt[cell_of(g, pos + 3 * p)] > max_pc;
}

// per-block totals: particle blocks count liquid and gas donors
// (markDonorsKernel, :1316-1327), cell blocks sum the split needs
// (splitNeedKernel, :1359-1368)
__global__ void __launch_bounds__(256) k_tp_sums(G3 g, long long n, const float *__restrict__ pos,
                                                 const float *__restrict__ phase, const int *__restrict__ cnt,
                                                 const int *__restrict__ need, int max_pc, int nbp,
                                                 long long *__restrict__ pl, long long *__restrict__ pg,
                                                 long long *__restrict__ cl, long long *__restrict__ cg) {
    const bool parts = (int)blockIdx.x < nbp;
    const long long b = parts ? blockIdx.x : blockIdx.x - nbp;
    const long long first = b * RS_CHUNK + (threadIdx.x >> 5) * RS_WARP_ITEMS + (threadIdx.x & 31);
    const long long nc = (long long)g.nx * g.ny * g.nz;
    long long ml = 0, mg = 0;
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const long long x = first + 32 * r;
        if (parts) {
            if (x < n && tp_over(g, pos, x, cnt, max_pc)) {
                if (phase[x] > 0.5f) ++ml;
                else ++mg;
            }
        } else if (x < nc) {
            const int q = need[x];
            ml += q > 0 ? q : 0;
            mg += q < 0 ? -q : 0;
        }
    }
    long long oa, ob, ta, tb;
    rs_warp_offset2(rs_warp_sum(ml), rs_warp_sum(mg), oa, ob, ta, tb);
    if (threadIdx.x == 0) {
        (parts ? pl : cl)[b] = ta;
        (parts ? pg : cg)[b] = tb;
    }
}

// scatterDonorsKernel (:1331-1355): liquid rank r -> pool[r], gas rank r ->
// pool[top - r], ranks at or past pool_half dropped
__global__ void __launch_bounds__(256) k_tp_scatter(G3 g, long long n, const float *__restrict__ pos,
                                                    const float *__restrict__ phase, const int *__restrict__ cnt,
                                                    int max_pc, const long long *__restrict__ pl,
                                                    const long long *__restrict__ pg, long long pool_half,
                                                    long long top, int *__restrict__ pool) {
    const int lane = threadIdx.x & 31;
    const long long first = blockIdx.x * (long long)RS_CHUNK + (threadIdx.x >> 5) * RS_WARP_ITEMS;
    unsigned bl[RS_ROUNDS], bg[RS_ROUNDS];
    long long ml = 0, mg = 0;
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const long long x = first + 32 * r + lane;
        const bool over = x < n && tp_over(g, pos, x, cnt, max_pc);
        const bool liq = over && phase[x] > 0.5f;
        bl[r] = __ballot_sync(0xffffffffu, liq);
        bg[r] = __ballot_sync(0xffffffffu, over && !liq);
        ml += __popc(bl[r]);
        mg += __popc(bg[r]);
    }
    long long oa, ob, ta, tb;
    rs_warp_offset2(ml, mg, oa, ob, ta, tb);
    long long rl = pl[blockIdx.x] + oa, rg = pg[blockIdx.x] + ob;
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const int p = (int)(first + 32 * r + lane);
        if ((bl[r] >> lane) & 1u) {
            const long long k = rl + __popc(bl[r] & below);
            if (k < pool_half) pool[k] = p;
        }
        if ((bg[r] >> lane) & 1u) {
            const long long k = rg + __popc(bg[r] & below);
            if (k < pool_half) pool[top - k] = p;
        }
        rl += __popc(bl[r]);
        rg += __popc(bg[r]);
    }
}

__device__ __forceinline__ long long warp_excl_scan(long long v, long long &total) {
    const int lane = threadIdx.x & 31;
    long long s = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += t;
    }
    total = __shfl_sync(0xffffffffu, s, 31);
    return s - v;
}

// claimDonorsKernel (:1453-1478) with buildClaimLoop (:1403-1451): a cell's
// slots in its phase's pool start at that phase's need before it; slots
// below min(donors, pool_half) move the donor to the cell centre with the
// face-centred velocity there
__global__ void __launch_bounds__(256) k_tp_claim(G3 g, const int *__restrict__ need,
                                                  const long long *__restrict__ cl, const long long *__restrict__ cg,
                                                  const long long *__restrict__ tot, long long pool_half, long long top,
                                                  const int *__restrict__ pool, const float *__restrict__ u,
                                                  const float *__restrict__ v, const float *__restrict__ w,
                                                  float *__restrict__ pos, float *__restrict__ vel) {
    const int lane = threadIdx.x & 31;
    const long long plane = (long long)g.nx * g.ny, nc = plane * g.nz;
    const long long first = blockIdx.x * (long long)RS_CHUNK + (threadIdx.x >> 5) * RS_WARP_ITEMS + lane;
    int q[RS_ROUNDS];
    long long ml = 0, mg = 0;
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const long long x = first + 32 * r;
        q[r] = x < nc ? need[x] : 0;
        ml += q[r] > 0 ? q[r] : 0;
        mg += q[r] < 0 ? -q[r] : 0;
    }
    long long oa, ob, ta, tb;
    rs_warp_offset2(rs_warp_sum(ml), rs_warp_sum(mg), oa, ob, ta, tb);
    if (ta == 0 && tb == 0) return;
    long long rl = cl[blockIdx.x] + oa, rg = cg[blockIdx.x] + ob;
    const long long avail_l = tot[0] < pool_half ? tot[0] : pool_half;
    const long long avail_g = tot[2] < pool_half ? tot[2] : pool_half;
    const float *comp[3] = {u, v, w};
#pragma unroll
    for (int r = 0; r < RS_ROUNDS; ++r) {
        const long long nl = q[r] > 0 ? q[r] : 0, ng = q[r] < 0 ? -q[r] : 0;
        long long tl, tg;
        const long long sl = rl + warp_excl_scan(nl, tl), sg = rg + warp_excl_scan(ng, tg);
        rl += tl;
        rg += tg;
        if (q[r] == 0) continue;
        const bool liquid = q[r] > 0;
        const long long needed = liquid ? nl : ng, slot0 = liquid ? sl : sg, avail = liquid ? avail_l : avail_g;
        if (slot0 >= avail) continue;
        const long long c = first + 32 * r;
        const int k = (int)(c / plane);
        const long long rem = c - (long long)k * plane;
        const int j = (int)(rem / g.nx), i = (int)(rem - (long long)j * g.nx);
        F3 qp = index_pos(g, comp_origin(g, 3), i, j, k);
        float vq[3];
        for (int a = 0; a < 3; ++a) {
            int sx, sy, sz;
            comp_shape(g, a, sx, sy, sz);
            vq[a] = trilinear(comp[a], sx, sy, sz, g, comp_origin(g, a), qp);
        }
        for (long long m = 0; m < needed && slot0 + m < avail; ++m) {
            const long long d = pool[liquid ? slot0 + m : top - (slot0 + m)];
            pos[3 * d] = qp.x;
            pos[3 * d + 1] = qp.y;
            pos[3 * d + 2] = qp.z;
            vel[3 * d] = vq[0];
            vel[3 * d + 1] = vq[1];
            vel[3 * d + 2] = vq[2];
        }
    }
}

int blocks_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16)); }

int post(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return ff_set_error(FF_E_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
    return FF_OK;
}

// mulberry32 (jitter_random.js:29-41)
struct Mulberry32 {
    uint32_t state;
    double next() {
        state = state + 0x6D2B79F5u;
        uint32_t t = state;
        t = (t ^ (t >> 15)) * (t | 1u);
        t ^= t + (t ^ (t >> 7)) * (t | 61u);
        return (double)(t ^ (t >> 14)) / 4294967296.0;
    }
};

}  // namespace

// ------------------------------------------------------------- host side --
extern "C" int ff_jitter_random(uint32_t seed, int n, double *out) {
    FF_CHECK(n >= 0 && (n == 0 || out), FF_E_ARG, "ff_jitter_random: bad arguments");
    Mulberry32 r{seed};
    for (int q = 0; q < n; ++q) out[q] = r.next();
    return FF_OK;
}

extern "C" int ff_flip_box_seed3(const double *bmin, const double *bmax, const double *h, int per_axis, double jitter,
                                 uint32_t seed, float *positions, int64_t capacity, int64_t *count) {
    FF_CHECK(bmin && bmax && h && count && per_axis > 0, FF_E_ARG, "computeFlipBoxSeed3: bad arguments");
    long long cells[3];
    double sub[3];
    for (int a = 0; a < 3; ++a) {
        const double c = std::floor((bmax[a] - bmin[a]) / h[a] + 0.5);   // Math.round
        cells[a] = c < 1 ? 1 : (long long)c;
        sub[a] = h[a] / per_axis;
    }
    const long long total = cells[0] * cells[1] * cells[2] * per_axis * per_axis * per_axis;
    *count = total;
    if (!positions) return FF_OK;
    FF_CHECK(capacity >= total, FF_E_LIMIT, "computeFlipBoxSeed3: %lld particles exceed the capacity %lld", total,
             (long long)capacity);
    Mulberry32 r{seed};
    long long n = 0;
    for (long long ck = 0; ck < cells[2]; ++ck)
        for (long long cj = 0; cj < cells[1]; ++cj)
            for (long long ci = 0; ci < cells[0]; ++ci)
                for (int sk = 0; sk < per_axis; ++sk)
                    for (int sj = 0; sj < per_axis; ++sj)
                        for (int si = 0; si < per_axis; ++si) {
                            const double jx = (r.next() * 2 - 1) * jitter * sub[0];
                            const double jy = (r.next() * 2 - 1) * jitter * sub[1];
                            const double jz = (r.next() * 2 - 1) * jitter * sub[2];
                            positions[3 * n] = (float)(bmin[0] + (double)ci * h[0] + (si + 0.5) * sub[0] + jx);
                            positions[3 * n + 1] = (float)(bmin[1] + (double)cj * h[1] + (sj + 0.5) * sub[1] + jy);
                            positions[3 * n + 2] = (float)(bmin[2] + (double)ck * h[2] + (sk + 0.5) * sub[2] + jz);
                            ++n;
                        }
    return FF_OK;
}

extern "C" void ff_flip_desc_default(ff_flip_desc *d, const int *res, const double *h, int max_particles, double dt) {
    std::memset(d, 0, sizeof *d);
    for (int a = 0; a < 3; ++a) {
        d->resolution[a] = res ? res[a] : 1;
        d->grid_spacing[a] = h ? h[a] : 1.0;
    }
    d->max_particles = max_particles;
    d->dt = dt;
    d->gravity[1] = -9.81;
    d->reduced_pressure = 1;
    d->flip_ratio = 0.97;
    d->velocity_damping = 0.02;
    d->p2g_atomic_scale = 65536.0;
    d->weight_epsilon = 1e-4;
    d->closed_flags = FF_DIRECTION_ALL_3D;
    d->max_substeps = 32;
    d->concentration_atomic_scale = 4096.0;
    d->extrapolation_depth = 5;
    d->resample_enabled = 1;   // resample defaults (:178-180)
    d->min_particles_per_cell = 4;
    d->max_particles_per_cell = 8;
    ff_pressure_desc_default(&d->pressure, res, h);
    d->pressure.max_plausible_pressure = 0.0;   // derived from dt, gravity and the domain
}

struct ff_flip_s {
    ff_ctx ctx = nullptr;
    ff_flip_desc desc{};
    G3 g{};
    int count = 0;
    ff_field u = nullptr, v = nullptr, w = nullptr;   // the velocity grid (borrowed)
    ff_field phi = nullptr;                           // collider (borrowed)
    ff_field pos = nullptr, vel = nullptr, conc = nullptr, mask = nullptr, active = nullptr, target = nullptr;
    ff_field cell_conc = nullptr, cell_rho = nullptr, beta[3] = {};
    float *old[3] = {};
    int *num[3] = {}, *den[3] = {}, *valid[3] = {}, *adj[3] = {}, *vtmp[2][3] = {};
    float *scratch[3] = {};
    int *ccnt = nullptr, *cacc = nullptr;
    // resampling: per-cell counts, the donor pool, block totals (particle
    // blocks then cell blocks) and the two totals
    int *rs_cnt = nullptr, *rs_pool = nullptr;
    long long *rs_bsum = nullptr, *rs_tot = nullptr;
    int rs_nbp = 0;
    ff_bc bc = nullptr;
    ff_advect adv = nullptr;
    ff_pressure ps = nullptr;
    bool density = false;
    float r0 = 0, r1 = 0, rref = 1;
    ff_diag last{};
};

static long long comp_n(const G3 &g, int a) {
    if (a == 3) return (long long)g.nx * g.ny * g.nz;
    int sx, sy, sz;
    comp_shape(g, a, sx, sy, sz);
    return (long long)sx * sy * sz;
}

extern "C" int ff_flip3_destroy(ff_flip f) {
    if (!f) return FF_OK;
    cudaStreamSynchronize(f->ctx->stream);
    ff_pressure3_destroy(f->ps);
    ff_advect3_destroy(f->adv);
    ff_bc3_destroy(f->bc);
    ff_field fs[] = {f->pos, f->vel, f->conc, f->mask, f->active, f->target, f->cell_conc, f->cell_rho,
                     f->beta[0], f->beta[1], f->beta[2]};
    for (ff_field x : fs) ff_field_destroy(x);
    for (int a = 0; a < 3; ++a) {
        ff_dev_free(f->old[a]);
        ff_dev_free(f->num[a]);
        ff_dev_free(f->den[a]);
        ff_dev_free(f->valid[a]);
        ff_dev_free(f->adj[a]);
        ff_dev_free(f->vtmp[0][a]);
        ff_dev_free(f->vtmp[1][a]);
        ff_dev_free(f->scratch[a]);
    }
    ff_dev_free(f->ccnt);
    ff_dev_free(f->cacc);
    ff_dev_free(f->rs_cnt);
    ff_dev_free(f->rs_pool);
    ff_dev_free(f->rs_bsum);
    ff_dev_free(f->rs_tot);
    delete f;
    return FF_OK;
}

extern "C" int ff_flip3_create(ff_ctx ctx, const ff_flip_desc *d, ff_field u, ff_field v, ff_field w, ff_flip *out) {
    FF_CHECK(ctx && d && out, FF_E_ARG, "ff_flip3_create: NULL argument");
    FF_CHECK(d->max_particles > 0, FF_E_ARG, "createGridFlipSolver3: options.maxParticles is required.");
    FF_CHECK(d->max_substeps > 0, FF_E_ARG, "createGridFlipSolver3: maxSubsteps must be positive");
    FF_TRY(check_grid32(d->resolution, "createGridFlipSolver3"));
    const bool density = d->ambient_density != 0.0 || d->component_density != 0.0;
    FF_CHECK(!density || d->carry_concentration, FF_E_ARG,
             "createGridFlipSolver3: ambientDensity/componentDensity require carryConcentration: true -- there is no "
             "concentration field to build a density from otherwise.");
    FF_CHECK(!density || (d->ambient_density > 0 && d->component_density > 0), FF_E_ARG,
             "createGridFlipSolver3: ambientDensity and componentDensity must be > 0.");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    ff_flip f = new ff_flip_s();
    f->ctx = ctx;
    f->desc = *d;
    f->g.nx = d->resolution[0];
    f->g.ny = d->resolution[1];
    f->g.nz = d->resolution[2];
    f->g.hx = (float)d->grid_spacing[0];
    f->g.hy = (float)d->grid_spacing[1];
    f->g.hz = (float)d->grid_spacing[2];
    f->g.ox = (float)d->origin[0];
    f->g.oy = (float)d->origin[1];
    f->g.oz = (float)d->origin[2];
    for (int a = 0; a < 3; ++a) {
        ff_field x = a == 0 ? u : (a == 1 ? v : w);
        if (!x || x->dtype != FF_FLOAT || x->count != comp_n(f->g, a)) {
            delete f;
            return ff_set_error(FF_E_ARG, "createGridFlipSolver3: velocity component %d has the wrong shape", a);
        }
    }
    f->u = u;
    f->v = v;
    f->w = w;
    f->count = d->max_particles;
    f->density = density;
    cudaStream_t s = ctx->stream;
    int st = FF_OK;
    auto bail = [&](int code) { ff_flip3_destroy(f); return code; };
    const int np[1] = {d->max_particles};
    const int cs[3] = {f->g.nx, f->g.ny, f->g.nz};
    if ((st = ff_field_create(ctx, FF_VEC3, 1, np, &f->pos))) return bail(st);
    if ((st = ff_field_create(ctx, FF_VEC3, 1, np, &f->vel))) return bail(st);
    if (d->carry_concentration && (st = ff_field_create(ctx, FF_FLOAT, 1, np, &f->conc))) return bail(st);
    if ((st = ff_field_create(ctx, FF_FLOAT, 3, cs, &f->mask))) return bail(st);
    if ((st = ff_field_create(ctx, FF_UINT8, 3, cs, &f->active))) return bail(st);
    if ((st = ff_field_create(ctx, FF_FLOAT, 3, cs, &f->target))) return bail(st);
    if (d->carry_concentration) {
        if ((st = ff_field_create(ctx, FF_FLOAT, 3, cs, &f->cell_conc))) return bail(st);
        if ((st = ff_field_create(ctx, FF_FLOAT, 3, cs, &f->cell_rho))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->ccnt, (size_t)comp_n(f->g, 3) * 4, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->cacc, (size_t)comp_n(f->g, 3) * 4, s))) return bail(st);
    }
    for (int a = 0; a < 3; ++a) {
        const size_t b = (size_t)comp_n(f->g, a) * 4;
        if ((st = ff_dev_alloc((void **)&f->old[a], b, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->num[a], b, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->den[a], b, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->valid[a], b, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->adj[a], b, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->vtmp[0][a], b, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->vtmp[1][a], b, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->scratch[a], b, s))) return bail(st);
        if (density) {
            const int fs3[3] = {f->g.nx + (a == 0), f->g.ny + (a == 1), f->g.nz + (a == 2)};
            if ((st = ff_field_create(ctx, FF_FLOAT, 3, fs3, &f->beta[a]))) return bail(st);
            if ((st = ff_field_fill(f->beta[a], 1.0f))) return bail(st);
        }
    }
    if (d->resample_enabled) {
        const long long nc = comp_n(f->g, 3);
        f->rs_nbp = (int)(((long long)d->max_particles + RS_CHUNK - 1) / RS_CHUNK);
        const long long nb = f->rs_nbp + (nc + RS_CHUNK - 1) / RS_CHUNK;
        if ((st = ff_dev_alloc((void **)&f->rs_cnt, (size_t)nc * 4, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->rs_pool, (size_t)d->max_particles * 4, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->rs_bsum, (size_t)nb * 8, s))) return bail(st);
        if ((st = ff_dev_alloc((void **)&f->rs_tot, 16, s))) return bail(st);
        if (cudaMemsetAsync(f->rs_tot, 0, 16, s) != cudaSuccess) return bail(ff_set_error(FF_E_CUDA, "flip create"));
    }
    if (density) {
        f->r0 = std::max((float)d->ambient_density, MIN_DENSITY);
        f->r1 = std::max((float)d->component_density, MIN_DENSITY);
        f->rref = std::max(f->r0, f->r1);
    }
    // boundary solver (no collider face weights), advection (trace), pressure
    if ((st = ff_bc3_create(ctx, d->resolution, d->grid_spacing, d->origin, &f->bc))) return bail(st);
    if ((st = ff_bc3_set_closed(f->bc, d->closed_flags))) return bail(st);
    ff_advect_desc ad{};
    for (int a = 0; a < 3; ++a) {
        ad.resolution[a] = d->resolution[a];
        ad.grid_spacing[a] = d->grid_spacing[a];
        ad.origin[a] = d->origin[a];
    }
    ad.dt = d->dt;
    ad.max_substeps = d->max_substeps;
    ad.order = 1;
    if ((st = ff_advect3_create(ctx, &ad, &f->adv))) return bail(st);
    ff_pressure_desc pd = d->pressure;
    for (int a = 0; a < 3; ++a) {
        pd.resolution[a] = d->resolution[a];
        pd.grid_spacing[a] = d->grid_spacing[a];
        pd.origin[a] = d->origin[a];
    }
    if (!(pd.max_plausible_pressure > 0)) {
        // derivedMaxPlausiblePressure (:361-366), in doubles as the reference
        const double gm = std::hypot(std::hypot(d->gravity[0], d->gravity[1]), d->gravity[2]);
        const double ext = d->resolution[0] * d->grid_spacing[0] + d->resolution[1] * d->grid_spacing[1] +
                           d->resolution[2] * d->grid_spacing[2];
        pd.max_plausible_pressure =
            (d->reduced_pressure && gm > 0) ? PRESSURE_BOUND_HEADROOM * d->dt * gm * ext : 1e6;
    }
    if ((st = ff_pressure3_create(ctx, &pd, &f->ps))) return bail(st);
    if ((st = ff_pressure3_set_dirichlet(f->ps, f->active, f->target))) return bail(st);
    if (density && (st = ff_pressure3_set_face_weights(f->ps, f->beta[0], f->beta[1], f->beta[2]))) return bail(st);
    if (cudaStreamSynchronize(s) != cudaSuccess) return bail(ff_set_error(FF_E_CUDA, "flip create sync"));
    *out = f;
    return FF_OK;
}

extern "C" int ff_flip3_set_collider(ff_flip f, ff_field phi) {
    FF_CHECK(f, FF_E_ARG, "NULL FLIP solver");
    FF_CHECK(!phi || (phi->dtype == FF_FLOAT && phi->count == comp_n(f->g, 3)), FF_E_ARG,
             "FLIP collider must be a float cell SDF");
    f->phi = phi;
    FF_TRY(ff_bc3_set_collider(f->bc, phi, nullptr, nullptr, nullptr));
    return ff_advect3_set_collider(f->adv, phi);
}

extern "C" int ff_flip3_set_count(ff_flip f, int n) {
    FF_CHECK(f && n >= 0 && n <= f->desc.max_particles, FF_E_ARG, "FLIP particle count out of range");
    f->count = n;
    return FF_OK;
}

extern "C" int ff_flip3_fields(ff_flip f, ff_field *positions, ff_field *velocities, ff_field *concentration,
                               ff_field *fluid_mask, ff_pressure *pressure) {
    FF_CHECK(f, FF_E_ARG, "NULL FLIP solver");
    if (positions) *positions = f->pos;
    if (velocities) *velocities = f->vel;
    if (concentration) *concentration = f->conc;
    if (fluid_mask) *fluid_mask = f->mask;
    if (pressure) *pressure = f->ps;
    return FF_OK;
}

extern "C" int ff_flip3_grid_fields(ff_flip f, ff_field *cell_concentration, ff_field *cell_density, ff_field *beta_u,
                                    ff_field *beta_v, ff_field *beta_w, ff_field *dirichlet_active,
                                    ff_field *dirichlet_target) {
    FF_CHECK(f, FF_E_ARG, "NULL FLIP solver");
    if (cell_concentration) *cell_concentration = f->cell_conc;
    if (cell_density) *cell_density = f->density ? f->cell_rho : nullptr;
    if (beta_u) *beta_u = f->beta[0];
    if (beta_v) *beta_v = f->beta[1];
    if (beta_w) *beta_w = f->beta[2];
    if (dirichlet_active) *dirichlet_active = f->active;
    if (dirichlet_target) *dirichlet_target = f->target;
    return FF_OK;
}

static int extrapolate(ff_flip f, float *data, const int *marker, int a) {
    cudaStream_t s = f->ctx->stream;
    int sx, sy, sz;
    comp_shape(f->g, a, sx, sy, sz);
    const long long n = comp_n(f->g, a);
    FF_CUDA(cudaMemcpyAsync(f->vtmp[0][a], marker, n * 4, cudaMemcpyDeviceToDevice, s));
    float *src = data, *dst = f->scratch[a];
    int *vs = f->vtmp[0][a], *vd = f->vtmp[1][a];
    for (int it = 0; it < f->desc.extrapolation_depth; ++it) {
        k_extrapolate<<<blocks_for(n), 256, 0, s>>>(sx, sy, sz, src, dst, vs, vd);
        std::swap(src, dst);
        std::swap(vs, vd);
    }
    if (src != data) FF_CUDA(cudaMemcpyAsync(data, src, n * 4, cudaMemcpyDeviceToDevice, s));
    return post("extrapolate");
}

// One stage of onAdvanceTimeStep (:1110-1150).
extern "C" int ff_flip3_stage(ff_flip f, int stage) {
    FF_CHECK(f, FF_E_ARG, "NULL FLIP solver");
    cudaSetDevice(f->ctx->device);
    cudaStream_t s = f->ctx->stream;
    const ff_flip_desc &d = f->desc;
    const G3 &g = f->g;
    const long long n = f->count;
    float *uvw[3] = {(float *)f->u->d, (float *)f->v->d, (float *)f->w->d};
    float *pos = (float *)f->pos->d, *vel = (float *)f->vel->d;
    const F3 grav{(float)d.gravity[0], (float)d.gravity[1], (float)d.gravity[2]};
    switch (stage) {
    case FF_FLIP_ADVECT_PARTICLES: {
        if (n == 0) return FF_OK;
        VelField F{g, uvw[0], uvw[1], uvw[2], f->phi ? (const float *)f->phi->d : nullptr};
        // minPos / maxPos (:927-929): the extent in doubles, stored as f32
        const F3 ext{(float)(d.resolution[0] * d.grid_spacing[0]), (float)(d.resolution[1] * d.grid_spacing[1]),
                     (float)(d.resolution[2] * d.grid_spacing[2])};
        const F3 mn{g.ox + 1e-4f, g.oy + 1e-4f, g.oz + 1e-4f};
        const F3 mx{(g.ox + ext.x) - 1e-4f, (g.oy + ext.y) - 1e-4f, (g.oz + ext.z) - 1e-4f};
        k_flip_advect<<<blocks_for(n), 256, 0, s>>>(F, n, pos, (float)d.dt, d.max_substeps, mn, mx,
                                                    (float)d.collider_push_thresh, (float)d.collider_push_shift, 0);
        return post("advectParticles");
    }
    case FF_FLIP_P2G: {
        for (int a = 0; a < 3; ++a) {
            FF_CUDA(cudaMemsetAsync(f->num[a], 0, comp_n(g, a) * 4, s));
            FF_CUDA(cudaMemsetAsync(f->den[a], 0, comp_n(g, a) * 4, s));
        }
        const float S = (float)d.p2g_atomic_scale;
        if (n) k_flip_scatter<<<blocks_for(n), 256, 0, s>>>(g, n, pos, vel, S, f->num[0], f->den[0], f->num[1],
                                                            f->den[1], f->num[2], f->den[2], 3);
        for (int a = 0; a < 3; ++a)
            k_flip_finalize<<<blocks_for(comp_n(g, a)), 256, 0, s>>>(comp_n(g, a), f->num[a], f->den[a], S,
                                                                     (float)d.weight_epsilon, uvw[a], f->valid[a]);
        return post("P2G");
    }
    case FF_FLIP_SNAPSHOT:
        for (int a = 0; a < 3; ++a)
            FF_CUDA(cudaMemcpyAsync(f->old[a], uvw[a], comp_n(g, a) * 4, cudaMemcpyDeviceToDevice, s));
        return FF_OK;
    case FF_FLIP_EXTRAPOLATE_WEIGHT:
        for (int a = 0; a < 3; ++a) FF_TRY(extrapolate(f, uvw[a], f->valid[a], a));
        return FF_OK;
    case FF_FLIP_CONSTRAIN:
        return ff_bc3_constrain(f->bc, f->u, f->v, f->w, d.extrapolation_depth);
    case FF_FLIP_MARK_FLUID:
        FF_CUDA(cudaMemsetAsync(f->mask->d, 0, comp_n(g, 3) * 4, s));
        if (n) k_flip_mark<<<blocks_for(n), 256, 0, s>>>(g, n, pos, (float *)f->mask->d);
        for (int a = 0; a < 3; ++a)
            k_flip_adjacent<<<blocks_for(comp_n(g, a)), 256, 0, s>>>(g, a, (const float *)f->mask->d, f->adj[a]);
        return post("markFluidCells");
    case FF_FLIP_CONCENTRATION_GRID: {
        if (!d.carry_concentration) return FF_OK;
        const long long nc = comp_n(g, 3);
        FF_CUDA(cudaMemsetAsync(f->ccnt, 0, nc * 4, s));
        FF_CUDA(cudaMemsetAsync(f->cacc, 0, nc * 4, s));
        const float cscale = (float)d.concentration_atomic_scale;
        if (n) k_flip_conc_accum<<<blocks_for(n), 256, 0, s>>>(g, n, pos, (const float *)f->conc->d, cscale, f->ccnt,
                                                               f->cacc);
        k_flip_conc_resolve<<<blocks_for(nc), 256, 0, s>>>(nc, f->ccnt, f->cacc, cscale, f->density, f->r0, f->r1,
                                                           (float *)f->cell_conc->d, (float *)f->cell_rho->d);
        if (f->density)
            for (int a = 0; a < 3; ++a)
                k_flip_beta<<<blocks_for(comp_n(g, a)), 256, 0, s>>>(g, a, (const float *)f->cell_rho->d,
                                                                     (const float *)f->mask->d, f->rref,
                                                                     (float *)f->beta[a]->d);
        return post("concentration");
    }
    case FF_FLIP_GRAVITY:
        // reduced pressure puts gravity in the air cells' Dirichlet target;
        // with the density coupling the grid still takes the beta term
        if (d.reduced_pressure && !f->density) return FF_OK;
        for (int a = 0; a < 3; ++a)
            k_flip_gravity<<<blocks_for(comp_n(g, a)), 256, 0, s>>>(
                g, a, f->density ? (const float *)f->cell_rho->d : nullptr,
                (d.reduced_pressure && f->density) ? (const float *)f->beta[a]->d : nullptr, grav, (float)d.dt,
                f->rref, uvw[a]);
        return post("gravity");
    case FF_FLIP_PROJECT: {
        k_flip_dirichlet<<<blocks_for(comp_n(g, 3)), 256, 0, s>>>(g, (const float *)f->mask->d, grav, (float)d.dt,
                                                                  d.reduced_pressure, (uint8_t *)f->active->d,
                                                                  (float *)f->target->d);
        FF_TRY(post("dirichlet"));
        return ff_pressure3_project(f->ps, f->u, f->v, f->w, f->u, f->v, f->w, &f->last);
    }
    case FF_FLIP_EXTRAPOLATE_PRESSURE:
        for (int a = 0; a < 3; ++a) FF_TRY(extrapolate(f, uvw[a], f->adj[a], a));
        return FF_OK;
    case FF_FLIP_G2P:
        if (n) k_flip_g2p<<<blocks_for(n), 256, 0, s>>>(g, n, pos, vel, uvw[0], uvw[1], uvw[2], f->old[0], f->old[1],
                                                        f->old[2], (float)d.flip_ratio,
                                                        std::min(std::max((float)d.velocity_damping, 0.0f), 1.0f),
                                                        nullptr, 0.0f);
        return post("G2P");
    case FF_FLIP_CONCENTRATION_PARTICLE:
        if (!d.carry_concentration || !n) return FF_OK;
        k_flip_mix_fade<<<blocks_for(n), 256, 0, s>>>(g, n, pos, (const float *)f->cell_conc->d,
                                                      std::min(std::max((float)d.mixing, 0.0f), 1.0f),
                                                      std::min(std::max((float)d.fade, 0.0f), 1.0f),
                                                      (float *)f->conc->d);
        return post("mixAndFade");
    case FF_FLIP_RESAMPLE: {
        // resamplePass (:813-816): counts, donors, needs, claims, then the
        // fluid mask and face adjacency again (:806-810)
        if (!d.resample_enabled) return FF_OK;
        const long long nc = comp_n(g, 3);
        const int nbp = (int)((n + RS_CHUNK - 1) / RS_CHUNK), nbc = (int)((nc + RS_CHUNK - 1) / RS_CHUNK);
        long long *bsum_c = f->rs_bsum + f->rs_nbp;
        FF_CUDA(cudaMemsetAsync(f->rs_cnt, 0, nc * 4, s));
        if (n) k_rs_count<<<blocks_for(n), 256, 0, s>>>(g, n, pos, f->rs_cnt);
        k_rs_sums<<<nbp + nbc, 256, 0, s>>>(g, n, pos, f->rs_cnt, d.min_particles_per_cell,
                                            d.max_particles_per_cell, nbp, f->rs_bsum, bsum_c);
        k_rs_scan<<<1, 1024, 0, s>>>(f->rs_bsum, nbp, bsum_c, nbc, f->rs_tot);
        if (nbp) k_rs_scatter<<<nbp, 256, 0, s>>>(g, n, pos, f->rs_cnt, d.max_particles_per_cell, f->rs_bsum,
                                                  f->rs_pool);
        k_rs_claim<<<nbc, 256, 0, s>>>(g, f->rs_cnt, d.min_particles_per_cell, bsum_c, f->rs_tot, f->rs_pool,
                                       uvw[0], uvw[1], uvw[2], pos, vel);
        FF_TRY(post("resample"));
        return ff_flip3_stage(f, FF_FLIP_MARK_FLUID);
    }
    default:
        return ff_set_error(FF_E_ARG, "ff_flip3_stage: unknown stage %d", stage);
    }
}

// onAdvanceTimeStep (:1137-1144): pre-P2G, P2G and grid stages (resampling
// after the fluid mask, :1087-1093), the projection, then the
// post-projection stages.
extern "C" int ff_flip3_step(ff_flip f, ff_diag *diag) {
    FF_CHECK(f, FF_E_ARG, "NULL FLIP solver");
    static const int order[] = {FF_FLIP_ADVECT_PARTICLES, FF_FLIP_P2G,         FF_FLIP_SNAPSHOT,
                                FF_FLIP_EXTRAPOLATE_WEIGHT, FF_FLIP_CONSTRAIN,   FF_FLIP_MARK_FLUID,
                                FF_FLIP_RESAMPLE,           FF_FLIP_CONCENTRATION_GRID, FF_FLIP_GRAVITY,
                                FF_FLIP_CONSTRAIN,
                                FF_FLIP_PROJECT,            FF_FLIP_CONSTRAIN,   FF_FLIP_EXTRAPOLATE_PRESSURE,
                                FF_FLIP_G2P,                FF_FLIP_CONCENTRATION_PARTICLE};
    for (int st : order) FF_TRY(ff_flip3_stage(f, st));
    if (diag) *diag = f->last;
    return FF_OK;
}

extern "C" int ff_flip3_resample_stats(ff_flip f, int64_t *donors, int64_t *requested) {
    FF_CHECK(f, FF_E_ARG, "NULL FLIP solver");
    long long t[2] = {0, 0};
    if (f->rs_tot) {
        cudaSetDevice(f->ctx->device);
        FF_CUDA(cudaMemcpyAsync(t, f->rs_tot, sizeof t, cudaMemcpyDeviceToHost, f->ctx->stream));
        FF_CUDA(cudaStreamSynchronize(f->ctx->stream));
    }
    if (donors) *donors = t[0];
    if (requested) *requested = t[1];
    return FF_OK;
}

// ----------------------------------------------------------- two-phase 2D --
// createGridTwoPhaseFlipSolver2 (src/grid/grid_two_phase_flip_solver2.js:
// 479-1622) on a one-cell-thick 3D grid: the 2D u and v arrays are the
// k = 0 planes of (nx+1, ny, 1) and (nx, ny+1, 1) face arrays, particles
// sit on the plane z = hz/2 through the cell centres, and the z velocity is
// an internal zero field.  With those, every z term of the 3D kernels is an
// exact +0 or x1 and they compute the 2D expressions operation for
// operation (bilinear = trilinear at fz = 0; hz = max(hx, hy) keeps the
// trace's min spacing).  Every cell is fluid; the pressure is pinned to 0
// at one cell (pressurePin, :767-797); beta = rho_max / face density
// (:750-762); gravity is uniform (:932-944); the FLIP/PIC blend follows the
// particle's concentration (:966-992); resampling keeps two pools by phase.
extern "C" void ff_twophase_desc_default(ff_twophase_desc *d, const int *res, const double *h, int max_particles,
                                         double dt) {
    std::memset(d, 0, sizeof *d);
    for (int a = 0; a < 2; ++a) {
        d->resolution[a] = res ? res[a] : 1;
        d->grid_spacing[a] = h ? h[a] : 1.0;
    }
    d->max_particles = max_particles;
    d->dt = dt;
    d->gravity[1] = -9.81;
    d->ambient_density = 0.01;   // gasDensity (:496)
    d->component_density = 1.0;  // liquidDensity (:495)
    d->concentration_atomic_scale = 4096.0;
    d->flip_ratio = 0.97;
    d->gas_flip_ratio = 0.90;
    d->velocity_damping = 0.02;
    d->p2g_atomic_scale = 65536.0;
    d->weight_epsilon = 1e-4;
    d->closed_flags = 15;   // DIRECTION_ALL in 2D
    d->max_substeps = 32;
    d->pin_cell[0] = d->resolution[0] / 2;   // 'topCenter' (:770-772)
    d->pin_cell[1] = d->resolution[1] - 1;
    d->resample_enabled = 1;   // resample defaults (:535-539)
    d->min_particles_per_cell = 3;
    d->max_particles_per_cell = 8;
    d->extrapolation_depth = 5;
    const int r3[3] = {d->resolution[0], d->resolution[1], 1};
    const double h3[3] = {d->grid_spacing[0], d->grid_spacing[1], std::max(d->grid_spacing[0], d->grid_spacing[1])};
    ff_pressure_desc_default(&d->pressure, r3, h3);
    // defaultMultigridLevels (:372-384): deepest of up to 4 levels that
    // every axis divides into
    int levels = 1;
    while (levels < 4 && d->resolution[0] % (1 << levels) == 0 && d->resolution[1] % (1 << levels) == 0) ++levels;
    d->pressure.mg_levels = levels;
}

struct ff_twophase_s {
    ff_ctx ctx = nullptr;
    int dims = 2;                   // 2: the one-cell-thick stand-in of the 2D solver; 3: a full grid
    ff_twophase_desc desc{};        // the 2D solver's options as given
    ff_twophase3_desc d{};          // the options on three axes (the 2D ones with nz = 1)
    G3 g{};
    int count = 0;
    ff_field u = nullptr, v = nullptr, w = nullptr, phi = nullptr;   // borrowed (w owned in 2D)
    ff_field pos = nullptr, vel = nullptr, phase = nullptr, frac = nullptr, rho = nullptr, beta[3] = {};
    ff_field active = nullptr, target = nullptr;
    float *old[3] = {};
    int *num[3] = {}, *den[3] = {}, *valid[3] = {}, *vtmp[2][3] = {};
    float *scratch[3] = {};
    int *ccnt = nullptr, *cacc = nullptr;
    int *rs_need = nullptr, *rs_pool = nullptr;
    long long *rs_bsum = nullptr, *rs_tot = nullptr;
    int rs_nbp = 0, rs_nbc = 0;
    ff_bc bc = nullptr;
    ff_pressure ps = nullptr;
    float r0 = 0, r1 = 0, rref = 1;
    ff_diag last{};
};

extern "C" int ff_twophase2_destroy(ff_twophase t) {
    if (!t) return FF_OK;
    cudaStreamSynchronize(t->ctx->stream);
    ff_pressure3_destroy(t->ps);
    ff_bc3_destroy(t->bc);
    ff_field fs[] = {t->dims == 2 ? t->w : nullptr, t->pos, t->vel, t->phase, t->frac, t->rho, t->beta[0],
                     t->beta[1], t->beta[2], t->active, t->target};
    for (ff_field x : fs) ff_field_destroy(x);
    for (int a = 0; a < 3; ++a) {
        ff_dev_free(t->old[a]);
        ff_dev_free(t->num[a]);
        ff_dev_free(t->den[a]);
        ff_dev_free(t->valid[a]);
        ff_dev_free(t->vtmp[0][a]);
        ff_dev_free(t->vtmp[1][a]);
        ff_dev_free(t->scratch[a]);
    }
    void *ps[] = {t->ccnt, t->cacc, t->rs_need, t->rs_pool, t->rs_bsum, t->rs_tot};
    for (void *p : ps) ff_dev_free(p);
    delete t;
    return FF_OK;
}

// The buffers, boundary solver and pressure solver of a two-phase solver
// whose t->d, t->g, t->dims, t->u, t->v (and t->w in 3D) are set.
static int tp_setup(ff_twophase t) {
    ff_ctx ctx = t->ctx;
    const ff_twophase3_desc &d = t->d;
    FF_TRY(check_grid32(d.resolution, "createGridTwoPhaseFlipSolver"));
    const int nx = t->g.nx, ny = t->g.ny, nz = t->g.nz;
    t->count = d.max_particles;
    t->r0 = std::max((float)d.ambient_density, MIN_DENSITY);
    t->r1 = std::max((float)d.component_density, MIN_DENSITY);
    t->rref = std::max(t->r0, t->r1);
    cudaStream_t s = ctx->stream;
    int st = FF_OK;
    const int np[1] = {d.max_particles};
    const int cs[3] = {nx, ny, nz};
    const long long nc = (long long)nx * ny * nz;
    if (t->dims == 2) {
        const int ws[3] = {nx, ny, 2};
        if ((st = ff_field_create(ctx, FF_FLOAT, 3, ws, &t->w))) return st;
    }
    if ((st = ff_field_create(ctx, FF_VEC3, 1, np, &t->pos))) return st;
    if ((st = ff_field_create(ctx, FF_VEC3, 1, np, &t->vel))) return st;
    if ((st = ff_field_create(ctx, FF_FLOAT, 1, np, &t->phase))) return st;
    if ((st = ff_field_create(ctx, FF_FLOAT, 3, cs, &t->frac))) return st;
    if ((st = ff_field_create(ctx, FF_FLOAT, 3, cs, &t->rho))) return st;
    if ((st = ff_field_create(ctx, FF_UINT8, 3, cs, &t->active))) return st;
    if ((st = ff_field_create(ctx, FF_FLOAT, 3, cs, &t->target))) return st;
    if ((st = ff_field_fill(t->rho, (float)d.component_density))) return st;
    // particles start at rest at the origin corner (on the centre plane in
    // 2D), all gas until seeded (:599-606)
    {
        std::vector<float> p3((size_t)3 * d.max_particles, 0.0f);
        for (size_t p = 0; p < (size_t)d.max_particles; ++p) {
            p3[3 * p] = t->dims == 2 ? 0.0f : t->g.ox;
            p3[3 * p + 1] = t->dims == 2 ? 0.0f : t->g.oy;
            p3[3 * p + 2] = t->dims == 2 ? t->g.oz + t->g.hz * 0.5f : t->g.oz;
        }
        if ((st = ff_field_upload(t->pos, p3.data(), p3.size() * 4))) return st;
        if (cudaMemsetAsync(t->vel->d, 0, t->vel->bytes, s) != cudaSuccess ||
            cudaMemsetAsync(t->phase->d, 0, t->phase->bytes, s) != cudaSuccess)
            return ff_set_error(FF_E_CUDA, "twophase");
    }
    for (int a = 0; a < 3; ++a) {
        const int fs3[3] = {nx + (a == 0), ny + (a == 1), nz + (a == 2)};
        if ((st = ff_field_create(ctx, FF_FLOAT, 3, fs3, &t->beta[a]))) return st;
        if ((st = ff_field_fill(t->beta[a], 1.0f))) return st;
    }
    for (int a = 0; a < t->dims; ++a) {
        const size_t b = (size_t)comp_n(t->g, a) * 4;
        if ((st = ff_dev_alloc((void **)&t->old[a], b, s))) return st;
        if ((st = ff_dev_alloc((void **)&t->num[a], b, s))) return st;
        if ((st = ff_dev_alloc((void **)&t->den[a], b, s))) return st;
        if ((st = ff_dev_alloc((void **)&t->valid[a], b, s))) return st;
        if ((st = ff_dev_alloc((void **)&t->vtmp[0][a], b, s))) return st;
        if ((st = ff_dev_alloc((void **)&t->vtmp[1][a], b, s))) return st;
        if ((st = ff_dev_alloc((void **)&t->scratch[a], b, s))) return st;
    }
    if ((st = ff_dev_alloc((void **)&t->ccnt, (size_t)nc * 4, s))) return st;
    if ((st = ff_dev_alloc((void **)&t->cacc, (size_t)nc * 4, s))) return st;
    if (d.resample_enabled) {
        t->rs_nbp = (int)(((long long)d.max_particles + RS_CHUNK - 1) / RS_CHUNK);
        t->rs_nbc = (int)((nc + RS_CHUNK - 1) / RS_CHUNK);
        if ((st = ff_dev_alloc((void **)&t->rs_need, (size_t)nc * 4, s))) return st;
        if ((st = ff_dev_alloc((void **)&t->rs_pool, (size_t)d.max_particles * 4, s))) return st;
        if ((st = ff_dev_alloc((void **)&t->rs_bsum, (size_t)2 * (t->rs_nbp + t->rs_nbc) * 8, s))) return st;
        if ((st = ff_dev_alloc((void **)&t->rs_tot, 32, s))) return st;
        if (cudaMemsetAsync(t->rs_tot, 0, 32, s) != cudaSuccess) return ff_set_error(FF_E_CUDA, "twophase");
    }
    // the pressure pin as a Dirichlet cell at 0 (dirichletAt, :786-795)
    {
        std::vector<uint8_t> act((size_t)nc, 0);
        if (d.pin_cell[0] >= 0)
            act[(size_t)d.pin_cell[0] + (size_t)nx * (d.pin_cell[1] + (size_t)ny * d.pin_cell[2])] = 1;
        if ((st = ff_field_upload(t->active, act.data(), act.size()))) return st;
        if (cudaMemsetAsync(t->target->d, 0, (size_t)nc * 4, s) != cudaSuccess)
            return ff_set_error(FF_E_CUDA, "twophase");
    }
    const int r3[3] = {nx, ny, nz};
    const double h3[3] = {d.grid_spacing[0], d.grid_spacing[1], d.grid_spacing[2]};
    const double o3[3] = {d.origin[0], d.origin[1], d.origin[2]};
    if ((st = ff_bc3_create(ctx, r3, h3, o3, &t->bc))) return st;
    if ((st = ff_bc3_set_closed(t->bc, t->dims == 2 ? (d.closed_flags & 15) | 48 : d.closed_flags))) return st;
    ff_pressure_desc pd = d.pressure;
    for (int a = 0; a < 3; ++a) {
        pd.resolution[a] = r3[a];
        pd.grid_spacing[a] = h3[a];
        pd.origin[a] = o3[a];
    }
    if ((st = ff_pressure3_create(ctx, &pd, &t->ps))) return st;
    if ((st = ff_pressure3_set_dirichlet(t->ps, t->active, t->target))) return st;
    if ((st = ff_pressure3_set_face_weights(t->ps, t->beta[0], t->beta[1], t->dims == 3 ? t->beta[2] : nullptr)))
        return st;
    if (cudaStreamSynchronize(s) != cudaSuccess) return ff_set_error(FF_E_CUDA, "two-phase create sync");
    return FF_OK;
}

extern "C" int ff_twophase2_create(ff_ctx ctx, const ff_twophase_desc *d, ff_field u, ff_field v, ff_twophase *out) {
    FF_CHECK(ctx && d && out, FF_E_ARG, "ff_twophase2_create: NULL argument");
    FF_CHECK(d->max_particles > 0, FF_E_ARG, "createGridTwoPhaseFlipSolver2: options.maxParticles is required.");
    FF_CHECK(d->resolution[0] > 0 && d->resolution[1] > 0, FF_E_ARG, "createGridTwoPhaseFlipSolver2: bad resolution");
    FF_CHECK(d->component_density > 0, FF_E_ARG,
             "createGridTwoPhaseFlipSolver2: the concentration-1 density (liquidDensity / componentDensity) must be "
             "> 0, got %g.", d->component_density);
    FF_CHECK(d->ambient_density > 0, FF_E_ARG,
             "createGridTwoPhaseFlipSolver2: the concentration-0 density (gasDensity / ambientDensity) must be > 0, "
             "got %g.", d->ambient_density);
    FF_CHECK(d->pin_cell[0] < 0 || (d->pin_cell[0] < d->resolution[0] && d->pin_cell[1] >= 0 &&
                                    d->pin_cell[1] < d->resolution[1]),
             FF_E_ARG, "createGridTwoPhaseFlipSolver2: pressurePin cell outside the grid");
    FF_CHECK(d->max_substeps > 0, FF_E_ARG, "createGridTwoPhaseFlipSolver2: maxSubsteps must be positive");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    const int nx = d->resolution[0], ny = d->resolution[1];
    if (!u || !v || u->dtype != FF_FLOAT || v->dtype != FF_FLOAT || u->count != (long long)(nx + 1) * ny ||
        v->count != (long long)nx * (ny + 1))
        return ff_set_error(FF_E_ARG, "createGridTwoPhaseFlipSolver2: velocity grid has the wrong shape");
    ff_twophase t = new ff_twophase_s();
    t->ctx = ctx;
    t->dims = 2;
    t->desc = *d;
    // the options on three axes: one cell thick, hz = max(hx, hy) (the
    // trace's minimum spacing), no z gravity, the pin on the plane k = 0
    ff_twophase3_desc &e = t->d;
    std::memset(&e, 0, sizeof e);
    for (int a = 0; a < 2; ++a) {
        e.resolution[a] = d->resolution[a];
        e.grid_spacing[a] = d->grid_spacing[a];
        e.origin[a] = d->origin[a];
        e.gravity[a] = d->gravity[a];
        e.pin_cell[a] = d->pin_cell[a];
    }
    e.resolution[2] = 1;
    e.grid_spacing[2] = std::max(d->grid_spacing[0], d->grid_spacing[1]);
    e.pin_cell[2] = d->pin_cell[0] < 0 ? -1 : 0;
    e.max_particles = d->max_particles;
    e.dt = d->dt;
    e.ambient_density = d->ambient_density;
    e.component_density = d->component_density;
    e.mixing = d->mixing;
    e.fade = d->fade;
    e.concentration_atomic_scale = d->concentration_atomic_scale;
    e.flip_ratio = d->flip_ratio;
    e.gas_flip_ratio = d->gas_flip_ratio;
    e.velocity_damping = d->velocity_damping;
    e.p2g_atomic_scale = d->p2g_atomic_scale;
    e.weight_epsilon = d->weight_epsilon;
    e.closed_flags = d->closed_flags;
    e.max_substeps = d->max_substeps;
    e.collider_push_thresh = d->collider_push_thresh;
    e.collider_push_shift = d->collider_push_shift;
    e.resample_enabled = d->resample_enabled;
    e.min_particles_per_cell = d->min_particles_per_cell;
    e.max_particles_per_cell = d->max_particles_per_cell;
    e.extrapolation_depth = d->extrapolation_depth;
    e.pressure = d->pressure;
    t->g.nx = nx;
    t->g.ny = ny;
    t->g.nz = 1;
    t->g.hx = (float)d->grid_spacing[0];
    t->g.hy = (float)d->grid_spacing[1];
    t->g.hz = (float)std::max(d->grid_spacing[0], d->grid_spacing[1]);
    t->g.ox = (float)d->origin[0];
    t->g.oy = (float)d->origin[1];
    t->g.oz = 0.0f;
    t->u = u;
    t->v = v;
    const int st = tp_setup(t);
    if (st != FF_OK) {
        ff_twophase2_destroy(t);
        return st;
    }
    *out = t;
    return FF_OK;
}

extern "C" void ff_twophase3_desc_default(ff_twophase3_desc *d, const int *res, const double *h, int max_particles,
                                          double dt) {
    std::memset(d, 0, sizeof *d);
    for (int a = 0; a < 3; ++a) {
        d->resolution[a] = res ? res[a] : 1;
        d->grid_spacing[a] = h ? h[a] : 1.0;
    }
    d->max_particles = max_particles;
    d->dt = dt;
    d->gravity[1] = -9.81;
    d->ambient_density = 0.01;
    d->component_density = 1.0;
    d->concentration_atomic_scale = 4096.0;
    d->flip_ratio = 0.97;
    d->gas_flip_ratio = 0.90;
    d->velocity_damping = 0.02;
    d->p2g_atomic_scale = 65536.0;
    d->weight_epsilon = 1e-4;
    d->closed_flags = 63;
    d->max_substeps = 32;
    d->pin_cell[0] = d->resolution[0] / 2;
    d->pin_cell[1] = d->resolution[1] - 1;
    d->pin_cell[2] = d->resolution[2] / 2;
    d->resample_enabled = 1;
    d->min_particles_per_cell = 3;
    d->max_particles_per_cell = 8;
    d->extrapolation_depth = 5;
    ff_pressure_desc_default(&d->pressure, d->resolution, d->grid_spacing);
    int levels = 1;
    while (levels < 5 && d->resolution[0] % (1 << levels) == 0 && d->resolution[1] % (1 << levels) == 0 &&
           d->resolution[2] % (1 << levels) == 0)
        ++levels;
    d->pressure.mg_levels = levels;
}

extern "C" int ff_twophase3_create(ff_ctx ctx, const ff_twophase3_desc *d, ff_field u, ff_field v, ff_field w,
                                   ff_twophase *out) {
    FF_CHECK(ctx && d && out, FF_E_ARG, "ff_twophase3_create: NULL argument");
    FF_CHECK(d->max_particles > 0, FF_E_ARG, "ff_twophase3_create: maxParticles is required.");
    FF_CHECK(d->resolution[0] > 0 && d->resolution[1] > 0 && d->resolution[2] > 1, FF_E_ARG,
             "ff_twophase3_create: bad resolution (nz must exceed 1; use ff_twophase2_create in 2D)");
    FF_CHECK(d->component_density > 0 && d->ambient_density > 0, FF_E_ARG,
             "ff_twophase3_create: both phase densities must be > 0, got %g and %g.", d->component_density,
             d->ambient_density);
    FF_CHECK(d->pin_cell[0] < 0 || (d->pin_cell[0] < d->resolution[0] && d->pin_cell[1] >= 0 &&
                                    d->pin_cell[1] < d->resolution[1] && d->pin_cell[2] >= 0 &&
                                    d->pin_cell[2] < d->resolution[2]),
             FF_E_ARG, "ff_twophase3_create: pressure pin cell outside the grid");
    FF_CHECK(d->max_substeps > 0, FF_E_ARG, "ff_twophase3_create: maxSubsteps must be positive");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    const int nx = d->resolution[0], ny = d->resolution[1], nz = d->resolution[2];
    const long long want[3] = {(long long)(nx + 1) * ny * nz, (long long)nx * (ny + 1) * nz,
                               (long long)nx * ny * (nz + 1)};
    const ff_field uvw[3] = {u, v, w};
    for (int a = 0; a < 3; ++a)
        FF_CHECK(uvw[a] && uvw[a]->dtype == FF_FLOAT && uvw[a]->count == want[a], FF_E_ARG,
                 "ff_twophase3_create: velocity grid has the wrong shape");
    ff_twophase t = new ff_twophase_s();
    t->ctx = ctx;
    t->dims = 3;
    t->d = *d;
    t->g.nx = nx;
    t->g.ny = ny;
    t->g.nz = nz;
    t->g.hx = (float)d->grid_spacing[0];
    t->g.hy = (float)d->grid_spacing[1];
    t->g.hz = (float)d->grid_spacing[2];
    t->g.ox = (float)d->origin[0];
    t->g.oy = (float)d->origin[1];
    t->g.oz = (float)d->origin[2];
    t->u = u;
    t->v = v;
    t->w = w;
    const int st = tp_setup(t);
    if (st != FF_OK) {
        ff_twophase2_destroy(t);
        return st;
    }
    *out = t;
    return FF_OK;
}

extern "C" int ff_twophase2_set_collider(ff_twophase t, ff_field phi) {
    FF_CHECK(t, FF_E_ARG, "NULL two-phase solver");
    FF_CHECK(!phi || (phi->dtype == FF_FLOAT && phi->count == (long long)t->g.nx * t->g.ny * t->g.nz), FF_E_ARG,
             "two-phase collider must be a float cell SDF");
    t->phi = phi;
    return ff_bc3_set_collider(t->bc, phi, nullptr, nullptr, nullptr);
}

extern "C" int ff_twophase2_set_count(ff_twophase t, int n) {
    FF_CHECK(t && n >= 0 && n <= t->d.max_particles, FF_E_ARG, "two-phase particle count out of range");
    t->count = n;
    return FF_OK;
}

extern "C" int ff_twophase2_set_particles(ff_twophase t, int n, const float *xy, const float *vxy,
                                          const float *phase) {
    FF_CHECK(t && n >= 0 && n <= t->d.max_particles, FF_E_ARG, "two-phase particle upload: bad count");
    FF_CHECK(t->dims == 2, FF_E_ARG, "two-phase particle upload: a 3D solver takes ff_twophase3_set_particles");
    cudaSetDevice(t->ctx->device);
    const float zc = t->g.oz + t->g.hz * 0.5f;
    std::vector<float> p3((size_t)3 * n), v3((size_t)3 * n);
    for (size_t p = 0; p < (size_t)n; ++p) {
        if (xy) {
            p3[3 * p] = xy[2 * p];
            p3[3 * p + 1] = xy[2 * p + 1];
            p3[3 * p + 2] = zc;
        }
        if (vxy) {
            v3[3 * p] = vxy[2 * p];
            v3[3 * p + 1] = vxy[2 * p + 1];
            v3[3 * p + 2] = 0.0f;
        }
    }
    cudaStream_t s = t->ctx->stream;
    if (n && xy) FF_CUDA(cudaMemcpyAsync(t->pos->d, p3.data(), p3.size() * 4, cudaMemcpyHostToDevice, s));
    if (n && vxy) FF_CUDA(cudaMemcpyAsync(t->vel->d, v3.data(), v3.size() * 4, cudaMemcpyHostToDevice, s));
    if (n && phase) FF_CUDA(cudaMemcpyAsync(t->phase->d, phase, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    FF_CUDA(cudaStreamSynchronize(s));
    return FF_OK;
}

extern "C" int ff_twophase2_get_particles(ff_twophase t, int n, float *xy, float *vxy, float *phase) {
    FF_CHECK(t && n >= 0 && n <= t->d.max_particles, FF_E_ARG, "two-phase particle download: bad count");
    FF_CHECK(t->dims == 2, FF_E_ARG, "two-phase particle download: a 3D solver takes ff_twophase3_get_particles");
    cudaSetDevice(t->ctx->device);
    cudaStream_t s = t->ctx->stream;
    std::vector<float> p3((size_t)3 * n), v3((size_t)3 * n);
    if (n && xy) FF_CUDA(cudaMemcpyAsync(p3.data(), t->pos->d, p3.size() * 4, cudaMemcpyDeviceToHost, s));
    if (n && vxy) FF_CUDA(cudaMemcpyAsync(v3.data(), t->vel->d, v3.size() * 4, cudaMemcpyDeviceToHost, s));
    if (n && phase) FF_CUDA(cudaMemcpyAsync(phase, t->phase->d, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    FF_CUDA(cudaStreamSynchronize(s));
    for (int p = 0; p < n; ++p)
        for (int a = 0; a < 2; ++a) {
            if (xy) xy[2 * (size_t)p + a] = p3[3 * (size_t)p + a];
            if (vxy) vxy[2 * (size_t)p + a] = v3[3 * (size_t)p + a];
        }
    return FF_OK;
}

extern "C" int ff_twophase3_set_particles(ff_twophase t, int n, const float *xyz, const float *vxyz,
                                          const float *phase) {
    FF_CHECK(t && n >= 0 && n <= t->d.max_particles, FF_E_ARG, "two-phase particle upload: bad count");
    FF_CHECK(t->dims == 3, FF_E_ARG, "two-phase particle upload: a 2D solver takes ff_twophase2_set_particles");
    cudaSetDevice(t->ctx->device);
    cudaStream_t s = t->ctx->stream;
    if (n && xyz) FF_CUDA(cudaMemcpyAsync(t->pos->d, xyz, (size_t)n * 12, cudaMemcpyHostToDevice, s));
    if (n && vxyz) FF_CUDA(cudaMemcpyAsync(t->vel->d, vxyz, (size_t)n * 12, cudaMemcpyHostToDevice, s));
    if (n && phase) FF_CUDA(cudaMemcpyAsync(t->phase->d, phase, (size_t)n * 4, cudaMemcpyHostToDevice, s));
    FF_CUDA(cudaStreamSynchronize(s));
    return FF_OK;
}

extern "C" int ff_twophase3_get_particles(ff_twophase t, int n, float *xyz, float *vxyz, float *phase) {
    FF_CHECK(t && n >= 0 && n <= t->d.max_particles, FF_E_ARG, "two-phase particle download: bad count");
    FF_CHECK(t->dims == 3, FF_E_ARG, "two-phase particle download: a 2D solver takes ff_twophase2_get_particles");
    cudaSetDevice(t->ctx->device);
    cudaStream_t s = t->ctx->stream;
    if (n && xyz) FF_CUDA(cudaMemcpyAsync(xyz, t->pos->d, (size_t)n * 12, cudaMemcpyDeviceToHost, s));
    if (n && vxyz) FF_CUDA(cudaMemcpyAsync(vxyz, t->vel->d, (size_t)n * 12, cudaMemcpyDeviceToHost, s));
    if (n && phase) FF_CUDA(cudaMemcpyAsync(phase, t->phase->d, (size_t)n * 4, cudaMemcpyDeviceToHost, s));
    FF_CUDA(cudaStreamSynchronize(s));
    return FF_OK;
}

extern "C" int ff_twophase2_fields(ff_twophase t, ff_field *phase, ff_field *liquid_fraction, ff_field *density,
                                   ff_field *beta_u, ff_field *beta_v, ff_pressure *pressure) {
    FF_CHECK(t, FF_E_ARG, "NULL two-phase solver");
    if (phase) *phase = t->phase;
    if (liquid_fraction) *liquid_fraction = t->frac;
    if (density) *density = t->rho;
    if (beta_u) *beta_u = t->beta[0];
    if (beta_v) *beta_v = t->beta[1];
    if (pressure) *pressure = t->ps;
    return FF_OK;
}

extern "C" int ff_twophase3_fields(ff_twophase t, ff_field *phase, ff_field *liquid_fraction, ff_field *density,
                                   ff_field *beta_u, ff_field *beta_v, ff_field *beta_w, ff_pressure *pressure) {
    FF_TRY(ff_twophase2_fields(t, phase, liquid_fraction, density, beta_u, beta_v, pressure));
    if (beta_w) *beta_w = t->beta[2];
    return FF_OK;
}

extern "C" int ff_twophase3_cell_counts(ff_twophase t, int32_t *count, int32_t *sum) {
    FF_CHECK(t, FF_E_ARG, "NULL two-phase solver");
    cudaSetDevice(t->ctx->device);
    cudaStream_t s = t->ctx->stream;
    const size_t nc = (size_t)t->g.nx * t->g.ny * t->g.nz;
    if (count) FF_CUDA(cudaMemcpyAsync(count, t->ccnt, nc * 4, cudaMemcpyDeviceToHost, s));
    if (sum) FF_CUDA(cudaMemcpyAsync(sum, t->cacc, nc * 4, cudaMemcpyDeviceToHost, s));
    FF_CUDA(cudaStreamSynchronize(s));
    return FF_OK;
}

static int tp_extrapolate(ff_twophase t, float *data, const int *marker, int a) {
    cudaStream_t s = t->ctx->stream;
    int sx, sy, sz;
    comp_shape(t->g, a, sx, sy, sz);
    const long long n = comp_n(t->g, a);
    FF_CUDA(cudaMemcpyAsync(t->vtmp[0][a], marker, n * 4, cudaMemcpyDeviceToDevice, s));
    float *src = data, *dst = t->scratch[a];
    int *vs = t->vtmp[0][a], *vd = t->vtmp[1][a];
    for (int it = 0; it < t->d.extrapolation_depth; ++it) {
        k_extrapolate<<<blocks_for(n), 256, 0, s>>>(sx, sy, sz, src, dst, vs, vd);
        std::swap(src, dst);
        std::swap(vs, vd);
    }
    if (src != data) FF_CUDA(cudaMemcpyAsync(data, src, n * 4, cudaMemcpyDeviceToDevice, s));
    return post("extrapolate");
}

// One stage of onAdvanceTimeStep (:1505-1592).  The 2D solver's grid is one
// cell thick with an internal zero w; the 3D solver moves all three
// components.
extern "C" int ff_twophase2_stage(ff_twophase t, int stage) {
    FF_CHECK(t, FF_E_ARG, "NULL two-phase solver");
    cudaSetDevice(t->ctx->device);
    cudaStream_t s = t->ctx->stream;
    const ff_twophase3_desc &d = t->d;
    const G3 &g = t->g;
    const bool three = t->dims == 3;
    const int na = t->dims;
    const long long n = t->count, nc = (long long)g.nx * g.ny * g.nz;
    float *uvw[3] = {(float *)t->u->d, (float *)t->v->d, (float *)t->w->d};
    float *w = uvw[2];
    float *pos = (float *)t->pos->d, *vel = (float *)t->vel->d, *ph = (float *)t->phase->d;
    const float cscale = (float)d.concentration_atomic_scale;
    switch (stage) {
    case FF_TP_ADVECT: {
        // advectParticles + pushOutOfCollider (:1098-1124)
        if (!three) FF_CUDA(cudaMemsetAsync(w, 0, comp_n(g, 2) * 4, s));
        if (n == 0) return FF_OK;
        VelField F{g, uvw[0], uvw[1], w, t->phi ? (const float *)t->phi->d : nullptr};
        const F3 mn{g.ox + 1e-4f, g.oy + 1e-4f, g.oz + 1e-4f};
        const F3 mx{(g.ox + (float)(d.resolution[0] * d.grid_spacing[0])) - 1e-4f,
                    (g.oy + (float)(d.resolution[1] * d.grid_spacing[1])) - 1e-4f,
                    three ? (g.oz + (float)(d.resolution[2] * d.grid_spacing[2])) - 1e-4f : (g.oz + g.hz) - 1e-4f};
        k_flip_advect<<<blocks_for(n), 256, 0, s>>>(F, n, pos, (float)d.dt, d.max_substeps, mn, mx,
                                                    (float)d.collider_push_thresh, (float)d.collider_push_shift,
                                                    three ? 0 : 1);
        return post("advectParticles");
    }
    case FF_TP_DENSITY:
        // countPhasesKernel, computeDensityKernel, computeBetaU/V (:646-762)
        FF_CUDA(cudaMemsetAsync(t->ccnt, 0, nc * 4, s));
        FF_CUDA(cudaMemsetAsync(t->cacc, 0, nc * 4, s));
        if (n) k_flip_conc_accum<<<blocks_for(n), 256, 0, s>>>(g, n, pos, ph, cscale, t->ccnt, t->cacc);
        k_flip_conc_resolve<<<blocks_for(nc), 256, 0, s>>>(nc, t->ccnt, t->cacc, cscale, 1, t->r0, t->r1,
                                                           (float *)t->frac->d, (float *)t->rho->d);
        for (int a = 0; a < na; ++a)
            k_flip_beta<<<blocks_for(comp_n(g, a)), 256, 0, s>>>(g, a, (const float *)t->rho->d, nullptr, t->rref,
                                                                 (float *)t->beta[a]->d);
        return post("density");
    case FF_TP_P2G: {
        // scatterU/V(/W), finalizeU/V(/W) (:850-930)
        const float S = (float)d.p2g_atomic_scale;
        for (int a = 0; a < na; ++a) {
            FF_CUDA(cudaMemsetAsync(t->num[a], 0, comp_n(g, a) * 4, s));
            FF_CUDA(cudaMemsetAsync(t->den[a], 0, comp_n(g, a) * 4, s));
        }
        if (n) k_flip_scatter<<<blocks_for(n), 256, 0, s>>>(g, n, pos, vel, S, t->num[0], t->den[0], t->num[1],
                                                            t->den[1], t->num[2], t->den[2], na);
        for (int a = 0; a < na; ++a)
            k_flip_finalize<<<blocks_for(comp_n(g, a)), 256, 0, s>>>(comp_n(g, a), t->num[a], t->den[a], S,
                                                                     (float)d.weight_epsilon, uvw[a], t->valid[a]);
        return post("P2G");
    }
    case FF_TP_SNAPSHOT:
        for (int a = 0; a < na; ++a)
            FF_CUDA(cudaMemcpyAsync(t->old[a], uvw[a], comp_n(g, a) * 4, cudaMemcpyDeviceToDevice, s));
        return FF_OK;
    case FF_TP_EXTRAPOLATE_WEIGHT:
        for (int a = 0; a < na; ++a) FF_TRY(tp_extrapolate(t, uvw[a], t->valid[a], a));
        return FF_OK;
    case FF_TP_CONSTRAIN:
        // in 2D the grid's u and v are the 3D arrays' k = 0 planes
        return ff_bc3_constrain(t->bc, t->u, t->v, t->w, d.extrapolation_depth);
    case FF_TP_GRAVITY: {
        const F3 grav{(float)d.gravity[0], (float)d.gravity[1], three ? (float)d.gravity[2] : 0.0f};
        for (int a = 0; a < na; ++a)
            k_flip_gravity<<<blocks_for(comp_n(g, a)), 256, 0, s>>>(g, a, nullptr, nullptr, grav, (float)d.dt, 1.0f,
                                                                    uvw[a]);
        return post("gravity");
    }
    case FF_TP_PROJECT:
        return ff_pressure3_project(t->ps, t->u, t->v, t->w, t->u, t->v, t->w, &t->last);
    case FF_TP_G2P: {
        if (!three) FF_CUDA(cudaMemsetAsync(w, 0, comp_n(g, 2) * 4, s));
        if (!n) return FF_OK;
        const float clamp01[3] = {std::min(std::max((float)d.flip_ratio, 0.0f), 1.0f),
                                  std::min(std::max((float)d.gas_flip_ratio, 0.0f), 1.0f),
                                  std::min(std::max((float)d.velocity_damping, 0.0f), 1.0f)};
        k_flip_g2p<<<blocks_for(n), 256, 0, s>>>(g, n, pos, vel, uvw[0], uvw[1], w, t->old[0], t->old[1],
                                                 three ? t->old[2] : w, clamp01[0], clamp01[2], ph, clamp01[1]);
        return post("G2P");
    }
    case FF_TP_MIX:
        // mixConcentration (:1055-1073), skipped when both controls are 0
        if (!n || (d.mixing == 0.0 && d.fade == 0.0)) return FF_OK;
        k_flip_mix_fade<<<blocks_for(n), 256, 0, s>>>(g, n, pos, (const float *)t->frac->d,
                                                      std::min(std::max((float)d.mixing, 0.0f), 1.0f),
                                                      std::min(std::max((float)d.fade, 0.0f), 1.0f), ph);
        return post("mixConcentration");
    case FF_TP_RESAMPLE: {
        // resamplePassNow (:1480-1494) on the counts of this frame's DENSITY stage
        if (!d.resample_enabled) return FF_OK;
        const int nbp = (int)((n + RS_CHUNK - 1) / RS_CHUNK), nbc = t->rs_nbc;
        long long *pl = t->rs_bsum, *pg = pl + t->rs_nbp, *cl = pg + t->rs_nbp, *cg = cl + nbc;
        const long long half = std::max(1, d.max_particles / 2), top = d.max_particles - 1;
        k_tp_need<<<blocks_for(nc), 256, 0, s>>>(g, t->ccnt, t->cacc, cscale, d.min_particles_per_cell, t->rs_need);
        k_tp_sums<<<nbp + nbc, 256, 0, s>>>(g, n, pos, ph, t->ccnt, t->rs_need, d.max_particles_per_cell, nbp, pl, pg,
                                            cl, cg);
        k_rs_scan<<<1, 1024, 0, s>>>(pl, nbp, cl, nbc, t->rs_tot);
        k_rs_scan<<<1, 1024, 0, s>>>(pg, nbp, cg, nbc, t->rs_tot + 2);
        if (nbp)
            k_tp_scatter<<<nbp, 256, 0, s>>>(g, n, pos, ph, t->ccnt, d.max_particles_per_cell, pl, pg, half, top,
                                             t->rs_pool);
        k_tp_claim<<<nbc, 256, 0, s>>>(g, t->rs_need, cl, cg, t->rs_tot, half, top, t->rs_pool, uvw[0], uvw[1], w,
                                       pos, vel);
        return post("resample");
    }
    default:
        return ff_set_error(FF_E_ARG, "ff_twophase2_stage: unknown stage %d", stage);
    }
}

// onAdvanceTimeStep (:1505-1592)
extern "C" int ff_twophase2_step(ff_twophase t, ff_diag *diag) {
    FF_CHECK(t, FF_E_ARG, "NULL two-phase solver");
    static const int order[] = {FF_TP_ADVECT,    FF_TP_DENSITY, FF_TP_P2G,       FF_TP_SNAPSHOT,
                                FF_TP_EXTRAPOLATE_WEIGHT,       FF_TP_CONSTRAIN, FF_TP_GRAVITY,
                                FF_TP_CONSTRAIN, FF_TP_PROJECT, FF_TP_CONSTRAIN, FF_TP_G2P,
                                FF_TP_MIX,       FF_TP_RESAMPLE};
    for (int st : order) FF_TRY(ff_twophase2_stage(t, st));
    if (diag) *diag = t->last;
    return FF_OK;
}

extern "C" int ff_twophase2_resample_stats(ff_twophase t, int64_t *out4) {
    FF_CHECK(t && out4, FF_E_ARG, "NULL argument");
    long long v[4] = {0, 0, 0, 0};
    if (t->rs_tot) {
        cudaSetDevice(t->ctx->device);
        FF_CUDA(cudaMemcpyAsync(v, t->rs_tot, sizeof v, cudaMemcpyDeviceToHost, t->ctx->stream));
        FF_CUDA(cudaStreamSynchronize(t->ctx->stream));
    }
    for (int q = 0; q < 4; ++q) out4[q] = v[q];
    return FF_OK;
}
