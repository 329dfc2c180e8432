// CG vector kernels with fused FP64 reductions and the GPU-resident scalar
// logic of fluxflow's PCG (src/linalg/linalg.js:1147-1311), plus the
// pressure-projection build / correct / circuit-breaker kernels
// (src/grid/grid_pressure_solver3.js:163-494).
#include "ff_device.cuh"
#include <cstdio>

using namespace ffd;

namespace {

constexpr double MAX_BETA_MAGNITUDE = 10.0;     // linalg.js:226
constexpr double MAX_ALPHA_MAGNITUDE = 1e6;     // linalg.js:244
constexpr double MAX_PAP_GROWTH_FACTOR = 1e8;   // linalg.js:284
constexpr double PAP_BASELINE_FLOOR = 1e-12;    // linalg.js:1052
constexpr double MAX_RESIDUAL_GROWTH = 100.0;   // linalg.js:1095

struct Cell {
    int i, j, k;
    long long c;
    bool ok;
};
__device__ __forceinline__ Cell cell3(const Dims &d) {
    Cell q;
    q.i = blockIdx.x * blockDim.x + threadIdx.x;
    q.j = blockIdx.y * blockDim.y + threadIdx.y;
    q.k = blockIdx.z;
    q.ok = q.i < d.nx && q.j < d.ny;
    q.c = (long long)q.i + (long long)d.nx * ((long long)q.j + (long long)d.ny * q.k);
    return q;
}

// Plain FP32 operator, difference form: sum_f K_f (v_n - v_c) - E v_c.
// V(idx) must return the operand at a linear cell index.
template <class VF>
__device__ __forceinline__ float apply_plain(const Dims &d, const Cell &q, const float4 *coef,
                                             float vc, VF V) {
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    float4 kc = __ldg(coef + q.c);
    float s = -kc.w * vc;
    if (q.i > 0) s += kc.x * (V(q.c - 1) - vc);
    if (q.i < d.nx - 1) s += __ldg(&coef[q.c + 1].x) * (V(q.c + 1) - vc);
    if (q.j > 0) s += kc.y * (V(q.c - sy) - vc);
    if (q.j < d.ny - 1) s += __ldg(&coef[q.c + sy].y) * (V(q.c + sy) - vc);
    if (q.k > 0) s += kc.z * (V(q.c - sz) - vc);
    if (q.k < d.nz - 1) s += __ldg(&coef[q.c + sz].z) * (V(q.c + sz) - vc);
    return s;
}

// Compensated operator on a double-single operand (hi + lo): every product
// and sum is carried as an unevaluated pair (TwoProd / TwoSum), so the
// result is accurate to ~eps^2 of the individual flux terms.  Returns b - Ax
// rounded to FP32.
template <class XF>
__device__ __forceinline__ float residual_ds(const Dims &d, const Cell &q, const float4 *coef,
                                             float b, float hc, float lc, XF X) {
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    float4 kc = __ldg(coef + q.c);
    float S = 0.f, Se = 0.f;
    auto term = [&](float K, long long n) {
        float hn, ln;
        X(n, hn, ln);
        float dh, de;
        two_sum(hn, -hc, dh, de);
        de = __fadd_rn(de, __fsub_rn(ln, lc));
        float p, pe;
        two_prod(K, dh, p, pe);
        pe = __fmaf_rn(K, de, pe);
        float s, e;
        two_sum(S, p, s, e);
        S = s;
        Se = __fadd_rn(Se, __fadd_rn(e, pe));
    };
    if (q.i > 0) term(kc.x, q.c - 1);
    if (q.i < d.nx - 1) term(__ldg(&coef[q.c + 1].x), q.c + 1);
    if (q.j > 0) term(kc.y, q.c - sy);
    if (q.j < d.ny - 1) term(__ldg(&coef[q.c + sy].y), q.c + sy);
    if (q.k > 0) term(kc.z, q.c - sz);
    if (q.k < d.nz - 1) term(__ldg(&coef[q.c + sz].z), q.c + sz);
    {   // - E * (hc + lc)
        float p, pe;
        two_prod(-kc.w, hc, p, pe);
        pe = __fmaf_rn(-kc.w, lc, pe);
        float s, e;
        two_sum(S, p, s, e);
        S = s;
        Se = __fadd_rn(Se, __fadd_rn(e, pe));
    }
    float r0, e0;
    two_sum(b, -S, r0, e0);
    return __fadd_rn(r0, __fsub_rn(e0, Se));
}

// ----------------------------------------------------------------- setup --
// Ax, r = b - Ax, r.r and b.b (linalg.js:1627-1637 setupSequence, first half).
__global__ void k_setup_residual(Dims d, const float4 *__restrict__ coef,
                                 const float *__restrict__ b, const float *__restrict__ xh,
                                 const float *__restrict__ xl, float *__restrict__ r,
                                 PcgState *st, double *partials, int ds) {
    Cell q = cell3(d);
    double v[2] = {0.0, 0.0};
    if (q.ok) {
        float bc = __ldg(b + q.c);
        float rc;
        if (ds) {
            rc = residual_ds(d, q, coef, bc, __ldg(xh + q.c), __ldg(xl + q.c),
                             [&](long long n, float &h, float &l) { h = __ldg(xh + n); l = __ldg(xl + n); });
        } else {
            float xc = __ldg(xh + q.c);
            rc = bc - apply_plain(d, q, coef, xc, [&](long long n) { return __ldg(xh + n); });
        }
        r[q.c] = rc;
        v[0] = (double)rc * (double)rc;
        v[1] = (double)bc * (double)bc;
    }
    double tot[2];
    if (grid_reduce<2>(v, partials, &st->ticket[0], tot)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
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
}

// ------------------------------------------------------ p = z + beta p; pAp --
template <class ZT>
__global__ void k_update_p_pap(Dims d, const float4 *__restrict__ coef, const ZT *__restrict__ z,
                               float *p0, float *p1, PcgState *st, double *partials) {
    if (st->stop) return;
    const int pc = st->p_cur;
    const float *pold = pc ? p1 : p0;
    float *pnew = pc ? p0 : p1;
    const float beta = (float)st->beta;
    const bool first = st->first != 0;
    Cell q = cell3(d);
    double v[1] = {0.0};
    if (q.ok) {
        auto P = [&](long long n) {
            float zn = ld(z, n);
            return first ? zn : __fmaf_rn(beta, __ldg(pold + n), zn);
        };
        float pc_ = P(q.c);
        float ap = apply_plain(d, q, coef, pc_, P);
        pnew[q.c] = pc_;
        v[0] = (double)pc_ * (double)ap;
    }
    double tot[1];
    if (grid_reduce<1>(v, partials, &st->ticket[1], tot)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
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

// ------------------------------------ x += alpha p; r = b - A x; r.r; stop test
__global__ void k_update_x_residual(Dims d, const float4 *__restrict__ coef,
                                    const float *__restrict__ b, const float *p0,
                                    const float *p1, float *xh0, float *xl0, float *xh1,
                                    float *xl1, float *__restrict__ r, PcgState *st,
                                    double *partials, int ds) {
    if (st->stop) return;
    const int xc = st->x_cur;
    const float *p = st->p_cur ? p1 : p0;
    const float *xh = xc ? xh1 : xh0;
    const float *xl = xc ? xl1 : xl0;
    float *oh = xc ? xh0 : xh1;
    float *ol = xc ? xl0 : xl1;
    const double alpha = st->alpha;
    const float ahi = (float)alpha;
    const float alo = (float)(alpha - (double)ahi);
    Cell q = cell3(d);
    double v[1] = {0.0};
    if (q.ok) {
        float bc = __ldg(b + q.c);
        float rc;
        if (ds) {
            auto XN = [&](long long n, float &h, float &l) {
                ds_axpy(xh[n], xl[n], ahi, alo, p[n], h, l);
            };
            float hc, lc;
            XN(q.c, hc, lc);
            rc = residual_ds(d, q, coef, bc, hc, lc, XN);
            oh[q.c] = hc;
            ol[q.c] = lc;
        } else {
            auto XN = [&](long long n) { return __fmaf_rn(ahi, p[n], xh[n]); };
            float x_c = XN(q.c);
            rc = bc - apply_plain(d, q, coef, x_c, XN);
            oh[q.c] = x_c;
        }
        r[q.c] = rc;
        v[0] = (double)rc * (double)rc;
    }
    double tot[1];
    if (grid_reduce<1>(v, partials, &st->ticket[2], tot)) {
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            double rr = tot[0];
            st->rr = rr;
            st->x_cur = xc ^ 1;
            st->iter += 1;
            // residual-growing (linalg.js:1864-1882), sampled where the
            // reference's host reads the residual: at its chunk ends
            if (!nonfinite_d(rr) && st->iter >= st->guard_next) {
                st->guard_next += GROWTH_SAMPLE;
                if (st->best_rr < 0.0 || fabs(rr) < st->best_rr) st->best_rr = fabs(rr);
                else if (st->best_rr > 0.0 && fabs(rr) > st->best_rr * MAX_RESIDUAL_GROWTH &&
                         st->stop == 0) {
                    st->growth_stop = 1;
                }
            }
            // convergenceKernel (linalg.js:1283-1311)
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

// ----------------------------------------------------------- r.z and beta --
template <class ZT>
__global__ void k_rz_beta(Dims d, const float *__restrict__ r, const ZT *__restrict__ z,
                          PcgState *st, double *partials, int setup) {
    if (!setup && st->stop) return;
    long long n = d.n();
    long long i0 = (long long)blockIdx.x * blockDim.x * 4 + threadIdx.x;
    double v[1] = {0.0};
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        long long i = i0 + (long long)u * blockDim.x;
        if (i < n) v[0] += (double)__ldg(r + i) * (double)ld(z, i);
    }
    double tot[1];
    if (grid_reduce<1>(v, partials, &st->ticket[3], tot)) {
        if (threadIdx.x == 0) {
            double rz = tot[0];
            st->rz = rz;
            if (setup) {
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

__global__ void k_state_init(PcgState *st, double tol, int maxiter, int relative) {
    const int last_valid = st->last_valid, last = last_valid ? st->last_iters : GROWTH_FIRST_DEFAULT;
    PcgState s = {};
    s.tol = tol;
    s.maxiter = maxiter;
    s.relative = relative;
    s.best_rr = -1.0;
    s.last_iters = last;
    s.last_valid = last_valid;
    s.guard_next = growth_first_check(last);
    *st = s;
}

__global__ void k_loop_control(PcgState *st, cudaGraphConditionalHandle h, int use_handle) {
    if (threadIdx.x != 0) return;
    st->launched += 1;
    int cont = (st->stop == 0) && (st->err == 0) && (st->iter < st->maxiter) && (st->launched < st->maxiter + 4);
    if (!cont) {
        // the count the next solve's first chunk is sized by (linalg.js:1839-1905)
        st->last_iters = st->stop == FF_STOP_CONVERGED ? st->stop_iter : st->iter;
        st->last_valid = 1;
    }
    if (use_handle) cudaGraphSetConditional(h, cont ? 1u : 0u);
}

__global__ void k_laplacian(Dims d, const float4 *__restrict__ coef, const float *__restrict__ x,
                            float *__restrict__ y) {
    Cell q = cell3(d);
    if (!q.ok) return;
    float xc = __ldg(x + q.c);
    y[q.c] = apply_plain(d, q, coef, xc, [&](long long n) { return __ldg(x + n); });
}

// createJacobiPreconditioner (multigrid.js:568-604): z = r / diag, identity
// where the diagonal is zero.
template <class ZT>
__global__ void k_jacobi(Dims d, const float4 *__restrict__ coef, const float *__restrict__ r,
                         ZT *__restrict__ z, const PcgState *st) {
    if (st && st->stop) return;
    Cell q = cell3(d);
    if (!q.ok) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    float4 kc = __ldg(coef + q.c);
    float D = -(kc.x + kc.y + kc.z + kc.w);
    if (q.i < d.nx - 1) D -= __ldg(&coef[q.c + 1].x);
    if (q.j < d.ny - 1) D -= __ldg(&coef[q.c + sy].y);
    if (q.k < d.nz - 1) D -= __ldg(&coef[q.c + sz].z);
    float rc = __ldg(r + q.c);
    ffd::st(z, q.c, fabsf(D) > 0.f ? rc / D : rc);
}

template <class ZT>
__global__ void k_identity(long long n, const float *__restrict__ r, ZT *__restrict__ z,
                           const PcgState *st) {
    if (st && st->stop) return;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) ffd::st(z, i, __ldg(r + i));
}

__global__ void k_fill(float *p, long long n, float v) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

// ------------------------------------------------------ pressure build etc --
// updateDirichletFields (grid_pressure_solver3.js:163-206)
__global__ void k_dirichlet_fields(Dims d, const uint8_t *active, const float *target,
                                   const float *cwu, const float *cwv, const float *cww,
                                   uint8_t *mask, float *tgt, uint8_t *vent) {
    Cell q = cell3(d);
    if (!q.ok) return;
    bool enclosed = false;
    if (cwu) {
        long long fu = q.i + (long long)(d.nx + 1) * (q.j + (long long)d.ny * q.k);
        long long fv = q.i + (long long)d.nx * (q.j + (long long)(d.ny + 1) * q.k);
        float t = cwu[fu] + cwu[fu + 1] + cwv[fv] + cwv[fv + d.nx];
        if (d.nz > 1) t += cww[q.c] + cww[q.c + (long long)d.nx * d.ny];
        enclosed = t < 1e-6f;
    }
    bool act = active ? active[q.c] != 0 : false;
    mask[q.c] = (act || enclosed) ? 1 : 0;
    tgt[q.c] = act ? (target ? target[q.c] : 0.f) : 0.f;
    vent[q.c] = act ? 1 : 0;
}

// systemFaceWeights = faceWeights * colliderWeights (:217-229)
__global__ void k_system_weights(long long n, const float *fw, const float *cw, float *sw) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a = fw ? fw[i] : 1.f, c = cw ? cw[i] : 1.f;
    sw[i] = (fw && cw) ? a * c : (fw ? a : c);
}

// dispatchBuildSystem (:350-453)
// ihx, ihy, ihz: (float)(1 / (double)h^2) per axis, formed once on the host
// (FP64 arithmetic per cell would dominate the kernel on this part)
__global__ void k_build_system(Dims d, float hx, float hy, float hz, float ihx, float ihy, float ihz,
                               const float *u, const float *v, const float *w, const float *cwu,
                               const float *cwv, const float *cww, const float *swu,
                               const float *swv, const float *sww, const uint8_t *mask,
                               const float *tgt, float *b, float *xh, float *xl) {
    Cell q = cell3(d);
    if (!q.ok) return;
    const long long s = (long long)d.nx * d.ny;
    long long fu = q.i + (long long)(d.nx + 1) * (q.j + (long long)d.ny * q.k);
    long long fv = q.i + (long long)d.nx * (q.j + (long long)(d.ny + 1) * q.k);
    long long fw = q.c;
    float div;
    if (cwu) {
        float lu = u[fu] * cwu[fu], ru = u[fu + 1] * cwu[fu + 1];
        float lv = v[fv] * cwv[fv], rv = v[fv + d.nx] * cwv[fv + d.nx];
        div = (ru - lu) / hx + (rv - lv) / hy;
        if (d.nz > 1) {
            float lw = w[fw] * cww[fw], rw = w[fw + s] * cww[fw + s];
            div += (rw - lw) / hz;
        }
    } else {
        div = (u[fu + 1] - u[fu]) / hx + (v[fv + d.nx] - v[fv]) / hy;
        if (d.nz > 1) div += (w[fw + s] - w[fw]) / hz;
    }
    if (!mask) {
        b[q.c] = div;
        return;
    }
    if (mask[q.c]) {
        float t = tgt[q.c];
        b[q.c] = -t;
        xh[q.c] = t;
        if (xl) xl[q.c] = 0.f;
        return;
    }
    float acc = 0.f;
    if (q.i > 0 && mask[q.c - 1]) acc += (swu ? swu[fu] : 1.f) * tgt[q.c - 1] * ihx;
    if (q.i < d.nx - 1 && mask[q.c + 1]) acc += (swu ? swu[fu + 1] : 1.f) * tgt[q.c + 1] * ihx;
    if (q.j > 0 && mask[q.c - d.nx]) acc += (swv ? swv[fv] : 1.f) * tgt[q.c - d.nx] * ihy;
    if (q.j < d.ny - 1 && mask[q.c + d.nx]) acc += (swv ? swv[fv + d.nx] : 1.f) * tgt[q.c + d.nx] * ihy;
    if (d.nz > 1) {
        if (q.k > 0 && mask[q.c - s]) acc += (sww ? sww[fw] : 1.f) * tgt[q.c - s] * ihz;
        if (q.k < d.nz - 1 && mask[q.c + s]) acc += (sww ? sww[fw + s] : 1.f) * tgt[q.c + s] * ihz;
    }
    b[q.c] = div - acc;
}

// countBadPressureCells (:297-304): non-finite or |p| > maxPlausiblePressure
__global__ void k_count_bad(long long n, const float *xh0, const float *xh1, PcgState *st,
                            float maxp) {
    const float *x = st->x_cur ? xh1 : xh0;
    // four cells per thread (float4 when the count allows)
    long long i = 4 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    int bad = 0;
    auto test = [&](float v) { return (int)(nonfinite_f(v) || !(fabsf(v) <= maxp)); };
    if (i + 3 < n && (n & 3) == 0) {
        const float4 v = *reinterpret_cast<const float4 *>(x + i);
        bad = test(v.x) + test(v.y) + test(v.z) + test(v.w);
    } else {
        for (long long q = i; q < i + 4 && q < n; ++q) bad += test(x[q]);
    }
    const int tot = __reduce_add_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd(&st->bad_cells, tot);
}

// finishAccepted / finishRejected (:499-500, :553-554): restore the snapshot
// when the breaker fired, else take a new one; leave the result in slot 0.
// Four cells a thread (16-byte accesses when n % 4 == 0: every array is
// 256-byte aligned); slot 0 is not rewritten when the result is already
// there.
__global__ void k_commit(long long n, float *xh0, float *xl0, const float *xh1,
                         const float *xl1, float *sh, float *sl, const PcgState *st) {
    const long long i = 4 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    const bool restore = st->bad_cells > 0, cur1 = st->x_cur != 0;
    if ((n & 3) == 0) {
        auto ld = [](const float *p, long long i) { return *reinterpret_cast<const float4 *>(p + i); };
        auto stq = [](float *p, long long i, const float4 &v) { *reinterpret_cast<float4 *>(p + i) = v; };
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        if (restore) {
            stq(xh0, i, ld(sh, i));
            if (xl0) stq(xl0, i, sl ? ld(sl, i) : z);
            return;
        }
        const float4 h = ld(cur1 ? xh1 : xh0, i);
        const float4 l = xl0 ? ld(cur1 ? xl1 : xl0, i) : z;
        if (cur1) {
            stq(xh0, i, h);
            if (xl0) stq(xl0, i, l);
        }
        stq(sh, i, h);
        if (sl) stq(sl, i, l);
        return;
    }
    for (long long c = i; c < i + 4 && c < n; ++c) {
        if (restore) {
            xh0[c] = sh[c];
            if (xl0) xl0[c] = sl ? sl[c] : 0.f;
            continue;
        }
        const float h = cur1 ? xh1[c] : xh0[c];
        const float l = xl0 ? (cur1 ? xl1[c] : xl0[c]) : 0.f;
        xh0[c] = h;
        if (xl0) xl0[c] = l;
        sh[c] = h;
        if (sl) sl[c] = l;
    }
}

// dispatchCorrectU/V/W (:457-494): interior faces only, gated by the
// collider weight, scaled by the face weight (beta).
// All axes of the correction in one pass: thread (i, j, k) over
// [0, nx] x [0, ny] x [0, nz] takes the u, v and w faces indexed (i, j, k)
// that exist (p difference over h, times the face weight, zero where the
// collider weight is zero; boundary faces copied); the pressure at cell
// (i, j, k) is read once for the three.
__global__ void k_correct3(Dims d, int naxes, float hx, float hy, float hz, const float *xh, const float *xl,
                           const float *fwu, const float *fwv, const float *fww, const float *cwu,
                           const float *cwv, const float *cww, const float *uin, const float *vin,
                           const float *win, float *uout, float *vout, float *wout) {
    // one thread per cell: its lower face on each axis, and the upper
    // domain-edge face when the cell is the last along that axis
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= d.nx || j >= d.ny) return;
    const long long c = i + (long long)d.nx * (j + (long long)d.ny * k);
    const float pc = xh[c];
    const float pcl = xl ? xl[c] : 0.f;
    // a face strictly inside the domain along its axis (m > 0)
    auto face = [&](int m, long long f, long long off, float h, const float *fw, const float *cw, const float *in,
                    float *out) {
        if (m == 0) {
            if (in != out) out[f] = in[f];
            return;
        }
        float dp = pc - xh[c - off];
        if (xl) dp += pcl - xl[c - off];
        float g = dp / h;
        if (fw) g = g * fw[f];
        if (cw) g = g * (cw[f] > 0.f ? 1.f : 0.f);
        out[f] = in[f] - g;
    };
    const long long fu = i + (long long)(d.nx + 1) * (j + (long long)d.ny * k);
    face(i, fu, 1, hx, fwu, cwu, uin, uout);
    if (i == d.nx - 1 && uin != uout) uout[fu + 1] = uin[fu + 1];
    const long long fv = i + (long long)d.nx * (j + (long long)(d.ny + 1) * k);
    face(j, fv, d.nx, hy, fwv, cwv, vin, vout);
    if (j == d.ny - 1 && vin != vout) vout[fv + d.nx] = vin[fv + d.nx];
    if (naxes == 3) {
        const long long plane = (long long)d.nx * d.ny;
        face(k, c, plane, hz, fww, cww, win, wout);
        if (k == d.nz - 1 && win != wout) wout[c + plane] = win[c + plane];
    }
}

// k_correct3 over x-quads (nx % 4 == 0): one thread per four cells of a
// row; the pressure and its y and z neighbours, the v and w faces as 16-byte
// accesses, the u faces (rows of nx + 1) as scalars.  Per face the same
// operations in the same order as k_correct3.
__global__ void k_correct4(Dims d, int naxes, float hx, float hy, float hz, const float *xh, const float *xl,
                           const float *fwu, const float *fwv, const float *fww, const float *cwu,
                           const float *cwv, const float *cww, const float *uin, const float *vin,
                           const float *win, float *uout, float *vout, float *wout) {
    const int qx = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z, i0 = 4 * qx;
    if (i0 >= d.nx || j >= d.ny) return;
    const long long c0 = i0 + (long long)d.nx * (j + (long long)d.ny * k);
    auto ld4 = [](const float *p, long long i) { return *reinterpret_cast<const float4 *>(p + i); };
    auto el = [](const float4 &q, int m) { return m == 0 ? q.x : m == 1 ? q.y : m == 2 ? q.z : q.w; };
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 pc = ld4(xh, c0), pcl = xl ? ld4(xl, c0) : z4;
    // one face: p difference over h, times the face weight, zero where the
    // collider weight is zero (k_correct3's face())
    auto grad = [&](float p, float pl, float q, float ql, float h, const float *fw, const float *cw, long long f) {
        float dp = p - q;
        if (xl) dp += pl - ql;
        float g = dp / h;
        if (fw) g = g * fw[f];
        if (cw) g = g * (cw[f] > 0.f ? 1.f : 0.f);
        return g;
    };
    // x faces i0 .. i0+3 (and the domain's upper one after the last cell)
    const long long fu = i0 + (long long)(d.nx + 1) * (j + (long long)d.ny * k);
    const float pw = i0 > 0 ? xh[c0 - 1] : 0.f, pwl = (xl && i0 > 0) ? xl[c0 - 1] : 0.f;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const long long f = fu + m;
        if (i0 + m == 0) {
            if (uin != uout) uout[f] = uin[f];
        } else {
            const float q = m == 0 ? pw : el(pc, m - 1), ql = m == 0 ? pwl : el(pcl, m - 1);
            uout[f] = uin[f] - grad(el(pc, m), el(pcl, m), q, ql, hx, fwu, cwu, f);
        }
    }
    if (i0 + 4 == d.nx && uin != uout) uout[fu + 4] = uin[fu + 4];
    // y faces
    const long long fv = i0 + (long long)d.nx * (j + (long long)(d.ny + 1) * k);
    if (j == 0) {
        if (vin != vout) *reinterpret_cast<float4 *>(vout + fv) = ld4(vin, fv);
    } else {
        const float4 ps = ld4(xh, c0 - d.nx), psl = xl ? ld4(xl, c0 - d.nx) : z4, vi = ld4(vin, fv);
        float o[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) o[m] = el(vi, m) - grad(el(pc, m), el(pcl, m), el(ps, m), el(psl, m), hy, fwv, cwv, fv + m);
        *reinterpret_cast<float4 *>(vout + fv) = make_float4(o[0], o[1], o[2], o[3]);
    }
    if (j == d.ny - 1 && vin != vout) *reinterpret_cast<float4 *>(vout + fv + d.nx) = ld4(vin, fv + d.nx);
    if (naxes == 3) {
        const long long plane = (long long)d.nx * d.ny;
        if (k == 0) {
            if (win != wout) *reinterpret_cast<float4 *>(wout + c0) = ld4(win, c0);
        } else {
            const float4 ps = ld4(xh, c0 - plane), psl = xl ? ld4(xl, c0 - plane) : z4, wi = ld4(win, c0);
            float o[4];
#pragma unroll
            for (int m = 0; m < 4; ++m) o[m] = el(wi, m) - grad(el(pc, m), el(pcl, m), el(ps, m), el(psl, m), hz, fww, cww, c0 + m);
            *reinterpret_cast<float4 *>(wout + c0) = make_float4(o[0], o[1], o[2], o[3]);
        }
        if (k == d.nz - 1 && win != wout) *reinterpret_cast<float4 *>(wout + c0 + plane) = ld4(win, c0 + plane);
    }
}

}  // namespace

namespace ffk {

static int post(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return ff_set_error(FF_E_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
    return FF_OK;
}
static unsigned nblocks1(long long n, int t) { return (unsigned)((n + t - 1) / t); }

int fill_f32(float *p, long long n, float v, cudaStream_t s) {
    if (n <= 0) return FF_OK;
    // +0.0 is all-zero bits: a memset (copy engine rate, no kernel)
    if (v == 0.f && !signbit(v)) {
        FF_CUDA(cudaMemsetAsync(p, 0, (size_t)n * sizeof(float), s));
        return FF_OK;
    }
    k_fill<<<nblocks1(n, 256), 256, 0, s>>>(p, n, v);
    return post("fill");
}
int copy_bytes(void *dst, const void *src, size_t bytes, cudaStream_t s) {
    FF_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s));
    return FF_OK;
}

int dirichlet_fields(Dims d, const uint8_t *active, const float *target, const float *cwu,
                     const float *cwv, const float *cww, uint8_t *mask, float *tgt,
                     uint8_t *vent, cudaStream_t s) {
    auto L = launch3(d.nx, d.ny, d.nz);
    k_dirichlet_fields<<<L.grid, L.block, 0, s>>>(d, active, target, cwu, cwv, cww, mask, tgt, vent);
    return post("dirichlet_fields");
}

int system_weights(Dims d, const float *fw[3], const float *cw[3], float *sw[3], cudaStream_t s) {
    long long nf[3] = {d.nu(), d.nv(), d.nw()};
    for (int a = 0; a < 3; ++a) {
        if (!sw[a]) continue;
        k_system_weights<<<nblocks1(nf[a], 256), 256, 0, s>>>(nf[a], fw[a], cw[a], sw[a]);
    }
    return post("system_weights");
}

int build_system(Dims d, float hx, float hy, float hz, const float *u, const float *v,
                 const float *w, const float *cw[3], const float *fw[3], const float *sw[3],
                 const uint8_t *mask, const float *tgt, float *b, float *x_hi, float *x_lo,
                 cudaStream_t s) {
    (void)fw;
    auto L = launch3(d.nx, d.ny, d.nz);
    const float ihx = (float)(1.0 / ((double)hx * hx)), ihy = (float)(1.0 / ((double)hy * hy)),
                ihz = (float)(1.0 / ((double)hz * hz));
    k_build_system<<<L.grid, L.block, 0, s>>>(d, hx, hy, hz, ihx, ihy, ihz, u, v, w, cw[0], cw[1], cw[2],
                                              sw[0], sw[1], sw[2], mask, tgt, b, x_hi, x_lo);
    return post("build_system");
}

int count_bad_and_commit(Dims d, float *x_hi0, float *x_lo0, float *x_hi1, float *x_lo1,
                         float *snap_hi, float *snap_lo, PcgState *st, float max_plausible,
                         int *bad_count, cudaStream_t s) {
    (void)bad_count;
    long long n = d.n();
    FF_CUDA(cudaMemsetAsync(&st->bad_cells, 0, sizeof(int), s));
    k_count_bad<<<nblocks1((n + 3) / 4, 256), 256, 0, s>>>(n, x_hi0, x_hi1, st, max_plausible);
    FF_TRY(post("count_bad"));
    k_commit<<<nblocks1((n + 3) / 4, 256), 256, 0, s>>>(n, x_hi0, x_lo0, x_hi1, x_lo1, snap_hi, snap_lo, st);
    return post("commit");
}

int correct(Dims d, float hx, float hy, float hz, const float *x_hi, const float *x_lo,
            const float *fw[3], const float *cw[3], const float *uin, const float *vin,
            const float *win, float *uout, float *vout, float *wout, cudaStream_t s) {
    const float *ins[3] = {uin, vin, win};
    float *outs[3] = {uout, vout, wout};
    const int naxes = d.nz > 1 ? 3 : 2;
    auto L = launch3(d.nx, d.ny, d.nz);
    if (d.nx % 4 == 0) {
        auto L4 = launch3(d.nx / 4, d.ny, d.nz);
        k_correct4<<<L4.grid, L4.block, 0, s>>>(d, naxes, hx, hy, hz, x_hi, x_lo, fw[0], fw[1], fw[2], cw[0], cw[1],
                                                cw[2], ins[0], ins[1], ins[2], outs[0], outs[1], outs[2]);
    } else {
        k_correct3<<<L.grid, L.block, 0, s>>>(d, naxes, hx, hy, hz, x_hi, x_lo, fw[0], fw[1], fw[2], cw[0], cw[1],
                                              cw[2], ins[0], ins[1], ins[2], outs[0], outs[1], outs[2]);
    }
    return post("correct");
}

int cg_setup_residual(Dims d, const float4 *coef, const float *b, const float *xh,
                      const float *xl, float *r, PcgState *st, double *partials, int ds,
                      cudaStream_t s) {
    auto L = launch3(d.nx, d.ny, d.nz);
    k_setup_residual<<<L.grid, L.block, 0, s>>>(d, coef, b, xh, xl, r, st, partials, ds);
    return post("setup_residual");
}

int cg_update_p_pap(Dims d, const float4 *coef, const void *z, int zbf16, float *p0, float *p1,
                    PcgState *st, double *partials, cudaStream_t s) {
    auto L = launch3(d.nx, d.ny, d.nz);
    if (zbf16)
        k_update_p_pap<__nv_bfloat16><<<L.grid, L.block, 0, s>>>(d, coef, (const __nv_bfloat16 *)z, p0, p1, st, partials);
    else
        k_update_p_pap<float><<<L.grid, L.block, 0, s>>>(d, coef, (const float *)z, p0, p1, st, partials);
    return post("update_p_pap");
}

int cg_update_x_residual(Dims d, const float4 *coef, const float *b, const float *p0,
                         const float *p1, float *xh0, float *xl0, float *xh1, float *xl1,
                         float *r, PcgState *st, double *partials, int ds, cudaStream_t s) {
    auto L = launch3(d.nx, d.ny, d.nz);
    k_update_x_residual<<<L.grid, L.block, 0, s>>>(d, coef, b, p0, p1, xh0, xl0, xh1, xl1, r, st, partials, ds);
    return post("update_x_residual");
}

int cg_rz_beta(Dims d, const float *r, const void *z, int zbf16, PcgState *st,
               double *partials, int setup, cudaStream_t s) {
    long long n = d.n();
    unsigned g = nblocks1(n, 256 * 4);
    if (zbf16)
        k_rz_beta<__nv_bfloat16><<<g, 256, 0, s>>>(d, r, (const __nv_bfloat16 *)z, st, partials, setup);
    else
        k_rz_beta<float><<<g, 256, 0, s>>>(d, r, (const float *)z, st, partials, setup);
    return post("rz_beta");
}

int state_init(PcgState *st, double tol, int maxiter, int relative, cudaStream_t s) {
    k_state_init<<<1, 1, 0, s>>>(st, tol, maxiter, relative);
    return post("state_init");
}

int loop_control(PcgState *st, unsigned long long handle, int use_handle, cudaStream_t s) {
    k_loop_control<<<1, 32, 0, s>>>(st, (cudaGraphConditionalHandle)handle, use_handle);
    return post("loop_control");
}

int laplacian_apply(Dims d, const float4 *coef, const float *x, float *y, cudaStream_t s) {
    auto L = launch3(d.nx, d.ny, d.nz);
    k_laplacian<<<L.grid, L.block, 0, s>>>(d, coef, x, y);
    return post("laplacian");
}

int jacobi_apply(Dims d, const float4 *coef, const float *r, void *z, int zbf16,
                 const PcgState *st, cudaStream_t s) {
    auto L = launch3(d.nx, d.ny, d.nz);
    if (zbf16) k_jacobi<__nv_bfloat16><<<L.grid, L.block, 0, s>>>(d, coef, r, (__nv_bfloat16 *)z, st);
    else k_jacobi<float><<<L.grid, L.block, 0, s>>>(d, coef, r, (float *)z, st);
    return post("jacobi");
}

int identity_apply(Dims d, const float *r, void *z, int zbf16, const PcgState *st,
                   cudaStream_t s) {
    long long n = d.n();
    if (zbf16) k_identity<__nv_bfloat16><<<nblocks1(n, 256), 256, 0, s>>>(n, r, (__nv_bfloat16 *)z, st);
    else k_identity<float><<<nblocks1(n, 256), 256, 0, s>>>(n, r, (float *)z, st);
    return post("identity");
}

}  // namespace ffk
