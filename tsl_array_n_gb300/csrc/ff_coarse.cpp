// FP64 direct solve of the coarsest multigrid level.
//
// The reference relaxes the coarsest level with numberOfCoarsestIterations
// red-black sweeps (fluxflow src/linalg/multigrid.js:679-737), which is not a
// symmetric operator (multigrid.js:1647-1676 records the consequence).  This
// replaces it, when selected, with an exact solve: the coarsest operator A
// (negative semidefinite, often singular: pure Neumann once a thin Dirichlet
// region has coarsened away) is negated to B = -A and factored B = L D L^T
// without pivoting.  A pivot that vanishes relative to its original diagonal
// marks a null direction; its D^+ entry is set to 0.  G = -L^-T D^+ L^-1 is a
// symmetric generalised inverse (A G A = A), so the V-cycle stays symmetric.
// G is formed explicitly so the device applies it as one dense FP64 matvec.
// The matrix is banded (bandwidth nx ny in lexicographic order) and its
// factor keeps that band, so the factorisation and the column solves run
// over the band only.
#include "ff_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>

int ff_coarse_inverse(int nx, int ny, int nz, const float4 *coef, std::vector<double> &G) {
    const int n = nx * ny * nz;
    const long long sy = nx, sz = (long long)nx * ny;
    // lexicographic order: every coupling lies within `band` of the diagonal,
    // and so does every nonzero of L (no fill outside the band)
    const int band = nz > 1 ? (int)sz : (ny > 1 ? (int)sy : 1);
    const int W = band + 1;   // Lb[r * W + d] = B[r][r - d] (d = 0: the diagonal), then L[r][r - d]
    std::vector<double> Lb((size_t)n * W, 0.0);
    auto at = [&](long long r, long long c) -> double & { return Lb[(size_t)r * W + (r - c)]; };
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                long long c = i + sy * (j + (long long)ny * k);
                float4 kc = coef[c];
                double diag = (double)kc.w + kc.x + kc.y + kc.z;
                // B = -A: off-diagonal -K (the lower couplings; B is symmetric)
                if (i > 0) at(c, c - 1) -= kc.x;
                if (j > 0) at(c, c - sy) -= kc.y;
                if (k > 0) at(c, c - sz) -= kc.z;
                if (i < nx - 1) diag += coef[c + 1].x;
                if (j < ny - 1) diag += coef[c + sy].y;
                if (k < nz - 1) diag += coef[c + sz].z;
                at(c, c) += diag;
            }
    std::vector<double> orig(n), D(n);
    for (int j = 0; j < n; ++j) orig[j] = at(j, j);
    // in-place L D L^T (unit L below the diagonal) over the band; the terms
    // outside it are exact zeros, so this equals the dense factorisation
    std::vector<double> tmp(n);
    for (int j = 0; j < n; ++j) {
        const int lo = std::max(0, j - band);
        for (int k = lo; k < j; ++k) tmp[k] = at(j, k) * D[k];
        double d = at(j, j);
        for (int k = lo; k < j; ++k) d -= at(j, k) * tmp[k];
        bool zero = !(d > 1e-10 * std::fabs(orig[j])) || orig[j] == 0.0;
        D[j] = zero ? 0.0 : d;
        const int hi = std::min(n - 1, j + band);
        for (int i = j + 1; i <= hi; ++i) {
            if (zero) { at(i, j) = 0.0; continue; }
            double s = at(i, j);
            for (int k = std::max(lo, i - band); k < j; ++k) s -= at(i, k) * tmp[k];
            at(i, j) = s / d;
        }
    }
    // G = -L^-T D^+ L^-1, column by column (independent: spread over the
    // host's cores), each solve within the band
    G.assign((size_t)n * n, 0.0);
    auto columns = [&](int c0, int c1) {
        std::vector<double> y(n);
        for (int col = c0; col < c1; ++col) {
            std::fill(y.begin(), y.end(), 0.0);
            y[col] = 1.0;
            for (int i = col + 1; i < n; ++i) {   // forward: L y = e_col
                double s = 0.0;
                for (int k = std::max(col, i - band); k < i; ++k) s += at(i, k) * y[k];
                y[i] = -s;
            }
            for (int i = 0; i < n; ++i) y[i] = D[i] > 0.0 ? y[i] / D[i] : 0.0;
            for (int i = n - 1; i >= 0; --i) {   // backward: L^T x = y
                double s = y[i];
                const int kh = std::min(n - 1, i + band);
                for (int k = i + 1; k <= kh; ++k) s -= at(k, i) * y[k];
                y[i] = s;
            }
            for (int i = 0; i < n; ++i) G[(size_t)i * n + col] = -y[i];
        }
    };
    const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (nt == 1 || n < 256) {
        columns(0, n);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) pool.emplace_back(columns, (int)((long long)n * t / nt), (int)((long long)n * (t + 1) / nt));
        for (std::thread &th : pool) th.join();
    }
    // exact symmetry in FP64 (the column solves agree with the rows to rounding)
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            double a = 0.5 * (G[(size_t)i * n + j] + G[(size_t)j * n + i]);
            G[(size_t)i * n + j] = a;
            G[(size_t)j * n + i] = a;
        }
    return FF_OK;
}
