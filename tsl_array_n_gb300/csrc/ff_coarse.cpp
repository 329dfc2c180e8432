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
#include "ff_internal.h"
#include <cmath>
#include <cstring>

int ff_coarse_inverse(int nx, int ny, int nz, const float4 *coef, std::vector<double> &G) {
    const int n = nx * ny * nz;
    const long long sy = nx, sz = (long long)nx * ny;
    std::vector<double> B((size_t)n * n, 0.0);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                long long c = i + sy * (j + (long long)ny * k);
                float4 kc = coef[c];
                double diag = (double)kc.w + kc.x + kc.y + kc.z;
                auto couple = [&](long long m, double K) {
                    B[(size_t)c * n + m] -= K;   // B = -A, off-diagonal -K
                };
                if (i > 0) couple(c - 1, kc.x);
                if (j > 0) couple(c - sy, kc.y);
                if (k > 0) couple(c - sz, kc.z);
                if (i < nx - 1) { double K = coef[c + 1].x; diag += K; couple(c + 1, K); }
                if (j < ny - 1) { double K = coef[c + sy].y; diag += K; couple(c + sy, K); }
                if (k < nz - 1) { double K = coef[c + sz].z; diag += K; couple(c + sz, K); }
                B[(size_t)c * n + c] += diag;
            }
    std::vector<double> orig(n), D(n);
    for (int j = 0; j < n; ++j) orig[j] = B[(size_t)j * n + j];
    // in-place L D L^T in the lower triangle (unit L below the diagonal)
    std::vector<double> tmp(n);
    for (int j = 0; j < n; ++j) {
        double *rj = &B[(size_t)j * n];
        for (int k = 0; k < j; ++k) tmp[k] = rj[k] * D[k];
        double d = rj[j];
        for (int k = 0; k < j; ++k) d -= rj[k] * tmp[k];
        bool zero = !(d > 1e-10 * std::fabs(orig[j])) || orig[j] == 0.0;
        D[j] = zero ? 0.0 : d;
        for (int i = j + 1; i < n; ++i) {
            double *ri = &B[(size_t)i * n];
            if (zero) { ri[j] = 0.0; continue; }
            double s = ri[j];
            for (int k = 0; k < j; ++k) s -= ri[k] * tmp[k];
            ri[j] = s / d;
        }
    }
    // G = -L^-T D^+ L^-1, column by column
    G.assign((size_t)n * n, 0.0);
    std::vector<double> y(n);
    for (int col = 0; col < n; ++col) {
        std::fill(y.begin(), y.end(), 0.0);
        y[col] = 1.0;
        for (int i = col + 1; i < n; ++i) {   // forward: L y = e_col
            const double *ri = &B[(size_t)i * n];
            double s = 0.0;
            for (int k = col; k < i; ++k) s += ri[k] * y[k];
            y[i] = -s;
        }
        for (int i = 0; i < n; ++i) y[i] = D[i] > 0.0 ? y[i] / D[i] : 0.0;
        for (int i = n - 1; i >= 0; --i) {   // backward: L^T x = y
            double s = y[i];
            for (int k = i + 1; k < n; ++k) s -= B[(size_t)k * n + i] * y[k];
            y[i] = s;
        }
        for (int i = 0; i < n; ++i) G[(size_t)i * n + col] = -y[i];
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
