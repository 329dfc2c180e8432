// Internal declarations shared by the libff translation units.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "../../include/ff.h"

// ---------------------------------------------------------------- errors --
int ff_set_error(int code, const char *fmt, ...);
#define FF_CUDA(call)                                                            \
    do {                                                                         \
        cudaError_t _e = (call);                                                 \
        if (_e != cudaSuccess)                                                   \
            return ff_set_error(FF_E_CUDA, "%s:%d %s: %s", __FILE__, __LINE__,   \
                                #call, cudaGetErrorString(_e));                  \
    } while (0)
#define FF_CHECK(cond, code, ...)                                                \
    do {                                                                         \
        if (!(cond)) return ff_set_error(code, __VA_ARGS__);                     \
    } while (0)
#define FF_TRY(call)                                                             \
    do {                                                                         \
        int _s = (call);                                                         \
        if (_s != FF_OK) return _s;                                              \
    } while (0)

// The grid-velocity and FLIP kernels index their arrays in 32 bits, as the
// reference's WGSL does (u32 indices): every face or cell array of a grid
// must hold fewer than 2^31 elements.
inline int check_grid32(const int *res, const char *who) {
    const long long big = ((long long)res[0] + 1) * ((long long)res[1] + 1) * ((long long)res[2] + 1);
    FF_CHECK(big < 0x7fffffffLL, FF_E_LIMIT, "%s: a %dx%dx%d grid exceeds 2^31 elements per array", who, res[0],
             res[1], res[2]);
    return FF_OK;
}

// residual-growing stop: the squared residual is compared with the best one
// seen where the reference's host reads it, at the end of each chunk
// (linalg.js:942-943, 1839-1882): the first chunk ends at the previous
// solve's iteration count + 2 (4 before any solve), at least MIN_CHUNK,
// and every MIN_CHUNK iterations after it
constexpr int GROWTH_SAMPLE = 4;
constexpr int GROWTH_FIRST_DEFAULT = 4;
__host__ __device__ inline int growth_first_check(int last_iters) {
    return last_iters + 2 > GROWTH_SAMPLE ? last_iters + 2 : GROWTH_SAMPLE;
}

// --------------------------------------------------------------- handles --
struct ff_ctx_s {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t events[16] = {};
    // copy streams of the host-buffer entry points (created on first use):
    // uploads and downloads run beside the compute stream
    cudaStream_t up = nullptr, down = nullptr;
};
int ff_ctx_copy_streams(ff_ctx ctx);

struct ff_field_s {
    ff_ctx ctx = nullptr;
    int dtype = FF_FLOAT;
    int ndim = 1;
    int shape[3] = {1, 1, 1};
    int64_t count = 0;
    size_t bytes = 0;
    void *d = nullptr;
    bool owned = true;
};

size_t ff_dtype_size(int dtype);
// device allocation with 256-byte alignment and zero fill
int ff_dev_alloc(void **p, size_t bytes, cudaStream_t s);
void ff_dev_free(void *p);

// ------------------------------------------------------------ grid shapes --
#ifdef __CUDACC__
#define FF_HD __host__ __device__
#else
#define FF_HD
#endif
struct Dims {
    int nx, ny, nz;
    FF_HD long long n() const { return (long long)nx * ny * nz; }
    FF_HD long long nu() const { return (long long)(nx + 1) * ny * nz; }
    FF_HD long long nv() const { return (long long)nx * (ny + 1) * nz; }
    FF_HD long long nw() const { return (long long)nx * ny * (nz + 1); }
};

// ------------------------------------------------------- PCG device state --
// One struct in device memory holds every scalar the iteration needs; the
// host reads it once at the end of a solve.  Mirrors the reference's 9-slot
// scalar buffer (fluxflow src/linalg/linalg.js:1030-1065) in FP64.
struct PcgState {
    double pAp, rr, rz, rz_old, pap_baseline, bb;
    double alpha, beta, thr, tol, best_rr;
    int stop, iter, stop_iter, first;
    int maxiter, relative, p_cur, x_cur;
    int launched, bad_cells, growth_stop;
    int guard_next;             // iteration of the next residual-growing check
    int last_iters, last_valid; // the previous solve's iteration count (kept across solves)
    int err;   // nonzero: a kernel gave up on a bounded wait (bit 0: TMA staging, bit 1: grid barrier)
    unsigned ticket[4];
};

// Per-level data of the multigrid hierarchy.  Coefficients are stored per
// cell as (Kx, Ky, Kz, E): K_a is the coupling through the cell's LOWER face
// on axis a (w_face / h_a^2, zero when either cell is pinned or the face is a
// domain edge) and E collects the faces to pinned neighbours (1 for a pinned
// cell).  (A x)_c = sum_f K_f (x_n - x_c) - E_c x_c reproduces laplacianAt
// (fluxflow src/linalg/multigrid.js:273-339) exactly, and the diagonal is
// -(sum of the six K + E), laplacianDiagonalAt (:399-437).
struct Level {
    Dims d{};
    float h2inv[3] = {1, 1, 1};
    float *w[3] = {nullptr, nullptr, nullptr};   // face weights (fp32), may be null
    uint8_t *mask = nullptr;                       // may be null
    float4 *coef = nullptr;                        // fp32 coefficients
    uint2 *coef16 = nullptr;                       // bf16 coefficients (4 x bf16)
    void *x = nullptr, *b = nullptr, *buf = nullptr;  // storage type per mode
};

// TMA descriptors of one level's sweep operands: the two x buffers (ping-pong)
// and b, each as a 3D FP32 tensor with the staged box of the TMA sweep.
// cls: one byte per x-quad, two bits per cell (0 interior with the plain
// coefficients, 1 Dirichlet, 2 domain edge with the plain coefficients,
// 3 anything else), rows padded to 16 bytes.
struct SweepMaps {
    CUtensorMap x[2];
    CUtensorMap b;
    CUtensorMap cls;
    CUtensorMap cls_cg;   // the same class bytes in the level-0 CG kernels' (shorter) boxes
    const float *xp[2] = {nullptr, nullptr};
    uint8_t *cls_ptr = nullptr;
    int cls_pitch = 0;
    // per cell of class 3: couplings across the upper x, y, z faces and the
    // reciprocal of the diagonal (other cells' entries are not written)
    float4 *gco = nullptr;
    // work order of the sweep's blocks (tile columns x z-chunks, those with
    // non-plain cells first)
    int *order = nullptr;
    // level 0: the work orders of the two TMA CG kernels
    int *order_pap = nullptr, *order_xr = nullptr;
    bool ok = false;
};

// Tensor maps of the level-0 CG operands for the TMA CG kernels: plane
// regions of 18 rows (16 for b) and 72 columns.
struct CgMaps {
    CUtensorMap z[2];          // preconditioned residual, in either sweep buffer
    CUtensorMap p[2];          // search directions (ping-pong)
    CUtensorMap xh[2], xl[2];  // iterate, high and low words (ping-pong)
    CUtensorMap b;             // right-hand side of the solve
    const float *zp[2] = {nullptr, nullptr};
    bool ds = false;
    bool ok = false;
};

// --------------------------------------------------------- kernel launchers --
namespace ffk {
// generic
int fill_f32(float *p, long long n, float v, cudaStream_t s);
int copy_bytes(void *dst, const void *src, size_t bytes, cudaStream_t s);

// coefficient / hierarchy preparation
int dirichlet_fields(Dims d, const uint8_t *active, const float *target, const float *cwu,
                     const float *cwv, const float *cww, uint8_t *mask, float *tgt,
                     uint8_t *vent, cudaStream_t s);
int system_weights(Dims d, const float *fw[3], const float *cw[3], float *sw[3], cudaStream_t s);
int build_coef(const Level &L, int dims, int want16, cudaStream_t s);
int coarsen_weights(const Level &f, Level &c, int dims, cudaStream_t s);
int coarsen_mask(const Level &f, const uint8_t *src, Level &c, int dims, cudaStream_t s);

// pressure build / correct / breaker
int build_system(Dims d, float hx, float hy, float hz, const float *u, const float *v,
                 const float *w, const float *cw[3], const float *fw[3], const float *sw[3],
                 const uint8_t *mask, const float *tgt, float *b, float *x_hi, float *x_lo,
                 cudaStream_t s);
int count_bad_and_commit(Dims d, float *x_hi0, float *x_lo0, float *x_hi1, float *x_lo1,
                         float *snap_hi, float *snap_lo, PcgState *st, float max_plausible,
                         int *bad_count, cudaStream_t s);
int correct(Dims d, float hx, float hy, float hz, const float *x_hi, const float *x_lo,
            const float *fw[3], const float *cw[3], const float *uin, const float *vin,
            const float *win, float *uout, float *vout, float *wout, cudaStream_t s);

// CG kernels (storage: 0 fp32, 1 bf16 for z)
int cg_setup_residual(Dims d, const float4 *coef, const float *b, const float *xh,
                      const float *xl, float *r, PcgState *st, double *partials, int ds,
                      cudaStream_t s);
int cg_update_p_pap(Dims d, const float4 *coef, const void *z, int zbf16, float *p0,
                    float *p1, PcgState *st, double *partials, cudaStream_t s);
int cg_update_x_residual(Dims d, const float4 *coef, const float *b, const float *p0,
                         const float *p1, float *xh0, float *xl0, float *xh1, float *xl1,
                         float *r, PcgState *st, double *partials, int ds, cudaStream_t s);
int cg_rz_beta(Dims d, const float *r, const void *z, int zbf16, PcgState *st,
               double *partials, int setup, cudaStream_t s);
int state_init(PcgState *st, double tol, int maxiter, int relative, cudaStream_t s);
int loop_control(PcgState *st, unsigned long long handle, int use_handle, cudaStream_t s);
int laplacian_apply(Dims d, const float4 *coef, const float *x, float *y, cudaStream_t s);
int jacobi_apply(Dims d, const float4 *coef, const float *r, void *z, int zbf16,
                 const PcgState *st, cudaStream_t s);
int identity_apply(Dims d, const float *r, void *z, int zbf16, const PcgState *st,
                   cudaStream_t s);

// multigrid kernels.  xbf/bbf: storage is bf16 when set.
int mg_relax(const Level &L, int dims, int colour, float sor, int first, int xbf, int bbf,
             int coef16, const PcgState *st, cudaStream_t s);
int mg_residual(const Level &L, int dims, int xbf, int bbf, int rbf, int coef16, const PcgState *st,
                cudaStream_t s);
int mg_restrict(const Level &f, Level &c, int dims, int fbf, int cbf, int zero_x,
                const PcgState *st, cudaStream_t s);
int mg_prolong(const Level &c, Level &f, int dims, int cbf, int fbf, const PcgState *st,
               cudaStream_t s);
int mg_coarse_sweeps(const Level &L, int dims, int sweeps, float sor, int xbf, int bbf,
                     int coef16, const PcgState *st, cudaStream_t s);
int mg_coarse_direct(const Level &L, const double *G, int n, int xbf, int bbf,
                     const PcgState *st, cudaStream_t s);
// fused FP32 kernels (ff_fused.cu)
size_t brick_count(const Dims &d);
bool fused_ok(const Dims &d);
int fused_configure();
size_t fused_blocks(const Dims &d, int sm_count);
int brick_flags(const Level &L, uint8_t *bricks, cudaStream_t s);
int sweep(const Level &L, const uint8_t *bricks, const float *x_in, float *x_out, int colour_a, float sor,
          int first, const Level *coarse, int dims, PcgState *st, double *partials, int rz_mode,
          int sm_count, cudaStream_t s);
// TMA-staged sweep (levels with nx % 4 == 0 and nx >= 32): x_in is the
// buffer maps.xp[in] (in < 0: x_in identically zero), x_out the other one
// residual r = b - A x and its restriction into the coarse b in two
// streaming passes through rx (nx/2 x ny x nz floats); needs cell classes
int res_restrict2(const Level &f, const SweepMaps &m, const float *x, float *rx, Level &c, int dims,
                  const PcgState *st, cudaStream_t s);
// x_f += P x_c on an FP32 level with nx % 4 == 0 (one thread per x-quad)
int prolong4(const Level &c, const Level &f, int dims, float *fine_x, const PcgState *st, cudaStream_t s);
bool sweep_tma_ok(const Dims &d);
size_t sweep_tma_cls_bytes(const Dims &d);
int sweep_tma_maps(const Level &L, const float *x0, const float *x1, uint8_t *cls, SweepMaps &m);
// the level's coefficients (as build_coef), classes, brick flags from the
// classes (when bricks is non-null) and work orders in one pass over the
// weights and mask
int coef_classes(const Level &L, const SweepMaps &m, uint8_t *bricks, int dims, int want16, int sm_count,
                 cudaStream_t s);
size_t cls_row_pitch(const Dims &d);
// the V-cycle from level lv[0] down to the coarsest lv[nl-1] and back, one
// cooperative launch (coarse_sweeps > 0: sweeps instead of G b at the bottom)
// bar: three words (arrivals, generation, abort), zero before the first
// launch and after a failed one; st may be null (no stop or error flags)
int vcycle_tail(const Level *lv, const SweepMaps *sm, int nl, int dims, int down, int up, float sor,
                const double *G, int nG, int coarse_sweeps, PcgState *st, unsigned *bar, int sm_count,
                cudaStream_t s);
int cg_tma_maps(const Level &L0, const float *z0, const float *z1, const float *p0, const float *p1,
                const float *xh0, const float *xl0, const float *xh1, const float *xl1, const float *b, bool ds,
                CgMaps &m);
int p_pap_tma(const Level &L0, const SweepMaps &sm, const CgMaps &m, const float *z, float *p0, float *p1,
              PcgState *st, double *partials, int sm_count, cudaStream_t s);
int x_residual_tma(const Level &L0, const SweepMaps &sm, const CgMaps &m, float *xh0, float *xl0, float *xh1,
                   float *xl1, float *r, PcgState *st, double *partials, int setup, int sm_count, cudaStream_t s);
int sweep_tma(const Level &L, const SweepMaps &m, const uint8_t *bricks, int in, int colour_a, float sor,
              PcgState *st, double *partials, int rz_mode, int sm_count, cudaStream_t s);
size_t sweep_tma_blocks(const Dims &d, int sm_count);
// work items of the level-0 TMA CG kernels (which: 0 p.Ap, 1 x + alpha p)
size_t cg_tma_items(const Dims &d, int sm_count, int which);
int res_restrict(const Level &f, const uint8_t *bricks, const float *x, Level &c, int dims,
                 const PcgState *st, int sm_count, cudaStream_t s);
int fused_p_pap(const Level &L0, const uint8_t *bricks, const float *z, float *p0, float *p1,
                PcgState *st, double *partials, int sm_count, cudaStream_t s);
int fused_x_residual(const Level &L0, const uint8_t *bricks, const float *p0, const float *p1,
                     const float *b, float *xh0, float *xl0, float *xh1, float *xl1, float *r,
                     PcgState *st, double *partials, int ds, int setup, int sm_count, cudaStream_t s);
// standalone restrict/prolong on fp32 fields (test hooks)
int mg_restrict_f32(Dims fd, int dims, const float *fine, const uint8_t *fmask,
                    const uint8_t *cmask, float *coarse, cudaStream_t s);
int mg_prolong_f32(Dims fd, int dims, const float *coarse, const uint8_t *fmask, float *fine,
                   cudaStream_t s);
}  // namespace ffk

// host-side FP64 factorisation of the coarsest level (ff_coarse.cpp)
int ff_coarse_inverse(int nx, int ny, int nz, const float4 *coef, std::vector<double> &G);
