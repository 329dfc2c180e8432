// Pressure projection: the host side of createGridPressureSolver3
// (fluxflow src/grid/grid_pressure_solver3.js:66-574) and of the GPU-resident
// PCG it drives (src/linalg/linalg.js:782-2469).
//
// A solve is two CUDA graphs: the setup sequence (linalg.js:1627-1637) and a
// conditional WHILE node whose body is one PCG iteration (linalg.js:1404-1436
// order).  The loop stops itself on the device (convergence, a guard, or the
// iteration cap), so the host waits once per solve instead of once per chunk
// (linalg.js:1817-1911).
#include "ff_internal.h"
#include <nvtx3/nvToolsExt.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdio>

namespace {
int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }
}

struct ff_pressure_s {
    ff_ctx ctx = nullptr;
    ff_pressure_desc desc{};
    Dims d{};
    int dims = 3;
    float hx = 1, hy = 1, hz = 1;
    int maxiter = 0;
    int check_bad = 1;
    int use_graph = 1;
    // FP32 V-cycle storage on the fused kernels (needs nx % 4 == 0 on every
    // level the sweeps run on); otherwise the per-colour kernels
    bool fused = false;

    // caller-owned inputs (borrowed handles)
    ff_field cw[3] = {nullptr, nullptr, nullptr};
    ff_field fw[3] = {nullptr, nullptr, nullptr};
    ff_field active = nullptr, target = nullptr;

    // owned fields
    ff_field pressure = nullptr, bfield = nullptr, maskf = nullptr, ventf = nullptr;
    float *tgt = nullptr;
    float *x_lo0 = nullptr, *x_hi1 = nullptr, *x_lo1 = nullptr;
    float *r = nullptr, *p0 = nullptr, *p1 = nullptr, *snap_hi = nullptr, *snap_lo = nullptr;
    void *z = nullptr;
    float *sw[3] = {nullptr, nullptr, nullptr};
    std::vector<Level> lv;
    bool has_mask = false, has_w = false;
    PcgState *st = nullptr;
    PcgState *st_host = nullptr;
    double *partials = nullptr;
    // FP32 fused path: a second x buffer per level (sweeps are out of
    // place), per-level regular-brick flags, and where z ends up
    std::vector<float *> x2;
    std::vector<uint8_t *> bricks;
    float *z_final = nullptr;
    // TMA descriptors per level (levels where the TMA sweep applies)
    SweepMaps *smaps = nullptr;
    CgMaps cgm;              // level-0 CG operands for the TMA CG kernels
    bool use_tma = true;
    // first level of the coarse V-cycle run as one cooperative launch (-1: none)
    int tail_l = -1;
    bool use_tail = true;
    unsigned *tail_bar = nullptr;   // its grid barrier: arrivals, generation, abort
    // learned warm start (borrowed network), its guess field, last choice
    ff_unet net = nullptr;
    ff_field guess = nullptr;
    int warm_used = -1;
    // reportNoiseFloor (grid_pressure_solver3.js:118-131, 517-542): off by
    // default; when on, the start's norm before the solve and max |r| after it
    bool report_floor = false;
    // ff_pressure3_project_host: the previous call's compute and download
    cudaEvent_t ev_compute = nullptr, ev_up = nullptr, ev_down = nullptr;
    bool host_started = false;
    double x0_norm = 0.0;
    unsigned *maxbits = nullptr, *maxbits_host = nullptr;

    // hash of the operator's inputs (Dirichlet active/target, collider and
    // face weights) at the last prepare, to skip rebuilding an unchanged
    // operator; a set_* call clears `prepared`
    unsigned long long *hash_dev = nullptr, *hash_host = nullptr;
    unsigned long long input_hash = 0;
    int rebuilds = 0;

    // coarsest direct solve
    double *G = nullptr;
    int nG = 0;
    std::vector<float4> coarse_key;

    // graphs
    cudaGraphExec_t setup_exec = nullptr, loop_exec = nullptr;
    cudaGraph_t setup_graph = nullptr, loop_graph = nullptr;
    bool prepared = false;

    int vbf() const { return desc.vcycle_storage == FF_STORE_BF16; }
    int ds() const { return desc.iterate == FF_ITERATE_DS; }
    cudaStream_t s() const { return ctx->stream; }
    float *xh0() const { return (float *)pressure->d; }
};

static void destroy_graphs(ff_pressure ps) {
    if (ps->setup_exec) cudaGraphExecDestroy(ps->setup_exec);
    if (ps->loop_exec) cudaGraphExecDestroy(ps->loop_exec);
    if (ps->setup_graph) cudaGraphDestroy(ps->setup_graph);
    if (ps->loop_graph) cudaGraphDestroy(ps->loop_graph);
    ps->setup_exec = ps->loop_exec = nullptr;
    ps->setup_graph = ps->loop_graph = nullptr;
}

extern "C" void ff_pressure_desc_default(ff_pressure_desc *d, const int *res, const double *h) {
    std::memset(d, 0, sizeof *d);
    for (int a = 0; a < 3; ++a) {
        d->resolution[a] = res ? res[a] : 1;
        d->grid_spacing[a] = h ? h[a] : 1.0;
    }
    d->preconditioner = FF_PRE_MULTIGRID;
    d->tolerance = 1e-6;
    d->max_iterations = 0;
    d->max_iterations_factor = 1.5;
    d->relative_tolerance = 1;
    d->max_plausible_pressure = 1e6;
    d->mg_levels = 1;
    d->mg_down = 2;
    d->mg_up = 2;
    d->mg_coarsest = 20;
    d->mg_final = 2;
    d->mg_sor = 1.0;
    d->mg_coarsen_mask = 1;
    d->mg_coarsen_weights = 1;
    d->mg_coarse_mode = FF_COARSE_SWEEPS;
    d->vcycle_storage = FF_STORE_FP32;
    d->iterate = FF_ITERATE_FP32;
}

static int alloc_f(float **p, long long n, cudaStream_t s) { return ff_dev_alloc((void **)p, (size_t)n * 4, s); }

static int compute_maxiter(const ff_pressure_desc &d, int dims) {
    if (d.max_iterations > 0) return d.max_iterations;
    int m = std::max(d.resolution[0], std::max(d.resolution[1], dims == 3 ? d.resolution[2] : 0));
    // grid_pressure_solver3.js:133 (factor 1 in 3D), grid_pressure_solver2.js:398 (4 in 2D)
    return (int)std::ceil(d.max_iterations_factor * m * (dims == 3 ? 1 : 4));
}

extern "C" int ff_pressure3_create(ff_ctx ctx, const ff_pressure_desc *desc, ff_pressure *out) {
    FF_CHECK(ctx && desc && out, FF_E_ARG, "ff_pressure3_create: NULL argument");
    *out = nullptr;
    const int *r = desc->resolution;
    FF_CHECK(r[0] > 0 && r[1] > 0 && r[2] > 0, FF_E_ARG, "grid_pressure_solver3: resolution must be positive");
    FF_CHECK(desc->preconditioner >= 0 && desc->preconditioner <= 2, FF_E_ARG,
             "grid_pressure_solver3: unknown preconditioner '%d' (expected multigrid, jacobi, none)",
             desc->preconditioner);
    int dims = r[2] > 1 ? 3 : 2;
    int L = std::max(1, desc->mg_levels);
    int div = 1 << (L - 1);
    FF_CHECK(r[0] % div == 0 && r[1] % div == 0 && (dims == 2 || r[2] % div == 0), FF_E_ARG,
             "multigrid: shape [%d, %d, %d] is not divisible by 2^(numberOfLevels-1)=%d (numberOfLevels=%d).",
             r[0], r[1], r[2], div, L);
    FF_CHECK(L <= 12, FF_E_LIMIT, "multigrid: at most 12 levels");
    if (desc->mg_coarse_mode == FF_COARSE_DIRECT) {
        long long nc = (long long)(r[0] / div) * (r[1] / div) * (dims == 3 ? r[2] / div : 1);
        FF_CHECK(nc <= 4096, FF_E_LIMIT, "multigrid: direct coarsest solve limited to 4096 cells, got %lld", nc);
    }
    cudaSetDevice(ctx->device);
    ff_pressure ps = new ff_pressure_s();
    ps->ctx = ctx;
    ps->desc = *desc;
    ps->desc.mg_levels = L;
    ps->d = Dims{r[0], r[1], r[2]};
    ps->dims = dims;
    ps->hx = (float)desc->grid_spacing[0];
    ps->hy = (float)desc->grid_spacing[1];
    ps->hz = (float)desc->grid_spacing[2];
    ps->maxiter = compute_maxiter(*desc, dims);
    if (desc->vcycle_storage == FF_STORE_FP32) {
        bool ok = true;
        for (int l = 0; l < L; ++l)
            if (l < L - 1 || l == 0) ok = ok && ffk::fused_ok(Dims{r[0] >> l, r[1] >> l, dims == 3 ? r[2] >> l : 1});
        ps->fused = ok;
        if (ok) {
            int rc = ffk::fused_configure();
            if (rc != FF_OK) { delete ps; return rc; }
        }
    }
    cudaStream_t s = ctx->stream;
    const long long n = ps->d.n();
    int shape[3] = {r[0], r[1], r[2]};
    int st = FF_OK;
    auto bail = [&](int code) { ff_pressure3_destroy(ps); return code; };
    if ((st = ff_field_create(ctx, FF_FLOAT, 3, shape, &ps->pressure))) return bail(st);
    if ((st = ff_field_create(ctx, FF_FLOAT, 3, shape, &ps->bfield))) return bail(st);
    if ((st = ff_field_create(ctx, FF_UINT8, 3, shape, &ps->maskf))) return bail(st);
    if ((st = ff_field_create(ctx, FF_UINT8, 3, shape, &ps->ventf))) return bail(st);
    if ((st = alloc_f(&ps->tgt, n, s))) return bail(st);
    if ((st = alloc_f(&ps->x_hi1, n, s))) return bail(st);
    if (ps->ds()) {
        if ((st = alloc_f(&ps->x_lo0, n, s))) return bail(st);
        if ((st = alloc_f(&ps->x_lo1, n, s))) return bail(st);
        if ((st = alloc_f(&ps->snap_lo, n, s))) return bail(st);
    }
    if ((st = alloc_f(&ps->r, n, s))) return bail(st);
    if ((st = alloc_f(&ps->p0, n, s))) return bail(st);
    if ((st = alloc_f(&ps->p1, n, s))) return bail(st);
    if ((st = alloc_f(&ps->snap_hi, n, s))) return bail(st);
    // the preconditioner output z (level-0 x of the V-cycle) stays FP32:
    // rounding it to BF16 quadruples the PCG iteration count, while BF16 on
    // the coarse levels and residual buffers costs about one iteration in ten
    const size_t vsz = ps->vbf() ? 2 : 4;
    if ((st = ff_dev_alloc(&ps->z, (size_t)n * 4, s))) return bail(st);
    long long nf[3] = {ps->d.nu(), ps->d.nv(), ps->d.nw()};
    for (int a = 0; a < dims; ++a)
        if ((st = alloc_f(&ps->sw[a], nf[a], s))) return bail(st);
    // hierarchy
    ps->lv.resize(L);
    for (int l = 0; l < L; ++l) {
        Level &v = ps->lv[l];
        int sc = 1 << l;
        v.d = Dims{r[0] / sc, r[1] / sc, dims == 3 ? r[2] / sc : 1};
        double hs[3] = {desc->grid_spacing[0] * sc, desc->grid_spacing[1] * sc, desc->grid_spacing[2] * sc};
        for (int a = 0; a < 3; ++a) v.h2inv[a] = (float)(1.0 / (hs[a] * hs[a]));
        long long ln = v.d.n();
        if ((st = ff_dev_alloc((void **)&v.coef, (size_t)ln * sizeof(float4), s))) return bail(st);
        if (ps->vbf() && (st = ff_dev_alloc((void **)&v.coef16, (size_t)ln * sizeof(uint2), s))) return bail(st);
        if (l > 0) {
            if ((st = ff_dev_alloc(&v.x, (size_t)ln * vsz, s))) return bail(st);
            if ((st = ff_dev_alloc(&v.b, (size_t)ln * vsz, s))) return bail(st);
            if ((st = ff_dev_alloc((void **)&v.mask, (size_t)ln, s))) return bail(st);
            long long lf[3] = {v.d.nu(), v.d.nv(), v.d.nw()};
            for (int a = 0; a < dims; ++a)
                if ((st = alloc_f(&v.w[a], lf[a], s))) return bail(st);
        } else {
            v.x = ps->z;
            v.b = ps->r;
        }
        if (l < L - 1 && (st = ff_dev_alloc(&v.buf, (size_t)ln * vsz, s))) return bail(st);
        float *x2 = nullptr;
        uint8_t *br = nullptr;
        if (ps->fused) {
            if ((st = alloc_f(&x2, ln, s))) return bail(st);
            if ((st = ff_dev_alloc((void **)&br, ffk::brick_count(v.d), s))) { ff_dev_free(x2); return bail(st); }
        }
        ps->x2.push_back(x2);
        ps->bricks.push_back(br);
    }
    if ((st = ff_dev_alloc((void **)&ps->st, sizeof(PcgState), s))) return bail(st);
    if ((st = ff_dev_alloc((void **)&ps->hash_dev, sizeof(unsigned long long), s))) return bail(st);
    if (cudaMallocHost(&ps->hash_host, sizeof(unsigned long long)) != cudaSuccess)
        return bail(ff_set_error(FF_E_NOMEM, "cudaMallocHost"));
    if (cudaMallocHost(&ps->st_host, sizeof(PcgState)) != cudaSuccess) return bail(ff_set_error(FF_E_NOMEM, "cudaMallocHost"));
    auto g = Dims{r[0], r[1], r[2]};
    long long blocks = (long long)div_up(g.nx, g.nx >= 128 ? 128 : g.nx >= 64 ? 64 : 32) *
                       div_up(g.ny, 256 / (g.nx >= 128 ? 128 : g.nx >= 64 ? 64 : 32)) * g.nz;
    blocks = std::max(blocks, (long long)div_up(n, 1024));
    blocks = std::max(blocks, (long long)ffk::fused_blocks(ps->d, ctx->sm_count));
    if (ps->fused) {
        ps->smaps = new SweepMaps[L];
        for (int l = 0; l < L; ++l) {
            Level &v = ps->lv[l];
            if (l == L - 1 || !ffk::sweep_tma_ok(v.d)) continue;
            uint8_t *cls = nullptr;
            if ((st = ff_dev_alloc((void **)&cls, ffk::sweep_tma_cls_bytes(v.d), s))) return bail(st);
            ps->smaps[l].cls_ptr = cls;
            float4 *gco = nullptr;
            if ((st = ff_dev_alloc((void **)&gco, (size_t)v.d.n() * sizeof(float4), s))) return bail(st);
            ps->smaps[l].gco = gco;
            int *order = nullptr;
            if ((st = ff_dev_alloc((void **)&order, ffk::sweep_tma_blocks(v.d, ctx->sm_count) * sizeof(int), s)))
                return bail(st);
            ps->smaps[l].order = order;
            if (l == 0) {
                for (int w = 0; w < 2; ++w) {
                    const size_t items = ffk::cg_tma_items(v.d, ctx->sm_count, w);
                    if ((st = ff_dev_alloc((void **)&order, items * sizeof(int), s))) return bail(st);
                    (w == 0 ? ps->smaps[l].order_pap : ps->smaps[l].order_xr) = order;
                    blocks = std::max(blocks, (long long)items);
                }
            }
            if ((st = ffk::sweep_tma_maps(v, (const float *)v.x, ps->x2[l], cls, ps->smaps[l]))) return bail(st);
            blocks = std::max(blocks, (long long)ffk::sweep_tma_blocks(v.d, ctx->sm_count));
        }
        // the coarse V-cycle in one launch: from the first level of at most
        // 64^3 cells (below level 0) whose levels down to the last but one
        // all have nx % 4 == 0 (class bytes per x-quad) and a residual buffer
        for (int l = 1; l < L - 1 && ps->tail_l < 0; ++l) {
            if (ps->lv[l].d.n() > (1LL << 18)) continue;
            bool ok = true;
            for (int q = l; q < L - 1; ++q) ok = ok && ps->lv[q].d.nx % 4 == 0 && ps->lv[q].buf;
            if (ok) ps->tail_l = l;
        }
        if (ps->tail_l >= 0 && (st = ff_dev_alloc((void **)&ps->tail_bar, 4 * sizeof(unsigned), s))) return bail(st);
        for (int l = ps->tail_l; l >= 0 && l < L - 1; ++l) {
            SweepMaps &m = ps->smaps[l];
            if (m.cls_ptr) continue;
            if ((st = ff_dev_alloc((void **)&m.cls_ptr, ffk::sweep_tma_cls_bytes(ps->lv[l].d), s))) return bail(st);
            if ((st = ff_dev_alloc((void **)&m.gco, (size_t)ps->lv[l].d.n() * sizeof(float4), s))) return bail(st);
            m.cls_pitch = (int)ffk::cls_row_pitch(ps->lv[l].d);
        }
    }
    if ((st = ff_dev_alloc((void **)&ps->partials, (size_t)blocks * 2 * sizeof(double), s))) return bail(st);
    if (ps->smaps && ps->smaps[0].ok &&
        (st = ffk::cg_tma_maps(ps->lv[0], (const float *)ps->z, ps->x2[0], ps->p0, ps->p1, ps->xh0(), ps->x_lo0,
                               ps->x_hi1, ps->x_lo1, (const float *)ps->bfield->d, ps->ds(), ps->cgm)))
        return bail(st);
    if (cudaStreamSynchronize(s) != cudaSuccess) return bail(ff_set_error(FF_E_CUDA, "sync after create"));
    *out = ps;
    return FF_OK;
}

extern "C" int ff_pressure3_destroy(ff_pressure ps) {
    if (!ps) return FF_OK;
    cudaStreamSynchronize(ps->ctx->stream);
    destroy_graphs(ps);
    ff_field_destroy(ps->guess);
    if (ps->smaps)
        for (size_t l = 0; l < ps->lv.size(); ++l) {
            ff_dev_free(ps->smaps[l].cls_ptr);
            ff_dev_free(ps->smaps[l].gco);
            ff_dev_free(ps->smaps[l].order);
            ff_dev_free(ps->smaps[l].order_pap);
            ff_dev_free(ps->smaps[l].order_xr);
        }
    delete[] ps->smaps;
    ff_dev_free(ps->tail_bar);
    ff_field_destroy(ps->pressure);
    ff_field_destroy(ps->bfield);
    ff_field_destroy(ps->maskf);
    ff_field_destroy(ps->ventf);
    float *fs[] = {ps->tgt, ps->x_lo0, ps->x_hi1, ps->x_lo1, ps->r, ps->p0, ps->p1, ps->snap_hi, ps->snap_lo};
    for (float *p : fs) ff_dev_free(p);
    ff_dev_free(ps->z);
    for (int a = 0; a < 3; ++a) ff_dev_free(ps->sw[a]);
    for (size_t l = 0; l < ps->lv.size(); ++l) {
        Level &v = ps->lv[l];
        ff_dev_free(v.coef);
        ff_dev_free(v.coef16);
        ff_dev_free(v.buf);
        if (l > 0) {
            ff_dev_free(v.x);
            ff_dev_free(v.b);
            ff_dev_free(v.mask);
            for (int a = 0; a < 3; ++a) ff_dev_free(v.w[a]);
        }
    }
    ff_dev_free(ps->st);
    if (ps->st_host) cudaFreeHost(ps->st_host);
    ff_dev_free(ps->hash_dev);
    for (cudaEvent_t e : {ps->ev_compute, ps->ev_up, ps->ev_down})
        if (e) cudaEventDestroy(e);
    ff_dev_free(ps->maxbits);
    if (ps->maxbits_host) cudaFreeHost(ps->maxbits_host);
    if (ps->hash_host) cudaFreeHost(ps->hash_host);
    ff_dev_free(ps->partials);
    for (float *p : ps->x2) ff_dev_free(p);
    for (uint8_t *p : ps->bricks) ff_dev_free(p);
    ff_dev_free(ps->G);
    delete ps;
    return FF_OK;
}

static int check_face_field(ff_pressure ps, ff_field f, int axis) {
    if (!f) return FF_OK;
    int want[3] = {ps->d.nx + (axis == 0), ps->d.ny + (axis == 1), ps->d.nz + (axis == 2)};
    if (ps->dims == 2 && axis == 2) return FF_OK;
    FF_CHECK(f->dtype == FF_FLOAT, FF_E_ARG, "face weights must be float fields");
    FF_CHECK(f->shape[0] == want[0] && f->shape[1] == want[1] && f->shape[2] == want[2], FF_E_ARG,
             "face field for axis %d has shape [%d, %d, %d], expected [%d, %d, %d]", axis, f->shape[0],
             f->shape[1], f->shape[2], want[0], want[1], want[2]);
    return FF_OK;
}

extern "C" int ff_pressure3_set_collider_weights(ff_pressure ps, ff_field u, ff_field v, ff_field w) {
    FF_CHECK(ps, FF_E_ARG, "NULL solver");
    FF_CHECK((u && v && (w || ps->dims == 2)) || (!u && !v && !w), FF_E_ARG,
             "collider weights need all of u, v%s or none", ps->dims == 3 ? ", w" : "");
    FF_TRY(check_face_field(ps, u, 0));
    FF_TRY(check_face_field(ps, v, 1));
    FF_TRY(check_face_field(ps, w, 2));
    ps->cw[0] = u; ps->cw[1] = v; ps->cw[2] = ps->dims == 3 ? w : nullptr;
    ps->prepared = false;
    return FF_OK;
}

extern "C" int ff_pressure3_set_face_weights(ff_pressure ps, ff_field u, ff_field v, ff_field w) {
    FF_CHECK(ps, FF_E_ARG, "NULL solver");
    FF_CHECK((u && v && (w || ps->dims == 2)) || (!u && !v && !w), FF_E_ARG,
             "face weights need all of u, v%s or none", ps->dims == 3 ? ", w" : "");
    FF_TRY(check_face_field(ps, u, 0));
    FF_TRY(check_face_field(ps, v, 1));
    FF_TRY(check_face_field(ps, w, 2));
    ps->fw[0] = u; ps->fw[1] = v; ps->fw[2] = ps->dims == 3 ? w : nullptr;
    ps->prepared = false;
    return FF_OK;
}

extern "C" int ff_pressure3_set_dirichlet(ff_pressure ps, ff_field active, ff_field target) {
    FF_CHECK(ps, FF_E_ARG, "NULL solver");
    if (active) {
        FF_CHECK(active->dtype == FF_UINT8 && active->count == ps->d.n(), FF_E_ARG,
                 "dirichlet active must be a u8 cell field of the solver's resolution");
    }
    if (target) {
        FF_CHECK(active, FF_E_ARG, "dirichlet target given without active");
        FF_CHECK(target->dtype == FF_FLOAT && target->count == ps->d.n(), FF_E_ARG,
                 "dirichlet target must be a float cell field of the solver's resolution");
    }
    ps->active = active;
    ps->target = target;
    ps->prepared = false;
    return FF_OK;
}

extern "C" int ff_pressure3_set(ff_pressure ps, const char *key, double value) {
    FF_CHECK(ps && key, FF_E_ARG, "NULL argument");
    std::string k(key);
    if (k == "tolerance") { ps->desc.tolerance = value; destroy_graphs(ps); }
    else if (k == "maxIterations") { ps->maxiter = (int)value; destroy_graphs(ps); }
    else if (k == "relativeTolerance") { ps->desc.relative_tolerance = value != 0; destroy_graphs(ps); }
    else if (k == "checkBadCells") ps->check_bad = value != 0;
    else if (k == "useGraph") { ps->use_graph = value != 0; }
    else if (k == "useTma") { ps->use_tma = value != 0; destroy_graphs(ps); }
    else if (k == "coarseTail") { ps->use_tail = value != 0; destroy_graphs(ps); }
    else if (k == "preconditioner") {
        FF_CHECK(value >= 0 && value <= 2, FF_E_ARG, "unknown preconditioner %g", value);
        ps->desc.preconditioner = (int)value;
        destroy_graphs(ps);
    } else if (k == "sorFactor") { ps->desc.mg_sor = value; destroy_graphs(ps); }
    else if (k == "reportNoiseFloor") ps->report_floor = value != 0;
    else return ff_set_error(FF_E_ARG, "unknown setting '%s'", key);
    return FF_OK;
}

extern "C" int ff_pressure3_fields(ff_pressure ps, ff_field *pressure, ff_field *b, ff_field *mask,
                                   ff_field *vent) {
    FF_CHECK(ps, FF_E_ARG, "NULL solver");
    if (pressure) *pressure = ps->pressure;
    if (b) *b = ps->bfield;
    if (mask) *mask = ps->maskf;
    if (vent) *vent = ps->ventf;
    return FF_OK;
}

// --------------------------------------------------------------- prepare --
static const float *fptr(ff_field f) { return f ? (const float *)f->d : nullptr; }

// a level's coefficients, brick flags, classes and work orders: one fused
// pass where the level keeps classes, else the coefficient kernels
static int build_level(ff_pressure ps, int l, cudaStream_t s) {
    Level &L = ps->lv[l];
    if (ps->smaps && ps->smaps[l].cls_ptr)
        return ffk::coef_classes(L, ps->smaps[l], ps->bricks[l], ps->dims, ps->vbf(), ps->ctx->sm_count, s);
    FF_TRY(ffk::build_coef(L, ps->dims, ps->vbf(), s));
    if (ps->bricks[l]) FF_TRY(ffk::brick_flags(L, ps->bricks[l], s));
    return FF_OK;
}

namespace {
// splitmix64 finaliser (Steele, Lea & Flood 2014)
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// acc += sum over each array's bytes, taken as 32-bit words (the last few
// bytes on their own), of mix64(position, word, salt): a sum, so the order
// in which blocks add does not matter.  All the arrays in one launch:
// blockIdx.y picks the array.
// (16-byte loads, two in flight a thread: the fields are 256-byte aligned;
// the words past the last whole 16 bytes and the last few bytes are taken
// by block 0 of the array)
struct HashFields {
    const unsigned char *p[8];
    long long nbytes[8];
    unsigned long long salt[8];
};
__device__ __forceinline__ unsigned long long hash16(const uint4 &q, long long i, unsigned long long salt) {
    const unsigned long long b = (unsigned long long)(4 * i) << 32;
    return mix64((b | q.x) ^ salt) + mix64(((b + (1ull << 32)) | q.y) ^ salt) +
           mix64(((b + (2ull << 32)) | q.z) ^ salt) + mix64(((b + (3ull << 32)) | q.w) ^ salt);
}
__global__ void k_hash_bytes(HashFields f, unsigned long long *__restrict__ acc) {
    const unsigned char *p = f.p[blockIdx.y];
    const long long nbytes = f.nbytes[blockIdx.y];
    const unsigned long long salt = f.salt[blockIdx.y];
    const long long nw = nbytes >> 2, n4 = nbytes >> 4;
    const uint32_t *w = reinterpret_cast<const uint32_t *>(p);
    const uint4 *w4 = reinterpret_cast<const uint4 *>(p);
    unsigned long long h = 0;
    const long long step = (long long)gridDim.x * blockDim.x;
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    for (; i + step < n4; i += 2 * step) {
        const uint4 q0 = __ldg(w4 + i), q1 = __ldg(w4 + i + step);
        h += hash16(q0, i, salt) + hash16(q1, i + step, salt);
    }
    if (i < n4) h += hash16(__ldg(w4 + i), i, salt);
    if (blockIdx.x == 0 && threadIdx.x < nw - 4 * n4) {
        const long long i = 4 * n4 + threadIdx.x;
        h += mix64(((unsigned long long)i << 32 | __ldg(w + i)) ^ salt);
    }
    if (blockIdx.x == 0 && threadIdx.x < (nbytes & 3))
        h += mix64(((unsigned long long)(nw * 4 + threadIdx.x) << 40 | p[nw * 4 + threadIdx.x]) ^ ~salt);
    for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc, h);
}
}  // namespace

// One hash of every input the operator and its hierarchy derive from (the
// Dirichlet active mask and targets, collider and face weights), read back
// to the host: equal hashes and no set_* call since the last prepare mean
// the Dirichlet fields, system weights, coarse levels, coefficients,
// classes, work orders and coarsest factorisation all still hold.
static int input_hash(ff_pressure ps, unsigned long long *out) {
    cudaStream_t s = ps->s();
    FF_CUDA(cudaMemsetAsync(ps->hash_dev, 0, sizeof(unsigned long long), s));
    ff_field fs[8] = {ps->active, ps->target, ps->cw[0], ps->cw[1], ps->cw[2], ps->fw[0], ps->fw[1], ps->fw[2]};
    HashFields hf;
    int nf = 0;
    long long most = 0;
    for (int q = 0; q < 8; ++q) {
        if (!fs[q]) continue;
        hf.p[nf] = (const unsigned char *)fs[q]->d;
        hf.nbytes[nf] = (long long)fs[q]->bytes;
        hf.salt[nf] = 0x5851F42D4C957F2Dull * (q + 1);
        most = std::max(most, hf.nbytes[nf]);
        ++nf;
    }
    if (nf > 0) {
        // about eight blocks an SM in all, two 16-byte loads a thread per round
        const long long want = std::max(1LL, (long long)ps->ctx->sm_count * 8 / nf);
        const int blocks = (int)std::max(1LL, std::min<long long>((most / 32 + 255) / 256, want));
        k_hash_bytes<<<dim3((unsigned)blocks, (unsigned)nf), 256, 0, s>>>(hf, ps->hash_dev);
    }
    FF_CUDA(cudaGetLastError());
    FF_CUDA(cudaMemcpyAsync(ps->hash_host, ps->hash_dev, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    FF_CUDA(cudaStreamSynchronize(s));
    *out = *ps->hash_host;
    return FF_OK;
}

static int prepare(ff_pressure ps, ff_field u, ff_field v, ff_field w) {
    cudaStream_t s = ps->s();
    const Dims &d = ps->d;
    Level &L0 = ps->lv[0];
    const float *cw[3] = {fptr(ps->cw[0]), fptr(ps->cw[1]), fptr(ps->cw[2])};
    const float *fw[3] = {fptr(ps->fw[0]), fptr(ps->fw[1]), fptr(ps->fw[2])};
    // the operator's inputs unchanged since the last prepare: only b is new
    unsigned long long h = 0;
    FF_TRY(input_hash(ps, &h));
    const bool reuse = ps->prepared && h == ps->input_hash;
    // updateDirichletFields (grid_pressure_solver3.js:171-206)
    ps->has_mask = ps->active || cw[0];
    // a zero mask is the same operator as no mask, so level 0 always reads
    // the solver's mask field and the graph's pointers never change
    uint8_t *mask = (uint8_t *)ps->maskf->d;
    if (reuse) {
    } else if (ps->has_mask) {
        FF_TRY(ffk::dirichlet_fields(d, ps->active ? (const uint8_t *)ps->active->d : nullptr,
                                     fptr(ps->target), cw[0], cw[1], cw[2], mask, ps->tgt,
                                     (uint8_t *)ps->ventf->d, s));
    } else {
        FF_CUDA(cudaMemsetAsync(ps->maskf->d, 0, ps->maskf->bytes, s));
        FF_CUDA(cudaMemsetAsync(ps->ventf->d, 0, ps->ventf->bytes, s));
    }
    // systemFaceWeights (:217-229)
    ps->has_w = fw[0] || cw[0];
    float *sw[3] = {nullptr, nullptr, nullptr};
    if (ps->has_w) {
        if (fw[0] && cw[0]) {
            for (int a = 0; a < ps->dims; ++a) sw[a] = ps->sw[a];
            if (!reuse) FF_TRY(ffk::system_weights(d, fw, cw, sw, s));
        } else {
            // one factor only: the system weights are those arrays themselves
            for (int a = 0; a < ps->dims; ++a) sw[a] = (float *)(fw[0] ? fw[a] : cw[a]);
        }
    }
    // the solve starts from the pressure field as the caller sees it: the
    // low word of the double-single iterate left by the previous solve is
    // cleared (the caller may have rewritten the high word)
    if (ps->x_lo0) FF_CUDA(cudaMemsetAsync(ps->x_lo0, 0, (size_t)d.n() * sizeof(float), s));
    // dispatchBuildSystem (:429-453); pins p at Dirichlet cells
    if (u) {
        FF_TRY(ffk::build_system(d, ps->hx, ps->hy, ps->hz, fptr(u), fptr(v), fptr(w), cw, fw,
                                 (const float **)sw, mask, ps->tgt, (float *)ps->bfield->d,
                                 ps->xh0(), ps->x_lo0, s));
    }
    // level 0 of the hierarchy reads the caller's mask and the system weights
    L0.mask = mask;
    for (int a = 0; a < 3; ++a) L0.w[a] = sw[a];
    const int Ln = (int)ps->lv.size();
    const bool cmask = ps->desc.mg_coarsen_mask != 0, cwgt = ps->desc.mg_coarsen_weights != 0;
    const bool coarsening_masks = (ps->has_mask && cmask) || (ps->has_w && cwgt);
    const bool use_coarse_w = ps->has_w && cwgt;
    if (reuse) return FF_OK;
    // refreshCoarseLevels (multigrid.js:416-452): weights before masks
    for (int l = 1; l < Ln; ++l) {
        Level &f = ps->lv[l - 1], &c = ps->lv[l];
        // unweighted coarse levels are weight 1 everywhere (multigrid.js:360-380)
        if (use_coarse_w) {
            FF_TRY(ffk::coarsen_weights(f, c, ps->dims, s));
        } else {
            long long lf[3] = {c.d.nu(), c.d.nv(), c.d.nw()};
            for (int a = 0; a < ps->dims; ++a) FF_TRY(ffk::fill_f32(c.w[a], lf[a], 1.f, s));
        }
        if (coarsening_masks) {
            const uint8_t *src = (!ps->has_mask || !cmask) ? nullptr
                                 : (l == 1 ? (const uint8_t *)ps->ventf->d : f.mask);
            // coarsen_mask reads the level's own weights for the enclosed guard
            // only when the level is weighted
            float *keep[3] = {c.w[0], c.w[1], c.w[2]};
            if (!use_coarse_w) c.w[0] = c.w[1] = c.w[2] = nullptr;
            int rc = ffk::coarsen_mask(f, src, c, ps->dims, s);
            for (int a = 0; a < 3; ++a) c.w[a] = keep[a];
            FF_TRY(rc);
        } else {
            FF_CUDA(cudaMemsetAsync(c.mask, 0, (size_t)c.d.n(), s));
        }
        FF_TRY(build_level(ps, l, s));
    }
    FF_TRY(build_level(ps, 0, s));
    ps->prepared = true;
    ps->input_hash = h;
    ++ps->rebuilds;
    // FP64 direct coarsest solve: refactor when the coarsest operator changed
    if (ps->desc.preconditioner == FF_PRE_MULTIGRID && ps->desc.mg_coarse_mode == FF_COARSE_DIRECT) {
        Level &c = ps->lv[Ln - 1];
        int nc = (int)c.d.n();
        std::vector<float4> key(nc);
        FF_CUDA(cudaMemcpyAsync(key.data(), c.coef, nc * sizeof(float4), cudaMemcpyDeviceToHost, s));
        FF_CUDA(cudaStreamSynchronize(s));
        bool same = ps->G && (int)ps->coarse_key.size() == nc &&
                    std::memcmp(key.data(), ps->coarse_key.data(), nc * sizeof(float4)) == 0;
        if (!same) {
            std::vector<double> G;
            FF_TRY(ff_coarse_inverse(c.d.nx, c.d.ny, c.d.nz, key.data(), G));
            if (!ps->G) FF_TRY(ff_dev_alloc((void **)&ps->G, (size_t)nc * nc * sizeof(double), s));
            FF_CUDA(cudaMemcpyAsync(ps->G, G.data(), (size_t)nc * nc * sizeof(double), cudaMemcpyHostToDevice, s));
            FF_CUDA(cudaStreamSynchronize(s));
            ps->nG = nc;
            ps->coarse_key.swap(key);
        }
    }
    return FF_OK;
}

extern "C" int ff_pressure3_prepare(ff_pressure ps, ff_field u, ff_field v, ff_field w) {
    FF_CHECK(ps, FF_E_ARG, "NULL solver");
    cudaSetDevice(ps->ctx->device);
    return prepare(ps, u, v, w);
}

// --------------------------------------------------------------- V-cycle --
static int relax_level(ff_pressure ps, int l, int iters, bool reversed, bool &first,
                       const PcgState *st) {
    Level &v = ps->lv[l];
    const int xbf = l == 0 ? 0 : ps->vbf(), bbf = l == 0 ? 0 : ps->vbf();
    const float sor = (float)ps->desc.mg_sor;
    for (int it = 0; it < iters; ++it) {
        for (int h = 0; h < 2; ++h) {
            int colour = reversed ? 1 - h : h;
            FF_TRY(ffk::mg_relax(v, ps->dims, colour, sor, first ? 1 : 0, xbf, bbf, ps->vbf(), st, ps->s()));
            first = false;
        }
    }
    return FF_OK;
}

static int zero_x(ff_pressure ps, int l) {
    Level &v = ps->lv[l];
    FF_CUDA(cudaMemsetAsync(v.x, 0, (size_t)v.d.n() * (ps->vbf() && l > 0 ? 2 : 4), ps->s()));
    return FF_OK;
}

// vCycle (multigrid.js:1609-1642); x of `l` is zero on entry.  Storage:
// level-0 x (z) and b (r) are FP32; coarse x, b and every residual buffer
// take the V-cycle storage type.
static int vcycle(ff_pressure ps, int l, const PcgState *st) {
    const int Ln = (int)ps->lv.size();
    const int vb = ps->vbf();
    Level &v = ps->lv[l];
    const int xbf = l == 0 ? 0 : vb, bbf = l == 0 ? 0 : vb;
    if (l == Ln - 1) {
        if (ps->desc.mg_coarse_mode == FF_COARSE_DIRECT) {
            return ffk::mg_coarse_direct(v, ps->G, ps->nG, xbf, bbf, st, ps->s());
        }
        long long n = v.d.n();
        if (n <= 16384) {
            if (l == 0) FF_TRY(zero_x(ps, 0));
            return ffk::mg_coarse_sweeps(v, ps->dims, ps->desc.mg_coarsest, (float)ps->desc.mg_sor, xbf,
                                         bbf, vb, st, ps->s());
        }
        bool first = true;
        return relax_level(ps, l, ps->desc.mg_coarsest, false, first, st);
    }
    Level &c = ps->lv[l + 1];
    bool first = true;
    if (ps->desc.mg_down <= 0 && l == 0) FF_TRY(zero_x(ps, 0));
    if (ps->desc.mg_down <= 0) first = false;
    FF_TRY(relax_level(ps, l, ps->desc.mg_down, false, first, st));
    FF_TRY(ffk::mg_residual(v, ps->dims, xbf, bbf, vb, vb, st, ps->s()));
    // the next level's x must be zero unless its own first relax pass or a
    // direct solve overwrites it
    bool next_is_coarsest = (l + 1 == Ln - 1);
    bool need_zero = next_is_coarsest ? (ps->desc.mg_coarse_mode != FF_COARSE_DIRECT &&
                                         c.d.n() <= 16384)
                                      : (ps->desc.mg_down <= 0);
    FF_TRY(ffk::mg_restrict(v, c, ps->dims, vb, vb, need_zero ? 1 : 0, st, ps->s()));
    FF_TRY(vcycle(ps, l + 1, st));
    FF_TRY(ffk::mg_prolong(c, v, ps->dims, vb, xbf, st, ps->s()));
    bool nf = false;
    return relax_level(ps, l, l > 0 ? ps->desc.mg_up : ps->desc.mg_final, true, nf, st);
}

// The FP32 V-cycle on fused sweeps.  Every sweep is out of place, so each
// level alternates between its two x buffers; the sequence is static, so
// where each level's result lands is known when the work is enqueued.
// `out` receives the buffer holding level l's final x.  rz_mode (level 0
// only): 0 none, 1 r.z + beta, 2 r.z + seed, fused into the last sweep; the
// return flag `rz_done` says whether it was.
// One fused sweep on level l from bufs[cur] (cur < 0: x = 0) into
// bufs[nxt]: the TMA-staged kernel where the level has descriptors, the
// cp.async kernel elsewhere.
static int level_sweep(ff_pressure ps, int l, PcgState *st, float *const bufs[2], int cur, int nxt, int colour_a,
                       int rz_mode) {
    Level &v = ps->lv[l];
    const float sor = (float)ps->desc.mg_sor;
    if (ps->use_tma && ps->smaps && ps->smaps[l].ok) {
        // descriptors index the buffers as {level x, second buffer}
        const int in = cur < 0 ? -1 : (bufs[cur] == ps->smaps[l].xp[0] ? 0 : 1);
        const int out = in == 0 ? 1 : 0;
        FF_CHECK(bufs[nxt] == ps->smaps[l].xp[out], FF_E_STATE, "sweep buffers do not match the TMA descriptors");
        return ffk::sweep_tma(v, ps->smaps[l], ps->bricks[l], in, colour_a, sor, st, ps->partials, rz_mode,
                              ps->ctx->sm_count, ps->s());
    }
    return ffk::sweep(v, ps->bricks[l], cur < 0 ? nullptr : bufs[cur], bufs[nxt], colour_a, sor, cur < 0, nullptr,
                      ps->dims, st, ps->partials, rz_mode, ps->ctx->sm_count, ps->s());
}

static int vcycle_fused(ff_pressure ps, int l, PcgState *st, int rz_mode, float **out, bool *rz_done) {
    const int Ln = (int)ps->lv.size();
    Level &v = ps->lv[l];
    cudaStream_t s = ps->s();
    const float sor = (float)ps->desc.mg_sor;
    float *bufs[2] = {(float *)v.x, ps->x2[l]};
    int cur = -1;   // -1: x is identically zero
    *rz_done = false;
    const bool direct = ps->desc.mg_coarse_mode == FF_COARSE_DIRECT;
    if (l == ps->tail_l && ps->use_tail && l > 0 && ps->tail_bar &&
        (direct ? ps->G != nullptr : ps->desc.mg_coarsest > 0)) {
        // this level and every coarser one in one cooperative launch
        FF_TRY(ffk::vcycle_tail(&ps->lv[l], &ps->smaps[l], Ln - l, ps->dims, ps->desc.mg_down, ps->desc.mg_up, sor,
                                direct ? ps->G : nullptr, direct ? ps->nG : 0, direct ? 0 : ps->desc.mg_coarsest, st,
                                ps->tail_bar, ps->ctx->sm_count, s));
        *out = (float *)v.x;
        return FF_OK;
    }
    if (l == Ln - 1) {
        if (ps->desc.mg_coarse_mode == FF_COARSE_DIRECT) {
            FF_TRY(ffk::mg_coarse_direct(v, ps->G, ps->nG, 0, 0, st, s));
        } else if (v.d.n() <= 16384) {
            FF_CUDA(cudaMemsetAsync(v.x, 0, (size_t)v.d.n() * 4, s));
            FF_TRY(ffk::mg_coarse_sweeps(v, ps->dims, ps->desc.mg_coarsest, sor, 0, 0, 0, st, s));
        } else {
            for (int it = 0; it < ps->desc.mg_coarsest; ++it) {
                int nxt = cur < 0 ? 0 : 1 - cur;
                FF_TRY(level_sweep(ps, l, st, bufs, cur, nxt, 0, 0));
                cur = nxt;
            }
            if (cur == 1) FF_CUDA(cudaMemcpyAsync(v.x, bufs[1], (size_t)v.d.n() * 4, cudaMemcpyDeviceToDevice, s));
        }
        *out = (float *)v.x;
        return FF_OK;
    }
    Level &c = ps->lv[l + 1];
    // pre-smoothing, colour 0 then 1 (relax, multigrid.js:1589-1607)
    for (int it = 0; it < ps->desc.mg_down; ++it) {
        int nxt = cur < 0 ? 0 : 1 - cur;
        FF_TRY(level_sweep(ps, l, st, bufs, cur, nxt, 0, 0));
        cur = nxt;
    }
    if (cur < 0) {
        FF_CUDA(cudaMemsetAsync(bufs[0], 0, (size_t)v.d.n() * 4, s));
        cur = 0;
    }
    // residual and restriction into the coarse b, fused (the fine residual
    // never reaches memory)
    if (ps->use_tma && ps->smaps && ps->smaps[l].ok && v.buf)
        FF_TRY(ffk::res_restrict2(v, ps->smaps[l], bufs[cur], (float *)v.buf, c, ps->dims, st, s));
    else
        FF_TRY(ffk::res_restrict(v, ps->bricks[l], bufs[cur], c, ps->dims, st, ps->ctx->sm_count, s));
    float *coarse_x = nullptr;
    bool dummy;
    FF_TRY(vcycle_fused(ps, l + 1, st, 0, &coarse_x, &dummy));
    Level coarse = c;
    coarse.x = coarse_x;
    // post-smoothing, colours reversed (1 then 0); the coarse-grid
    // correction rides on the first one
    const int up = l > 0 ? ps->desc.mg_up : ps->desc.mg_final;
    {
        // x += P e (buildCorrectKernel, multigrid.js:990-1040)
        Level tmp = v;
        tmp.x = bufs[cur];
        FF_TRY(ffk::prolong4(coarse, tmp, ps->dims, bufs[cur], st, s));
    }
    for (int it = 0; it < up; ++it) {
        int nxt = 1 - cur;
        bool last = it == up - 1;
        int rz = (l == 0 && last) ? rz_mode : 0;
        FF_TRY(level_sweep(ps, l, st, bufs, cur, nxt, 1, rz));
        if (rz) *rz_done = true;
        cur = nxt;
    }
    *out = bufs[cur];
    return FF_OK;
}

// z = M r.  rz_mode as in vcycle_fused; returns whether r.z was fused.
static int precondition_rz(ff_pressure ps, PcgState *st, int rz_mode, bool *rz_done) {
    const Dims &d = ps->d;
    *rz_done = false;
    if (ps->desc.preconditioner == FF_PRE_MULTIGRID) {
        if (!ps->fused) {
            ps->z_final = (float *)ps->z;
            return vcycle(ps, 0, st);
        }
        float *zf = nullptr;
        FF_TRY(vcycle_fused(ps, 0, st, rz_mode, &zf, rz_done));
        ps->z_final = zf;
        return FF_OK;
    }
    ps->z_final = (float *)ps->z;
    if (ps->desc.preconditioner == FF_PRE_JACOBI)
        return ffk::jacobi_apply(d, ps->lv[0].coef, ps->r, ps->z, 0, st, ps->s());
    return ffk::identity_apply(d, ps->r, ps->z, 0, st, ps->s());
}

static int precondition(ff_pressure ps, PcgState *st) {
    bool done;
    return precondition_rz(ps, st, 0, &done);
}

// ------------------------------------------------------------------ solve --
// clears the coarse V-cycle's barrier words (after a launch that gave up
// they keep its arrivals and abort flag)
static int reset_tail_bar(ff_pressure ps) {
    if (ps->tail_bar) FF_CUDA(cudaMemsetAsync(ps->tail_bar, 0, 4 * sizeof(unsigned), ps->s()));
    return FF_OK;
}

// the level-0 CG kernels run in the TMA layout when the sweep does
static bool cg_tma(const ff_pressure ps) { return ps->use_tma && ps->cgm.ok && ps->smaps && ps->smaps[0].ok; }

static int enqueue_setup(ff_pressure ps) {
    const Dims &d = ps->d;
    cudaStream_t s = ps->s();
    FF_TRY(ffk::state_init(ps->st, ps->desc.tolerance, ps->maxiter, ps->desc.relative_tolerance, s));
    FF_TRY(reset_tail_bar(ps));
    if (!ps->fused) {
        FF_TRY(ffk::cg_setup_residual(d, ps->lv[0].coef, (const float *)ps->bfield->d, ps->xh0(),
                                      ps->x_lo0, ps->r, ps->st, ps->partials, ps->ds(), s));
    } else {
        if (cg_tma(ps))
            FF_TRY(ffk::x_residual_tma(ps->lv[0], ps->smaps[0], ps->cgm, ps->xh0(), ps->x_lo0, ps->x_hi1, ps->x_lo1,
                                       ps->r, ps->st, ps->partials, 1, ps->ctx->sm_count, s));
        else
            FF_TRY(ffk::fused_x_residual(ps->lv[0], ps->bricks[0], ps->p0, ps->p1, (const float *)ps->bfield->d,
                                         ps->xh0(), ps->x_lo0, ps->x_hi1, ps->x_lo1, ps->r, ps->st, ps->partials,
                                         ps->ds(), 1, ps->ctx->sm_count, s));
    }
    bool rz_done;
    FF_TRY(precondition_rz(ps, ps->st, 2, &rz_done));
    if (!rz_done) FF_TRY(ffk::cg_rz_beta(d, ps->r, ps->z_final, 0, ps->st, ps->partials, 1, s));
    return FF_OK;
}

static int enqueue_iteration(ff_pressure ps, unsigned long long handle, int use_handle) {
    const Dims &d = ps->d;
    cudaStream_t s = ps->s();
    if (!ps->fused) {
        FF_TRY(ffk::cg_update_p_pap(d, ps->lv[0].coef, ps->z, 0, ps->p0, ps->p1, ps->st,
                                    ps->partials, s));
        FF_TRY(ffk::cg_update_x_residual(d, ps->lv[0].coef, (const float *)ps->bfield->d, ps->p0,
                                         ps->p1, ps->xh0(), ps->x_lo0, ps->x_hi1, ps->x_lo1, ps->r,
                                         ps->st, ps->partials, ps->ds(), s));
    } else {
        // z_final is static for a configuration: the setup's V-cycle left it
        const float *zf = ps->z_final ? ps->z_final : (const float *)ps->z;
        if (cg_tma(ps)) {
            FF_TRY(ffk::p_pap_tma(ps->lv[0], ps->smaps[0], ps->cgm, zf, ps->p0, ps->p1, ps->st, ps->partials,
                                  ps->ctx->sm_count, s));
            FF_TRY(ffk::x_residual_tma(ps->lv[0], ps->smaps[0], ps->cgm, ps->xh0(), ps->x_lo0, ps->x_hi1, ps->x_lo1,
                                       ps->r, ps->st, ps->partials, 0, ps->ctx->sm_count, s));
        } else {
            FF_TRY(ffk::fused_p_pap(ps->lv[0], ps->bricks[0], zf, ps->p0, ps->p1, ps->st, ps->partials,
                                    ps->ctx->sm_count, s));
            FF_TRY(ffk::fused_x_residual(ps->lv[0], ps->bricks[0], ps->p0, ps->p1, (const float *)ps->bfield->d,
                                         ps->xh0(), ps->x_lo0, ps->x_hi1, ps->x_lo1, ps->r, ps->st, ps->partials,
                                         ps->ds(), 0, ps->ctx->sm_count, s));
        }
    }
    bool rz_done;
    FF_TRY(precondition_rz(ps, ps->st, 1, &rz_done));
    if (!rz_done) FF_TRY(ffk::cg_rz_beta(d, ps->r, ps->z_final, 0, ps->st, ps->partials, 0, s));
    FF_TRY(ffk::loop_control(ps->st, handle, use_handle, s));
    return FF_OK;
}

static int build_graphs(ff_pressure ps) {
    destroy_graphs(ps);
    cudaStream_t s = ps->s();
    // setup graph
    FF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int st = enqueue_setup(ps);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (st != FF_OK) { if (g) cudaGraphDestroy(g); return st; }
    FF_CUDA(e);
    ps->setup_graph = g;
    FF_CUDA(cudaGraphInstantiate(&ps->setup_exec, g, 0));
    // loop graph: one conditional WHILE node
    cudaGraph_t lg = nullptr;
    FF_CUDA(cudaGraphCreate(&lg, 0));
    ps->loop_graph = lg;
    cudaGraphConditionalHandle h;
    FF_CUDA(cudaGraphConditionalHandleCreate(&h, lg, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    FF_CUDA(cudaGraphAddNode(&node, lg, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    FF_CUDA(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    st = enqueue_iteration(ps, (unsigned long long)h, 1);
    e = cudaStreamEndCapture(s, &body);
    FF_TRY(st);
    FF_CUDA(e);
    FF_CUDA(cudaGraphInstantiate(&ps->loop_exec, lg, 0));
    return FF_OK;
}

static int run_solve(ff_pressure ps) {
    cudaStream_t s = ps->s();
    if (ps->use_graph) {
        if (!ps->setup_exec) FF_TRY(build_graphs(ps));
        FF_CUDA(cudaGraphLaunch(ps->setup_exec, s));
        if (ps->maxiter > 0) FF_CUDA(cudaGraphLaunch(ps->loop_exec, s));
        return FF_OK;
    }
    // host-driven chunks (linalg.js:1817-1911), for comparison and fallback
    FF_TRY(enqueue_setup(ps));
    int ran = 0;
    while (ran < ps->maxiter) {
        int chunk = std::min(8, ps->maxiter - ran);
        for (int i = 0; i < chunk; ++i) FF_TRY(enqueue_iteration(ps, 0, 0));
        ran += chunk;
        FF_CUDA(cudaMemcpyAsync(ps->st_host, ps->st, sizeof(PcgState), cudaMemcpyDeviceToHost, s));
        FF_CUDA(cudaStreamSynchronize(s));
        if (ps->st_host->stop != 0) break;
    }
    return FF_OK;
}

static int read_diag(ff_pressure ps, ff_diag *diag, int extra_launches);
static int prepare_launches(ff_pressure ps, bool build);

namespace {
// sum over cells of (b - Ax)^2 into FP64 block partials
__global__ void k_res_sumsq(long long n, const float *__restrict__ b, const float *__restrict__ ax,
                            double *__restrict__ partial) {
    __shared__ double sred[256];
    double acc = 0.0;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const double r = (double)b[c] - (double)ax[c];
        acc += r * r;
    }
    sred[threadIdx.x] = acc;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) sred[threadIdx.x] += sred[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sred[0];
}
// sum over cells of (hi + lo)^2, the double-single iterate, into FP64 partials
__global__ void k_iterate_sumsq(long long n, const float *__restrict__ hi, const float *__restrict__ lo,
                                double *__restrict__ partial) {
    __shared__ double sred[256];
    double acc = 0.0;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const double x = (double)hi[c] + (lo ? (double)lo[c] : 0.0);
        acc += x * x;
    }
    sred[threadIdx.x] = acc;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) sred[threadIdx.x] += sred[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sred[0];
}
// createMaxAbsReducer (reduction.js:43-77): max over cells of |r| as the bits
// of a non-negative float, which order like the floats
__global__ void k_max_abs_bits(long long n, const float *__restrict__ r, unsigned *__restrict__ bits) {
    unsigned m = 0u;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        m = max(m, __float_as_uint(fabsf(r[c])));
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(bits, m);
}
// the network's guess pinned to the targets at Dirichlet cells
__global__ void k_guess_pin(long long n, const uint8_t *__restrict__ mask, const float *__restrict__ tgt,
                            float *__restrict__ g) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        if (mask[c]) g[c] = tgt[c];
}
// r = b - A g (zero on Dirichlet rows, whose residual the pin makes zero)
__global__ void k_guess_residual(long long n, const float *__restrict__ b, const float *__restrict__ ag,
                                 const uint8_t *__restrict__ mask, float *__restrict__ r) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        r[c] = mask[c] ? 0.0f : b[c] - ag[c];
}
// g += z off the Dirichlet cells
__global__ void k_guess_correct(long long n, const float *__restrict__ z, const uint8_t *__restrict__ mask,
                                float *__restrict__ g) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        if (!mask[c]) g[c] += z[c];
}
// the iterate becomes the guess; Dirichlet cells keep their targets
__global__ void k_apply_guess(long long n, const float *__restrict__ guess, const uint8_t *__restrict__ mask,
                              const float *__restrict__ tgt, float *__restrict__ hi, float *__restrict__ lo) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        hi[c] = mask[c] ? tgt[c] : guess[c];
        if (lo) lo[c] = 0.0f;
    }
}
}  // namespace

extern "C" int ff_pressure3_set_warm_start(ff_pressure ps, ff_unet net) {
    FF_CHECK(ps, FF_E_ARG, "NULL pressure solver");
    ps->net = net;
    if (net && !ps->guess) {
        int shape[3] = {ps->d.nx, ps->d.ny, ps->d.nz};
        FF_TRY(ff_field_create(ps->ctx, FF_FLOAT, 3, shape, &ps->guess));
    }
    return FF_OK;
}

// ||b - A x||^2 with the level-0 operator (x in `ax` scratch afterwards)
static int residual_sq(ff_pressure ps, const float *x, float *ax, double *out) {
    cudaStream_t s = ps->s();
    const long long n = ps->d.n();
    FF_TRY(ffk::laplacian_apply(ps->d, ps->lv[0].coef, x, ax, s));
    const int nb = 256;
    k_res_sumsq<<<nb, 256, 0, s>>>(n, (const float *)ps->bfield->d, ax, ps->partials);
    FF_CUDA(cudaGetLastError());
    std::vector<double> hp(nb);
    FF_CUDA(cudaMemcpyAsync(hp.data(), ps->partials, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
    FF_CUDA(cudaStreamSynchronize(s));
    double t = 0;
    for (double x2 : hp) t += x2;
    *out = t;
    return FF_OK;
}

// |x| of the start the solve runs from (estimateNoiseFloor's dotXX read,
// linalg.js:884-905)
static int start_norm(ff_pressure ps) {
    cudaStream_t s = ps->s();
    const int nb = 256;
    k_iterate_sumsq<<<nb, 256, 0, s>>>(ps->d.n(), ps->xh0(), ps->x_lo0, ps->partials);
    FF_CUDA(cudaGetLastError());
    std::vector<double> hp(nb);
    FF_CUDA(cudaMemcpyAsync(hp.data(), ps->partials, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
    FF_CUDA(cudaStreamSynchronize(s));
    double t = 0;
    for (double x2 : hp) t += x2;
    ps->x0_norm = std::sqrt(t);
    return FF_OK;
}

// max |r| of the last true residual, enqueued after the solve
static int enqueue_max_residual(ff_pressure ps) {
    cudaStream_t s = ps->s();
    if (!ps->maxbits) {
        FF_TRY(ff_dev_alloc((void **)&ps->maxbits, sizeof(unsigned), s));
        FF_CHECK(cudaMallocHost(&ps->maxbits_host, sizeof(unsigned)) == cudaSuccess, FF_E_NOMEM, "cudaMallocHost");
    }
    FF_CUDA(cudaMemsetAsync(ps->maxbits, 0, sizeof(unsigned), s));
    k_max_abs_bits<<<std::max(1, ps->ctx->sm_count * 4), 256, 0, s>>>(ps->d.n(), ps->r, ps->maxbits);
    FF_CUDA(cudaGetLastError());
    FF_CUDA(cudaMemcpyAsync(ps->maxbits_host, ps->maxbits, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    return FF_OK;
}

// learned warm start: predict, compare residuals, keep the better start
static int warm_start(ff_pressure ps) {
    ps->warm_used = -1;
    if (!ps->net) return FF_OK;
    cudaStream_t s = ps->s();
    int res[3] = {ps->d.nx, ps->d.ny, ps->d.nz};
    FF_TRY(ff_unet_forward(ps->net, res, (double)ps->hx, ps->bfield, ps->maskf, ps->pressure, ps->guess));
    // The network supplies the smooth part of the pressure; its error at the
    // grid scale, which the operator amplifies in the residual, is removed by
    // one preconditioner application: g += M^-1 (b - A g).
    if (ps->desc.preconditioner == FF_PRE_MULTIGRID) {
        const long long n = ps->d.n();
        float *g = (float *)ps->guess->d;
        const uint8_t *mask = (const uint8_t *)ps->maskf->d;
        k_guess_pin<<<256, 256, 0, s>>>(n, mask, ps->tgt, g);
        FF_TRY(ffk::laplacian_apply(ps->d, ps->lv[0].coef, g, ps->p0, s));
        k_guess_residual<<<256, 256, 0, s>>>(n, (const float *)ps->bfield->d, ps->p0, mask, ps->r);
        FF_CUDA(cudaGetLastError());
        FF_TRY(reset_tail_bar(ps));
        FF_TRY(precondition(ps, nullptr));
        k_guess_correct<<<256, 256, 0, s>>>(n, ps->z_final ? ps->z_final : (const float *)ps->z, mask, g);
        FF_CUDA(cudaGetLastError());
    }
    double r_prev, r_net;
    FF_TRY(residual_sq(ps, ps->xh0(), ps->r, &r_prev));
    FF_TRY(residual_sq(ps, (const float *)ps->guess->d, ps->p0, &r_net));
    ps->warm_used = 0;
    if (r_net < r_prev) {
        const long long n = ps->d.n();
        k_apply_guess<<<256, 256, 0, s>>>(n, (const float *)ps->guess->d, (const uint8_t *)ps->maskf->d, ps->tgt,
                                          ps->xh0(), ps->x_lo0);
        FF_CUDA(cudaGetLastError());
        ps->warm_used = 1;
    }
    return FF_OK;
}

extern "C" int ff_pressure3_project(ff_pressure ps, ff_field u_in, ff_field v_in, ff_field w_in,
                                    ff_field u_out, ff_field v_out, ff_field w_out, ff_diag *diag) {
    FF_CHECK(ps && u_in && v_in && u_out && v_out, FF_E_ARG, "project: NULL field");
    FF_CHECK(ps->dims == 2 || (w_in && w_out), FF_E_ARG, "project: 3D needs w fields");
    const Dims &d = ps->d;
    FF_CHECK(u_in->count == d.nu() && v_in->count == d.nv() && u_out->count == d.nu() &&
                 v_out->count == d.nv() && (ps->dims == 2 || (w_in->count == d.nw() && w_out->count == d.nw())),
             FF_E_ARG,
             "createGridPressureSolver3: project() input resolution does not match constructed resolution [%d, %d, %d].",
             d.nx, d.ny, d.nz);
    cudaSetDevice(ps->ctx->device);
    cudaStream_t s = ps->s();
    FF_TRY(prepare(ps, u_in, v_in, w_in));
    FF_TRY(warm_start(ps));
    if (ps->report_floor) FF_TRY(start_norm(ps));
    FF_TRY(run_solve(ps));
    if (ps->report_floor) FF_TRY(enqueue_max_residual(ps));
    // circuit breaker + snapshot (:289-336, :547-554), then the correction
    FF_TRY(ffk::count_bad_and_commit(d, ps->xh0(), ps->x_lo0, ps->x_hi1, ps->x_lo1, ps->snap_hi,
                                     ps->snap_lo, ps->st,
                                     ps->check_bad ? (float)ps->desc.max_plausible_pressure : INFINITY,
                                     nullptr, s));
    const float *cw[3] = {fptr(ps->cw[0]), fptr(ps->cw[1]), fptr(ps->cw[2])};
    const float *fw[3] = {fptr(ps->fw[0]), fptr(ps->fw[1]), fptr(ps->fw[2])};
    FF_TRY(ffk::correct(d, ps->hx, ps->hy, ps->hz, ps->xh0(), ps->x_lo0, fw, cw, fptr(u_in),
                        fptr(v_in), fptr(w_in), (float *)u_out->d, (float *)v_out->d,
                        w_out ? (float *)w_out->d : nullptr, s));
    // prepare + finish (count, commit, correct per axis)
    return read_diag(ps, diag, prepare_launches(ps, true) + 2 + ps->dims);
}

// project() with the velocity coming from and going to host memory: the
// upload runs on the context's upload stream after the previous call's
// compute (its last reads of the inputs), the projection on the compute
// stream after the upload and after the previous call's download (its outputs
// are about to be overwritten), the download on the download stream after the
// projection.  So a call's upload overlaps the previous call's download.  The
// host buffers should be page-locked; the downloaded values are in place after
// ff_ctx_synchronize (or after the next call's projection has started).
extern "C" int ff_pressure3_project_host(ff_pressure ps, ff_field u_in, ff_field v_in, ff_field w_in,
                                         const void *hu, const void *hv, const void *hw, ff_field u_out,
                                         ff_field v_out, ff_field w_out, void *hu_out, void *hv_out, void *hw_out,
                                         ff_diag *diag) {
    FF_CHECK(ps && u_in && v_in && u_out && v_out && hu && hv && hu_out && hv_out, FF_E_ARG,
             "project_host: NULL argument");
    FF_CHECK(ps->dims == 2 || (w_in && w_out && hw && hw_out), FF_E_ARG, "project_host: 3D needs w fields and buffers");
    cudaSetDevice(ps->ctx->device);
    FF_TRY(ff_ctx_copy_streams(ps->ctx));
    for (cudaEvent_t *e : {&ps->ev_compute, &ps->ev_up, &ps->ev_down})
        if (!*e) FF_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    cudaStream_t s = ps->s(), up = ps->ctx->up, down = ps->ctx->down;
    ff_field fin[3] = {u_in, v_in, ps->dims == 3 ? w_in : nullptr};
    ff_field fout[3] = {u_out, v_out, ps->dims == 3 ? w_out : nullptr};
    const void *hin[3] = {hu, hv, hw};
    void *hout[3] = {hu_out, hv_out, hw_out};
    if (ps->host_started) FF_CUDA(cudaStreamWaitEvent(up, ps->ev_compute, 0));
    for (int a = 0; a < 3; ++a)
        if (fin[a]) FF_CUDA(cudaMemcpyAsync(fin[a]->d, hin[a], fin[a]->bytes, cudaMemcpyHostToDevice, up));
    FF_CUDA(cudaEventRecord(ps->ev_up, up));
    FF_CUDA(cudaStreamWaitEvent(s, ps->ev_up, 0));
    if (ps->host_started) FF_CUDA(cudaStreamWaitEvent(s, ps->ev_down, 0));
    FF_TRY(ff_pressure3_project(ps, u_in, v_in, w_in, u_out, v_out, w_out, diag));
    FF_CUDA(cudaEventRecord(ps->ev_compute, s));
    FF_CUDA(cudaStreamWaitEvent(down, ps->ev_compute, 0));
    for (int a = 0; a < 3; ++a)
        if (fout[a]) FF_CUDA(cudaMemcpyAsync(hout[a], fout[a]->d, fout[a]->bytes, cudaMemcpyDeviceToHost, down));
    FF_CUDA(cudaEventRecord(ps->ev_down, down));
    ps->host_started = true;
    return FF_OK;
}

// kernel launches of one V-cycle, as vcycle() below enqueues them
static int vcycle_launches(ff_pressure ps) {
    const int Ln = (int)ps->lv.size();
    int n = 0;
    for (int l = 0; l < Ln - 1; ++l) {
        n += 2 * ps->desc.mg_down + 3 + 2 * (l > 0 ? ps->desc.mg_up : ps->desc.mg_final);
    }
    const Level &c = ps->lv[Ln - 1];
    if (ps->desc.mg_coarse_mode == FF_COARSE_DIRECT || c.d.n() <= 16384) n += 1;
    else n += 2 * ps->desc.mg_coarsest;
    return n;
}

static int precond_launches(ff_pressure ps) {
    return ps->desc.preconditioner == FF_PRE_MULTIGRID ? vcycle_launches(ps) : 1;
}

// prepare(): Dirichlet fields, system weights, build, per-level coarsening
static int prepare_launches(ff_pressure ps, bool build) {
    int n = (ps->has_mask ? 1 : 0) + (ps->has_w ? 1 : 0) + (build ? 1 : 0) + 1;
    n += ((int)ps->lv.size() - 1) * 2;   // coarsen weights (or fill), build_coef
    if ((ps->has_mask && ps->desc.mg_coarsen_mask) || (ps->has_w && ps->desc.mg_coarsen_weights))
        n += (int)ps->lv.size() - 1;
    return n;
}

static int read_diag(ff_pressure ps, ff_diag *diag, int extra_launches) {
    cudaStream_t s = ps->s();
    FF_CUDA(cudaMemcpyAsync(ps->st_host, ps->st, sizeof(PcgState), cudaMemcpyDeviceToHost, s));
    FF_CUDA(cudaStreamSynchronize(s));
    FF_CHECK(ps->st_host->err == 0, FF_E_CUDA,
             "a solver kernel gave up waiting for its staged data (error bits 0x%x); the result is invalid",
             ps->st_host->err);
    if (diag) {
        const PcgState &h = *ps->st_host;
        diag->converged = h.stop == FF_STOP_CONVERGED;
        diag->iterations = h.stop == FF_STOP_CONVERGED ? h.stop_iter : h.iter;
        diag->residual = std::sqrt(std::fabs(h.rr));
        diag->b_norm = std::sqrt(std::fabs(h.bb));
        // a guard that fired below the tolerance is a non-event (linalg.js:1702-1710)
        int sb = FF_STOP_NONE;
        if (h.stop != FF_STOP_NONE && h.stop != FF_STOP_CONVERGED && !(diag->residual < h.thr)) sb = h.stop;
        diag->stopped_by = sb;
        diag->bad_cells = h.bad_cells;
        diag->rejected = ps->check_bad && h.bad_cells > 0;
        diag->max_iterations = ps->maxiter;
        diag->warm_start = ps->warm_used;
        // reportNoiseFloor (linalg.js:884-905; grid_pressure_solver3.js:271-282,
        // 517-542): floor = eps_f32 * operatorScale * |x0|, operatorScale the
        // sum over the axes of 2 / h^2
        diag->report_floor = ps->report_floor ? 1 : 0;
        diag->max_residual = diag->noise_floor = diag->noise_floor_relative = 0.0;
        diag->tolerance_below_floor = 0;
        diag->floor_threshold = 0.0;
        if (ps->report_floor) {
            float mr;
            std::memcpy(&mr, ps->maxbits_host, sizeof(float));
            diag->max_residual = (double)mr;
            double scale = 2.0 / ((double)ps->hx * ps->hx) + 2.0 / ((double)ps->hy * ps->hy);
            if (ps->dims == 3) scale += 2.0 / ((double)ps->hz * ps->hz);
            const double fl = std::ldexp(1.0, -24) * scale * ps->x0_norm;
            diag->noise_floor = fl;
            diag->noise_floor_relative = diag->b_norm > 0 ? fl / diag->b_norm : 0.0;
            const double thr = ps->desc.relative_tolerance
                                   ? std::max(ps->desc.tolerance * diag->b_norm, ps->desc.tolerance)
                                   : ps->desc.tolerance;
            diag->floor_threshold = thr;
            diag->tolerance_below_floor = thr < fl ? 1 : 0;
        }
        // setup: state init, residual, preconditioner, r.z; then each loop
        // body the device ran: p/pAp, x/residual, preconditioner, r.z, control
        int per_iter = 4 + precond_launches(ps);
        diag->kernel_launches = extra_launches + 3 + precond_launches(ps) + h.launched * per_iter;
    }
    return FF_OK;
}

// solve(A p = b) for a given right-hand side: createPreconditionedConjugate-
// GradientSolver(...).solve (linalg.js:2176) on the solver's current system.
extern "C" int ff_pressure3_solve(ff_pressure ps, ff_field b, ff_diag *diag) {
    FF_CHECK(ps && b, FF_E_ARG, "NULL argument");
    FF_CHECK(b->count == ps->d.n() && b->dtype == FF_FLOAT, FF_E_ARG, "b must be a float cell field");
    cudaSetDevice(ps->ctx->device);
    cudaStream_t s = ps->s();
    FF_TRY(prepare(ps, nullptr, nullptr, nullptr));
    FF_CUDA(cudaMemcpyAsync(ps->bfield->d, b->d, b->bytes, cudaMemcpyDeviceToDevice, s));
    FF_TRY(warm_start(ps));
    if (ps->report_floor) FF_TRY(start_norm(ps));
    FF_TRY(run_solve(ps));
    if (ps->report_floor) FF_TRY(enqueue_max_residual(ps));
    FF_TRY(ffk::count_bad_and_commit(ps->d, ps->xh0(), ps->x_lo0, ps->x_hi1, ps->x_lo1, ps->snap_hi,
                                     ps->snap_lo, ps->st,
                                     ps->check_bad ? (float)ps->desc.max_plausible_pressure : INFINITY,
                                     nullptr, s));
    return read_diag(ps, diag, prepare_launches(ps, false) + 2);
}

// ------------------------------------------------------------- test hooks --
extern "C" int ff_laplacian_apply(ff_pressure ps, ff_field x, ff_field y) {
    FF_CHECK(ps && x && y, FF_E_ARG, "NULL argument");
    FF_CHECK(ps->prepared, FF_E_STATE, "call ff_pressure3_prepare first");
    FF_CHECK(x->count == ps->d.n() && y->count == ps->d.n(), FF_E_ARG, "field size mismatch");
    FF_TRY(ffk::laplacian_apply(ps->d, ps->lv[0].coef, (const float *)x->d, (float *)y->d, ps->s()));
    FF_CUDA(cudaStreamSynchronize(ps->s()));
    return FF_OK;
}

extern "C" int ff_precondition_apply(ff_pressure ps, ff_field r, ff_field z) {
    FF_CHECK(ps && r && z, FF_E_ARG, "NULL argument");
    FF_CHECK(ps->prepared, FF_E_STATE, "call ff_pressure3_prepare first");
    FF_CHECK(r->count == ps->d.n() && z->count == ps->d.n(), FF_E_ARG, "field size mismatch");
    cudaStream_t s = ps->s();
    FF_CUDA(cudaMemcpyAsync(ps->r, r->d, r->bytes, cudaMemcpyDeviceToDevice, s));
    FF_TRY(reset_tail_bar(ps));
    FF_TRY(precondition(ps, nullptr));
    long long n = ps->d.n();
    FF_CUDA(cudaMemcpyAsync(z->d, ps->z_final ? ps->z_final : ps->z, (size_t)n * 4, cudaMemcpyDeviceToDevice, s));
    FF_CUDA(cudaStreamSynchronize(s));
    if (ps->tail_bar) {
        // the coarse V-cycle's abort flag (this path has no solver state)
        unsigned abort_flag = 0;
        FF_CUDA(cudaMemcpy(&abort_flag, ps->tail_bar + 2, sizeof(unsigned), cudaMemcpyDeviceToHost));
        FF_CHECK(abort_flag == 0, FF_E_CUDA, "coarse V-cycle: a grid barrier timed out");
    }
    return FF_OK;
}

extern "C" int ff_mg_level_info(ff_pressure ps, int level, int *shape3) {
    FF_CHECK(ps && shape3, FF_E_ARG, "NULL argument");
    FF_CHECK(level >= 0 && level < (int)ps->lv.size(), FF_E_ARG, "level %d out of range", level);
    shape3[0] = ps->lv[level].d.nx;
    shape3[1] = ps->lv[level].d.ny;
    shape3[2] = ps->lv[level].d.nz;
    return FF_OK;
}

extern "C" int ff_mg_level_download(ff_pressure ps, int level, uint8_t *mask, float *wu, float *wv,
                                    float *ww) {
    FF_CHECK(ps, FF_E_ARG, "NULL solver");
    FF_CHECK(ps->prepared, FF_E_STATE, "call ff_pressure3_prepare first");
    FF_CHECK(level >= 0 && level < (int)ps->lv.size(), FF_E_ARG, "level %d out of range", level);
    Level &v = ps->lv[level];
    cudaStream_t s = ps->s();
    const Dims &d = v.d;
    if (mask) {
        if (v.mask) FF_CUDA(cudaMemcpyAsync(mask, v.mask, (size_t)d.n(), cudaMemcpyDeviceToHost, s));
        else std::memset(mask, 0, (size_t)d.n());
    }
    float *outs[3] = {wu, wv, ww};
    long long nf[3] = {d.nu(), d.nv(), d.nw()};
    bool weighted = ps->has_w && (level == 0 || ps->desc.mg_coarsen_weights);
    for (int a = 0; a < 3; ++a) {
        if (!outs[a]) continue;
        if (weighted && v.w[a]) FF_CUDA(cudaMemcpyAsync(outs[a], v.w[a], (size_t)nf[a] * 4, cudaMemcpyDeviceToHost, s));
        else std::fill(outs[a], outs[a] + nf[a], 1.0f);
    }
    FF_CUDA(cudaStreamSynchronize(s));
    return FF_OK;
}

extern "C" int ff_mg_restrict(ff_pressure ps, int fine_level, ff_field fine, ff_field coarse) {
    FF_CHECK(ps && fine && coarse, FF_E_ARG, "NULL argument");
    FF_CHECK(ps->prepared, FF_E_STATE, "call ff_pressure3_prepare first");
    FF_CHECK(fine_level >= 0 && fine_level + 1 < (int)ps->lv.size(), FF_E_ARG, "bad level");
    Level &f = ps->lv[fine_level], &c = ps->lv[fine_level + 1];
    FF_CHECK(fine->count == f.d.n() && coarse->count == c.d.n(), FF_E_ARG, "field size mismatch");
    FF_TRY(ffk::mg_restrict_f32(f.d, ps->dims, (const float *)fine->d, f.mask, c.mask, (float *)coarse->d, ps->s()));
    FF_CUDA(cudaStreamSynchronize(ps->s()));
    return FF_OK;
}

extern "C" int ff_mg_prolong_add(ff_pressure ps, int fine_level, ff_field coarse, ff_field fine) {
    FF_CHECK(ps && fine && coarse, FF_E_ARG, "NULL argument");
    FF_CHECK(ps->prepared, FF_E_STATE, "call ff_pressure3_prepare first");
    FF_CHECK(fine_level >= 0 && fine_level + 1 < (int)ps->lv.size(), FF_E_ARG, "bad level");
    Level &f = ps->lv[fine_level], &c = ps->lv[fine_level + 1];
    FF_CHECK(fine->count == f.d.n() && coarse->count == c.d.n(), FF_E_ARG, "field size mismatch");
    FF_TRY(ffk::mg_prolong_f32(f.d, ps->dims, (const float *)coarse->d, f.mask, (float *)fine->d, ps->s()));
    FF_CUDA(cudaStreamSynchronize(ps->s()));
    return FF_OK;
}

// Per-kernel device timing on the solver's own buffers (the role of
// fluxflow src/profiling.js:92-149 dispatch timing).  Each repetition is
// bracketed by CUDA events on the context stream; the PCG stop flag is
// cleared between repetitions so no launch exits early.
extern "C" int ff_pressure3_profile(ff_pressure ps, int which, int reps, float *avg_ms) {
    FF_CHECK(ps && avg_ms && reps > 0, FF_E_ARG, "NULL argument");
    FF_CHECK(ps->prepared, FF_E_STATE, "call ff_pressure3_prepare or project first");
    FF_CHECK(which >= 0 && which <= FF_PROF_ITERATION, FF_E_ARG, "unknown kernel id %d", which);
    cudaStream_t s = ps->s();
    const Dims &d = ps->d;
    Level &L0 = ps->lv[0];
    cudaEvent_t a, b;
    FF_CUDA(cudaEventCreate(&a));
    FF_CUDA(cudaEventCreate(&b));
    float total = 0.f;
    const int vb = ps->vbf();
    const bool nf = !ps->fused;   // profile the per-colour kernels when not fused
    // an NVTX range lets a profiler select exactly these launches
    FF_TRY(reset_tail_bar(ps));
    nvtxRangePushA("ff_profile");
    for (int r = 0; r < reps; ++r) {
        FF_CUDA(cudaMemsetAsync(&ps->st->stop, 0, sizeof(int), s));
        FF_CUDA(cudaEventRecord(a, s));
        int rc = FF_OK;
        switch (which) {
        case FF_PROF_P_PAP:
            rc = nf ? ffk::cg_update_p_pap(d, L0.coef, ps->z, 0, ps->p0, ps->p1, ps->st, ps->partials, s)
                 : cg_tma(ps) ? ffk::p_pap_tma(L0, ps->smaps[0], ps->cgm, (const float *)ps->z, ps->p0, ps->p1,
                                               ps->st, ps->partials, ps->ctx->sm_count, s)
                    : ffk::fused_p_pap(L0, ps->bricks[0], (float *)ps->z, ps->p0, ps->p1, ps->st, ps->partials,
                                       ps->ctx->sm_count, s);
            break;
        case FF_PROF_X_RESIDUAL:
            rc = nf ? ffk::cg_update_x_residual(d, L0.coef, (const float *)ps->bfield->d, ps->p0, ps->p1, ps->xh0(),
                                                ps->x_lo0, ps->x_hi1, ps->x_lo1, ps->r, ps->st, ps->partials,
                                                ps->ds(), s)
                 : cg_tma(ps) ? ffk::x_residual_tma(L0, ps->smaps[0], ps->cgm, ps->xh0(), ps->x_lo0, ps->x_hi1,
                                                    ps->x_lo1, ps->r, ps->st, ps->partials, 0, ps->ctx->sm_count, s)
                    : ffk::fused_x_residual(L0, ps->bricks[0], ps->p0, ps->p1, (const float *)ps->bfield->d,
                                            ps->xh0(), ps->x_lo0, ps->x_hi1, ps->x_lo1, ps->r, ps->st,
                                            ps->partials, ps->ds(), 0, ps->ctx->sm_count, s);
            break;
        case FF_PROF_RELAX:
            // BF16 path: one colour pass; FP32 path: one fused sweep (both colours)
            rc = nf ? ffk::mg_relax(L0, ps->dims, r & 1, (float)ps->desc.mg_sor, 0, 0, 0, vb, ps->st, s)
                    : [&] {
                          float *const bufs[2] = {(float *)L0.x, ps->x2[0]};
                          return level_sweep(ps, 0, ps->st, bufs, 0, 1, 0, 0);
                      }();
            break;
        case FF_PROF_RESIDUAL:
            // fused path: residual + restriction in one kernel
            if (nf) rc = ffk::mg_residual(L0, ps->dims, 0, 0, vb, vb, ps->st, s);
            else if (ps->lv.size() > 1 && ps->use_tma && ps->smaps && ps->smaps[0].ok && L0.buf)
                rc = ffk::res_restrict2(L0, ps->smaps[0], (const float *)L0.x, (float *)L0.buf, ps->lv[1], ps->dims,
                                        ps->st, s);
            else if (ps->lv.size() > 1)
                rc = ffk::res_restrict(L0, ps->bricks[0], (const float *)L0.x, ps->lv[1], ps->dims, ps->st,
                                       ps->ctx->sm_count, s);
            break;
        case FF_PROF_RESTRICT:
            rc = ps->lv.size() > 1 ? ffk::mg_restrict(L0, ps->lv[1], ps->dims, vb, vb, 0, ps->st, s) : FF_OK;
            break;
        case FF_PROF_PROLONG:
            if (ps->lv.size() > 1)
                rc = nf ? ffk::mg_prolong(ps->lv[1], L0, ps->dims, vb, 0, ps->st, s)
                        : ffk::prolong4(ps->lv[1], L0, ps->dims, (float *)L0.x, ps->st, s);
            break;
        case FF_PROF_RZ:
            rc = ffk::cg_rz_beta(d, ps->r, ps->z, 0, ps->st, ps->partials, 0, s);
            break;
        case FF_PROF_PRECONDITIONER:
            rc = precondition(ps, ps->st);
            break;
        case FF_PROF_ITERATION:
            rc = enqueue_iteration(ps, 0, 0);
            break;
        }
        FF_TRY(rc);
        FF_CUDA(cudaEventRecord(b, s));
        FF_CUDA(cudaEventSynchronize(b));
        float ms = 0.f;
        FF_CUDA(cudaEventElapsedTime(&ms, a, b));
        total += ms;
    }
    nvtxRangePop();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *avg_ms = total / reps;
    return FF_OK;
}
