// Static SDF collider bake and fractional face weights, on the device in
// FP64 (the reference does both on the CPU in JS doubles and stores f32):
//   createSDFStaticCollider3.addShapes  (fluxflow src/grid/sdf_collider3.js:69-99)
//   computeFaceWeights                  (sdf_collider3.js:131-254)
//   fractionInsideCpu / fractionInsideSdfCpu (src/grid/level_set_utils.js:51-161)
//   primitiveDistanceCpu                (src/grid/primitive_sdf3.js:169-208)
#include "ff_internal.h"
#include <atomic>
#include <cmath>
#include <cstring>

namespace {

constexpr double MIN_FACE_WEIGHT = 0.01;   // sdf_collider3.js:23

struct Shape {
    int type;            // 0 sphere, 1 box
    int has_rotation;
    double center[3];
    double radius;
    double half[3];
    double axis[3];      // normalised
    double angle;
};

__device__ double prim_distance(const Shape &s, double x, double y, double z) {
    double lx = x - s.center[0], ly = y - s.center[1], lz = z - s.center[2];
    if (s.type == 0) return sqrt(lx * lx + ly * ly + lz * lz) - s.radius;
    double qx = lx, qy = ly, qz = lz;
    if (s.has_rotation) {
        // rotateAroundAxisCpu(v, axis, -angle): Rodrigues rotation
        double a = -s.angle, c = cos(a), sn = sin(a);
        double kx = s.axis[0], ky = s.axis[1], kz = s.axis[2];
        double cx = ky * lz - kz * ly, cy = kz * lx - kx * lz, cz = kx * ly - ky * lx;
        double kd = kx * lx + ky * ly + kz * lz;
        qx = lx * c + cx * sn + kx * kd * (1 - c);
        qy = ly * c + cy * sn + ky * kd * (1 - c);
        qz = lz * c + cz * sn + kz * kd * (1 - c);
    }
    double dx = fabs(qx) - s.half[0], dy = fabs(qy) - s.half[1], dz = fabs(qz) - s.half[2];
    double mx = fmax(dx, 0.0), my = fmax(dy, 0.0), mz = fmax(dz, 0.0);
    double outside = sqrt(mx * mx + my * my + mz * mz);
    double inside = fmin(fmax(dx, fmax(dy, dz)), 0.0);
    return outside + inside;
}

__device__ double shapes_distance(const Shape *sh, int n, double x, double y, double z, double sign) {
    double d = INFINITY;
    for (int q = 0; q < n; ++q) d = fmin(d, prim_distance(sh[q], x, y, z));
    return sign * d;
}

__device__ double frac_sdf(double p0, double p1) {
    bool i0 = p0 < 0, i1 = p1 < 0;
    if (i0 && i1) return 1.0;
    if (i0 && !i1) return p0 / (p0 - p1);
    if (!i0 && i1) return p1 / (p1 - p0);
    return 0.0;
}

__device__ void cycle4(double *a) {
    double t = a[0];
    a[0] = a[1]; a[1] = a[2]; a[2] = a[3]; a[3] = t;
}

// fractionInsideCpu (level_set_utils.js:89-161)
__device__ double fraction_inside(double bl, double br, double tl, double tr) {
    int cnt = (bl < 0) + (tl < 0) + (br < 0) + (tr < 0);
    double L[4] = {bl, br, tr, tl};
    if (cnt == 4) return 1.0;
    if (cnt == 3) {
        for (int g = 0; g < 4 && L[0] < 0; ++g) cycle4(L);
        double s0 = 1 - frac_sdf(L[0], L[3]);
        double s1 = 1 - frac_sdf(L[0], L[1]);
        return 1 - 0.5 * s0 * s1;
    }
    if (cnt == 2) {
        for (int g = 0; g < 4 && (L[0] >= 0 || !(L[1] < 0 || L[2] < 0)); ++g) cycle4(L);
        if (L[1] < 0) {
            double sl = frac_sdf(L[0], L[3]);
            double sr = frac_sdf(L[1], L[2]);
            return 0.5 * (sl + sr);
        }
        double mid = 0.25 * (L[0] + L[1] + L[2] + L[3]);
        if (mid < 0) {
            double area = 0;
            double s1 = 1 - frac_sdf(L[0], L[3]);
            double s3 = 1 - frac_sdf(L[2], L[3]);
            area += 0.5 * s1 * s3;
            double s2 = 1 - frac_sdf(L[2], L[1]);
            double s0 = 1 - frac_sdf(L[0], L[1]);
            area += 0.5 * s0 * s2;
            return 1 - area;
        }
        double area = 0;
        double s0 = frac_sdf(L[0], L[1]);
        double s1 = frac_sdf(L[0], L[3]);
        area += 0.5 * s0 * s1;
        double s2 = frac_sdf(L[2], L[1]);
        double s3 = frac_sdf(L[2], L[3]);
        area += 0.5 * s2 * s3;
        return area;
    }
    if (cnt == 1) {
        for (int g = 0; g < 4 && L[0] >= 0; ++g) cycle4(L);
        double s0 = frac_sdf(L[0], L[3]);
        double s1 = frac_sdf(L[0], L[1]);
        return 0.5 * s0 * s1;
    }
    return 0.0;
}

__global__ void k_bake_phi(const Shape *sh, int ns, double sign, int nx, int ny, int nz,
                           double ox, double oy, double oz, double hx, double hy, double hz,
                           float *phi) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y,
        k = blockIdx.z;
    if (i >= nx || j >= ny) return;
    // originXCpu = originX + 0.5 gridSpacingX; x = originXCpu + i gridSpacingX
    double x = (ox + 0.5 * hx) + i * hx, y = (oy + 0.5 * hy) + j * hy, z = (oz + 0.5 * hz) + k * hz;
    phi[i + (long long)nx * (j + (long long)ny * k)] = (float)shapes_distance(sh, ns, x, y, z, sign);
}

__global__ void k_face_weights(const Shape *sh, int ns, double sign, int axis, int fx, int fy,
                               int fz, double ox, double oy, double oz, double gx, double gy,
                               double gz, float *w) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y,
        k = blockIdx.z;
    if (i >= fx || j >= fy) return;
    const double hx = 0.5 * gx, hy = 0.5 * gy, hz = 0.5 * gz;
    double x = ox + i * gx, y = oy + j * gy, z = oz + k * gz;
    double off[4][3];
    if (axis == 0) {
        double o[4][3] = {{0, -hy, -hz}, {0, hy, -hz}, {0, -hy, hz}, {0, hy, hz}};
        memcpy(off, o, sizeof o);
    } else if (axis == 1) {
        double o[4][3] = {{-hx, 0, -hz}, {hx, 0, -hz}, {-hx, 0, hz}, {hx, 0, hz}};
        memcpy(off, o, sizeof o);
    } else {
        double o[4][3] = {{-hx, -hy, 0}, {hx, -hy, 0}, {-hx, hy, 0}, {hx, hy, 0}};
        memcpy(off, o, sizeof o);
    }
    double c[4];
    for (int q = 0; q < 4; ++q)
        c[q] = shapes_distance(sh, ns, x + off[q][0], y + off[q][1], z + off[q][2], sign);
    double frac = fraction_inside(c[0], c[1], c[2], c[3]);
    double wv = fmin(1.0, fmax(0.0, 1.0 - frac));
    if (c[0] <= 0 && c[1] <= 0 && c[2] <= 0 && c[3] <= 0) wv = 0.0;
    else if (wv > 0 && wv < MIN_FACE_WEIGHT) wv = MIN_FACE_WEIGHT;
    w[i + (long long)fx * (j + (long long)fy * k)] = (float)wv;
}

}  // namespace

// Host records of the caller's shapes as the kernels read them
// (primitive_sdf3.js:169-200); rejects unknown types.
static int shape_records(const ff_shape *shapes, int nshapes, Shape *out) {
    for (int q = 0; q < nshapes; ++q) {
        const ff_shape &src = shapes[q];
        FF_CHECK(src.type == FF_SHAPE_SPHERE || src.type == FF_SHAPE_BOX, FF_E_ARG,
                 "primitive_sdf3: unknown shape type '%d'.", src.type);
        Shape &dst = out[q];
        dst.type = src.type == FF_SHAPE_SPHERE ? 0 : 1;
        dst.has_rotation = src.has_rotation;
        for (int c = 0; c < 3; ++c) {
            dst.center[c] = src.center[c];
            dst.half[c] = src.half_extents[c];
        }
        dst.radius = src.radius;
        const double len = std::sqrt(src.rotation_axis[0] * src.rotation_axis[0] +
                                     src.rotation_axis[1] * src.rotation_axis[1] +
                                     src.rotation_axis[2] * src.rotation_axis[2]);
        for (int c = 0; c < 3; ++c) dst.axis[c] = len > 0 ? src.rotation_axis[c] / len : (c == 2 ? 1.0 : 0.0);
        dst.angle = src.rotation_angle;
    }
    return FF_OK;
}

// Output fields must be float fields of the cell / face sizes (any may be NULL).
static int check_bake_fields(const int *res, ff_field phi, const ff_field ws[3]) {
    const int nx = res[0], ny = res[1], nz = res[2];
    FF_CHECK(!phi || (phi->count == (long long)nx * ny * nz && phi->dtype == FF_FLOAT), FF_E_ARG, "phi field shape");
    for (int a = 0; a < 3; ++a)
        FF_CHECK(!ws[a] || (ws[a]->count == (long long)(nx + (a == 0)) * (ny + (a == 1)) * (nz + (a == 2)) &&
                            ws[a]->dtype == FF_FLOAT),
                 FF_E_ARG, "face weight field %d shape", a);
    return FF_OK;
}

// phi and the face weights from a device shape table, on stream s
static void launch_bake(const Shape *table, int nshapes, int invert, const int *res, const double *h,
                        const double *origin, ff_field phi, const ff_field ws[3], cudaStream_t s) {
    const int nx = res[0], ny = res[1], nz = res[2];
    const double sign = invert ? -1.0 : 1.0;
    const dim3 blk(64, 4, 1);
    if (phi) {
        dim3 g((nx + 63) / 64, (ny + 3) / 4, nz);
        k_bake_phi<<<g, blk, 0, s>>>(table, nshapes, sign, nx, ny, nz, origin[0], origin[1], origin[2], h[0], h[1],
                                     h[2], (float *)phi->d);
    }
    for (int a = 0; a < 3; ++a) {
        if (!ws[a]) continue;
        const int fx = nx + (a == 0), fy = ny + (a == 1), fz = nz + (a == 2);
        // dataOriginU/V/W (sdf_collider3.js:226-228)
        const double o[3] = {origin[0] + (a != 0 ? 0.5 * h[0] : 0.0), origin[1] + (a != 1 ? 0.5 * h[1] : 0.0),
                             origin[2] + (a != 2 ? 0.5 * h[2] : 0.0)};
        dim3 g((fx + 63) / 64, (fy + 3) / 4, fz);
        k_face_weights<<<g, blk, 0, s>>>(table, nshapes, sign, a, fx, fy, fz, o[0], o[1], o[2], h[0], h[1], h[2],
                                         (float *)ws[a]->d);
    }
}

extern "C" int ff_collider3_bake(ff_ctx ctx, const ff_shape *shapes, int nshapes, int invert,
                                 const int *res, const double *h, const double *origin,
                                 ff_field phi, ff_field wu, ff_field wv, ff_field ww) {
    FF_CHECK(ctx && res && h && origin, FF_E_ARG, "ff_collider3_bake: NULL argument");
    FF_CHECK(nshapes >= 0 && nshapes <= 64, FF_E_LIMIT, "ff_collider3_bake: at most 64 shapes");
    FF_CHECK(nshapes == 0 || shapes, FF_E_ARG, "ff_collider3_bake: shapes is NULL");
    const ff_field ws[3] = {wu, wv, ww};
    FF_TRY(check_bake_fields(res, phi, ws));
    Shape hs[64];
    FF_TRY(shape_records(shapes, nshapes, hs));
    cudaStream_t s = ctx->stream;
    Shape *dsh = nullptr;
    FF_CUDA(cudaMalloc(&dsh, sizeof(Shape) * (nshapes > 0 ? nshapes : 1)));
    cudaError_t e = cudaSuccess;
    if (nshapes) e = cudaMemcpyAsync(dsh, hs, sizeof(Shape) * nshapes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        launch_bake(dsh, nshapes, invert, res, h, origin, phi, ws, s);
        e = cudaGetLastError();
    }
    // the kernels read dsh: wait for them before freeing it
    const cudaError_t es = cudaStreamSynchronize(s);
    cudaFree(dsh);
    FF_CUDA(e);
    FF_CUDA(es);
    return FF_OK;
}

// ---------------------------------------------------------------------------
// ff_collider3_bake_noalloc: the same bake with its shape table in a
// fixed-size device array instead of a per-call cudaMalloc/cudaFree.
//
// Who needs it: a host that bakes colliders inside a loop where a device
// allocation is not allowed -- a process running under a fixed device-memory
// budget managed by someone else's pool, or a frame loop where the implicit
// device-wide synchronisation of cudaMalloc/cudaFree would stall work queued
// on other streams.  This entry point makes no allocation and no allocating
// library call; its only device scratch is g_bake_shapes below.
//
// Setup: the first call on each device looks up the array's device address
// (cudaGetSymbolAddress, which may load the module); make that first call
// before any stream capture.  Later calls launch three kinds of kernels
// only: the table travels to the device as a kernel parameter (no host copy,
// no host buffer that has to outlive the call), k_store_shapes writes it into
// g_bake_shapes, and the bake kernels read it from there, in stream order.
//
// Nothing in the table has to start at zero: the kernels read entries
// 0..nshapes-1 only, and this call writes exactly those before its kernels
// run.  There is one table per device and calls return before their kernels
// finish, so two calls are safe only when they are ordered on the GPU: the
// same stream, or the second caller waits for the first call's stream (an
// event or a synchronize) before it calls.  Calls from two contexts' streams
// or two host threads on one device without such an order race on it.
namespace {
constexpr int BAKE_NOALLOC_MAX_SHAPES = FF_BAKE_NOALLOC_MAX_SHAPES;
static __device__ __align__(256) Shape g_bake_shapes[BAKE_NOALLOC_MAX_SHAPES];

// the whole table as one kernel parameter (7 KB, below the 32 KB limit)
struct ShapeTable {
    Shape s[BAKE_NOALLOC_MAX_SHAPES];
};

__global__ void k_store_shapes(const __grid_constant__ ShapeTable t, int n, Shape *dst) {
    const int q = threadIdx.x;
    if (q < n) dst[q] = t.s[q];
}

constexpr int MAX_DEVICES = 64;
std::atomic<void *> g_bake_table[MAX_DEVICES] = {};

// device address of g_bake_shapes on `device` (the current device), looked up
// once per device
int bake_table(int device, Shape **out) {
    FF_CHECK(device >= 0 && device < MAX_DEVICES, FF_E_LIMIT, "ff_collider3_bake_noalloc: device %d out of range",
             device);
    void *p = g_bake_table[device].load(std::memory_order_acquire);
    if (!p) {
        cudaError_t e = cudaGetSymbolAddress(&p, g_bake_shapes);
        FF_CHECK(e == cudaSuccess && p, FF_E_CUDA, "ff_collider3_bake_noalloc: cudaGetSymbolAddress: %s",
                 cudaGetErrorString(e));
        g_bake_table[device].store(p, std::memory_order_release);
    }
    *out = static_cast<Shape *>(p);
    return FF_OK;
}

// makes `device` current for the call and gives the caller's current device
// back on every return path
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != device) cudaSetDevice(device);
    }
    ~DeviceScope() {
        int now = -1;
        if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
    }
};
}  // namespace

extern "C" int ff_collider3_bake_noalloc(ff_ctx ctx, const ff_shape *shapes, int nshapes, int invert,
                                         const int *res, const double *h, const double *origin, ff_field phi,
                                         ff_field wu, ff_field wv, ff_field ww) {
    FF_CHECK(ctx && res && h && origin, FF_E_ARG, "ff_collider3_bake_noalloc: NULL argument");
    FF_CHECK(nshapes >= 0 && nshapes <= BAKE_NOALLOC_MAX_SHAPES, FF_E_LIMIT,
             "ff_collider3_bake_noalloc: %d shapes exceed the fixed table of %d (use ff_collider3_bake)", nshapes,
             BAKE_NOALLOC_MAX_SHAPES);
    FF_CHECK(nshapes == 0 || shapes, FF_E_ARG, "ff_collider3_bake_noalloc: shapes is NULL");
    const ff_field ws[3] = {wu, wv, ww};
    FF_TRY(check_bake_fields(res, phi, ws));
    ShapeTable t;
    std::memset(&t, 0, sizeof t);
    FF_TRY(shape_records(shapes, nshapes, t.s));
    DeviceScope scope(ctx->device);
    Shape *table = nullptr;
    FF_TRY(bake_table(ctx->device, &table));
    cudaStream_t s = ctx->stream;
    if (nshapes) k_store_shapes<<<1, BAKE_NOALLOC_MAX_SHAPES, 0, s>>>(t, nshapes, table);
    launch_bake(table, nshapes, invert, res, h, origin, phi, ws, s);
    FF_CUDA(cudaGetLastError());
    return FF_OK;
}
