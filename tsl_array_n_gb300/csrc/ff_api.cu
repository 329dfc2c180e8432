// Context, field and error entry points of the C ABI (include/ff.h).
#include "ff_internal.h"
#include <cstdarg>
#include <cstdio>
#include <cstring>

static thread_local char g_err[512] = "";

int ff_set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

extern "C" const char *ff_last_error(void) { return g_err; }
extern "C" const char *ff_version(void) { return "ff 0.1 sm_103a"; }

size_t ff_dtype_size(int dtype) {
    switch (dtype) {
    case FF_FLOAT: return 4;
    case FF_INT: return 4;
    case FF_UINT8: return 1;
    case FF_VEC3: return 12;
    default: return 0;
    }
}

int ff_dev_alloc(void **p, size_t bytes, cudaStream_t s) {
    *p = nullptr;
    if (bytes == 0) bytes = 256;
    size_t padded = (bytes + 255) & ~size_t(255);
    cudaError_t e = cudaMalloc(p, padded);
    if (e != cudaSuccess) {
        *p = nullptr;
        return ff_set_error(e == cudaErrorMemoryAllocation ? FF_E_NOMEM : FF_E_CUDA,
                            "cudaMalloc(%zu): %s", padded, cudaGetErrorString(e));
    }
    e = cudaMemsetAsync(*p, 0, padded, s);
    if (e != cudaSuccess) return ff_set_error(FF_E_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    return FF_OK;
}

void ff_dev_free(void *p) {
    if (p) cudaFree(p);
}

extern "C" int ff_ctx_create(int device, ff_ctx *out) {
    FF_CHECK(out, FF_E_ARG, "ff_ctx_create: out is NULL");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return ff_set_error(FF_E_CUDA, "ff_ctx_create: no CUDA device (%s)", cudaGetErrorString(e));
    FF_CHECK(device >= 0 && device < n, FF_E_ARG, "ff_ctx_create: device %d out of range (%d)", device, n);
    FF_CUDA(cudaSetDevice(device));
    ff_ctx c = new ff_ctx_s();
    c->device = device;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return ff_set_error(FF_E_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    *out = c;
    return FF_OK;
}

int ff_ctx_copy_streams(ff_ctx ctx) {
    if (ctx->up && ctx->down) return FF_OK;
    FF_CUDA(cudaSetDevice(ctx->device));
    if (!ctx->up) FF_CUDA(cudaStreamCreateWithFlags(&ctx->up, cudaStreamNonBlocking));
    if (!ctx->down) FF_CUDA(cudaStreamCreateWithFlags(&ctx->down, cudaStreamNonBlocking));
    return FF_OK;
}

extern "C" int ff_ctx_join_copies(ff_ctx ctx) {
    FF_CHECK(ctx, FF_E_ARG, "ff_ctx_join_copies: NULL context");
    for (cudaStream_t c : {ctx->up, ctx->down}) {
        if (!c) continue;
        cudaEvent_t e;
        FF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        cudaError_t r = cudaEventRecord(e, c);
        if (r == cudaSuccess) r = cudaStreamWaitEvent(ctx->stream, e, 0);
        cudaEventDestroy(e);
        FF_CUDA(r);
    }
    return FF_OK;
}

extern "C" int ff_ctx_destroy(ff_ctx ctx) {
    if (!ctx) return FF_OK;
    cudaSetDevice(ctx->device);
    for (cudaStream_t c : {ctx->up, ctx->down}) {
        if (!c) continue;
        cudaStreamSynchronize(c);
        cudaStreamDestroy(c);
    }
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->stream);
    for (auto &e : ctx->events) if (e) cudaEventDestroy(e);
    delete ctx;
    return FF_OK;
}

extern "C" int ff_ctx_synchronize(ff_ctx ctx) {
    FF_CHECK(ctx, FF_E_ARG, "ff_ctx_synchronize: NULL context");
    FF_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->up) FF_CUDA(cudaStreamSynchronize(ctx->up));
    if (ctx->down) FF_CUDA(cudaStreamSynchronize(ctx->down));
    return FF_OK;
}

extern "C" int ff_ctx_event_record(ff_ctx ctx, int slot) {
    FF_CHECK(ctx && slot >= 0 && slot < 16, FF_E_ARG, "ff_ctx_event_record: bad slot");
    if (!ctx->events[slot]) FF_CUDA(cudaEventCreate(&ctx->events[slot]));
    FF_CUDA(cudaEventRecord(ctx->events[slot], ctx->stream));
    return FF_OK;
}

extern "C" int ff_ctx_event_elapsed(ff_ctx ctx, int a, int b, float *ms) {
    FF_CHECK(ctx && ms && a >= 0 && a < 16 && b >= 0 && b < 16, FF_E_ARG, "ff_ctx_event_elapsed: bad slot");
    FF_CHECK(ctx->events[a] && ctx->events[b], FF_E_STATE, "event slot not recorded");
    FF_CUDA(cudaEventSynchronize(ctx->events[b]));
    FF_CUDA(cudaEventElapsedTime(ms, ctx->events[a], ctx->events[b]));
    return FF_OK;
}

extern "C" int ff_host_alloc(size_t bytes, void **out) {
    FF_CHECK(out, FF_E_ARG, "ff_host_alloc: out is NULL");
    FF_CUDA(cudaMallocHost(out, bytes));
    return FF_OK;
}

extern "C" int ff_host_free(void *p) {
    if (p) FF_CUDA(cudaFreeHost(p));
    return FF_OK;
}

// arrayN (tsl_array_n src/array.js:94-133); shape validation as array.js:4-20
extern "C" int ff_field_create(ff_ctx ctx, int dtype, int ndim, const int *shape, ff_field *out) {
    FF_CHECK(ctx && out && shape, FF_E_ARG, "ff_field_create: NULL argument");
    *out = nullptr;
    FF_CHECK(ff_dtype_size(dtype) > 0, FF_E_ARG, "tsl_array_n: unsupported type %d", dtype);
    FF_CHECK(ndim >= 1 && ndim <= 3, FF_E_ARG, "tsl_array_n: shape must have 1-3 dimensions, got %d", ndim);
    int64_t count = 1;
    for (int a = 0; a < ndim; ++a) {
        FF_CHECK(shape[a] > 0, FF_E_ARG, "tsl_array_n: shape[%d] must be a positive integer, got %d", a, shape[a]);
        count *= shape[a];
    }
    ff_field f = new ff_field_s();
    f->ctx = ctx;
    f->dtype = dtype;
    f->ndim = ndim;
    for (int a = 0; a < 3; ++a) f->shape[a] = a < ndim ? shape[a] : 1;
    f->count = count;
    f->bytes = (size_t)count * ff_dtype_size(dtype);
    int s = ff_dev_alloc(&f->d, f->bytes, ctx->stream);
    if (s != FF_OK) {
        delete f;
        return s;
    }
    *out = f;
    return FF_OK;
}

extern "C" int ff_field_destroy(ff_field f) {
    if (!f) return FF_OK;
    if (f->owned) {
        cudaStreamSynchronize(f->ctx->stream);
        ff_dev_free(f->d);
    }
    delete f;
    return FF_OK;
}

extern "C" int ff_field_upload(ff_field f, const void *host, size_t bytes) {
    FF_CHECK(f && host, FF_E_ARG, "ff_field_upload: NULL argument");
    FF_CHECK(bytes == f->bytes, FF_E_ARG, "fromArray: %zu bytes given, field holds %zu", bytes, f->bytes);
    FF_CUDA(cudaMemcpyAsync(f->d, host, bytes, cudaMemcpyHostToDevice, f->ctx->stream));
    FF_CUDA(cudaStreamSynchronize(f->ctx->stream));
    return FF_OK;
}

extern "C" int ff_field_download(ff_field f, void *host, size_t bytes) {
    FF_CHECK(f && host, FF_E_ARG, "ff_field_download: NULL argument");
    FF_CHECK(bytes == f->bytes, FF_E_ARG, "toArray: %zu bytes requested, field holds %zu", bytes, f->bytes);
    FF_CUDA(cudaMemcpyAsync(host, f->d, bytes, cudaMemcpyDeviceToHost, f->ctx->stream));
    FF_CUDA(cudaStreamSynchronize(f->ctx->stream));
    return FF_OK;
}

extern "C" int ff_field_upload_async(ff_field f, const void *host, size_t bytes) {
    FF_CHECK(f && host, FF_E_ARG, "ff_field_upload_async: NULL argument");
    FF_CHECK(bytes == f->bytes, FF_E_ARG, "fromArray: %zu bytes given, field holds %zu", bytes, f->bytes);
    FF_CUDA(cudaMemcpyAsync(f->d, host, bytes, cudaMemcpyHostToDevice, f->ctx->stream));
    return FF_OK;
}

extern "C" int ff_field_download_async(ff_field f, void *host, size_t bytes) {
    FF_CHECK(f && host, FF_E_ARG, "ff_field_download_async: NULL argument");
    FF_CHECK(bytes == f->bytes, FF_E_ARG, "toArray: %zu bytes requested, field holds %zu", bytes, f->bytes);
    FF_CUDA(cudaMemcpyAsync(host, f->d, bytes, cudaMemcpyDeviceToHost, f->ctx->stream));
    return FF_OK;
}

extern "C" int ff_field_copy(ff_field dst, ff_field src) {
    FF_CHECK(dst && src, FF_E_ARG, "ff_field_copy: NULL field");
    FF_CHECK(dst->bytes == src->bytes && dst->dtype == src->dtype, FF_E_ARG,
             "ff_field_copy: fields differ in type or size");
    FF_CUDA(cudaMemcpyAsync(dst->d, src->d, dst->bytes, cudaMemcpyDeviceToDevice, dst->ctx->stream));
    return FF_OK;
}

extern "C" int ff_field_fill(ff_field f, float value) {
    FF_CHECK(f, FF_E_ARG, "ff_field_fill: NULL field");
    if (f->dtype == FF_FLOAT || f->dtype == FF_VEC3) {
        FF_TRY(ffk::fill_f32((float *)f->d, (long long)(f->bytes / 4), value, f->ctx->stream));
    } else if (f->dtype == FF_UINT8) {
        FF_CUDA(cudaMemsetAsync(f->d, value != 0.f ? 1 : 0, f->bytes, f->ctx->stream));
    } else {
        FF_CHECK(value == 0.f, FF_E_ARG, "ff_field_fill: int fields only fill with 0");
        FF_CUDA(cudaMemsetAsync(f->d, 0, f->bytes, f->ctx->stream));
    }
    return FF_OK;
}

extern "C" int ff_field_info(ff_field f, int *dtype, int *ndim, int *shape3, int64_t *count) {
    FF_CHECK(f, FF_E_ARG, "ff_field_info: NULL field");
    if (dtype) *dtype = f->dtype;
    if (ndim) *ndim = f->ndim;
    if (shape3) for (int a = 0; a < 3; ++a) shape3[a] = f->shape[a];
    if (count) *count = f->count;
    return FF_OK;
}

extern "C" void *ff_field_device_ptr(ff_field f) { return f ? f->d : nullptr; }
