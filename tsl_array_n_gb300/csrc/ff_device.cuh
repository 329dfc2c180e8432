// Device helpers shared by the libff kernels.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include "ff_internal.h"

namespace ffd {

// ---- storage loads / stores (fp32 or bf16, FP32 arithmetic) --------------
__device__ __forceinline__ float ld(const float *p, long long i) { return __ldg(p + i); }
__device__ __forceinline__ float ld(const __nv_bfloat16 *p, long long i) {
    unsigned short u = __ldg(reinterpret_cast<const unsigned short *>(p) + i);
    return __uint_as_float((unsigned)u << 16);
}
// plain (non-__ldg) loads for arrays written by the same kernel launch
__device__ __forceinline__ float ldw(const float *p, long long i) { return p[i]; }
__device__ __forceinline__ float ldw(const __nv_bfloat16 *p, long long i) {
    unsigned short u = reinterpret_cast<const unsigned short *>(p)[i];
    return __uint_as_float((unsigned)u << 16);
}
__device__ __forceinline__ void st(float *p, long long i, float v) { p[i] = v; }
__device__ __forceinline__ void st(__nv_bfloat16 *p, long long i, float v) { p[i] = __float2bfloat16_rn(v); }

__device__ __forceinline__ float bf_lo(unsigned v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(unsigned v) { return __uint_as_float(v & 0xffff0000u); }

template <bool C16>
__device__ __forceinline__ float4 ldcoef(const float4 *c32, const uint2 *c16, long long i) {
    if (C16) {
        uint2 r = __ldg(c16 + i);
        return make_float4(bf_lo(r.x), bf_hi(r.x), bf_lo(r.y), bf_hi(r.y));
    } else {
        return __ldg(c32 + i);
    }
}
template <bool C16>
__device__ __forceinline__ float ldkx(const float4 *c32, const uint2 *c16, long long i) {
    if (C16) return bf_lo(__ldg(&c16[i].x));
    return __ldg(&c32[i].x);
}
template <bool C16>
__device__ __forceinline__ float ldky(const float4 *c32, const uint2 *c16, long long i) {
    if (C16) return bf_hi(__ldg(&c16[i].x));
    return __ldg(&c32[i].y);
}
template <bool C16>
__device__ __forceinline__ float ldkz(const float4 *c32, const uint2 *c16, long long i) {
    if (C16) return bf_lo(__ldg(&c16[i].y));
    return __ldg(&c32[i].z);
}

// ---- error-free transformations (Knuth TwoSum, FMA TwoProd) --------------
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void two_prod(float a, float b, float &p, float &e) {
    p = __fmul_rn(a, b);
    e = __fmaf_rn(a, b, -p);
}
// (hi, lo) + alpha * p with alpha split into two floats; renormalised.
__device__ __forceinline__ void ds_axpy(float hi, float lo, float ahi, float alo, float p,
                                        float &ohi, float &olo) {
    float ph, pl;
    two_prod(ahi, p, ph, pl);
    pl = __fmaf_rn(alo, p, pl);
    float s, e;
    two_sum(hi, ph, s, e);
    e = __fadd_rn(e, __fadd_rn(lo, pl));
    ohi = __fadd_rn(s, e);
    olo = __fsub_rn(e, __fsub_rn(ohi, s));
}

// ---- float guards (fluxflow src/float_guards.js:78-111) ------------------
__device__ __forceinline__ bool nonfinite_d(double v) {
    unsigned long long u = __double_as_longlong(v);
    return ((u >> 52) & 0x7ffull) == 0x7ffull;
}
__device__ __forceinline__ bool nonfinite_or_above(double v, double limit) {
    return nonfinite_d(v) || !(fabs(v) <= limit);
}
__device__ __forceinline__ bool nonfinite_f(float v) {
    return (__float_as_uint(v) & 0x7f800000u) == 0x7f800000u;
}

// ---- deterministic block + grid reduction (FP64) --------------------------
// Each block writes its partial sums to partials[v * nblocks + block]; the
// last block to arrive (ticket) sums them in a fixed order.  Returns true in
// every thread of the last block, with the totals in tot[].
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <int NV>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], double *partials, unsigned *ticket,
                                            double (&tot)[NV], int slot = -1) {
    __shared__ double sred[NV][32];
    __shared__ bool last;
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int nthr = blockDim.x * blockDim.y * blockDim.z;
    const int lane = tid & 31, warp = tid >> 5, nwarp = (nthr + 31) >> 5;
    const unsigned nblocks = gridDim.x * gridDim.y * gridDim.z;
    // the block's partial goes to `slot` when given (a work-item index), else
    // to its linear block index
    const unsigned bid =
        slot >= 0 ? (unsigned)slot : blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double w = warp_sum(v[q]);
        if (lane == 0) sred[q][warp] = w;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double w = lane < nwarp ? sred[q][lane] : 0.0;
            w = warp_sum(w);
            if (lane == 0) partials[(size_t)q * nblocks + bid] = w;
        }
        if (lane == 0) {
            __threadfence();
            unsigned t = atomicAdd(ticket, 1u);
            last = (t == nblocks - 1);
        }
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = 0.0;
        for (unsigned b = tid; b < nblocks; b += nthr) s += __ldcg(partials + (size_t)q * nblocks + b);
        s = warp_sum(s);
        __syncthreads();
        if (lane == 0) sred[q][warp] = s;
        __syncthreads();
        double w = lane < nwarp ? sred[q][lane] : 0.0;
        tot[q] = warp_sum(w);
    }
    if (tid == 0) *ticket = 0u;
    return true;
}

// grid helpers: 3D launch over a (nx, ny, nz) box
struct Launch3 {
    dim3 grid, block;
};
inline Launch3 launch3(int nx, int ny, int nz) {
    int bx = nx >= 128 ? 128 : (nx >= 64 ? 64 : 32);
    int by = 256 / bx;
    Launch3 L;
    L.block = dim3(bx, by, 1);
    L.grid = dim3((nx + bx - 1) / bx, (ny + by - 1) / by, nz);
    return L;
}

}  // namespace ffd
