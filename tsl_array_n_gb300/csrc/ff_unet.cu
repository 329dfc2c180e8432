// Learned warm start for the pressure solve: a 3-level 3D U-Net (16/32/64
// channels, 3x3x3 convolutions, GELU, ~0.35M parameters) that maps
// (divergence, solid mask, previous pressure) to a pressure guess.  No
// reference counterpart: fluxflow has no network.
//
// Activations are stored channels-last (z, y, x, c) in BF16; convolutions
// are implicit GEMMs (M = voxels, K = 27 taps x Cin, N = Cout) on the
// tensor cores with BF16 operands and FP32 accumulation; pre-activations
// are kept in FP32 for the backward pass; master weights, gradients and the
// Adam moments are FP32, with a BF16 copy of the weights for the GEMMs.
// The input-gradient convolution reuses the forward kernel with the taps
// flipped and the weight matrix transposed; weight gradients accumulate
// per-tap [Cin x Cout] tiles over voxel chunks with FP32 atomics.
#include "ff_internal.h"
#include <mma.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

using namespace nvcuda;
typedef __nv_bfloat16 bf16;

namespace {

constexpr int MT = 64;   // voxels per conv block (4 warps x 16)

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

struct Vol {
    int nx, ny, nz;
    __host__ __device__ long long n() const { return (long long)nx * ny * nz; }
};

// offset of tap t (0..26) in (dz, dy, dx) = (t/9 - 1, (t/3)%3 - 1, t%3 - 1)
__device__ __forceinline__ void tap_offset(int t, int &dx, int &dy, int &dz) {
    dz = t / 9 - 1;
    dy = (t / 3) % 3 - 1;
    dx = t % 3 - 1;
}

// 3x3x3 convolution, zero padding 1: Y[v, co] = act(sum_{t, ci} X[v + off(t), ci] W[t, ci, co] + bias[co]).
// X has CIN channels (a multiple of 16), W is [27][CIN][COUT] BF16.  Writes
// the FP32 pre-activation Z (if given) and the BF16 output Y (if given).
template <int COUT>
__global__ void __launch_bounds__(128) k_conv3(Vol v, const bf16 *__restrict__ X, int cin, const bf16 *__restrict__ W,
                                              const float *__restrict__ bias, int act, float *__restrict__ Z,
                                              bf16 *__restrict__ Y) {
    constexpr int LDA = 16 + 8, LDB = COUT + 8, LDC = COUT + 4;
    __shared__ __align__(32) bf16 As[MT * LDA];
    __shared__ __align__(32) bf16 Bs[16 * LDB];
    __shared__ __align__(32) float Cs[MT * LDC];
    const int tid = threadIdx.x, warp = tid >> 5;
    const long long v0 = (long long)blockIdx.x * MT;
    const long long nvox = v.n();
    // this thread's A rows: row r = tid / 2, 8 channels at half (tid & 1)
    const int ar = tid >> 1, ah = tid & 1;
    const long long av = v0 + ar;
    int ax = 0, ay = 0, az = 0;
    if (av < nvox) {
        ax = (int)(av % v.nx);
        ay = (int)((av / v.nx) % v.ny);
        az = (int)(av / ((long long)v.nx * v.ny));
    }
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc[COUT / 16];
#pragma unroll
    for (int j = 0; j < COUT / 16; ++j) wmma::fill_fragment(acc[j], 0.0f);
    for (int t = 0; t < 27; ++t) {
        int dx, dy, dz;
        tap_offset(t, dx, dy, dz);
        const int sx = ax + dx, sy = ay + dy, sz = az + dz;
        const bool in = av < nvox && sx >= 0 && sx < v.nx && sy >= 0 && sy < v.ny && sz >= 0 && sz < v.nz;
        const long long src = in ? (sx + (long long)v.nx * (sy + (long long)v.ny * sz)) : 0;
        for (int c0 = 0; c0 < cin; c0 += 16) {
            uint4 a = make_uint4(0, 0, 0, 0);
            if (in) a = *reinterpret_cast<const uint4 *>(X + src * cin + c0 + 8 * ah);
            *reinterpret_cast<uint4 *>(As + ar * LDA + 8 * ah) = a;
            for (int q = tid; q < 16 * COUT / 8; q += 128) {
                const int k = q / (COUT / 8), n8 = q % (COUT / 8);
                *reinterpret_cast<uint4 *>(Bs + k * LDB + 8 * n8) =
                    *reinterpret_cast<const uint4 *>(W + ((long long)(t * cin + c0 + k)) * COUT + 8 * n8);
            }
            __syncthreads();
            wmma::fragment<wmma::matrix_a, 16, 16, 16, bf16, wmma::row_major> fa;
            wmma::load_matrix_sync(fa, As + warp * 16 * LDA, LDA);
#pragma unroll
            for (int j = 0; j < COUT / 16; ++j) {
                wmma::fragment<wmma::matrix_b, 16, 16, 16, bf16, wmma::row_major> fb;
                wmma::load_matrix_sync(fb, Bs + 16 * j, LDB);
                wmma::mma_sync(acc[j], fa, fb, acc[j]);
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int j = 0; j < COUT / 16; ++j)
        wmma::store_matrix_sync(Cs + warp * 16 * LDC + 16 * j, acc[j], LDC, wmma::mem_row_major);
    __syncthreads();
    for (int q = tid; q < MT * COUT; q += 128) {
        const int r = q / COUT, c = q % COUT;
        const long long vv = v0 + r;
        if (vv >= nvox) continue;
        float z = Cs[r * LDC + c] + (bias ? bias[c] : 0.0f);
        if (Z) Z[vv * COUT + c] = z;
        if (Y) Y[vv * COUT + c] = __float2bfloat16_rn(act ? gelu(z) : z);
    }
}

// weight gradient: dW[t, ci, co] += sum_v X[v + off(t), ci] G[v, co] over a
// chunk of 256 voxels; block = (chunk, tap)
template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3_wgrad(Vol v, const bf16 *__restrict__ X, const bf16 *__restrict__ G,
                                                    float *__restrict__ dW) {
    constexpr int LDX = CIN + 8, LDG = COUT + 8, NT = (CIN / 16) * (COUT / 16), PER = (NT + 3) / 4;
    __shared__ __align__(32) bf16 Xs[16 * LDX];
    __shared__ __align__(32) bf16 Gs[16 * LDG];
    __shared__ __align__(32) float Cs[4][16 * 16];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int t = blockIdx.y;
    int dx, dy, dz;
    tap_offset(t, dx, dy, dz);
    const long long nvox = v.n();
    wmma::fragment<wmma::accumulator, 16, 16, 16, float> acc[PER];
#pragma unroll
    for (int p = 0; p < PER; ++p) wmma::fill_fragment(acc[p], 0.0f);
    const long long vbeg = (long long)blockIdx.x * 256;
    for (long long k0 = vbeg; k0 < vbeg + 256; k0 += 16) {
        // stage 16 voxels of shifted X and of G
        for (int q = tid; q < 16 * (CIN / 8); q += 128) {
            const int r = q / (CIN / 8), c8 = q % (CIN / 8);
            const long long vv = k0 + r;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (vv < nvox) {
                const int x = (int)(vv % v.nx), y = (int)((vv / v.nx) % v.ny), z = (int)(vv / ((long long)v.nx * v.ny));
                const int sx = x + dx, sy = y + dy, sz = z + dz;
                if (sx >= 0 && sx < v.nx && sy >= 0 && sy < v.ny && sz >= 0 && sz < v.nz)
                    val = *reinterpret_cast<const uint4 *>(X + (sx + (long long)v.nx * (sy + (long long)v.ny * sz)) * CIN + 8 * c8);
            }
            *reinterpret_cast<uint4 *>(Xs + r * LDX + 8 * c8) = val;
        }
        for (int q = tid; q < 16 * (COUT / 8); q += 128) {
            const int r = q / (COUT / 8), c8 = q % (COUT / 8);
            const long long vv = k0 + r;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (vv < nvox) val = *reinterpret_cast<const uint4 *>(G + vv * COUT + 8 * c8);
            *reinterpret_cast<uint4 *>(Gs + r * LDG + 8 * c8) = val;
        }
        __syncthreads();
#pragma unroll
        for (int p = 0; p < PER; ++p) {
            const int tile = warp + 4 * p;
            if (tile < NT) {
                const int ci = tile / (COUT / 16), co = tile % (COUT / 16);
                wmma::fragment<wmma::matrix_a, 16, 16, 16, bf16, wmma::col_major> fa;   // X^T: [ci x v]
                wmma::fragment<wmma::matrix_b, 16, 16, 16, bf16, wmma::row_major> fb;   // G: [v x co]
                wmma::load_matrix_sync(fa, Xs + 16 * ci, LDX);
                wmma::load_matrix_sync(fb, Gs + 16 * co, LDG);
                wmma::mma_sync(acc[p], fa, fb, acc[p]);
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < PER; ++p) {
        const int tile = warp + 4 * p;
        if (tile >= NT) continue;
        const int ci = tile / (COUT / 16), co = tile % (COUT / 16);
        wmma::store_matrix_sync(Cs[warp], acc[p], 16, wmma::mem_row_major);
        __syncwarp();
        for (int e = lane; e < 256; e += 32) {
            const int r = e / 16, c = e % 16;
            atomicAdd(dW + ((long long)t * CIN + 16 * ci + r) * COUT + 16 * co + c, Cs[warp][e]);
        }
        __syncwarp();
    }
}

// G = dY * gelu'(Z) in BF16 (the GEMM operand of both backward convolutions);
// with act == 0, G = dY
__global__ void k_act_grad(long long n, const float *__restrict__ dY, const float *__restrict__ Z, int act,
                           bf16 *__restrict__ G) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        G[i] = __float2bfloat16_rn(act ? dY[i] * gelu_grad(Z[i]) : dY[i]);
}

// bias gradient: db[c] += sum_v G[v, c]
__global__ void k_bias_grad(long long nvox, int C, const bf16 *__restrict__ G, float *__restrict__ db) {
    extern __shared__ float sb[];
    for (int c = threadIdx.x; c < C; c += blockDim.x) sb[c] = 0.f;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nvox * C; i += (long long)gridDim.x * blockDim.x)
        atomicAdd(&sb[i % C], __bfloat162float(G[i]));
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) atomicAdd(&db[c], sb[c]);
}

// W'[t', co, ci] = W[26 - t', ci, co]: the input-gradient convolution's
// weights (flipped taps, transposed channels), BF16
__global__ void k_flip_transpose(int cin_real, int cin, int cout, const float *__restrict__ W, bf16 *__restrict__ Wt) {
    const long long n = 27LL * cin * cout;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(i / ((long long)cin * cout));
        const int r = (int)(i % ((long long)cin * cout));
        const int co = r / cin, ci = r % cin;   // Wt layout [t][co][ci]
        const float w = ci < cin_real ? W[((long long)(26 - t) * cin_real + ci) * cout + co] : 0.0f;
        Wt[i] = __float2bfloat16_rn(w);
    }
}

// BF16 copy of the master weights [27][cin_real][cout] padded to cin rows
__global__ void k_weights_bf16(int cin_real, int cin, int cout, const float *__restrict__ W, bf16 *__restrict__ Wb) {
    const long long n = 27LL * cin * cout;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(i / ((long long)cin * cout));
        const int r = (int)(i % ((long long)cin * cout));
        const int ci = r / cout, co = r % cout;
        Wb[i] = __float2bfloat16_rn(ci < cin_real ? W[((long long)t * cin_real + ci) * cout + co] : 0.0f);
    }
}

// dst[t][ci][co] (ci < cin_real) += src[t][ci][co] over cin padded rows
__global__ void k_gather_rows(int cin_real, int cin, int cout, const float *__restrict__ src, float *__restrict__ dst) {
    const long long n = 27LL * cin_real * cout;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(i / ((long long)cin_real * cout));
        const int r = (int)(i % ((long long)cin_real * cout));
        dst[i] += src[((long long)t * cin + r / cout) * cout + r % cout];
    }
}

// 2x average pooling (channels-last)
__global__ void k_pool(Vol c, int C, const bf16 *__restrict__ X, bf16 *__restrict__ Y) {
    const long long n = c.n() * C;
    const int fx = 2 * c.nx, fy = 2 * c.ny;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long vv = i / C;
        const int ch = (int)(i % C);
        const int x = (int)(vv % c.nx), y = (int)((vv / c.nx) % c.ny), z = (int)(vv / ((long long)c.nx * c.ny));
        float s = 0.f;
        for (int q = 0; q < 8; ++q) {
            const long long f = (2 * x + (q & 1)) + (long long)fx * ((2 * y + ((q >> 1) & 1)) + (long long)fy * (2 * z + (q >> 2)));
            s += __bfloat162float(X[f * C + ch]);
        }
        Y[i] = __float2bfloat16_rn(s * 0.125f);
    }
}
__global__ void k_pool_grad(Vol c, int C, const float *__restrict__ dY, float *__restrict__ dX, int accumulate) {
    const long long n = c.n() * C;
    const int fx = 2 * c.nx, fy = 2 * c.ny;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long vv = i / C;
        const int ch = (int)(i % C);
        const int x = (int)(vv % c.nx), y = (int)((vv / c.nx) % c.ny), z = (int)(vv / ((long long)c.nx * c.ny));
        const float g = dY[i] * 0.125f;
        for (int q = 0; q < 8; ++q) {
            const long long f = (2 * x + (q & 1)) + (long long)fx * ((2 * y + ((q >> 1) & 1)) + (long long)fy * (2 * z + (q >> 2)));
            dX[f * C + ch] = (accumulate ? dX[f * C + ch] : 0.f) + g;
        }
    }
}

// nearest 2x upsampling of X (C1 channels) into channels [0, C1) of the
// concat buffer Y (C1 + C2 channels); channels [C1, C1 + C2) take the skip S
__global__ void k_up_concat(Vol f, int C1, int C2, const bf16 *__restrict__ X, const bf16 *__restrict__ S,
                            bf16 *__restrict__ Y) {
    const int C = C1 + C2;
    const long long n = f.n() * C;
    const int cx = f.nx / 2, cy = f.ny / 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long vv = i / C;
        const int ch = (int)(i % C);
        if (ch < C1) {
            const int x = (int)(vv % f.nx), y = (int)((vv / f.nx) % f.ny), z = (int)(vv / ((long long)f.nx * f.ny));
            Y[i] = X[((x / 2) + (long long)cx * ((y / 2) + (long long)cy * (z / 2))) * C1 + ch];
        } else {
            Y[i] = S[vv * C2 + (ch - C1)];
        }
    }
}
// backward of k_up_concat: dX (coarse, C1) = sum over the 8 children, and
// the skip part added into dS (C2)
__global__ void k_up_concat_grad(Vol c, int C1, int C2, const float *__restrict__ dY, float *__restrict__ dX) {
    const int C = C1 + C2;
    const long long n = c.n() * C1;
    const int fx = 2 * c.nx, fy = 2 * c.ny;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long vv = i / C1;
        const int ch = (int)(i % C1);
        const int x = (int)(vv % c.nx), y = (int)((vv / c.nx) % c.ny), z = (int)(vv / ((long long)c.nx * c.ny));
        float s = 0.f;
        for (int q = 0; q < 8; ++q) {
            const long long f = (2 * x + (q & 1)) + (long long)fx * ((2 * y + ((q >> 1) & 1)) + (long long)fy * (2 * z + (q >> 2)));
            s += dY[f * C + ch];
        }
        dX[i] = s;
    }
}
__global__ void k_skip_grad_add(long long nvox, int C1, int C2, const float *__restrict__ dY, float *__restrict__ dS) {
    const int C = C1 + C2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nvox * C2; i += (long long)gridDim.x * blockDim.x) {
        const long long vv = i / C2;
        const int ch = (int)(i % C2);
        dS[i] += dY[vv * C + C1 + ch];
    }
}

// network input: channels (b / sb, mask, p_prev / sp, 0 ... 0), 16 wide
__global__ void k_input(long long n, const float *__restrict__ b, const uint8_t *__restrict__ mask,
                        const float *__restrict__ pp, const float *__restrict__ scales, bf16 *__restrict__ X) {
    const float isb = 1.0f / scales[0], isp = 1.0f / scales[1];
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        bf16 *x = X + v * 16;
        x[0] = __float2bfloat16_rn(b[v] * isb);
        x[1] = __float2bfloat16_rn(mask ? (float)mask[v] : 0.0f);
        x[2] = __float2bfloat16_rn(pp ? pp[v] * isp : 0.0f);
        for (int c = 3; c < 16; ++c) x[c] = __float2bfloat16_rn(0.0f);
    }
}

// 1x1x1 output layer (16 -> 1) in FP32 on the last convolution's FP32
// pre-activations (no BF16 rounding reaches the guess, whose grid-scale
// noise the Laplacian would amplify): out = sp (w . gelu(z) + b)
__global__ void k_head(long long n, const float *__restrict__ Zin, const float *__restrict__ w,
                       const float *__restrict__ scales, float *__restrict__ out, float *__restrict__ raw) {
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        float s = w[16];
        for (int c = 0; c < 16; ++c) s += gelu(Zin[v * 16 + c]) * w[c];
        if (raw) raw[v] = s;
        if (out) out[v] = s * scales[1];
    }
}
// MSE loss in normalised units: L = mean((raw - t / sp)^2); dL/draw per
// voxel; the loss itself by a deterministic block-partial reduction
__global__ void k_loss(long long n, const float *__restrict__ raw, const float *__restrict__ target,
                       const float *__restrict__ scales, float *__restrict__ draw, double *__restrict__ partial) {
    __shared__ double sred[256];
    const float isp = 1.0f / scales[1];
    double acc = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const float d = raw[v] - target[v] * isp;
        draw[v] = 2.0f * d / (float)n;
        acc += (double)d * d;
    }
    sred[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sred[threadIdx.x] += sred[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sred[0] / (double)n;
}
// head backward: dY[v, c] = draw[v] w[c]; dw[c] += sum draw y; db += sum draw
__global__ void k_head_grad(long long n, const float *__restrict__ Zin, const float *__restrict__ w,
                            const float *__restrict__ draw, float *__restrict__ dY, float *__restrict__ dw) {
    __shared__ float sw[17];
    if (threadIdx.x < 17) sw[threadIdx.x] = 0.f;
    __syncthreads();
    float lw[17] = {};
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const float g = draw[v];
        for (int c = 0; c < 16; ++c) {
            dY[v * 16 + c] = g * w[c];
            lw[c] += g * gelu(Zin[v * 16 + c]);
        }
        lw[16] += g;
    }
    for (int c = 0; c < 17; ++c) atomicAdd(&sw[c], lw[c]);
    __syncthreads();
    if (threadIdx.x < 17) atomicAdd(&dw[threadIdx.x], sw[threadIdx.x]);
}

// per-field RMS (deterministic two-level reduction into FP64 partials)
__global__ void k_sumsq(long long n, const float *__restrict__ a, double *__restrict__ partial) {
    __shared__ double sred[256];
    double acc = 0.0;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
        acc += (double)a[v] * a[v];
    sred[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sred[threadIdx.x] += sred[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sred[0];
}

// Adam (Kingma & Ba 2015) on the FP32 master weights
__global__ void k_adam(long long n, float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

int gblocks(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 32)); }

int post(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return ff_set_error(FF_E_CUDA, "%s launch: %s", what, cudaGetErrorString(e));
    return FF_OK;
}

int launch_conv(int cout, Vol v, const bf16 *X, int cin, const bf16 *W, const float *bias, int act, float *Z, bf16 *Y,
                cudaStream_t s) {
    const int nb = (int)((v.n() + MT - 1) / MT);
    switch (cout) {
    case 16: k_conv3<16><<<nb, 128, 0, s>>>(v, X, cin, W, bias, act, Z, Y); break;
    case 32: k_conv3<32><<<nb, 128, 0, s>>>(v, X, cin, W, bias, act, Z, Y); break;
    case 48: k_conv3<48><<<nb, 128, 0, s>>>(v, X, cin, W, bias, act, Z, Y); break;
    case 64: k_conv3<64><<<nb, 128, 0, s>>>(v, X, cin, W, bias, act, Z, Y); break;
    case 96: k_conv3<96><<<nb, 128, 0, s>>>(v, X, cin, W, bias, act, Z, Y); break;
    default: return ff_set_error(FF_E_ARG, "unet: no conv kernel for %d output channels", cout);
    }
    return post("conv3");
}

int launch_wgrad(int cin, int cout, Vol v, const bf16 *X, const bf16 *G, float *dW, cudaStream_t s) {
    dim3 grid((unsigned)((v.n() + 255) / 256), 27);
#define WG(A, B) \
    if (cin == A && cout == B) { k_conv3_wgrad<A, B><<<grid, 128, 0, s>>>(v, X, G, dW); return post("conv3 wgrad"); }
    WG(16, 16) WG(16, 32) WG(32, 32) WG(32, 64) WG(64, 64) WG(96, 32) WG(48, 16)
#undef WG
    return ff_set_error(FF_E_ARG, "unet: no weight-gradient kernel for %d -> %d", cin, cout);
}

// deterministic Gaussian initialisation: mulberry32 + Box-Muller
struct InitRng {
    uint32_t s;
    double u() {
        s += 0x6D2B79F5u;
        uint32_t t = s;
        t = (t ^ (t >> 15)) * (t | 1u);
        t ^= t + (t ^ (t >> 7)) * (t | 61u);
        return ((double)(t ^ (t >> 14)) + 0.5) / 4294967296.0;
    }
    double normal() { return std::sqrt(-2.0 * std::log(u())) * std::cos(6.283185307179586 * u()); }
};

}  // namespace

// --------------------------------------------------------------------------
struct ConvLayer {
    int cin_real, cin, cout, act;
    long long w_off, b_off;   // into the parameter vector
};

struct ff_unet_s {
    ff_ctx ctx = nullptr;
    std::vector<ConvLayer> convs;   // 10 conv layers in network order
    long long head_off = 0, nparam = 0;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;   // master params, grads, Adam moments
    bf16 *wb = nullptr;             // BF16 weights (per conv, padded cin)
    bf16 *wt = nullptr;             // flipped/transposed BF16 weights (largest layer)
    float *g0 = nullptr;            // first layer's weight gradient over the padded 16 inputs
    std::vector<long long> wb_off;
    long long adam_t = 0;
    // per-shape buffers
    Vol vol{0, 0, 0};
    std::vector<bf16 *> act;        // activations (BF16) per tensor slot
    std::vector<float *> pre;       // FP32 pre-activations per conv
    std::vector<float *> grad;      // FP32 gradient buffers per tensor slot
    bf16 *gbuf = nullptr;           // BF16 GEMM operand for backward
    float *raw = nullptr, *draw = nullptr, *scales = nullptr;
    double *partial = nullptr;
    std::vector<void *> owned;
};

// tensor slots: 0 input(16) 1 e0a(16) 2 e0b=skip0(16) 3 p1(16) 4 e1a(32) 5 e1b=skip1(32)
// 6 p2(32) 7 ba(64) 8 bb(64) 9 cat1(96) 10 d1a(32) 11 d1b(32) 12 cat0(48) 13 d0a(16) 14 d0b(16)
static const int SLOT_C[15] = {16, 16, 16, 16, 32, 32, 32, 64, 64, 96, 32, 32, 48, 16, 16};
static const int SLOT_LEVEL[15] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 1, 1, 1, 0, 0, 0};
// conv layer l reads slot CONV_IN[l] and writes slot CONV_OUT[l]
static const int CONV_IN[10] = {0, 1, 3, 4, 6, 7, 9, 10, 12, 13};
static const int CONV_OUT[10] = {1, 2, 4, 5, 7, 8, 10, 11, 13, 14};

static void free_shape(ff_unet u) {
    for (void *p : u->owned) ff_dev_free(p);
    u->owned.clear();
    u->act.clear();
    u->pre.clear();
    u->grad.clear();
    u->gbuf = nullptr;
    u->raw = u->draw = u->scales = nullptr;
    u->partial = nullptr;
    u->vol = Vol{0, 0, 0};
}

static int alloc_owned(ff_unet u, void **p, size_t bytes) {
    FF_TRY(ff_dev_alloc(p, bytes, u->ctx->stream));
    u->owned.push_back(*p);
    return FF_OK;
}

static int ensure_shape(ff_unet u, Vol v) {
    if (u->vol.nx == v.nx && u->vol.ny == v.ny && u->vol.nz == v.nz) return FF_OK;
    FF_CHECK(v.nx % 4 == 0 && v.ny % 4 == 0 && v.nz % 4 == 0 && v.nx >= 4 && v.ny >= 4 && v.nz >= 4, FF_E_ARG,
             "unet: resolution must be a multiple of 4 on every axis, got %dx%dx%d", v.nx, v.ny, v.nz);
    free_shape(u);
    u->vol = v;
    const long long n0 = v.n();
    u->act.resize(15);
    u->grad.resize(15);
    long long maxc = 0;
    for (int s = 0; s < 15; ++s) {
        const long long nv = n0 >> (3 * SLOT_LEVEL[s]);
        FF_TRY(alloc_owned(u, (void **)&u->act[s], (size_t)nv * SLOT_C[s] * sizeof(bf16)));
        FF_TRY(alloc_owned(u, (void **)&u->grad[s], (size_t)nv * SLOT_C[s] * sizeof(float)));
        maxc = std::max(maxc, nv * SLOT_C[s]);
    }
    u->pre.resize(10);
    for (int l = 0; l < 10; ++l) {
        const int s = CONV_OUT[l];
        const long long nv = n0 >> (3 * SLOT_LEVEL[s]);
        FF_TRY(alloc_owned(u, (void **)&u->pre[l], (size_t)nv * SLOT_C[s] * sizeof(float)));
    }
    FF_TRY(alloc_owned(u, (void **)&u->gbuf, (size_t)maxc * sizeof(bf16)));
    FF_TRY(alloc_owned(u, (void **)&u->raw, (size_t)n0 * 4));
    FF_TRY(alloc_owned(u, (void **)&u->draw, (size_t)n0 * 4));
    FF_TRY(alloc_owned(u, (void **)&u->scales, 16));
    FF_TRY(alloc_owned(u, (void **)&u->partial, sizeof(double) * 152 * 32));
    return FF_OK;
}

extern "C" int ff_unet_create(ff_ctx ctx, uint32_t seed, ff_unet *out) {
    FF_CHECK(ctx && out, FF_E_ARG, "ff_unet_create: NULL argument");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    ff_unet u = new ff_unet_s();
    u->ctx = ctx;
    // (cin_real, cout) per conv in network order
    const int spec[10][2] = {{3, 16}, {16, 16}, {16, 32}, {32, 32}, {32, 64}, {64, 64}, {96, 32}, {32, 32}, {48, 16}, {16, 16}};
    long long off = 0, woff = 0;
    for (int l = 0; l < 10; ++l) {
        ConvLayer c;
        c.cin_real = spec[l][0];
        c.cin = (spec[l][0] + 15) / 16 * 16;
        c.cout = spec[l][1];
        c.act = 1;
        c.w_off = off;
        off += 27LL * c.cin_real * c.cout;
        c.b_off = off;
        off += c.cout;
        u->convs.push_back(c);
        u->wb_off.push_back(woff);
        woff += 27LL * c.cin * c.cout;
    }
    u->head_off = off;
    off += 17;
    u->nparam = off;
    cudaStream_t s = ctx->stream;
    int st = FF_OK;
    auto bail = [&](int code) { ff_unet_destroy(u); return code; };
    if ((st = ff_dev_alloc((void **)&u->w, off * 4, s)) || (st = ff_dev_alloc((void **)&u->g, off * 4, s)) ||
        (st = ff_dev_alloc((void **)&u->m, off * 4, s)) || (st = ff_dev_alloc((void **)&u->v, off * 4, s)) ||
        (st = ff_dev_alloc((void **)&u->wb, woff * sizeof(bf16), s)) ||
        (st = ff_dev_alloc((void **)&u->wt, 27LL * 96 * 64 * sizeof(bf16), s)) ||
        (st = ff_dev_alloc((void **)&u->g0, 27LL * 16 * 16 * sizeof(float), s)))
        return bail(st);
    // He-normal weights (std sqrt(2 / fan_in)), zero biases; head 0.1 / sqrt(16)
    std::vector<float> hw(off, 0.0f);
    InitRng rng{seed};
    for (const ConvLayer &c : u->convs) {
        const double sd = std::sqrt(2.0 / (27.0 * c.cin_real));
        for (long long i = 0; i < 27LL * c.cin_real * c.cout; ++i) hw[c.w_off + i] = (float)(sd * rng.normal());
    }
    for (int c = 0; c < 16; ++c) hw[u->head_off + c] = (float)(0.25 * rng.normal());
    if ((st = ff_unet_set_params(u, hw.data(), off))) return bail(st);
    *out = u;
    return FF_OK;
}

extern "C" int ff_unet_destroy(ff_unet u) {
    if (!u) return FF_OK;
    cudaStreamSynchronize(u->ctx->stream);
    free_shape(u);
    ff_dev_free(u->w);
    ff_dev_free(u->g);
    ff_dev_free(u->m);
    ff_dev_free(u->v);
    ff_dev_free(u->wb);
    ff_dev_free(u->wt);
    ff_dev_free(u->g0);
    delete u;
    return FF_OK;
}

extern "C" int ff_unet_param_count(ff_unet u, int64_t *n) {
    FF_CHECK(u && n, FF_E_ARG, "NULL argument");
    *n = u->nparam;
    return FF_OK;
}

static int refresh_bf16(ff_unet u) {
    cudaStream_t s = u->ctx->stream;
    for (size_t l = 0; l < u->convs.size(); ++l) {
        const ConvLayer &c = u->convs[l];
        k_weights_bf16<<<gblocks(27LL * c.cin * c.cout), 256, 0, s>>>(c.cin_real, c.cin, c.cout, u->w + c.w_off,
                                                                       u->wb + u->wb_off[l]);
    }
    return post("weights bf16");
}

extern "C" int ff_unet_set_params(ff_unet u, const float *host, int64_t n) {
    FF_CHECK(u && host && n == u->nparam, FF_E_ARG, "unet: expected %lld parameters", (long long)(u ? u->nparam : 0));
    cudaStream_t s = u->ctx->stream;
    FF_CUDA(cudaMemcpyAsync(u->w, host, n * 4, cudaMemcpyHostToDevice, s));
    FF_CUDA(cudaMemsetAsync(u->m, 0, n * 4, s));
    FF_CUDA(cudaMemsetAsync(u->v, 0, n * 4, s));
    u->adam_t = 0;
    FF_TRY(refresh_bf16(u));
    FF_CUDA(cudaStreamSynchronize(s));
    return FF_OK;
}

extern "C" int ff_unet_get_params(ff_unet u, float *host, int64_t n) {
    FF_CHECK(u && host && n == u->nparam, FF_E_ARG, "unet: expected %lld parameters", (long long)(u ? u->nparam : 0));
    FF_CUDA(cudaMemcpyAsync(host, u->w, n * 4, cudaMemcpyDeviceToHost, u->ctx->stream));
    FF_CUDA(cudaStreamSynchronize(u->ctx->stream));
    return FF_OK;
}

extern "C" int ff_unet_get_grads(ff_unet u, float *host, int64_t n) {
    FF_CHECK(u && host && n == u->nparam, FF_E_ARG, "unet: expected %lld parameters", (long long)(u ? u->nparam : 0));
    FF_CUDA(cudaMemcpyAsync(host, u->g, n * 4, cudaMemcpyDeviceToHost, u->ctx->stream));
    FF_CUDA(cudaStreamSynchronize(u->ctx->stream));
    return FF_OK;
}

// normalisation scales: sb = rms(b), sp = rms(p_prev), or rms(b) L^2 / (4 pi^2)
// (L the smallest domain extent) when p_prev is zero or absent
static int compute_scales(ff_unet u, const float *b, const float *pp, double h, float out[2]) {
    cudaStream_t s = u->ctx->stream;
    const long long n = u->vol.n();
    const int nb = std::min(152 * 32, gblocks(n));
    std::vector<double> hp(nb);
    double sums[2] = {0, 0};
    const float *arr[2] = {b, pp};
    for (int q = 0; q < 2; ++q) {
        if (!arr[q]) continue;
        k_sumsq<<<nb, 256, 0, s>>>(n, arr[q], u->partial);
        FF_TRY(post("sumsq"));
        FF_CUDA(cudaMemcpyAsync(hp.data(), u->partial, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
        FF_CUDA(cudaStreamSynchronize(s));
        for (double x : hp) sums[q] += x;
    }
    const double sb = std::sqrt(sums[0] / n);
    double sp = std::sqrt(sums[1] / n);
    const double L = h * std::min(u->vol.nx, std::min(u->vol.ny, u->vol.nz));
    if (!(sp > 0)) sp = sb * L * L / (4.0 * M_PI * M_PI);
    out[0] = (float)(sb > 0 ? sb : 1.0);
    out[1] = (float)(sp > 0 ? sp : 1.0);
    FF_CUDA(cudaMemcpyAsync(u->scales, out, 8, cudaMemcpyHostToDevice, s));
    return FF_OK;
}

static Vol level_vol(ff_unet u, int lev) { return Vol{u->vol.nx >> lev, u->vol.ny >> lev, u->vol.nz >> lev}; }

static int forward(ff_unet u, const float *b, const uint8_t *mask, const float *pp, double h, float *out) {
    cudaStream_t s = u->ctx->stream;
    float sc[2];
    FF_TRY(compute_scales(u, b, pp, h, sc));
    const long long n0 = u->vol.n();
    k_input<<<gblocks(n0), 256, 0, s>>>(n0, b, mask, pp, u->scales, u->act[0]);
    auto conv = [&](int l) {
        const ConvLayer &c = u->convs[l];
        const int si = CONV_IN[l], so = CONV_OUT[l];
        return launch_conv(c.cout, level_vol(u, SLOT_LEVEL[so]), u->act[si], c.cin, u->wb + u->wb_off[l],
                           u->w + c.b_off, c.act, u->pre[l], u->act[so], s);
    };
    FF_TRY(conv(0));
    FF_TRY(conv(1));
    k_pool<<<gblocks(level_vol(u, 1).n() * 16), 256, 0, s>>>(level_vol(u, 1), 16, u->act[2], u->act[3]);
    FF_TRY(conv(2));
    FF_TRY(conv(3));
    k_pool<<<gblocks(level_vol(u, 2).n() * 32), 256, 0, s>>>(level_vol(u, 2), 32, u->act[5], u->act[6]);
    FF_TRY(conv(4));
    FF_TRY(conv(5));
    k_up_concat<<<gblocks(level_vol(u, 1).n() * 96), 256, 0, s>>>(level_vol(u, 1), 64, 32, u->act[8], u->act[5], u->act[9]);
    FF_TRY(conv(6));
    FF_TRY(conv(7));
    k_up_concat<<<gblocks(n0 * 48), 256, 0, s>>>(level_vol(u, 0), 32, 16, u->act[11], u->act[2], u->act[12]);
    FF_TRY(conv(8));
    FF_TRY(conv(9));
    k_head<<<gblocks(n0), 256, 0, s>>>(n0, u->pre[9], u->w + u->head_off, u->scales, out, u->raw);
    return post("unet forward");
}

// gradient of conv l: input gradient into grad[CONV_IN[l]] (unless l == 0),
// weight and bias gradients; grad[CONV_OUT[l]] holds dL/d(output)
static int conv_backward(ff_unet u, int l, bool accumulate_input) {
    cudaStream_t s = u->ctx->stream;
    const ConvLayer &c = u->convs[l];
    const int si = CONV_IN[l], so = CONV_OUT[l];
    const Vol v = level_vol(u, SLOT_LEVEL[so]);
    const long long nout = v.n() * c.cout;
    k_act_grad<<<gblocks(nout), 256, 0, s>>>(nout, u->grad[so], u->pre[l], c.act, u->gbuf);
    FF_TRY(post("act grad"));
    if (c.cin == c.cin_real) {
        FF_TRY(launch_wgrad(c.cin, c.cout, v, u->act[si], u->gbuf, u->g + c.w_off, s));
    } else {
        // padded input channels: accumulate over all 16, keep the real ones
        FF_CUDA(cudaMemsetAsync(u->g0, 0, 27LL * c.cin * c.cout * 4, s));
        FF_TRY(launch_wgrad(c.cin, c.cout, v, u->act[si], u->gbuf, u->g0, s));
        k_gather_rows<<<gblocks(27LL * c.cin_real * c.cout), 256, 0, s>>>(c.cin_real, c.cin, c.cout, u->g0,
                                                                          u->g + c.w_off);
    }
    k_bias_grad<<<std::min(gblocks(nout), 1024), 256, c.cout * 4, s>>>(v.n(), c.cout, u->gbuf, u->g + c.b_off);
    FF_TRY(post("bias grad"));
    if (l == 0) return FF_OK;
    k_flip_transpose<<<gblocks(27LL * c.cin * c.cout), 256, 0, s>>>(c.cin_real, c.cin, c.cout, u->w + c.w_off, u->wt);
    // dX = conv(G, W') with cin = cout_fwd, cout = cin_fwd; written as FP32
    // through the pre-activation output of the conv kernel
    float *dst = u->grad[si];
    if (accumulate_input) return ff_set_error(FF_E_STATE, "unet: accumulate not supported");
    FF_TRY(launch_conv(c.cin, v, u->gbuf, c.cout, u->wt, nullptr, 0, dst, nullptr, s));
    return FF_OK;
}

static int backward(ff_unet u) {
    cudaStream_t s = u->ctx->stream;
    const long long n0 = u->vol.n();
    k_head_grad<<<std::min(gblocks(n0), 1024), 256, 0, s>>>(n0, u->pre[9], u->w + u->head_off, u->draw, u->grad[14],
                                                             u->g + u->head_off);
    FF_TRY(post("head grad"));
    FF_TRY(conv_backward(u, 9, false));   // grad[13]
    FF_TRY(conv_backward(u, 8, false));   // grad[12] (cat0: 32 up + 16 skip)
    const Vol v1 = level_vol(u, 1), v2 = level_vol(u, 2);
    k_up_concat_grad<<<gblocks(v1.n() * 32), 256, 0, s>>>(v1, 32, 16, u->grad[12], u->grad[11]);
    FF_TRY(conv_backward(u, 7, false));   // grad[10]
    FF_TRY(conv_backward(u, 6, false));   // grad[9] (cat1: 64 up + 32 skip)
    k_up_concat_grad<<<gblocks(v2.n() * 64), 256, 0, s>>>(v2, 64, 32, u->grad[9], u->grad[8]);
    FF_TRY(conv_backward(u, 5, false));   // grad[7]
    FF_TRY(conv_backward(u, 4, false));   // grad[6]
    // skip1 (slot 5) gets the pooled path and the concat path
    k_pool_grad<<<gblocks(v2.n() * 32), 256, 0, s>>>(v2, 32, u->grad[6], u->grad[5], 0);
    k_skip_grad_add<<<gblocks(v1.n() * 32), 256, 0, s>>>(v1.n(), 64, 32, u->grad[9], u->grad[5]);
    FF_TRY(conv_backward(u, 3, false));   // grad[4]
    FF_TRY(conv_backward(u, 2, false));   // grad[3]
    k_pool_grad<<<gblocks(v1.n() * 16), 256, 0, s>>>(v1, 16, u->grad[3], u->grad[2], 0);
    k_skip_grad_add<<<gblocks(n0 * 16), 256, 0, s>>>(n0, 32, 16, u->grad[12], u->grad[2]);
    FF_TRY(conv_backward(u, 1, false));   // grad[1]
    FF_TRY(conv_backward(u, 0, false));
    return post("unet backward");
}

static int field_ok(ff_field f, long long n, int dtype) { return f && f->count == n && f->dtype == dtype; }

extern "C" int ff_unet_forward(ff_unet u, const int *res, double h, ff_field b, ff_field mask, ff_field p_prev,
                               ff_field out) {
    FF_CHECK(u && res, FF_E_ARG, "NULL argument");
    cudaSetDevice(u->ctx->device);
    FF_TRY(ensure_shape(u, Vol{res[0], res[1], res[2]}));
    const long long n = u->vol.n();
    FF_CHECK(field_ok(b, n, FF_FLOAT) && field_ok(out, n, FF_FLOAT) && (!p_prev || field_ok(p_prev, n, FF_FLOAT)) &&
                 (!mask || field_ok(mask, n, FF_UINT8)),
             FF_E_ARG, "unet forward: fields must be cell fields of the resolution (mask uint8)");
    return forward(u, (const float *)b->d, mask ? (const uint8_t *)mask->d : nullptr,
                   p_prev ? (const float *)p_prev->d : nullptr, h, (float *)out->d);
}

// forward + MSE loss against `target` + backward: leaves dL/dparams in the
// gradient buffer (zeroed first) and the loss in *loss
extern "C" int ff_unet_loss_backward(ff_unet u, const int *res, double h, ff_field b, ff_field mask, ff_field p_prev,
                                     ff_field target, double *loss) {
    FF_CHECK(u && res && target, FF_E_ARG, "NULL argument");
    cudaSetDevice(u->ctx->device);
    FF_TRY(ensure_shape(u, Vol{res[0], res[1], res[2]}));
    const long long n = u->vol.n();
    FF_CHECK(field_ok(b, n, FF_FLOAT) && field_ok(target, n, FF_FLOAT) && (!p_prev || field_ok(p_prev, n, FF_FLOAT)) &&
                 (!mask || field_ok(mask, n, FF_UINT8)),
             FF_E_ARG, "unet loss: fields must be cell fields of the resolution (mask uint8)");
    cudaStream_t s = u->ctx->stream;
    FF_TRY(forward(u, (const float *)b->d, mask ? (const uint8_t *)mask->d : nullptr,
                   p_prev ? (const float *)p_prev->d : nullptr, h, nullptr));
    const int nb = std::min(152 * 32, gblocks(n));
    k_loss<<<nb, 256, 0, s>>>(n, u->raw, (const float *)target->d, u->scales, u->draw, u->partial);
    FF_TRY(post("loss"));
    FF_CUDA(cudaMemsetAsync(u->g, 0, u->nparam * 4, s));
    FF_TRY(backward(u));
    std::vector<double> hp(nb);
    FF_CUDA(cudaMemcpyAsync(hp.data(), u->partial, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
    FF_CUDA(cudaStreamSynchronize(s));
    double tot = 0;
    for (double x : hp) tot += x;
    if (loss) *loss = tot;
    return FF_OK;
}

extern "C" int ff_unet_adam_step(ff_unet u, double lr, double beta1, double beta2, double eps) {
    FF_CHECK(u, FF_E_ARG, "NULL argument");
    cudaSetDevice(u->ctx->device);
    u->adam_t += 1;
    const double c1 = 1.0 - std::pow(beta1, (double)u->adam_t), c2 = 1.0 - std::pow(beta2, (double)u->adam_t);
    k_adam<<<gblocks(u->nparam), 256, 0, u->ctx->stream>>>(u->nparam, u->w, u->g, u->m, u->v, (float)lr, (float)beta1,
                                                            (float)beta2, (float)eps, (float)c1, (float)c2);
    FF_TRY(post("adam"));
    return refresh_bf16(u);
}
