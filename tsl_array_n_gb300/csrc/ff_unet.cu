// Learned warm start for the pressure solve: a 3-level 3D U-Net (16/32/64
// channels, 3x3x3 convolutions, GELU, ~0.35M parameters) that maps
// (divergence, solid mask, previous pressure) to a pressure guess.  No
// reference counterpart: fluxflow has no network.
//
// Activations are stored channels-last (z, y, x, c) in BF16; convolutions
// are implicit GEMMs (M = voxels, K = 27 taps x Cin, N = Cout) with BF16
// operands and FP32 accumulation on tcgen05 (accumulators in TMEM):
// forward, input-gradient and weight-gradient convolutions; pre-activations
// are kept in FP32 for the backward pass only (inference stores none);
// master weights, gradients and the Adam moments are FP32, with a BF16 copy
// of the weights for the GEMMs.  Forward and input-gradient convolutions run
// in k_conv3_zm (a z-march over TMA-staged planes); the input-gradient one
// takes the taps flipped and the weight matrix transposed; weight gradients
// accumulate per-tap [Cin x Cout] tiles over voxel chunks with FP32 atomics.
#include "ff_internal.h"
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

typedef __nv_bfloat16 bf16;

namespace {


// GELU in its tanh form, 0.5 x (1 + tanh(sqrt(2 / pi) (x + 0.044715 x^3)))
// (Hendrycks & Gimpel 2016), with the hardware tanh approximation; the
// derivative of the same expression for the backward pass
__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float GELU_K0 = 0.7978845608028654f, GELU_K1 = 0.044715f;
__device__ __forceinline__ float gelu(float x) {
    const float t = tanh_hw(GELU_K0 * __fmaf_rn(GELU_K1 * x, x * x, x));
    return 0.5f * x * (1.0f + t);
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float x2 = x * x;
    const float t = tanh_hw(GELU_K0 * __fmaf_rn(GELU_K1 * x, x2, x));
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * GELU_K0 * __fmaf_rn(3.0f * GELU_K1, x2, 1.0f);
}

struct Vol {
    int nx, ny, nz;
    __host__ __device__ long long n() const { return (long long)nx * ny * nz; }
};

// BF16 activations are stored as planes of 8-channel groups: channel c of
// voxel v (x-fastest index over a volume of n voxels) at element
// ((c / 8) n + v) 8 + c % 8.  A group plane is a plain volume of 16-byte
// voxels, so a TMA box of one group reads whole rows of the tile, and a
// concatenation along channels is a run of consecutive group planes.
__host__ __device__ __forceinline__ long long g8(long long v, int c, long long n) {
    return ((long long)(c >> 3) * n + v) * 8 + (c & 7);
}

// offset of tap t (0..26) in (dz, dy, dx) = (t/9 - 1, (t/3)%3 - 1, t%3 - 1)
__device__ __forceinline__ void tap_offset(int t, int &dx, int &dy, int &dz) {
    dz = t / 9 - 1;
    dy = (t / 3) % 3 - 1;
    dx = t % 3 - 1;
}

// ---- tcgen05 helpers -----------------------------------------------------
// 3x3x3 convolutions, zero padding 1: Y[v, co] = act(sum_{t, ci} X[v + off(t),
// ci] W[t, ci, co] + bias[co]), as implicit GEMMs on the 5th-generation
// tensor cores: M = 128 output voxels (one TMEM lane each), N = output
// channels (FP32 accumulators in TMEM), K = 27 taps x Cin.  Operands sit in
// shared memory in the canonical no-swizzle K-major layout (8-row x 16-byte
// core matrices); one elected thread issues the MMAs and commits them to an
// mbarrier.  Waits are bounded (0.5 s of globaltimer).
constexpr int TC_M = 128;
// stride between 8-row groups of the packed weights (Cin / 8 core matrices each)
__device__ __forceinline__ uint32_t sbo_b(int cin) { return (uint32_t)(cin >> 3) * 128u; }

__device__ __forceinline__ unsigned long long tc_timer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// shared-memory matrix descriptor: start, leading (K) and stride (M/N)
// byte offsets >> 4, descriptor version 1 (bits 46-47), no swizzle
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, K-major
// (or, mn_major, both MN-major: bits 15 and 16), N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t tc_idesc(int m, int n, bool mn_major = false) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (mn_major ? (3u << 15) : 0u) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ void mbar_init(uint32_t bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
// true once the phase of the given parity completed; false after 0.5 s
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    const unsigned long long t0 = tc_timer();
    while (true) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (done) return true;
        if (tc_timer() - t0 > 500000000ull) return false;
    }
}
__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int acc) {
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
                 "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}
// 16 consecutive FP32 accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                 "%13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = __uint_as_float(r[q]);
}

// The B operands of k_conv3_zm in the canonical K-major layout, per chunk of
// C output channels: from W [27][cin][cout] (tap t = (dz+1) 9 + (dy+1) 3 +
// (dx+1)) to P[chunk][shift (dy+1) 3 + (dx+1)][n][k] with n = j C + c, the
// column blocks j = 0, 1, 2 holding dz = +1, 0, -1 (output planes q - 2,
// q - 1, q of input plane q), core matrix (n / 8, k / 8) at
// ((n / 8) (cin / 8) + k / 8) x 64 elements, row n % 8, column k % 8.
__global__ void k_pack_b(int cin, int cout, int C, const bf16 *__restrict__ W, bf16 *__restrict__ P) {
    const long long n_all = 27LL * cin * cout;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n_all;
         e += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(e / ((long long)cin * cout));
        const int rem = (int)(e - (long long)t * cin * cout);
        const int k = rem / cout, co = rem % cout;
        const int dz = t / 9 - 1, sh = t % 9, j = 1 - dz;
        const int ch = co / C, n = j * C + co % C;
        const long long dst = (long long)ch * 27 * C * cin + (long long)sh * 3 * C * cin +
                              ((long long)((n >> 3) * (cin >> 3) + (k >> 3)) << 6) + ((n & 7) << 3) + (k & 7);
        P[dst] = W[e];
    }
}

// ---- z-marching tcgen05 convolution --------------------------------------
// The implicit GEMM of a 3x3x3 convolution (M = 128 output voxels of an
// 8 x 16 tile, K = 27 taps x Cin) for a whole column of tiles along z: one
// CTA owns tile (x0, y0) for output planes zb .. ze-1 of one chunk of C
// output channels and streams the input planes zb-1 .. ze through a ring of
// R shared-memory slots, each plane's tile plus its one-voxel halo (10 x 18
// voxels) loaded by TMA as Cin / 8 boxes, one per 8-channel group plane of
// the input, i.e. in the layout [group][y][x][8 channels] (each box row is
// 10 voxels x 16 bytes, contiguous in the group plane): the A operand of
// in-plane shift (dy, dx) is a
// descriptor view of the slot at (dy + 1, dx + 1) with core matrices one
// group block (2944 B) apart along K and one halo line (160 B) apart along M.
//
// The three z-taps share that A operand: one MMA multiplies input plane q
// by [W(dz=+1) | W(dz=0) | W(dz=-1)] (N = 3C), whose column blocks are the
// contributions of plane q to output planes q-2, q-1, q (relative to zb).
// The accumulators are a ring of S output planes in TMEM (C columns each),
// so those three blocks are consecutive slots; an MMA whose blocks wrap past
// the last slot is split in two.  So each input plane's operand is read 9 x
// Cin / 16 times from shared memory instead of 27 x, and a plane is needed
// by the MMAs of one step only.  Slots are zeroed before their first
// writer, so every MMA accumulates.  The weights of the CTA's chunk stay in
// shared memory for the whole column.
//
// Warp roles, connected by mbarriers only: warp 4 loads planes (full[slot]
// when a plane has landed, empty[slot] when the MMAs that read it are done),
// warp 5 issues the MMAs (accf[s] when output plane s is complete, acce[s]
// when the epilogue has read and re-zeroed it), warps 0-3 read the
// accumulators back (one TMEM lane, i.e. one output voxel, per thread:
// bias, GELU, stores).  Every wait is bounded (0.5 s); a role that gives up
// raises a shared flag the others see, and after the roles end the MMA
// thread drains what was issued (again bounded), sets the error word, and
// the TMEM is freed.
// ZM_GB: bytes of one group of one plane as the TMA writes it; ZM_GP: its
// pitch in the slot (a multiple of 128 bytes, the TMA destination alignment)
constexpr int ZM_HX = 10, ZM_HY = 18, ZM_GB = ZM_HX * ZM_HY * 16, ZM_GP = (ZM_GB + 127) / 128 * 128, ZM_RMAX = 6;
constexpr int ZM_THREADS = 192, ZM_SMAX = 8;
// output-plane slots of a C-channel chunk (four: the three an MMA writes and
// the one the epilogue reads) and their TMEM columns
__host__ __device__ constexpr int zm_slots(int) { return 4; }
__host__ __device__ constexpr int zm_tcols(int c) {
    return zm_slots(c) * c <= 32 ? 32 : (zm_slots(c) * c <= 64 ? 64 : (zm_slots(c) * c <= 128 ? 128 : 256));
}

struct ZmArgs {
    Vol v;
    int cin;            // input channels (tensor map and K), a multiple of 16
    int cout;           // channel stride of the outputs
    int ring;           // resident planes, 4 .. ZM_RMAX
    int zseg, nzseg;    // planes per work item, work items along z
    int ncol, tiles_x;  // tile columns
    int act;            // GELU on Y (and the head)
    const bf16 *P;      // weights packed for the B operand (k_pack_b), all cout
    const float *bias;  // cout or null
    float *Z;           // FP32 result before the activation (stride cout) or null
    bf16 *Y;            // BF16 activated result (8-channel group planes) or null
    const float *head;  // 1x1 head (16 weights + bias) fused into the epilogue, or null
    const float *scales;
    float *out, *raw;   // head outputs: out = scales[1] raw
    int *err;
};

__device__ __forceinline__ void zm_expect(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void zm_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// one 8-channel group plane's box (8 channels x 10 x 18 x 1 x 1) at (x, y, z, group)
__device__ __forceinline__ void zm_tma5(uint32_t dst, const CUtensorMap *map, int x, int y, int z, int g,
                                        uint32_t bar) {
    const int c = 0;
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"(map), "r"(c), "r"(x), "r"(y), "r"(z), "r"(g), "r"(bar)
        : "memory");
}
__device__ __forceinline__ bool zm_failed(const int *flag) { return *reinterpret_cast<const volatile int *>(flag) != 0; }

// 16 consecutive FP32 TMEM columns of this thread's lane set to zero
__device__ __forceinline__ void tc_zero16(uint32_t taddr) {
    const uint32_t z = 0;
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
                 "%1, %1, %1};" ::"r"(taddr),
                 "r"(z)
                 : "memory");
}

template <int N>
__global__ void __launch_bounds__(ZM_THREADS) k_conv3_zm(const __grid_constant__ ZmArgs a,
                                                        const __grid_constant__ CUtensorMap xmap) {
    constexpr int S = zm_slots(N), TCOLS = zm_tcols(N);
    extern __shared__ unsigned char zm_smem[];
    __shared__ __align__(8) uint64_t full[ZM_RMAX], empty[ZM_RMAX], accf[ZM_SMAX], acce[ZM_SMAX], drain;
    __shared__ uint32_t tmem_slot;
    __shared__ int fail, issued_sh, waited_sh;
    __shared__ float bias_s[96];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int groups = a.cin >> 3;
    const uint32_t slot_bytes = (uint32_t)groups * ZM_GP, plane_tx = (uint32_t)groups * ZM_GB;
    const int R = a.ring;
    // work item: consecutive blocks take neighbouring columns of one z range
    const int bid = blockIdx.x;
    const int col = bid % a.ncol, zs = (bid / a.ncol) % a.nzseg, chunk = bid / (a.ncol * a.nzseg);
    const int x0 = 8 * (col % a.tiles_x), y0 = 16 * (col / a.tiles_x);
    const int zb = zs * a.zseg, ze = min(zb + a.zseg, a.v.nz);
    const int n0 = chunk * N;
    const int nplanes = ze - zb, nload = nplanes + 2;   // input planes zb - 1 .. ze
    // shared memory: weights of the chunk (9 shifts x 3N x cin BF16), then the ring
    const uint32_t raw_addr = smem_u32(zm_smem);
    unsigned char *wsm = zm_smem + (((raw_addr + 1023u) & ~1023u) - raw_addr);
    const uint32_t wbytes = 27u * N * a.cin * 2u;
    unsigned char *ring = wsm + ((wbytes + 1023u) & ~1023u);
    const uint32_t wbase = smem_u32(wsm), rbase = smem_u32(ring);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(TCOLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
        asm volatile("tcgen05.fence::before_thread_sync;");
    }
    if (tid == 0) {
        for (int q = 0; q < R; ++q) {
            mbar_init(smem_u32(&full[q]), 1);
            mbar_init(smem_u32(&empty[q]), 1);
        }
        for (int b = 0; b < S; ++b) {
            mbar_init(smem_u32(&accf[b]), 1);
            mbar_init(smem_u32(&acce[b]), 4);   // one arrival per epilogue warp
        }
        fail = 0;
        issued_sh = waited_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int c = tid; c < N; c += ZM_THREADS) bias_s[c] = a.bias ? __ldg(a.bias + n0 + c) : 0.0f;
    // the chunk's packed weights are contiguous
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(a.P + (long long)chunk * 27 * N * a.cin);
        for (uint32_t q = tid; q < wbytes / 16u; q += ZM_THREADS) reinterpret_cast<uint4 *>(wsm)[q] = __ldg(src + q);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;
    if (warp < 4) {
        // every accumulator slot starts at zero
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c = 0; c < TCOLS; c += 16) tc_zero16(lane_addr + (uint32_t)c);
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");

    if (warp == 4) {
        // ---- producer: input plane q (z = zb - 1 + q) into ring slot q % R
        if (lane == 0) {
            int q = 0;
            for (; q < nload; ++q) {
                if (zm_failed(&fail)) break;
                const int slot = q % R;
                if (q >= R && !mbar_wait(smem_u32(&empty[slot]), (uint32_t)(((q / R) - 1) & 1))) {
                    atomicExch(&fail, 1);
                    break;
                }
                const uint32_t bar = smem_u32(&full[slot]), dst = rbase + (uint32_t)slot * slot_bytes;
                zm_expect(bar, plane_tx);
                for (int g = 0; g < groups; ++g)
                    zm_tma5(dst + (uint32_t)g * ZM_GP, &xmap, x0 - 1, y0 - 1, zb - 1 + q, g, bar);
            }
            issued_sh = q;
        }
    } else if (warp == 5) {
        // ---- MMA issue: input plane q into output planes q - 2 .. q
        if (lane == 0) {
            // descriptors advance by adding (byte offset >> 4) to the start field
            const uint64_t ad0 = tc_sdesc(rbase, ZM_GP, ZM_HX * 16), bd0 = tc_sdesc(wbase, 128u, sbo_b(a.cin));
            const int ksteps = a.cin >> 4;
            const uint32_t shift_b = (uint32_t)(3 * N * a.cin * 2), blk_b = (uint32_t)(N * a.cin * 2);
            int waited = 0;
            for (int q = 0; q < nload; ++q) {
                bool ok = !zm_failed(&fail);
                if (ok) ok = mbar_wait(smem_u32(&full[q % R]), (uint32_t)((q / R) & 1));
                if (ok) ++waited;
                // output plane q's slot must have been read and re-zeroed
                if (ok && q < nplanes && q >= S) ok = mbar_wait(smem_u32(&acce[q % S]), (uint32_t)(((q / S) - 1) & 1));
                if (!ok) {
                    atomicExch(&fail, 1);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;");
                // the valid output planes q - 2 .. q, as one or two runs of slots
                const int olo = max(q - 2, 0), ohi = min(q, nplanes - 1);
                const int b0 = olo - (q - 2), nb = ohi - olo + 1;
                const int s0 = olo % S;
                const int nb1 = min(nb, S - s0), nb2 = nb - nb1;
                const uint32_t id1 = tc_idesc(TC_M, nb1 * N), id2 = tc_idesc(TC_M, (nb2 > 0 ? nb2 : 1) * N);
                const uint32_t d1 = tmem + (uint32_t)(s0 * N), d2 = tmem;
                const uint64_t ap = ad0 + (((uint32_t)(q % R) * slot_bytes) >> 4);
#pragma unroll
                for (int sh = 0; sh < 9; ++sh) {
                    const int dy = sh / 3 - 1, dx = sh % 3 - 1;
                    const uint64_t ad = ap + ((uint32_t)(((dy + 1) * ZM_HX + (dx + 1)) * 16) >> 4);
                    const uint64_t bd = bd0 + (((uint32_t)sh * shift_b + (uint32_t)b0 * blk_b) >> 4);
#pragma unroll 1
                    for (int kc = 0; kc < ksteps; ++kc) {
                        const uint64_t ak = ad + (uint64_t)((2u * ZM_GP * kc) >> 4), bk = bd + (uint64_t)((256u * kc) >> 4);
                        tc_mma(d1, ak, bk, id1, 1);
                        if (nb2 > 0) tc_mma(d2, ak, bk + (uint64_t)(((uint32_t)nb1 * blk_b) >> 4), id2, 1);
                    }
                }
                // the slot refills only if a later plane goes there
                if (q + R < nload) tc_commit(smem_u32(&empty[q % R]));
                // output plane q - 2 has all its contributions
                if (q >= 2) tc_commit(smem_u32(&accf[(q - 2) % S]));
            }
            waited_sh = waited;
        }
    } else {
        // ---- epilogue: thread tid reads TMEM lane tid = output voxel (x0 + tid % 8, y0 + tid / 8)
        const int ox = x0 + (tid & 7), oy = y0 + (tid >> 3);
        const bool in = ox < a.v.nx && oy < a.v.ny;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        const float hb = a.head ? __ldg(a.head + 16) : 0.0f;
        const long long nvox = a.v.n();
        for (int j = 0; j < nplanes; ++j) {
            const int sl = j % S;
            if (zm_failed(&fail) || !mbar_wait(smem_u32(&accf[sl]), (uint32_t)((j / S) & 1))) {
                atomicExch(&fail, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            // the whole chunk into registers, the slot re-zeroed and handed
            // back to the MMA warp before the arithmetic and the stores
            float acc[N];
#pragma unroll
            for (int c0 = 0; c0 < N; c0 += 16) {
                float t[16];
                tc_ld16(lane_addr + (uint32_t)(sl * N + c0), t);
                tc_zero16(lane_addr + (uint32_t)(sl * N + c0));
#pragma unroll
                for (int q = 0; q < 16; ++q) acc[c0 + q] = t[q];
            }
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) zm_arrive(smem_u32(&acce[sl]));
            if (in) {
                const int z = zb + j;
                const long long vox = ox + (long long)a.v.nx * (oy + (long long)a.v.ny * z);
                float hs = hb;
#pragma unroll
                for (int c0 = 0; c0 < N; c0 += 16) {
                    float zz[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) zz[q] = acc[c0 + q] + bias_s[c0 + q];
                    if (a.Z) {
                        float4 *zr = reinterpret_cast<float4 *>(a.Z + vox * a.cout + n0 + c0);
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            zr[q] = make_float4(zz[4 * q], zz[4 * q + 1], zz[4 * q + 2], zz[4 * q + 3]);
                    }
                    if (a.Y || a.head) {
                        float gz[16];
#pragma unroll
                        for (int q = 0; q < 16; ++q) gz[q] = a.act ? gelu(zz[q]) : zz[q];
                        if (a.Y) {
                            __nv_bfloat162 yb[8];
#pragma unroll
                            for (int q = 0; q < 8; ++q) yb[q] = __floats2bfloat162_rn(gz[2 * q], gz[2 * q + 1]);
                            *reinterpret_cast<uint4 *>(a.Y + g8(vox, n0 + c0, nvox)) = reinterpret_cast<const uint4 *>(yb)[0];
                            *reinterpret_cast<uint4 *>(a.Y + g8(vox, n0 + c0 + 8, nvox)) =
                                reinterpret_cast<const uint4 *>(yb)[1];
                        }
                        if (a.head) {
#pragma unroll
                            for (int q = 0; q < 16; ++q) hs += gz[q] * __ldg(a.head + c0 + q);
                        }
                    }
                }
                if (a.head) {
                    if (a.raw) a.raw[vox] = hs;
                    if (a.out) a.out[vox] = hs * __ldg(a.scales + 1);
                }
            }
        }
    }
    __syncthreads();
    if (fail && tid == 5 * 32) {
        // drain the loads and MMAs issued before the roles gave up (bounded):
        // every issued plane lands, and a last commit tracks all the MMAs
        for (int q = waited_sh; q < issued_sh; ++q) mbar_wait(smem_u32(&full[q % R]), (uint32_t)((q / R) & 1));
        mbar_init(smem_u32(&drain), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        tc_commit(smem_u32(&drain));
        mbar_wait(smem_u32(&drain), 0);
        atomicExch(a.err, 1);
    }
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS));
    }
}

// weight gradient on tcgen05: dW[t, ci, co] += sum_v X[v + off(t), ci] G[v, co]
// over a chunk of WG_VC voxels; block = (chunk, tap).  The GEMM runs
// transposed, D[co][ci] = sum_v G[v][co] X[v + off(t)][ci]: M = Cout padded
// to 128 (columns past Cout stay zero), N = Cin, K = the chunk's voxels in
// stages of 64.  Both operands are MN-major in the canonical no-swizzle
// layout: a core matrix is 8 K-rows (voxels) of 16 bytes (8 consecutive
// channels), i.e. rows of the 8-channel group planes copied as they are; core matrices 128
// bytes apart along K (LBO) and 1 KB apart along M / N (SBO).  The
// accumulators are added to dW with FP32 atomics (order-dependent in the
// last bits).
constexpr int WG_KC = 64, WG_VC = 1024, WG_MAXQ = 10;   // rows per thread: 64 (Cin + Cout) / 8 / 128

__global__ void __launch_bounds__(128) k_conv3_wgrad_tc(Vol v, const bf16 *__restrict__ X, int cin,
                                                       const bf16 *__restrict__ G, int cout, float *__restrict__ dW,
                                                       int *__restrict__ err) {
    extern __shared__ unsigned char tc_smem[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ uint32_t tmem_slot;
    const int tcols = cin <= 32 ? 32 : (cin <= 64 ? 64 : 128);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int a_bytes = TC_M * WG_KC * 2, b_bytes = cin * WG_KC * 2;
    const int stage_bytes = (a_bytes + b_bytes + 1023) & ~1023;
    const uint32_t raw = smem_u32(tc_smem);
    unsigned char *stages = tc_smem + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t bar0 = smem_u32(&bars[0]), bar1 = smem_u32(&bars[1]);
    // A rows at or past Cout are never written below: zero both stages' A once
    for (int q = tid; q < a_bytes / 16; q += TC_M) {
        reinterpret_cast<uint4 *>(stages)[q] = make_uint4(0, 0, 0, 0);
        reinterpret_cast<uint4 *>(stages + stage_bytes)[q] = make_uint4(0, 0, 0, 0);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(tcols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
        asm volatile("tcgen05.fence::before_thread_sync;");
    }
    if (tid == 0) {
        mbar_init(bar0, 1);
        mbar_init(bar1, 1);
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;
    const int t = blockIdx.y;
    int dx, dy, dz;
    tap_offset(t, dx, dy, dz);
    const long long nvox = v.n();
    const long long vbeg = (long long)blockIdx.x * WG_VC;
    const int nst = (int)std::min<long long>(WG_VC / WG_KC, (nvox - vbeg + WG_KC - 1) / WG_KC);
    const uint32_t idesc = tc_idesc(TC_M, cin, true);
    constexpr uint32_t SBO = (WG_KC / 8) * 128;   // 8-channel groups along M or N
    const int gco = cout >> 3, gci = cin >> 3;
    // a stage is 64 (Cout / 8) A rows then 64 (Cin / 8) B rows of 16 bytes;
    // thread tid moves rows tid + 128 j (the A/B boundary is a multiple of
    // 128, so row j is A or B for the whole block).  The next stage's rows
    // are loaded into registers while the current stage's MMAs run.
    const int na = WG_KC * gco, nrows = WG_KC * (gco + gci), nq = nrows / TC_M;
    uint4 pre[WG_MAXQ];
    auto fetch = [&](int sidx) {
        const long long k0 = vbeg + (long long)sidx * WG_KC;
#pragma unroll
        for (int j = 0; j < WG_MAXQ; ++j) {
            if (j >= nq) break;
            const int q = tid + TC_M * j;
            const bool isa = q < na;
            const int qq = isa ? q : q - na;
            const int r = qq % WG_KC, cg = qq / WG_KC;
            const long long vv = k0 + r;
            uint4 val = make_uint4(0, 0, 0, 0);
            if (vv < nvox) {
                if (isa) {
                    val = __ldg(reinterpret_cast<const uint4 *>(G + g8(vv, 8 * cg, nvox)));
                } else {
                    const int x = (int)(vv % v.nx), y = (int)((vv / v.nx) % v.ny),
                              z = (int)(vv / ((long long)v.nx * v.ny));
                    const int sx = x + dx, sy = y + dy, sz = z + dz;
                    if (sx >= 0 && sx < v.nx && sy >= 0 && sy < v.ny && sz >= 0 && sz < v.nz)
                        val = __ldg(reinterpret_cast<const uint4 *>(
                            X + g8(sx + (long long)v.nx * (sy + (long long)v.ny * sz), 8 * cg, nvox)));
                }
            }
            pre[j] = val;
        }
    };
    // row (cg, r) of A or B: one 16-byte row of core matrix (cg, r / 8)
    auto put = [&](unsigned char *stg) {
        uint4 *A = reinterpret_cast<uint4 *>(stg), *B = reinterpret_cast<uint4 *>(stg + a_bytes);
#pragma unroll
        for (int j = 0; j < WG_MAXQ; ++j) {
            if (j >= nq) break;
            const int q = tid + TC_M * j;
            const bool isa = q < na;
            const int qq = isa ? q : q - na;
            const int r = qq % WG_KC, cg = qq / WG_KC;
            (isa ? A : B)[(cg * (WG_KC / 8) + (r >> 3)) * 8 + (r & 7)] = pre[j];
        }
    };
    bool ok = true;
    int last = -1;
    fetch(0);
    for (int sidx = 0; sidx < nst; ++sidx) {
        const int st = sidx & 1;
        unsigned char *stg = stages + st * stage_bytes;
        // the stage's previous MMAs (stage sidx - 2) must be done before it is overwritten
        if (sidx >= 2) ok = mbar_wait(st ? bar1 : bar0, (uint32_t)(((sidx >> 1) - 1) & 1));
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
        put(stg);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;");
            const uint32_t a0 = smem_u32(stg), b0 = a0 + (uint32_t)a_bytes;
#pragma unroll
            for (int kc = 0; kc < WG_KC / 16; ++kc)
                tc_mma(tmem, tc_sdesc(a0 + 256u * kc, 128u, SBO), tc_sdesc(b0 + 256u * kc, 128u, SBO), idesc,
                       (sidx > 0 || kc > 0) ? 1 : 0);
            tc_commit(st ? bar1 : bar0);
        }
        last = sidx;
        if (sidx + 1 < nst) fetch(sidx + 1);
    }
    if (last >= 0) {
        const bool done = mbar_wait((last & 1) ? bar1 : bar0, (uint32_t)((last >> 1) & 1));
        ok = ok && done;
    }
    ok = __syncthreads_and(ok);
    if (ok && last >= 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        const int co = warp * 32 + lane;
        const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c0 = 0; c0 < cin; c0 += 16) {
            float acc[16];
            tc_ld16(lane_addr + (uint32_t)c0, acc);
            if (co < cout) {
#pragma unroll
                for (int q = 0; q < 16; ++q) atomicAdd(dW + ((long long)t * cin + c0 + q) * cout + co, acc[q]);
            }
        }
    } else if (!ok && tid == 0) {
        atomicExch(err, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tcols));
    }
}

// G = dY * gelu'(Z) in BF16 (the GEMM operand of both backward convolutions),
// from channels-last FP32 into 8-channel group planes; with act == 0, G = dY.
// One thread per voxel and group.
__global__ void k_act_grad(long long nvox, int C, const float *__restrict__ dY, const float *__restrict__ Z, int act,
                           bf16 *__restrict__ G) {
    const int ng = C >> 3;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nvox * ng;
         i += (long long)gridDim.x * blockDim.x) {
        const long long v = i / ng;
        const int g = (int)(i - v * ng);
        __align__(16) bf16 o[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long e = v * C + 8 * g + k;
            o[k] = __float2bfloat16_rn(act ? dY[e] * gelu_grad(Z[e]) : dY[e]);
        }
        *reinterpret_cast<uint4 *>(G + g8(v, 8 * g, nvox)) = *reinterpret_cast<const uint4 *>(o);
    }
}

// bias gradient: db[c] += sum_v G[v, c] (G in 8-channel group planes: the
// flat index i runs over group planes, channel (i / (8 nvox)) 8 + i % 8)
__global__ void k_bias_grad(long long nvox, int C, const bf16 *__restrict__ G, float *__restrict__ db) {
    extern __shared__ float sb[];
    for (int c = threadIdx.x; c < C; c += blockDim.x) sb[c] = 0.f;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nvox * C; i += (long long)gridDim.x * blockDim.x)
        atomicAdd(&sb[(int)(i / (8 * nvox)) * 8 + (int)(i & 7)], __bfloat162float(G[i]));
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

// 2x average pooling of 8-channel group planes: one thread per coarse voxel
// and group (16-byte loads and stores)
__global__ void k_pool(Vol c, int C, const bf16 *__restrict__ X, bf16 *__restrict__ Y) {
    const int G = C >> 3;
    const long long nc = c.n(), nf = 8 * nc, n = nc * G;
    const int fx = 2 * c.nx, fy = 2 * c.ny;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(i / nc);
        const long long vv = i - (long long)g * nc;
        const int x = (int)(vv % c.nx);
        const long long yz = vv / c.nx;
        const int y = (int)(yz % c.ny), z = (int)(yz / c.ny);
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const long long f = (2 * x + (q & 1)) + (long long)fx * ((2 * y + ((q >> 1) & 1)) + (long long)fy * (2 * z + (q >> 2)));
            const uint4 u = __ldg(reinterpret_cast<const uint4 *>(X + g8(f, 8 * g, nf)));
            const bf16 *e = reinterpret_cast<const bf16 *>(&u);
#pragma unroll
            for (int k = 0; k < 8; ++k) s[k] += __bfloat162float(e[k]);
        }
        __align__(16) bf16 o[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) o[k] = __float2bfloat16_rn(s[k] * 0.125f);
        *reinterpret_cast<uint4 *>(Y + g8(vv, 8 * g, nc)) = *reinterpret_cast<const uint4 *>(o);
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

// nearest 2x upsampling of X (C1 channels) into the first C1 / 8 group
// planes of the concat buffer Y; the skip tensor's planes follow them in
// the same allocation (it was written there by its convolution), so the
// concatenation copies nothing else.  One thread per fine voxel and group.
__global__ void k_up_concat(Vol f, int C1, const bf16 *__restrict__ X, bf16 *__restrict__ Y) {
    const int G1 = C1 >> 3;
    const long long nf = f.n(), nc = nf / 8, n = nf * G1;
    const int cx = f.nx / 2, cy = f.ny / 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(i / nf);
        const long long vv = i - (long long)g * nf;
        const int x = (int)(vv % f.nx);
        const long long yz = vv / f.nx;
        const int y = (int)(yz % f.ny), z = (int)(yz / f.ny);
        const long long cv = (x / 2) + (long long)cx * ((y / 2) + (long long)cy * (z / 2));
        *reinterpret_cast<uint4 *>(Y + g8(vv, 8 * g, nf)) = __ldg(reinterpret_cast<const uint4 *>(X + g8(cv, 8 * g, nc)));
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

// network input: channels (b / sb, mask, p_prev / sp, 0 ... 0), 16 wide;
// only the first group plane is written (the second, channels 8-15, is
// zeroed once when the buffer is allocated).  One voxel per thread.
__global__ void k_input(long long n, const float *__restrict__ b, const uint8_t *__restrict__ mask,
                        const float *__restrict__ pp, const float *__restrict__ scales, bf16 *__restrict__ X) {
    const float isb = 1.0f / scales[0], isp = 1.0f / scales[1];
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        __align__(16) bf16 x[8];
        x[0] = __float2bfloat16_rn(b[v] * isb);
        x[1] = __float2bfloat16_rn(mask ? (float)mask[v] : 0.0f);
        x[2] = __float2bfloat16_rn(pp ? pp[v] * isp : 0.0f);
#pragma unroll
        for (int c = 3; c < 8; ++c) x[c] = __float2bfloat16_rn(0.0f);
        *reinterpret_cast<uint4 *>(X + v * 8) = *reinterpret_cast<const uint4 *>(x);
    }
}

// Loss in normalised units with d = raw - t / sp:
//   L = mean(d^2) + LAP_W mean((D d)^2),
// D the 7-point graph Laplacian of the grid (sum over the existing face
// neighbours of d_nbr - d_v; no term across the domain edge).  The second
// term weighs the error's grid-scale part, which the pressure operator
// amplifies in the residual of a guess.  dL/draw = (2 d + 2 LAP_W D(D d)) / n
// (D is symmetric).  Three passes: d into draw; D d into raw with the loss
// partials; then dL/draw over draw.
constexpr float LAP_W = 0.25f;

__device__ __forceinline__ float graph_lap(const float *a, Vol v, int x, int y, int z, long long i) {
    const float c = a[i];
    float s = 0.0f;
    if (x > 0) s += a[i - 1] - c;
    if (x < v.nx - 1) s += a[i + 1] - c;
    if (y > 0) s += a[i - v.nx] - c;
    if (y < v.ny - 1) s += a[i + v.nx] - c;
    const long long pz = (long long)v.nx * v.ny;
    if (z > 0) s += a[i - pz] - c;
    if (z < v.nz - 1) s += a[i + pz] - c;
    return s;
}

__global__ void k_loss_d(long long n, const float *__restrict__ raw, const float *__restrict__ target,
                         const float *__restrict__ scales, float *__restrict__ d) {
    const float isp = 1.0f / scales[1];
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x)
        d[v] = raw[v] - target[v] * isp;
}
__global__ void k_loss_lap(Vol v, const float *__restrict__ d, float *__restrict__ e, double *__restrict__ partial) {
    __shared__ double sred[256];
    const long long n = v.n();
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % v.nx);
        const long long yz = i / v.nx;
        const int y = (int)(yz % v.ny), z = (int)(yz / v.ny);
        const float l = graph_lap(d, v, x, y, z, i);
        e[i] = l;
        acc += (double)d[i] * d[i] + (double)LAP_W * l * l;
    }
    sred[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sred[threadIdx.x] += sred[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sred[0] / (double)n;
}
__global__ void k_loss_grad(Vol v, const float *__restrict__ e, float *__restrict__ d_to_draw) {
    const long long n = v.n();
    const float inv = 1.0f / (float)n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % v.nx);
        const long long yz = i / v.nx;
        const int y = (int)(yz % v.ny), z = (int)(yz / v.ny);
        d_to_draw[i] = (2.0f * d_to_draw[i] + 2.0f * LAP_W * graph_lap(e, v, x, y, z, i)) * inv;
    }
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

// per-field sums of squares of b and p_prev (deterministic two-level
// reduction: FP64 block partials, then k_scales in one block)
__global__ void k_sumsq2(long long n, const float *__restrict__ a, const float *__restrict__ c,
                         double *__restrict__ partial) {
    // each thread sums a few dozen squares in FP32, the block in FP32, the
    // blocks in FP64 (k_scales)
    __shared__ float sa[256], sc[256];
    float xa = 0.0f, xc = 0.0f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
        const float p = a[v];
        xa = __fmaf_rn(p, p, xa);
        if (c) {
            const float q = c[v];
            xc = __fmaf_rn(q, q, xc);
        }
    }
    sa[threadIdx.x] = xa;
    sc[threadIdx.x] = xc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sa[threadIdx.x] += sa[threadIdx.x + s];
            sc[threadIdx.x] += sc[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = sa[0];
        partial[2 * blockIdx.x + 1] = sc[0];
    }
}
// normalisation scales: sb = rms(b), sp = rms(p_prev), or rms(b) L^2 /
// (4 pi^2) (L the smallest domain extent) when p_prev is zero or absent;
// one block of 256 threads
__global__ void k_scales(int nb, long long n, double L2, const double *__restrict__ partial, float *__restrict__ scales) {
    __shared__ double sa[256], sc[256];
    double xa = 0.0, xc = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        xa += partial[2 * b];
        xc += partial[2 * b + 1];
    }
    sa[threadIdx.x] = xa;
    sc[threadIdx.x] = xc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sa[threadIdx.x] += sa[threadIdx.x + s];
            sc[threadIdx.x] += sc[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double sb = sqrt(sa[0] / (double)n);
        double sp = sqrt(sc[0] / (double)n);
        if (!(sp > 0)) sp = sb * L2 / (4.0 * 3.14159265358979323846 * 3.14159265358979323846);
        scales[0] = (float)(sb > 0 ? sb : 1.0);
        scales[1] = (float)(sp > 0 ? sp : 1.0);
    }
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

int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 152;
    }
    return n;
}

PFN_cuTensorMapEncodeTiled_v12000 zm_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// shared memory of k_conv3_zm: weights of an N-channel chunk, a ring of R
// planes, 1 KB alignment slack
size_t zm_smem_bytes(int n, int cin, int ring) {
    return ((27u * n * cin * 2u + 1023u) & ~1023u) + (size_t)ring * (cin / 8) * ZM_GP + 1024;
}

// CTAs per SM the register file allows for k_conv3_zm<N>
template <int N>
int zm_reg_blocks() {
    static int b = 0;
    if (!b) {
        cudaFuncAttributes fa;
        b = 6;
        if (cudaFuncGetAttributes(&fa, k_conv3_zm<N>) == cudaSuccess && fa.numRegs > 0)
            b = std::max(1, 65536 / (((fa.numRegs + 7) / 8 * 8) * ZM_THREADS));
    }
    return b;
}
int zm_reg_blocks_for(int n) {
    switch (n) {
    case 16: return zm_reg_blocks<16>();
    case 32: return zm_reg_blocks<32>();
    case 48: return zm_reg_blocks<48>();
    default: return zm_reg_blocks<64>();
    }
}

template <int N>
int launch_zm(const ZmArgs &a, const CUtensorMap &map, int nchunks, size_t smem, cudaStream_t s) {
    static size_t configured = 0;
    if (smem > configured) {
        FF_CUDA(cudaFuncSetAttribute(k_conv3_zm<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        configured = smem;
    }
    const long long blocks = (long long)a.ncol * a.nzseg * nchunks;
    k_conv3_zm<N><<<(unsigned)blocks, ZM_THREADS, smem, s>>>(a, map);
    return post("conv3 z-march");
}

// Y = act(conv(X, W) + bias) and/or Z = conv(X, W) + bias, or the fused head
// (out, raw) on top of the activation.  X: BF16 in 8-channel group planes
// with cin channels (a multiple of 16, at most 96); Y in the same layout, Z
// channels-last FP32; W: [27][cin][cout] BF16, packed into pk (27 cin cout)
// for the B operand.
int launch_conv(int cout, Vol v, const bf16 *X, int cin, const bf16 *W, const float *bias, int act, float *Z, bf16 *Y,
                bf16 *pk, int *err, cudaStream_t s, const float *head = nullptr, const float *scales = nullptr,
                float *out = nullptr, float *raw = nullptr) {
    if (cin % 16 || cin > 96) return ff_set_error(FF_E_ARG, "unet: conv input channels %d (multiples of 16 to 96)", cin);
    if (cout % 16 || cout > 96) return ff_set_error(FF_E_ARG, "unet: conv output channels %d (multiples of 16 to 96)", cout);
    // the output-channel chunk C (3C <= 256 columns per MMA) and the ring
    // depth R: the widest chunk that reaches two or more CTAs per SM (else
    // one), then the deepest ring at that chunk's best occupancy.  CTAs per
    // SM are bounded by shared memory (228 KB less 1 KB per CTA), TMEM (512
    // columns) and the register file.
    auto occupancy = [&](int c, int r) {
        const size_t sm = zm_smem_bytes(c, cin, r);
        if (sm > 227 * 1024) return 0;
        return std::min({zm_reg_blocks_for(c), (int)(233472 / (sm + 1024)), 512 / zm_tcols(c)});
    };
    int n = 0, ring = 3, occ = 0;
    for (int want = 2; want >= 1 && !n; --want)
        for (int d : {1, 2, 3, 4, 6}) {
            if (cout % d || (cout / d) % 16 || cout / d > 80) continue;
            int best = 0;
            for (int r = 3; r <= ZM_RMAX; ++r) best = std::max(best, occupancy(cout / d, r));
            if (best >= want) {
                n = cout / d;
                occ = best;
                for (int r = ZM_RMAX; r >= 3; --r)
                    if (occupancy(n, r) == best) {
                        ring = r;
                        break;
                    }
                break;
            }
        }
    if (!n) return ff_set_error(FF_E_LIMIT, "unet: no shared-memory plan for a %d -> %d convolution", cin, cout);
    k_pack_b<<<gblocks(27LL * cin * cout), 256, 0, s>>>(cin, cout, n, W, pk);
    FF_TRY(post("pack weights"));
    const size_t smem = zm_smem_bytes(n, cin, ring);
    const int blocks_per_sm = occ;
    ZmArgs a;
    a.v = v;
    a.cin = cin;
    a.cout = cout;
    a.ring = ring;
    a.tiles_x = (v.nx + 7) / 8;
    a.ncol = a.tiles_x * ((v.ny + 15) / 16);
    const int nchunks = cout / n;
    // the z split: work items of at least 8 planes (or the whole column)
    // whose count fills the resident slots best, counting each item's two
    // extra halo planes and about two planes' worth of start-up
    const long long slots = (long long)sm_count() * blocks_per_sm;
    double best = 1e300;
    a.zseg = v.nz;
    for (int zs = v.nz; zs >= std::min(8, v.nz); --zs) {
        const long long items = (long long)a.ncol * nchunks * ((v.nz + zs - 1) / zs);
        const double cost = (double)((items + slots - 1) / slots) * (zs + 4);
        if (cost < best - 1e-9) {
            best = cost;
            a.zseg = zs;
        }
    }
    a.nzseg = (v.nz + a.zseg - 1) / a.zseg;
    a.act = act;
    a.P = pk;
    a.bias = bias;
    a.Z = Z;
    a.Y = Y;
    a.head = head;
    a.scales = scales;
    a.out = out;
    a.raw = raw;
    a.err = err;
    if (head && !(n == 16 && cout == 16)) return ff_set_error(FF_E_ARG, "unet: the fused head needs 16 channels");
    PFN_cuTensorMapEncodeTiled_v12000 enc = zm_encoder();
    FF_CHECK(enc, FF_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    CUtensorMap map;
    // the input's group planes: (8 channels, x, y, z, group), 16-byte voxels
    cuuint64_t dims[5] = {8, (cuuint64_t)v.nx, (cuuint64_t)v.ny, (cuuint64_t)v.nz, (cuuint64_t)(cin / 8)};
    cuuint64_t strides[4] = {16, (cuuint64_t)v.nx * 16, (cuuint64_t)v.nx * v.ny * 16, (cuuint64_t)v.n() * 16};
    cuuint32_t box[5] = {8, ZM_HX, ZM_HY, 1, 1};
    cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUresult r = enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, (void *)X, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    FF_CHECK(r == CUDA_SUCCESS, FF_E_CUDA, "unet: cuTensorMapEncodeTiled failed (%d) for %dx%dx%d x %d", (int)r, v.nx,
             v.ny, v.nz, cin);
    switch (n) {
    case 16: return launch_zm<16>(a, map, nchunks, smem, s);
    case 32: return launch_zm<32>(a, map, nchunks, smem, s);
    case 48: return launch_zm<48>(a, map, nchunks, smem, s);
    case 64: return launch_zm<64>(a, map, nchunks, smem, s);
    default: return ff_set_error(FF_E_ARG, "unet: no conv kernel for a %d-channel chunk", n);
    }
}

int launch_wgrad(int cin, int cout, Vol v, const bf16 *X, const bf16 *G, float *dW, int *err, cudaStream_t s) {
    if (cin % 16 || cin > 96 || cout % 16 || cout > TC_M || WG_KC * (cin + cout) / 8 > TC_M * WG_MAXQ)
        return ff_set_error(FF_E_ARG, "unet: no weight-gradient kernel for %d -> %d", cin, cout);
    // two stages of (128 x 64 A + cin x 64 B) BF16, 1 KB aligned, + alignment slack
    const int stage = (TC_M * WG_KC * 2 + cin * WG_KC * 2 + 1023) & ~1023;
    const int smem = 2 * stage + 1024;
    static int configured = 0;
    if (smem > configured) {
        FF_CUDA(cudaFuncSetAttribute(k_conv3_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        configured = smem;
    }
    dim3 grid((unsigned)((v.n() + WG_VC - 1) / WG_VC), 27);
    k_conv3_wgrad_tc<<<grid, TC_M, smem, s>>>(v, X, cin, G, cout, dW, err);
    return post("conv3 wgrad tcgen05");
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
    bf16 *wpk = nullptr;            // one layer's weights packed for the tcgen05 B operand
    int *tc_err = nullptr;          // set by a tcgen05 conv whose wait ran out
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
    bool has_train = false;         // pre, grad, gbuf, raw, draw allocated
    std::vector<void *> owned;
};

// tensor slots: 0 input(16) 1 e0a(16) 2 e0b=skip0(16) 3 p1(16) 4 e1a(32) 5 e1b=skip1(32)
// 6 p2(32) 7 ba(64) 8 bb(64) 9 cat1(96) 10 d1a(32) 11 d1b(32) 12 cat0(48) 13 d0a(16) 14 d0b(16);
// slots 2 and 5 are the last group planes of slots 12 and 9
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
    u->has_train = false;
}

static int alloc_owned(ff_unet u, void **p, size_t bytes) {
    FF_TRY(ff_dev_alloc(p, bytes, u->ctx->stream));
    u->owned.push_back(*p);
    return FF_OK;
}

// activations for a volume; with train, also the FP32 pre-activations and
// gradient buffers of the backward pass (inference never allocates them)
static int ensure_shape(ff_unet u, Vol v, bool train) {
    const bool same = u->vol.nx == v.nx && u->vol.ny == v.ny && u->vol.nz == v.nz;
    if (same && (!train || u->has_train)) return FF_OK;
    FF_CHECK(v.nx % 4 == 0 && v.ny % 4 == 0 && v.nz % 4 == 0 && v.nx >= 4 && v.ny >= 4 && v.nz >= 4, FF_E_ARG,
             "unet: resolution must be a multiple of 4 on every axis, got %dx%dx%d", v.nx, v.ny, v.nz);
    if (!same) {
        free_shape(u);
        u->vol = v;
    }
    const long long n0 = v.n();
    if (u->act.empty()) {
        u->act.resize(15);
        for (int s = 0; s < 15; ++s) {
            if (s == 2 || s == 5) continue;   // skip tensors: inside their concat buffers
            const long long nv = n0 >> (3 * SLOT_LEVEL[s]);
            FF_TRY(alloc_owned(u, (void **)&u->act[s], (size_t)nv * SLOT_C[s] * sizeof(bf16)));
        }
        // cat0 = [up(d1b): 4 group planes | skip0: 2], cat1 = [up(bb): 8 | skip1: 4]
        u->act[2] = u->act[12] + 4 * n0 * 8;
        u->act[5] = u->act[9] + 8 * (n0 >> 3) * 8;
        // channels 8-15 of the input are always zero
        FF_CUDA(cudaMemsetAsync(u->act[0] + n0 * 8, 0, (size_t)n0 * 8 * sizeof(bf16), u->ctx->stream));
        FF_TRY(alloc_owned(u, (void **)&u->scales, 16));
        FF_TRY(alloc_owned(u, (void **)&u->partial, sizeof(double) * 152 * 32));
    }
    if (train && !u->has_train) {
        u->grad.resize(15);
        long long maxc = 0;
        for (int s = 0; s < 15; ++s) {
            const long long nv = n0 >> (3 * SLOT_LEVEL[s]);
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
        u->has_train = true;
    }
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
        (st = ff_dev_alloc((void **)&u->wpk, 27LL * 96 * 64 * sizeof(bf16), s)) ||
        (st = ff_dev_alloc((void **)&u->tc_err, sizeof(int), s)) ||
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
    ff_dev_free(u->wpk);
    ff_dev_free(u->tc_err);
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

// normalisation scales into u->scales on the device (no host round trip)
static int compute_scales(ff_unet u, const float *b, const float *pp, double h) {
    cudaStream_t s = u->ctx->stream;
    const long long n = u->vol.n();
    const int nb = std::min(152 * 16, gblocks(n));
    k_sumsq2<<<nb, 256, 0, s>>>(n, b, pp, u->partial);
    FF_TRY(post("sumsq"));
    const double L = h * std::min(u->vol.nx, std::min(u->vol.ny, u->vol.nz));
    k_scales<<<1, 256, 0, s>>>(nb, n, L * L, u->partial, u->scales);
    return post("scales");
}

static Vol level_vol(ff_unet u, int lev) { return Vol{u->vol.nx >> lev, u->vol.ny >> lev, u->vol.nz >> lev}; }

// train: keep every convolution's FP32 pre-activation and the head's raw
// output for the backward pass; inference stores neither.  The last
// convolution feeds the 1x1 head in its epilogue (its BF16 output is never
// read, so it is not written).
static int forward(ff_unet u, const float *b, const uint8_t *mask, const float *pp, double h, float *out,
                   bool train) {
    cudaStream_t s = u->ctx->stream;
    FF_TRY(compute_scales(u, b, pp, h));
    const long long n0 = u->vol.n();
    k_input<<<gblocks(n0), 256, 0, s>>>(n0, b, mask, pp, u->scales, u->act[0]);
    auto conv = [&](int l) {
        const ConvLayer &c = u->convs[l];
        const int si = CONV_IN[l], so = CONV_OUT[l];
        const bool head = l == 9;
        return launch_conv(c.cout, level_vol(u, SLOT_LEVEL[so]), u->act[si], c.cin, u->wb + u->wb_off[l],
                           u->w + c.b_off, c.act, train ? u->pre[l] : nullptr, head ? nullptr : u->act[so], u->wpk,
                           u->tc_err, s, head ? u->w + u->head_off : nullptr, u->scales, out,
                           train ? u->raw : nullptr);
    };
    FF_TRY(conv(0));
    FF_TRY(conv(1));
    k_pool<<<gblocks(level_vol(u, 1).n() * 2), 256, 0, s>>>(level_vol(u, 1), 16, u->act[2], u->act[3]);
    FF_TRY(conv(2));
    FF_TRY(conv(3));
    k_pool<<<gblocks(level_vol(u, 2).n() * 4), 256, 0, s>>>(level_vol(u, 2), 32, u->act[5], u->act[6]);
    FF_TRY(conv(4));
    FF_TRY(conv(5));
    k_up_concat<<<gblocks(level_vol(u, 1).n() * 8), 256, 0, s>>>(level_vol(u, 1), 64, u->act[8], u->act[9]);
    FF_TRY(conv(6));
    FF_TRY(conv(7));
    k_up_concat<<<gblocks(n0 * 4), 256, 0, s>>>(level_vol(u, 0), 32, u->act[11], u->act[12]);
    FF_TRY(conv(8));
    FF_TRY(conv(9));
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
    k_act_grad<<<gblocks(nout / 8), 256, 0, s>>>(v.n(), c.cout, u->grad[so], u->pre[l], c.act, u->gbuf);
    FF_TRY(post("act grad"));
    if (c.cin == c.cin_real) {
        FF_TRY(launch_wgrad(c.cin, c.cout, v, u->act[si], u->gbuf, u->g + c.w_off, u->tc_err, s));
    } else {
        // padded input channels: accumulate over all 16, keep the real ones
        FF_CUDA(cudaMemsetAsync(u->g0, 0, 27LL * c.cin * c.cout * 4, s));
        FF_TRY(launch_wgrad(c.cin, c.cout, v, u->act[si], u->gbuf, u->g0, u->tc_err, s));
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
    FF_TRY(launch_conv(c.cin, v, u->gbuf, c.cout, u->wt, nullptr, 0, dst, nullptr, u->wpk, u->tc_err, s));
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

// a tcgen05 convolution whose bounded wait ran out leaves the error word
// set: report it (once) after the stream drains
static int tc_status(ff_unet u) {
    int e = 0;
    FF_CUDA(cudaMemcpyAsync(&e, u->tc_err, sizeof(int), cudaMemcpyDeviceToHost, u->ctx->stream));
    FF_CUDA(cudaStreamSynchronize(u->ctx->stream));
    if (e) {
        FF_CUDA(cudaMemsetAsync(u->tc_err, 0, sizeof(int), u->ctx->stream));
        return ff_set_error(FF_E_CUDA, "unet: a tensor-core convolution timed out waiting for its MMAs");
    }
    return FF_OK;
}

extern "C" int ff_unet_forward(ff_unet u, const int *res, double h, ff_field b, ff_field mask, ff_field p_prev,
                               ff_field out) {
    FF_CHECK(u && res, FF_E_ARG, "NULL argument");
    cudaSetDevice(u->ctx->device);
    FF_TRY(ensure_shape(u, Vol{res[0], res[1], res[2]}, false));
    const long long n = u->vol.n();
    FF_CHECK(field_ok(b, n, FF_FLOAT) && field_ok(out, n, FF_FLOAT) && (!p_prev || field_ok(p_prev, n, FF_FLOAT)) &&
                 (!mask || field_ok(mask, n, FF_UINT8)),
             FF_E_ARG, "unet forward: fields must be cell fields of the resolution (mask uint8)");
    FF_TRY(forward(u, (const float *)b->d, mask ? (const uint8_t *)mask->d : nullptr,
                   p_prev ? (const float *)p_prev->d : nullptr, h, (float *)out->d, false));
    return tc_status(u);
}

// forward + MSE loss against `target` + backward: leaves dL/dparams in the
// gradient buffer (zeroed first) and the loss in *loss
extern "C" int ff_unet_loss_backward(ff_unet u, const int *res, double h, ff_field b, ff_field mask, ff_field p_prev,
                                     ff_field target, double *loss) {
    FF_CHECK(u && res && target, FF_E_ARG, "NULL argument");
    cudaSetDevice(u->ctx->device);
    FF_TRY(ensure_shape(u, Vol{res[0], res[1], res[2]}, true));
    const long long n = u->vol.n();
    FF_CHECK(field_ok(b, n, FF_FLOAT) && field_ok(target, n, FF_FLOAT) && (!p_prev || field_ok(p_prev, n, FF_FLOAT)) &&
                 (!mask || field_ok(mask, n, FF_UINT8)),
             FF_E_ARG, "unet loss: fields must be cell fields of the resolution (mask uint8)");
    cudaStream_t s = u->ctx->stream;
    FF_TRY(forward(u, (const float *)b->d, mask ? (const uint8_t *)mask->d : nullptr,
                   p_prev ? (const float *)p_prev->d : nullptr, h, nullptr, true));
    const int nb = std::min(152 * 32, gblocks(n));
    k_loss_d<<<gblocks(n), 256, 0, s>>>(n, u->raw, (const float *)target->d, u->scales, u->draw);
    k_loss_lap<<<nb, 256, 0, s>>>(u->vol, u->draw, u->raw, u->partial);
    k_loss_grad<<<gblocks(n), 256, 0, s>>>(u->vol, u->raw, u->draw);
    FF_TRY(post("loss"));
    FF_CUDA(cudaMemsetAsync(u->g, 0, u->nparam * 4, s));
    FF_TRY(backward(u));
    std::vector<double> hp(nb);
    FF_CUDA(cudaMemcpyAsync(hp.data(), u->partial, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
    FF_CUDA(cudaStreamSynchronize(s));
    double tot = 0;
    for (double x : hp) tot += x;
    if (loss) *loss = tot;
    return tc_status(u);
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
