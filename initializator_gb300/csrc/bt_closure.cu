// Learned closure: kernels of the small 3-D CNN that corrects a 2x-coarse,
// 4x-time-step solve toward the fine solve (no counterpart in the reference).
//
// Net: 4 layers of 3x3x3 convolutions, 16 -> 16 channels (the input's 7
// feature channels padded to 16), GELU between layers, BF16 operands with
// FP32 accumulation.
//
// Convolution = implicit GEMM on the 5th-generation tensor cores (tcgen05):
//   * activations are channels-last BF16 in a zero-padded grid, flattened:
//     row q = voxel of [sample][z+1][y+1][x+1], 16 channels = 32 bytes a row,
//     with margin rows before and after so every shifted read stays inside;
//   * a CTA computes 128 consecutive rows (M = 128) x 16 output channels
//     (N = 16); for each of the 27 taps the A tile is the 128 rows shifted by
//     the tap's flat offset — one contiguous block, fetched by TMA straight
//     into the canonical no-swizzle K-major layout (two 2 KB blocks of 8x16-byte
//     core matrices, one per 8-channel half), K = 16 per MMA;
//   * the weights of all 27 taps (prepacked on the host in the same canonical
//     layout, 512 bytes a tap) arrive with one bulk copy;
//   * one thread issues the 27 tcgen05.mma (kind::f16, BF16 x BF16 -> FP32 in
//     TMEM, 128 lanes x 16 columns), commits to an mbarrier, and the four
//     warps read their 32 TMEM lanes back (tcgen05.ld 32x32b.x16) for the
//     epilogue: bias, GELU (or GELU' for the data gradient), store;
//   * rows that fall on the zero halo are written as zero, so the output is
//     again a valid padded input for the next layer.
// The data gradient is the same kernel with the taps reversed and the channel
// roles swapped (prepacked "dgrad" weights). The weight gradient is a CUDA-core
// reduction (weight_grad_kernel) with a fixed-order second stage.
// Every mbarrier wait is bounded; a CTA that gives up records status, waits
// (bounded) for its copies and MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/bt.h"

namespace {

constexpr int ROWS = 128;        // M: rows (voxels) per CTA
constexpr int CH = 16;           // channels in and out
constexpr int TAPS = 27;
constexpr int A_TAP_BYTES = ROWS * CH * 2;       // 4096
constexpr int B_TAP_BYTES = CH * CH * 2;         // 512
constexpr int OFF_A = 0;
constexpr int OFF_B = TAPS * A_TAP_BYTES;        // 110592
constexpr int OFF_BAR = OFF_B + TAPS * B_TAP_BYTES;  // 124416
constexpr int CONV_SMEM = OFF_BAR + 64 + 1024;   // + alignment slack
constexpr uint32_t WAIT_LIMIT = 1u << 22;

__device__ __forceinline__ uint32_t sa(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(sa(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t i = 0; i < WAIT_LIMIT; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            sa(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(sa(bar))
        : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     sa(dst)),
                 "l"(src), "r"(bytes), "r"(sa(bar))
                 : "memory");
}

// tcgen05 ------------------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sa(slot)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void umma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(sa(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
// 32 lanes x 16 columns of 32-bit words: thread i of the warp gets lane (base + i)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor, no swizzle, K-major canonical layout:
// core matrices of 8 rows x 16 bytes (128 contiguous bytes); lbo = bytes
// between core matrices along K, sbo = bytes between them along M/N.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for sm_100-family tensor cores
    // base offset 0, lbo mode 0, layout type 0 (no swizzle)
    return d;
}
// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 16, M = 128.
constexpr uint32_t IDESC_BF16_M128_N16 = (1u << 4)       // D format FP32
                                         | (1u << 7)     // A format BF16
                                         | (1u << 10)    // B format BF16
                                         | ((16u >> 3) << 17)   // N >> 3
                                         | ((128u >> 4) << 24); // M >> 4

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// one 128 x 16 x 16 MMA: D[m][n] = sum_k A[m][k] * B[n][k]; A, B row-major BF16
// in global memory, D FP32 [128][16]
__global__ void __launch_bounds__(128) umma_selftest_kernel(const __nv_bfloat16* A, const __nv_bfloat16* B, float* D,
                                                            int* status) {
    __shared__ __align__(1024) unsigned char sm[4096 + 512 + 64];
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + 4096 + 512);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + 4096 + 512 + 16);
    const int tid = threadIdx.x, warp = tid >> 5;
    // canonical K-major no-swizzle: chunk kc (8 K elements) of row r at kc*2048 + r*16
    {
        const uint4* src = reinterpret_cast<const uint4*>(A + tid * 16);
        *reinterpret_cast<uint4*>(sm + 0 * 2048 + tid * 16) = src[0];
        *reinterpret_cast<uint4*>(sm + 1 * 2048 + tid * 16) = src[1];
        if (tid < 16) {
            const uint4* sb = reinterpret_cast<const uint4*>(B + tid * 16);
            *reinterpret_cast<uint4*>(sm + 4096 + 0 * 256 + tid * 16) = sb[0];
            *reinterpret_cast<uint4*>(sm + 4096 + 1 * 256 + tid * 16) = sb[1];
        }
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(tslot, 32);
    // generic-proxy smem writes must be visible to the tensor core
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    if (tid == 0) {
        umma_f16(tmem, smem_desc(sa(sm), 2048, 128), smem_desc(sa(sm + 4096), 256, 128), IDESC_BF16_M128_N16, 0);
        umma_commit(bar);
    }
    const bool ok = mbar_wait(bar, 0);
    tc_fence_after();
    if (ok) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16), v);
        for (int n = 0; n < 16; ++n) D[tid * 16 + n] = v[n];
    } else if (tid == 0) {
        atomicOr(status, 8);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 32);
}

struct ConvParams {
    long long rows;          // padded voxels of the batch (valid rows start at the base row)
    long long base_row;      // margin rows before row 0 in the tensor map / allocations
    int xp, yp, zp;          // padded grid (x+2, y+2, z+2)
    int taps_off[TAPS];      // flat row offset of each tap
    const unsigned char* wpack;  // 27 x 512 bytes canonical BF16 weights
    const float* bias;       // 16 (forward) or null
    int mode;                // 0: out = GELU(acc + bias) bf16 padded, pre = acc + bias (fp32)
                             // 1: outf = acc + bias (fp32 rows)
                             // 2: out = acc * GELU'(pre) bf16 padded (data gradient through GELU)
                             // 3: outf = acc (fp32 rows; data gradient without GELU)
    __nv_bfloat16* out;      // padded bf16 rows (base_row margin applied inside)
    float* pre;              // fp32 [rows][16]: stored (mode 0) or read (mode 2)
    float* outf;             // fp32 [rows][16] (modes 1, 3)
    int* status;
};

__global__ void __launch_bounds__(128, 1) conv3d_kernel(const __grid_constant__ ConvParams P,
                                                        const __grid_constant__ CUtensorMap xmap) {
    extern __shared__ __align__(1024) unsigned char raw[];
    unsigned char* sm = raw + ((1024u - (sa(raw) & 1023u)) & 1023u);
    uint64_t* bar_full = reinterpret_cast<uint64_t*>(sm + OFF_BAR);
    uint64_t* bar_mma = reinterpret_cast<uint64_t*>(sm + OFF_BAR + 8);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + OFF_BAR + 16);
    int* s_ok = reinterpret_cast<int*>(sm + OFF_BAR + 24);
    const int tid = threadIdx.x, warp = tid >> 5;
    const long long q0 = (long long)blockIdx.x * ROWS;

    if (tid == 0) {
        mbar_init(bar_full, 1);
        mbar_init(bar_mma, 1);
        fence_mbar_init();
        *s_ok = 1;
    }
    if (warp == 0) tmem_alloc(tslot, 32);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (tid == 0) {
        mbar_expect_tx(bar_full, TAPS * A_TAP_BYTES + TAPS * B_TAP_BYTES);
        for (int t = 0; t < TAPS; ++t) {
            const int row = (int)(P.base_row + q0 + P.taps_off[t]);
            tma_load_2d(sm + OFF_A + t * A_TAP_BYTES, &xmap, bar_full, 0, row);
            tma_load_2d(sm + OFF_A + t * A_TAP_BYTES + 2048, &xmap, bar_full, 8, row);
        }
        bulk_load(sm + OFF_B, P.wpack, TAPS * B_TAP_BYTES, bar_full);
        if (!mbar_wait(bar_full, 0)) {
            *s_ok = 0;
        } else {
            tc_fence_after();
            for (int t = 0; t < TAPS; ++t)
                umma_f16(tmem, smem_desc(sa(sm + OFF_A + t * A_TAP_BYTES), 2048, 128),
                         smem_desc(sa(sm + OFF_B + t * B_TAP_BYTES), 256, 128), IDESC_BF16_M128_N16, t > 0);
            umma_commit(bar_mma);
            if (!mbar_wait(bar_mma, 0)) *s_ok = 0;
        }
    }
    __syncthreads();
    if (!*s_ok) {
        // a bounded wait gave up: record it, let the copies and MMAs in flight
        // land (bounded), free the TMEM and leave
        if (tid == 0) {
            atomicOr(P.status, 8);
            for (uint32_t i = 0; i < WAIT_LIMIT; ++i)
                if (mbar_try_wait(bar_full, 0)) break;
            for (uint32_t i = 0; i < WAIT_LIMIT; ++i)
                if (mbar_try_wait(bar_mma, 0)) break;
        }
        tc_fence_before();
        __syncthreads();
        if (warp == 0) tmem_dealloc(tmem, 32);
        return;
    }
    tc_fence_after();
    float v[16];
    tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16), v);
    const long long q = q0 + tid;
    if (q < P.rows) {
        // padded coordinates of row q
        const long long plane = (long long)P.xp * P.yp;
        const long long r = q % (plane * P.zp);
        const int z = (int)(r / plane), y = (int)((r / P.xp) % P.yp), x = (int)(r % P.xp);
        const bool interior = x >= 1 && x <= P.xp - 2 && y >= 1 && y <= P.yp - 2 && z >= 1 && z <= P.zp - 2;
        if (P.mode == 0 || P.mode == 2) {
            __align__(16) __nv_bfloat16 o[16];
            if (P.mode == 0) {
#pragma unroll
                for (int c = 0; c < 16; ++c) {
                    const float pre = v[c] + P.bias[c];
                    if (P.pre) P.pre[q * 16 + c] = interior ? pre : 0.f;
                    o[c] = __float2bfloat16(interior ? gelu(pre) : 0.f);
                }
            } else {
#pragma unroll
                for (int c = 0; c < 16; ++c)
                    o[c] = __float2bfloat16(interior ? v[c] * gelu_grad(P.pre[q * 16 + c]) : 0.f);
            }
            uint4* dst = reinterpret_cast<uint4*>(P.out + (P.base_row + q) * 16);
            dst[0] = reinterpret_cast<const uint4*>(o)[0];
            dst[1] = reinterpret_cast<const uint4*>(o)[1];
        } else {
#pragma unroll
            for (int c = 0; c < 16; ++c)
                P.outf[q * 16 + c] = interior ? v[c] + (P.mode == 1 ? P.bias[c] : 0.f) : 0.f;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 32);
}

// dW[t][ci][co] (+ db[co] as t = 27) partial sums over one chunk of rows:
// sum over interior rows q of x[q + off_t][ci] * dz[q][co]
constexpr int WG_ROWS = 1024;
__global__ void __launch_bounds__(256) weight_grad_kernel(const __nv_bfloat16* x, const __nv_bfloat16* dz,
                                                          long long rows, long long base_row,
                                                          const int* taps_off, float* partial) {
    const int t = blockIdx.y;  // 0..27 (27 = bias)
    const long long q0 = (long long)blockIdx.x * WG_ROWS;
    const int ci = threadIdx.x >> 4, co = threadIdx.x & 15;
    float acc = 0.f;
    const int off = t < TAPS ? taps_off[t] : 0;
    for (int i = 0; i < WG_ROWS; ++i) {
        const long long q = q0 + i;
        if (q >= rows) break;
        const float g = __bfloat162float(dz[(base_row + q) * 16 + co]);  // zero on the halo
        const float a = t < TAPS ? __bfloat162float(x[(base_row + q + off) * 16 + ci]) : (ci == 0 ? 1.f : 0.f);
        acc = fmaf(a, g, acc);
    }
    partial[((long long)blockIdx.x * (TAPS + 1) + t) * 256 + threadIdx.x] = acc;
}

// fixed-order sum of the chunk partials: grad[t][ci][co]
__global__ void weight_grad_reduce_kernel(const float* partial, int nchunks, float* grad) {
    const int t = blockIdx.x, k = threadIdx.x;
    float s = 0.f;
    for (int c = 0; c < nchunks; ++c) s += partial[((long long)c * (TAPS + 1) + t) * 256 + k];
    grad[t * 256 + k] = s;
}

// AdamW on FP32 master parameters
__global__ void adamw_kernel(float* p, const float* g, float* m, float* v, int n, float lr, float b1, float b2,
                             float eps, float wd, float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] = p[i] * (1.f - lr * wd) - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// canonical BF16 packing of w[t][ci][co] (FP32): forward B[n = co][k = ci];
// data-gradient B[n = ci][k = co] with the taps reversed
__global__ void pack_weights_kernel(const float* w, unsigned char* fwd, unsigned char* dgrad) {
    const int t = blockIdx.x, ci = threadIdx.x >> 4, co = threadIdx.x & 15;
    const float val = w[(t * 16 + ci) * 16 + co];
    __nv_bfloat16 b = __float2bfloat16(val);
    // forward: n = co, k = ci
    reinterpret_cast<__nv_bfloat16*>(fwd + t * 512 + (ci >> 3) * 256 + co * 16)[ci & 7] = b;
    // dgrad: tap 26 - t, n = ci, k = co
    reinterpret_cast<__nv_bfloat16*>(dgrad + (TAPS - 1 - t) * 512 + (co >> 3) * 256 + ci * 16)[co & 7] = b;
}

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

}  // namespace

extern "C" {

int bt_umma_selftest(const void* a_bf16, const void* b_bf16, float* d, int* status, void* stream) {
    if (!a_bf16 || !b_bf16 || !d || !status) return BT_E_ARG;
    umma_selftest_kernel<<<1, 128, 0, (cudaStream_t)stream>>>((const __nv_bfloat16*)a_bf16,
                                                              (const __nv_bfloat16*)b_bf16, d, status);
    return cudaGetLastError() == cudaSuccess ? BT_OK : BT_E_CUDA;
}

int bt_conv3d(const bt_conv3d_args* a, void* stream) {
    if (!a || !a->x || !a->wpack || a->nb <= 0 || a->nx <= 0 || a->ny <= 0 || a->nz <= 0) return BT_E_ARG;
    if (a->mode < 0 || a->mode > 3) return BT_E_ARG;
    if ((a->mode == 0 || a->mode == 2) && !a->out) return BT_E_ARG;
    if ((a->mode == 1 || a->mode == 3) && !a->outf) return BT_E_ARG;
    if ((a->mode == 0 || a->mode == 1) && !a->bias) return BT_E_ARG;
    if (a->mode == 2 && !a->pre) return BT_E_ARG;
    const int xp = a->nx + 2, yp = a->ny + 2, zp = a->nz + 2;
    ConvParams P{};
    P.xp = xp;
    P.yp = yp;
    P.zp = zp;
    P.rows = (long long)a->nb * xp * yp * zp;
    P.base_row = bt_conv3d_margin(a->nx, a->ny);
    int t = 0;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) P.taps_off[t++] = dz * xp * yp + dy * xp + dx;
    P.wpack = (const unsigned char*)a->wpack;
    P.bias = a->bias;
    P.mode = a->mode;
    P.out = (__nv_bfloat16*)a->out;
    P.pre = a->pre;
    P.outf = a->outf;
    P.status = a->status;
    // 2-D view of the whole allocation: 16 channels x (rows + 2 margins)
    auto fn = encoder();
    if (!fn) return BT_E_CUDA;
    CUtensorMap map;
    const cuuint64_t total_rows = (cuuint64_t)(P.rows + 2 * P.base_row);
    cuuint64_t dims[2] = {16, total_rows};
    cuuint64_t strides[1] = {32};
    cuuint32_t box[2] = {8, ROWS};
    cuuint32_t es[2] = {1, 1};
    if (fn(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(a->x), dims, strides, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return BT_E_CUDA;
    static bool configured = false;
    if (!configured) {
        if (cudaFuncSetAttribute(conv3d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, CONV_SMEM) != cudaSuccess)
            return BT_E_CUDA;
        configured = true;
    }
    const long long nblocks = (P.rows + ROWS - 1) / ROWS;
    conv3d_kernel<<<(unsigned)nblocks, 128, CONV_SMEM, (cudaStream_t)stream>>>(P, map);
    return cudaGetLastError() == cudaSuccess ? BT_OK : BT_E_CUDA;
}

long long bt_conv3d_margin(int nx, int ny) {
    // the largest tap offset plus one tile of rounding, rounded up to a tile
    const long long m = (long long)(nx + 2) * (ny + 2) + (nx + 2) + 1 + ROWS;
    return (m + ROWS - 1) / ROWS * ROWS;
}

int bt_conv3d_weight_grad(const void* x, const void* dz, int nb, int nx, int ny, int nz, float* partial,
                          float* grad, void* stream) {
    if (!x || !dz || !partial || !grad || nb <= 0) return BT_E_ARG;
    const int xp = nx + 2, yp = ny + 2, zp = nz + 2;
    const long long rows = (long long)nb * xp * yp * zp;
    int offs[TAPS];
    int t = 0;
    for (int dzz = -1; dzz <= 1; ++dzz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) offs[t++] = dzz * xp * yp + dy * xp + dx;
    // the offsets travel in the partial buffer's tail (caller sizes it with bt_conv3d_wgrad_scratch)
    const int nchunks = (int)((rows + WG_ROWS - 1) / WG_ROWS);
    int* d_offs = reinterpret_cast<int*>(partial + (size_t)nchunks * (TAPS + 1) * 256);
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemcpyAsync(d_offs, offs, sizeof(offs), cudaMemcpyHostToDevice, s) != cudaSuccess) return BT_E_CUDA;
    weight_grad_kernel<<<dim3(nchunks, TAPS + 1), 256, 0, s>>>((const __nv_bfloat16*)x, (const __nv_bfloat16*)dz,
                                                                rows, bt_conv3d_margin(nx, ny), d_offs, partial);
    weight_grad_reduce_kernel<<<TAPS + 1, 256, 0, s>>>(partial, nchunks, grad);
    return cudaGetLastError() == cudaSuccess ? BT_OK : BT_E_CUDA;
}

long long bt_conv3d_wgrad_scratch(int nb, int nx, int ny, int nz) {
    const long long rows = (long long)nb * (nx + 2) * (ny + 2) * (nz + 2);
    const long long nchunks = (rows + WG_ROWS - 1) / WG_ROWS;
    return nchunks * (TAPS + 1) * 256 + 64;  // floats, + room for the tap offsets
}

int bt_adamw(float* p, const float* g, float* m, float* v, int n, float lr, float beta1, float beta2, float eps,
             float weight_decay, int step, void* stream) {
    if (!p || !g || !m || !v || n <= 0 || step <= 0) return BT_E_ARG;
    const float bc1 = 1.f - std::pow(beta1, (float)step), bc2 = 1.f - std::pow(beta2, (float)step);
    adamw_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(p, g, m, v, n, lr, beta1, beta2, eps,
                                                                     weight_decay, bc1, bc2);
    return cudaGetLastError() == cudaSuccess ? BT_OK : BT_E_CUDA;
}

int bt_conv3d_pack_weights(const float* w, void* wpack_fwd, void* wpack_dgrad, void* stream) {
    if (!w || !wpack_fwd || !wpack_dgrad) return BT_E_ARG;
    pack_weights_kernel<<<TAPS, 256, 0, (cudaStream_t)stream>>>(w, (unsigned char*)wpack_fwd,
                                                               (unsigned char*)wpack_dgrad);
    return cudaGetLastError() == cudaSuccess ? BT_OK : BT_E_CUDA;
}

}  // extern "C"
