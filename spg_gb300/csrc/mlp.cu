// Per-vertex MLP of the learned warm start: 24 -> 128 -> 128 -> 128 -> 3 with GELU, BF16
// weights, FP32 accumulation.
//
// Inference (mlp_infer_tc_kernel) runs on the 5th-generation tensor cores: tcgen05.mma with
// BF16 operands in shared memory and the FP32 accumulator in tensor memory, one 128-row tile
// per CTA at a time; each layer's accumulator is read back with tcgen05.ld, biased, passed
// through GELU and rounded to BF16 as the next layer's operand.
//
// Training runs its eleven GEMMs on the tensor cores too (gemm_tc_kernel: BF16 operands, FP32
// accumulation) and GELU forward/backward, bias reductions and Adam as SIMT kernels, on FP32
// master weights whose BF16 rounding is used in the forward pass, so the trained network is
// the one the BF16 inference kernel evaluates (straight-through for the rounding).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <vector>

#include "api_internal.h"
#include "devbuf.h"
#include "mlp.h"

namespace spgx {

// ---------------------------------------------------------------------------------------
// Shared pieces

__device__ __forceinline__ float gelu(float x)
{
    // tanh approximation of GELU: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
    const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
    return 0.5f * x * (1.f + tanhf(u));
}

// The same GELU with the hardware's approximate tanh (PTX tanh.approx.f32, one instruction;
// its error, about 2^-11 relative, is below the BF16 rounding the inference kernel applies to
// every activation). The tcgen05 kernel's epilogue is bound by this function: with tanhf it
// took 136 us on 263k rows, with the hardware tanh 92 us.
__device__ __forceinline__ float gelu_fast(float x)
{
    const float u = 0.7978845608028654f * (x + 0.044715f * x * x * x);
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
    return 0.5f * x * (1.f + t);
}

__device__ __forceinline__ float gelu_grad(float x)
{
    const float x2 = x * x;
    const float u = 0.7978845608028654f * (x + 0.044715f * x2 * x);
    const float t = tanhf(u);
    const float du = 0.7978845608028654f * (1.f + 3.f * 0.044715f * x2);
    return 0.5f * (1.f + t) + 0.5f * x * (1.f - t * t) * du;
}

// ---------------------------------------------------------------------------------------
// Inference on the tensor cores

struct MlpDevWeights {
    const __nv_bfloat16 *w1t;  // [128][32]  (k padded 24 -> 32)
    const __nv_bfloat16 *w2t;  // [128][128]
    const __nv_bfloat16 *w3t;  // [128][128]
    const __nv_bfloat16 *w4t;  // [8][128]   (n padded 3 -> 8)
    const float *b1, *b2, *b3, *b4;  // 128, 128, 128, 8
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    uint32_t r;
    memcpy(&r, &v, sizeof(r));
    return r;
}

// ---------------------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores (tcgen05): a persistent kernel over tiles of
// 128 rows. Per tile and layer one thread issues the layer's tcgen05.mma instructions
// (M = 128 rows, N = 128 hidden units or 16 for the padded 3 outputs, K = 16 per
// instruction, BF16 operands from shared memory, FP32 accumulator in tensor memory) and
// commits them to an mbarrier; the four warps then read the accumulator rows back with
// tcgen05.ld (warp w owns tensor-memory lanes 32w..32w+31, one row per thread), add the bias,
// apply GELU (gelu_fast), round to BF16 and write the next layer's A operand into shared
// memory.
//
// Shared-memory operands use the K-major layout without swizzle: 8 x 8 BF16 core matrices
// of 128 contiguous bytes (8 rows of 16 bytes); core matrices adjacent along K are 128 bytes
// apart (the descriptor's leading byte offset) and adjacent 8-row groups K / 8 * 128 bytes
// apart (its stride byte offset).
namespace tc {

constexpr int kRows = 128;
constexpr int kThreads = 128;
constexpr int kW1 = 0;                       // W1^T: 128 x 32 (K padded 24 -> 32)
constexpr int kW2 = kW1 + 128 * 32 * 2;      // W2^T: 128 x 128
constexpr int kW3 = kW2 + 128 * 128 * 2;     // W3^T: 128 x 128
constexpr int kW4 = kW3 + 128 * 128 * 2;     // W4^T: 16 x 128 (N padded 3 -> 16)
constexpr int kA = kW4 + 16 * 128 * 2;       // activations: 128 x 128 (layer 1: 128 x 32)
constexpr int kBias = kA + 128 * 128 * 2;    // b1, b2, b3 (128 each), b4 (16)
constexpr int kBar = kBias + (3 * 128 + 16) * 4;
constexpr int kTmemSlot = kBar + 8;
constexpr size_t kSmem = size_t(kTmemSlot + 8) + 1024;  // + slack to align the base to 1 KB
constexpr int kTmemCols = 128;
constexpr int kMaxPolls = 1 << 22;

// Byte offset of element (r, k) of a K-major operand with K columns, in core matrices.
__device__ __forceinline__ int core_off(int r, int k, int K)
{
    return ((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// Shared-memory matrix descriptor: start address, leading byte offset (K direction), stride
// byte offset (8-row groups), descriptor version 1 (bits 46-47), no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return uint64_t((addr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and B (bits
// 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
                 : "memory");
}

// Bounded wait for the mbarrier phase `parity` to complete; false when the polls run out.
__device__ __forceinline__ bool wait_phase(uint32_t bar, uint32_t parity)
{
    for (int i = 0; i < kMaxPolls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (i > 64) __nanosleep(64);
    }
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// Shared-memory writes by the threads, made visible to the tensor cores' (async-proxy) reads.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 32 consecutive FP32 accumulator columns of this thread's row (tensor-memory lane).
__device__ __forceinline__ void ld32(uint32_t taddr, float *v)
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc

__global__ void __launch_bounds__(tc::kThreads) mlp_infer_tc_kernel(MlpDevWeights W, const float *__restrict__ X,
                                                                    int n, float *__restrict__ Y,
                                                                    unsigned int *status)
{
    extern __shared__ unsigned char smem_raw[];
    // The operand region starts on a 1 KB boundary.
    unsigned char *sm = smem_raw + ((1024 - (static_cast<uint32_t>(__cvta_generic_to_shared(smem_raw)) & 1023)) & 1023);
    const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(sm));
    float *s_b = reinterpret_cast<float *>(sm + tc::kBias);
    const uint32_t bar = sbase + tc::kBar;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(sm + tc::kTmemSlot);
    const int tid = threadIdx.x, warp = tid >> 5;

    // Weights into the core-matrix layout, 16 bytes (8 consecutive k of one row n) per copy.
    {
        const int K[4] = {32, 128, 128, 128}, Nr[4] = {128, 128, 128, 16}, off[4] = {tc::kW1, tc::kW2, tc::kW3, tc::kW4};
        const __nv_bfloat16 *src[4] = {W.w1t, W.w2t, W.w3t, W.w4t};
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const int chunks = Nr[m] * K[m] / 8;
            for (int i = tid; i < chunks; i += blockDim.x) {
                const int nn = i / (K[m] / 8), k = (i % (K[m] / 8)) * 8;
                uint4 v = make_uint4(0u, 0u, 0u, 0u);
                if (m < 3 || nn < 8) v = __ldg(reinterpret_cast<const uint4 *>(src[m] + nn * K[m] + k));
                *reinterpret_cast<uint4 *>(sm + off[m] + tc::core_off(nn, k, K[m])) = v;
            }
        }
        for (int i = tid; i < 128; i += blockDim.x) {
            s_b[i] = W.b1[i];
            s_b[128 + i] = W.b2[i];
            s_b[256 + i] = W.b3[i];
        }
        if (tid < 16) s_b[384 + tid] = tid < 8 ? W.b4[tid] : 0.f;
    }
    if (warp == 0) {
        const uint32_t slot = static_cast<uint32_t>(__cvta_generic_to_shared(tmem_slot));
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot),
                     "r"(tc::kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t lane_base = uint32_t(warp * 32) << 16;  // this warp's tensor-memory lanes
    uint32_t phase = 0;
    bool ok = true;
    const int tiles = (n + tc::kRows - 1) / tc::kRows;
    for (int t = blockIdx.x; t < tiles && ok; t += gridDim.x) {
        const int row = t * tc::kRows + tid;
        // Layer-1 operand: the 24 features of this thread's row as BF16, K padded to 32.
        {
            float f[32];
#pragma unroll
            for (int k = 0; k < 32; ++k) f[k] = 0.f;
            if (row < n) {
                const float4 *xr = reinterpret_cast<const float4 *>(X + size_t(row) * 24);
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    const float4 v = __ldg(xr + q);
                    f[4 * q] = v.x, f[4 * q + 1] = v.y, f[4 * q + 2] = v.z, f[4 * q + 3] = v.w;
                }
            }
#pragma unroll
            for (int k = 0; k < 32; k += 8) {
                const uint4 v = make_uint4(pack_bf16(f[k], f[k + 1]), pack_bf16(f[k + 2], f[k + 3]),
                                           pack_bf16(f[k + 4], f[k + 5]), pack_bf16(f[k + 6], f[k + 7]));
                *reinterpret_cast<uint4 *>(sm + tc::kA + tc::core_off(tid, k, 32)) = v;
            }
        }
        for (int layer = 0; layer < 4; ++layer) {
            const int K = layer == 0 ? 32 : 128, N = layer == 3 ? 16 : 128;
            const int woff = layer == 0 ? tc::kW1 : layer == 1 ? tc::kW2 : layer == 2 ? tc::kW3 : tc::kW4;
            tc::fence_async_smem();
            tc::fence_before();
            __syncthreads();  // the operand is written and every read of the accumulator is done
            tc::fence_after();
            if (tid == 0) {
                const uint32_t idesc = tc::idesc_bf16(128, N);
                for (int ks = 0; ks < K / 16; ++ks) {
                    const uint64_t a = tc::smem_desc(sbase + tc::kA + ks * 256, 128, (K / 8) * 128);
                    const uint64_t b = tc::smem_desc(sbase + woff + ks * 256, 128, (K / 8) * 128);
                    tc::mma(tmem, a, b, idesc, ks > 0 ? 1u : 0u);
                }
                tc::commit(bar);
            }
            ok = __syncthreads_and(tc::wait_phase(bar, phase));  // the same verdict in every thread
            phase ^= 1u;
            tc::fence_after();
            if (!ok) break;
            if (layer < 3) {
                const float *bias = s_b + layer * 128;
#pragma unroll 1
                for (int c0 = 0; c0 < 128; c0 += 32) {
                    float v[32];
                    tc::ld32(tmem + lane_base + uint32_t(c0), v);
#pragma unroll
                    for (int k = 0; k < 32; k += 8) {
                        float g[8];
#pragma unroll
                        for (int q = 0; q < 8; ++q) g[q] = gelu_fast(v[k + q] + bias[c0 + k + q]);
                        const uint4 o = make_uint4(pack_bf16(g[0], g[1]), pack_bf16(g[2], g[3]),
                                                   pack_bf16(g[4], g[5]), pack_bf16(g[6], g[7]));
                        *reinterpret_cast<uint4 *>(sm + tc::kA + tc::core_off(tid, c0 + k, 128)) = o;
                    }
                }
            } else {
                float v[16];
                tc::ld16(tmem + lane_base, v);
                if (row < n) {
                    Y[size_t(row) * 3 + 0] = v[0] + s_b[384 + 0];
                    Y[size_t(row) * 3 + 1] = v[1] + s_b[384 + 1];
                    Y[size_t(row) * 3 + 2] = v[2] + s_b[384 + 2];
                }
            }
        }
    }
    if (!ok) {
        // A commit that never arrived: record it, and give the tensor cores a bounded while to
        // finish before the tensor memory is released.
        if (tid == 0) atomicOr(status, 1u);
        tc::wait_phase(bar, phase ^ 1u);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(tc::kTmemCols)
                     : "memory");
}

// BF16 transposed copies of the FP32 master weights for the inference kernel (row n of W^T
// holds the K inputs of output n; W4 is padded to 8 rows and W1 to K = 32).
__global__ void mlp_pack_kernel(const float *__restrict__ w, __nv_bfloat16 *w1t, __nv_bfloat16 *w2t,
                                __nv_bfloat16 *w3t, __nv_bfloat16 *w4t, float *b4pad)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const float *W1 = w + kMlpOffW1, *W2 = w + kMlpOffW2, *W3 = w + kMlpOffW3, *W4 = w + kMlpOffW4;
    if (i < 128 * 32) {
        const int nn = i / 32, k = i % 32;
        w1t[i] = __float2bfloat16_rn(k < 24 ? W1[k * 128 + nn] : 0.f);
    }
    if (i < 128 * 128) {
        const int nn = i / 128, k = i % 128;
        w2t[i] = __float2bfloat16_rn(W2[k * 128 + nn]);
        w3t[i] = __float2bfloat16_rn(W3[k * 128 + nn]);
    }
    if (i < 8 * 128) {
        const int nn = i / 128, k = i % 128;
        w4t[i] = __float2bfloat16_rn(nn < 3 ? W4[k * 3 + nn] : 0.f);
    }
    if (i < 8) b4pad[i] = i < 3 ? w[kMlpOffB4 + i] : 0.f;
}

// ---------------------------------------------------------------------------------------
// Training (FP32 SIMT)

// C[M x N] = op(A) * op(B) + beta * C on the tensor cores, row-major FP32 arrays, op =
// transpose when the flag is set. One CTA computes a 128 x NT tile (NT = 128, or 16 when
// N <= 16) over K in chunks of 64: the threads stage op(A) (128 x 64) and op(B)^T (NT x 64)
// as BF16 in the K-major core-matrix layout of the inference kernel (coalesced along
// whichever dimension is contiguous in memory; zeros outside the matrices), one thread issues
// the chunk's four tcgen05.mma (K = 16 each) into the FP32 accumulator in tensor memory and
// commits them to an mbarrier, and after the last chunk each warp reads its 32 rows back with
// tcgen05.ld. BF16 operands with FP32 accumulation, as the network's inference evaluates it.
// Long K (the weight gradients, summed over the batch) is split over gridDim.z CTAs whose
// partial tiles are added into C with atomics.
namespace tcg {

constexpr int kKC = 64;                          // K per chunk
constexpr int kA = 0;                            // 128 x 64 BF16
constexpr int kB = kA + 128 * kKC * 2;           // up to 128 x 64 BF16
constexpr int kBar = kB + 128 * kKC * 2;
constexpr int kSlot = kBar + 8;
// Padded so that at most four CTAs share an SM: four 128-column accumulators fill its tensor
// memory, so an allocation never waits on a CTA that is not resident.
constexpr size_t kSmem = 56 * 1024;

}  // namespace tcg

__global__ void __launch_bounds__(128) gemm_tc_kernel(int M, int N, int K, const float *__restrict__ A, int lda,
                                                      bool tA, const float *__restrict__ B, int ldb, bool tB,
                                                      float *C, int ldc, float beta, int NT, unsigned int *status)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char *sm = smem_raw + ((1024 - (static_cast<uint32_t>(__cvta_generic_to_shared(smem_raw)) & 1023)) & 1023);
    const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(sm));
    const uint32_t bar = sbase + tcg::kBar;
    uint32_t *slot = reinterpret_cast<uint32_t *>(sm + tcg::kSlot);
    __nv_bfloat16 *sA = reinterpret_cast<__nv_bfloat16 *>(sm + tcg::kA);
    __nv_bfloat16 *sB = reinterpret_cast<__nv_bfloat16 *>(sm + tcg::kB);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.y * 128, n0 = blockIdx.x * NT;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                         static_cast<uint32_t>(__cvta_generic_to_shared(slot))),
                     "r"(128)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *slot;
    // op(A)(m, k) and op(B)(k, n); the staging order follows the contiguous dimension.
    auto a_at = [&](int m, int k) -> float {
        return (m < M && k < K) ? (tA ? A[size_t(k) * lda + m] : A[size_t(m) * lda + k]) : 0.f;
    };
    auto b_at = [&](int k, int n) -> float {
        return (n < N && k < K) ? (tB ? B[size_t(n) * ldb + k] : B[size_t(k) * ldb + n]) : 0.f;
    };
    uint32_t phase = 0;
    bool ok = true;
    // Split K (gridDim.z > 1, beta = 0, C zeroed by the caller): this CTA sums its share of the
    // chunks and adds its partial tile into C.
    const int all_chunks = (K + tcg::kKC - 1) / tcg::kKC;
    const int per = (all_chunks + gridDim.z - 1) / gridDim.z;
    const int c_begin = blockIdx.z * per, c_end = min(all_chunks, c_begin + per);
    for (int c = c_begin; c < c_end && ok; ++c) {
        const int k0 = c * tcg::kKC;
#pragma unroll 16
        for (int e = tid; e < 128 * tcg::kKC; e += blockDim.x) {
            const int m = tA ? e % 128 : e / tcg::kKC, k = tA ? e / 128 : e % tcg::kKC;
            sA[tc::core_off(m, k, tcg::kKC) / 2] = __float2bfloat16_rn(a_at(m0 + m, k0 + k));
        }
#pragma unroll 16
        for (int e = tid; e < NT * tcg::kKC; e += blockDim.x) {
            const int n = tB ? e / tcg::kKC : e % NT, k = tB ? e % tcg::kKC : e / NT;
            sB[tc::core_off(n, k, tcg::kKC) / 2] = __float2bfloat16_rn(b_at(k0 + k, n0 + n));
        }
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        if (tid == 0) {
            const uint32_t idesc = tc::idesc_bf16(128, NT);
            for (int ks = 0; ks < tcg::kKC / 16; ++ks) {
                const uint64_t a = tc::smem_desc(sbase + tcg::kA + ks * 256, 128, (tcg::kKC / 8) * 128);
                const uint64_t bdesc = tc::smem_desc(sbase + tcg::kB + ks * 256, 128, (tcg::kKC / 8) * 128);
                tc::mma(tmem, a, bdesc, idesc, (c > c_begin || ks > 0) ? 1u : 0u);
            }
            tc::commit(bar);
        }
        // The chunk's operands are read before the next chunk overwrites them.
        ok = __syncthreads_and(tc::wait_phase(bar, phase));
        phase ^= 1u;
        tc::fence_after();
    }
    if (ok && c_end > c_begin) {
        const int m = m0 + tid;
        const uint32_t lane_base = uint32_t(warp * 32) << 16;
        for (int c0 = 0; c0 < NT; c0 += 16) {
            float v[16];
            tc::ld16(tmem + lane_base + uint32_t(c0), v);
            if (m < M)
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int n = n0 + c0 + j;
                    if (n < N) {
                        float *cp = C + size_t(m) * ldc + n;
                        if (gridDim.z > 1)
                            atomicAdd(cp, v[j]);
                        else
                            *cp = v[j] + (beta == 0.f ? 0.f : beta * *cp);
                    }
                }
        }
    } else {
        if (tid == 0) atomicOr(status, 1u);
        tc::wait_phase(bar, phase ^ 1u);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(128) : "memory");
}

// Z += bias (per column); A = gelu(Z) when act.
__global__ void bias_act_kernel(float *Z, float *A, const float *bias, int M, int N, bool act)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= size_t(M) * N) return;
    const float z = Z[i] + bias[i % N];
    Z[i] = z;
    if (act) A[i] = gelu(z);
}

// dZ = dA * gelu'(Z)
__global__ void gelu_back_kernel(float *dA, const float *Z, size_t count)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < count) dA[i] *= gelu_grad(Z[i]);
}

// dY = 2 (Y - T) / (M * 3) and the per-block partial sums of (Y - T)^2.
__global__ void mse_grad_kernel(const float *Y, const float *T, float *dY, int M, double *loss)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    double e2 = 0.0;
    if (i < size_t(M) * 3) {
        const float e = Y[i] - T[i];
        dY[i] = 2.f * e / float(M * 3);
        e2 = double(e) * e;
    }
    for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, e2);
}

// db[n] = sum over rows of dZ[:, n]
__global__ void col_sum_kernel(const float *dZ, float *db, int M, int N)
{
    const int nn = blockIdx.x;
    float s = 0.f;
    for (int m = threadIdx.x; m < M; m += blockDim.x) s += dZ[size_t(m) * N + nn];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ float part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int k = 0; k < (blockDim.x + 31) / 32; ++k) t += part[k];
        db[nn] = t;
    }
}

// BF16 rounding of the master weights used by the training forward pass (biases stay FP32).
__global__ void quantize_kernel(const float *w, float *wq, int count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const bool is_bias = (i >= kMlpOffB1 && i < kMlpOffW2) || (i >= kMlpOffB2 && i < kMlpOffW3) ||
                         (i >= kMlpOffB3 && i < kMlpOffW4) || i >= kMlpOffB4;
    wq[i] = is_bias ? w[i] : __bfloat162float(__float2bfloat16_rn(w[i]));
}

__global__ void adam_kernel(float *w, const float *g, float *m, float *v, int count, float lr, float b1, float b2,
                            float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// Gathers rows idx[0..M) of X (n x cols) into Xb.
__global__ void gather_rows_kernel(const float *X, const int *idx, float *Xb, int M, int cols)
{
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= size_t(M) * cols) return;
    Xb[i] = X[size_t(idx[i / cols]) * cols + i % cols];
}

static int blocks_for(size_t n, int t = 256) { return static_cast<int>((n + t - 1) / t); }

static void gemm(cudaStream_t st, int M, int N, int K, const float *A, int lda, bool tA, const float *B, int ldb,
                 bool tB, float *C, int ldc, float beta, unsigned int *status)
{
    const int NT = N <= 16 ? 16 : 128;
    // The weight gradients sum over the whole batch (K = rows): their K is split over CTAs.
    int splits = 1;
    if (beta == 0.f && ldc == N && K > 1024) splits = std::min(64, (K + 127) / 128);
    if (splits > 1) cudaMemsetAsync(C, 0, size_t(M) * N * sizeof(float), st);
    dim3 grid((N + NT - 1) / NT, (M + 127) / 128, splits);
    gemm_tc_kernel<<<grid, 128, tcg::kSmem, st>>>(M, N, K, A, lda, tA, B, ldb, tB, C, ldc, beta, NT, status);
}

spgx_status Mlp::init(uint64_t seed, int dev)
{
    device = dev;
    SPGX_TRY_STATUS(select_device(dev));
    SPGX_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    SPGX_TRY_STATUS(d_w.alloc(kMlpParams * sizeof(float)));
    SPGX_TRY_STATUS(d_wq.alloc(kMlpParams * sizeof(float)));
    SPGX_TRY_STATUS(d_g.alloc(kMlpParams * sizeof(float)));
    SPGX_TRY_STATUS(d_m.alloc(kMlpParams * sizeof(float)));
    SPGX_TRY_STATUS(d_v.alloc(kMlpParams * sizeof(float)));
    SPGX_TRY_STATUS(d_w1t.alloc(128 * 32 * 2));
    SPGX_TRY_STATUS(d_w2t.alloc(128 * 128 * 2));
    SPGX_TRY_STATUS(d_w3t.alloc(128 * 128 * 2));
    SPGX_TRY_STATUS(d_w4t.alloc(8 * 128 * 2));
    SPGX_TRY_STATUS(d_b4.alloc(8 * sizeof(float)));
    SPGX_TRY_STATUS(d_loss.alloc(sizeof(double)));
    SPGX_CUDA(cudaFuncSetAttribute(mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(tc::kSmem)));
    SPGX_CUDA(cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(tcg::kSmem)));
    SPGX_TRY_STATUS(d_status.alloc(sizeof(unsigned int)));
    SPGX_CUDA(cudaMemset(d_status.as<void>(), 0, sizeof(unsigned int)));
    SPGX_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
    // Xavier-uniform initialisation, zero biases.
    std::vector<float> w(kMlpParams, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int fan_in, int fan_out) {
        const float a = std::sqrt(6.f / float(fan_in + fan_out));
        std::uniform_real_distribution<float> U(-a, a);
        for (int i = 0; i < fan_in * fan_out; ++i) w[off + i] = U(rng);
    };
    fill(kMlpOffW1, kMlpIn, kMlpHidden);
    fill(kMlpOffW2, kMlpHidden, kMlpHidden);
    fill(kMlpOffW3, kMlpHidden, kMlpHidden);
    fill(kMlpOffW4, kMlpHidden, kMlpOut);
    return set_weights(w.data());
}

spgx_status Mlp::set_weights(const float *w)
{
    SPGX_CUDA(cudaMemcpyAsync(d_w.as<float>(), w, kMlpParams * sizeof(float), cudaMemcpyHostToDevice, stream));
    SPGX_CUDA(cudaMemsetAsync(d_m.as<float>(), 0, kMlpParams * sizeof(float), stream));
    SPGX_CUDA(cudaMemsetAsync(d_v.as<float>(), 0, kMlpParams * sizeof(float), stream));
    adam_t = 0;
    SPGX_TRY_STATUS(refresh());
    SPGX_CUDA(cudaStreamSynchronize(stream));
    return SPGX_OK;
}

spgx_status Mlp::refresh()
{
    mlp_pack_kernel<<<blocks_for(128 * 128), 256, 0, stream>>>(d_w.as<float>(), d_w1t.as<__nv_bfloat16>(),
                                                               d_w2t.as<__nv_bfloat16>(), d_w3t.as<__nv_bfloat16>(),
                                                               d_w4t.as<__nv_bfloat16>(), d_b4.as<float>());
    quantize_kernel<<<blocks_for(kMlpParams), 256, 0, stream>>>(d_w.as<float>(), d_wq.as<float>(), kMlpParams);
    SPGX_CUDA(cudaGetLastError());
    return SPGX_OK;
}

spgx_status Mlp::get_weights(float *w)
{
    SPGX_CUDA(cudaMemcpyAsync(w, d_w.as<float>(), kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, stream));
    SPGX_CUDA(cudaStreamSynchronize(stream));
    return SPGX_OK;
}

void Mlp::infer(const float *X, int n, float *Y, cudaStream_t st) const
{
    if (n <= 0) return;
    MlpDevWeights W{d_w1t.as<__nv_bfloat16>(), d_w2t.as<__nv_bfloat16>(), d_w3t.as<__nv_bfloat16>(),
                    d_w4t.as<__nv_bfloat16>(), d_w.as<float>() + kMlpOffB1, d_w.as<float>() + kMlpOffB2,
                    d_w.as<float>() + kMlpOffB3, d_b4.as<float>()};
    const int tiles = (n + tc::kRows - 1) / tc::kRows;
    const int grid = std::min(tiles, 2 * std::max(1, num_sms));  // two 110 KB CTAs per SM
    mlp_infer_tc_kernel<<<grid, tc::kThreads, tc::kSmem, st>>>(W, X, n, Y, d_status.as<unsigned int>());
}

spgx_status Mlp::take_status()
{
    unsigned int hs = 0;
    SPGX_CUDA(cudaMemcpy(&hs, d_status.as<void>(), sizeof(hs), cudaMemcpyDeviceToHost));
    if (hs & 1u) {
        SPGX_CUDA(cudaMemset(d_status.as<void>(), 0, sizeof(unsigned int)));
        set_error("MLP inference gave up waiting for the tensor cores (bounded wait)");
        return SPGX_ERR_TIMEOUT;
    }
    return SPGX_OK;
}

spgx_status Mlp::ensure_batch(int M)
{
    if (M <= batch_cap) return SPGX_OK;
    batch_cap = M;
    const size_t h = size_t(M) * kMlpHidden;
    for (DevBuf *b : {&z1, &a1, &z2, &a2, &z3, &a3}) SPGX_TRY_STATUS(b->alloc(h * sizeof(float)));
    SPGX_TRY_STATUS(yb.alloc(size_t(M) * 3 * sizeof(float)));
    SPGX_TRY_STATUS(dy.alloc(size_t(M) * 3 * sizeof(float)));
    SPGX_TRY_STATUS(da.alloc(h * sizeof(float)));
    SPGX_TRY_STATUS(db_.alloc(h * sizeof(float)));
    SPGX_TRY_STATUS(xb.alloc(size_t(M) * kMlpIn * sizeof(float)));
    SPGX_TRY_STATUS(tb.alloc(size_t(M) * 3 * sizeof(float)));
    SPGX_TRY_STATUS(ib.alloc(size_t(M) * sizeof(int)));
    return SPGX_OK;
}

// Loss and gradient over M device-resident rows X (M x 24), T (M x 3). Gradient -> d_g.
spgx_status Mlp::loss_grad_device(const float *X, const float *T, int M, double *loss_out)
{
    SPGX_TRY_STATUS(ensure_batch(M));
    const float *wq = d_wq.as<float>();
    float *g = d_g.as<float>();
    const int H = kMlpHidden;
    // forward
    gemm(stream, M, H, kMlpIn, X, kMlpIn, false, wq + kMlpOffW1, H, false, z1.as<float>(), H, 0.f, d_status.as<unsigned int>());
    bias_act_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(z1.as<float>(), a1.as<float>(), wq + kMlpOffB1, M, H, true);
    gemm(stream, M, H, H, a1.as<float>(), H, false, wq + kMlpOffW2, H, false, z2.as<float>(), H, 0.f, d_status.as<unsigned int>());
    bias_act_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(z2.as<float>(), a2.as<float>(), wq + kMlpOffB2, M, H, true);
    gemm(stream, M, H, H, a2.as<float>(), H, false, wq + kMlpOffW3, H, false, z3.as<float>(), H, 0.f, d_status.as<unsigned int>());
    bias_act_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(z3.as<float>(), a3.as<float>(), wq + kMlpOffB3, M, H, true);
    gemm(stream, M, 3, H, a3.as<float>(), H, false, wq + kMlpOffW4, 3, false, yb.as<float>(), 3, 0.f, d_status.as<unsigned int>());
    bias_act_kernel<<<blocks_for(size_t(M) * 3), 256, 0, stream>>>(yb.as<float>(), nullptr, wq + kMlpOffB4, M, 3, false);
    // loss
    SPGX_CUDA(cudaMemsetAsync(d_loss.as<double>(), 0, sizeof(double), stream));
    mse_grad_kernel<<<blocks_for(size_t(M) * 3), 256, 0, stream>>>(yb.as<float>(), T, dy.as<float>(), M,
                                                                    d_loss.as<double>());
    // backward
    gemm(stream, H, 3, M, a3.as<float>(), H, true, dy.as<float>(), 3, false, g + kMlpOffW4, 3, 0.f, d_status.as<unsigned int>());
    col_sum_kernel<<<3, 256, 0, stream>>>(dy.as<float>(), g + kMlpOffB4, M, 3);
    gemm(stream, M, H, 3, dy.as<float>(), 3, false, wq + kMlpOffW4, 3, true, da.as<float>(), H, 0.f, d_status.as<unsigned int>());
    gelu_back_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(da.as<float>(), z3.as<float>(), size_t(M) * H);
    gemm(stream, H, H, M, a2.as<float>(), H, true, da.as<float>(), H, false, g + kMlpOffW3, H, 0.f, d_status.as<unsigned int>());
    col_sum_kernel<<<H, 256, 0, stream>>>(da.as<float>(), g + kMlpOffB3, M, H);
    gemm(stream, M, H, H, da.as<float>(), H, false, wq + kMlpOffW3, H, true, db_.as<float>(), H, 0.f, d_status.as<unsigned int>());
    gelu_back_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(db_.as<float>(), z2.as<float>(), size_t(M) * H);
    gemm(stream, H, H, M, a1.as<float>(), H, true, db_.as<float>(), H, false, g + kMlpOffW2, H, 0.f, d_status.as<unsigned int>());
    col_sum_kernel<<<H, 256, 0, stream>>>(db_.as<float>(), g + kMlpOffB2, M, H);
    gemm(stream, M, H, H, db_.as<float>(), H, false, wq + kMlpOffW2, H, true, da.as<float>(), H, 0.f, d_status.as<unsigned int>());
    gelu_back_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(da.as<float>(), z1.as<float>(), size_t(M) * H);
    gemm(stream, kMlpIn, H, M, X, kMlpIn, true, da.as<float>(), H, false, g + kMlpOffW1, H, 0.f, d_status.as<unsigned int>());
    col_sum_kernel<<<H, 256, 0, stream>>>(da.as<float>(), g + kMlpOffB1, M, H);
    SPGX_CUDA(cudaGetLastError());
    if (loss_out) {
        double l = 0;
        SPGX_CUDA(cudaMemcpyAsync(&l, d_loss.as<double>(), sizeof(double), cudaMemcpyDeviceToHost, stream));
        SPGX_CUDA(cudaStreamSynchronize(stream));
        *loss_out = l / (double(M) * 3.0);
    }
    return SPGX_OK;
}

spgx_status Mlp::train(const float *X, const float *T, int n, int steps, int batch, float lr, uint64_t seed,
                       float *final_loss)
{
    DevBuf dX, dT;
    SPGX_TRY_STATUS(dX.alloc(size_t(n) * kMlpIn * sizeof(float)));
    SPGX_TRY_STATUS(dT.alloc(size_t(n) * 3 * sizeof(float)));
    SPGX_CUDA(cudaMemcpyAsync(dX.as<float>(), X, size_t(n) * kMlpIn * sizeof(float), cudaMemcpyHostToDevice, stream));
    SPGX_CUDA(cudaMemcpyAsync(dT.as<float>(), T, size_t(n) * 3 * sizeof(float), cudaMemcpyHostToDevice, stream));
    const int M = std::min(batch, n);
    SPGX_TRY_STATUS(ensure_batch(M));
    std::mt19937_64 rng(seed);
    std::uniform_int_distribution<int> U(0, n - 1);
    std::vector<int> idx(M);
    double loss = 0;
    for (int s = 0; s < steps; ++s) {
        for (int i = 0; i < M; ++i) idx[i] = U(rng);
        SPGX_CUDA(cudaMemcpyAsync(ib.as<int>(), idx.data(), M * sizeof(int), cudaMemcpyHostToDevice, stream));
        gather_rows_kernel<<<blocks_for(size_t(M) * kMlpIn), 256, 0, stream>>>(dX.as<float>(), ib.as<int>(),
                                                                              xb.as<float>(), M, kMlpIn);
        gather_rows_kernel<<<blocks_for(size_t(M) * 3), 256, 0, stream>>>(dT.as<float>(), ib.as<int>(), tb.as<float>(),
                                                                          M, 3);
        SPGX_TRY_STATUS(loss_grad_device(xb.as<float>(), tb.as<float>(), M, s + 1 == steps ? &loss : nullptr));
        ++adam_t;
        const float c1 = 1.f - std::pow(0.9f, float(adam_t)), c2 = 1.f - std::pow(0.999f, float(adam_t));
        adam_kernel<<<blocks_for(kMlpParams), 256, 0, stream>>>(d_w.as<float>(), d_g.as<float>(), d_m.as<float>(),
                                                                d_v.as<float>(), kMlpParams, lr, 0.9f, 0.999f, 1e-8f,
                                                                c1, c2);
        SPGX_TRY_STATUS(refresh());
    }
    SPGX_CUDA(cudaStreamSynchronize(stream));
    if (final_loss) *final_loss = static_cast<float>(loss);
    return SPGX_OK;
}

Mlp::~Mlp()
{
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
}

}  // namespace spgx

// =======================================================================================
// C ABI

extern "C" {

int32_t spgx_mlp_num_params(void) { return spgx::kMlpParams; }

spgx_status spgx_mlp_create(uint64_t seed, int32_t device, spgx_mlp **out)
{
    SPGX_GUARD_BEGIN
    if (!out) {
        spgx::set_error("out is NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    *out = nullptr;
    auto h = std::make_unique<spgx_mlp>();
    h->m = std::make_unique<spgx::Mlp>();
    SPGX_TRY_STATUS(h->m->init(seed, device));
    *out = h.release();
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_mlp_destroy(spgx_mlp *h)
{
    SPGX_GUARD_BEGIN
    if (h) {
        cudaSetDevice(h->m->device);
        delete h;
    }
    return SPGX_OK;
    SPGX_GUARD_END
}

#define SPGX_MHANDLE(h)                                \
    if (!(h)) {                                        \
        spgx::set_error("NULL MLP handle");            \
        return SPGX_ERR_INVALID_ARG;                   \
    }                                                  \
    SPGX_CUDA(cudaSetDevice((h)->m->device))

spgx_status spgx_mlp_get_weights(spgx_mlp *h, float *w)
{
    SPGX_GUARD_BEGIN
    SPGX_MHANDLE(h);
    if (!w) {
        spgx::set_error("weights pointer is NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    return h->m->get_weights(w);
    SPGX_GUARD_END
}

spgx_status spgx_mlp_set_weights(spgx_mlp *h, const float *w)
{
    SPGX_GUARD_BEGIN
    SPGX_MHANDLE(h);
    if (!w) {
        spgx::set_error("weights pointer is NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    return h->m->set_weights(w);
    SPGX_GUARD_END
}

spgx_status spgx_mlp_forward(spgx_mlp *h, int32_t n, const float *x, float *y)
{
    SPGX_GUARD_BEGIN
    SPGX_MHANDLE(h);
    if (n < 0 || (n > 0 && (!x || !y))) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    if (n == 0) return SPGX_OK;
    spgx::DevBuf dx, dy;
    SPGX_TRY_STATUS(dx.alloc(size_t(n) * spgx::kMlpIn * sizeof(float)));
    SPGX_TRY_STATUS(dy.alloc(size_t(n) * 3 * sizeof(float)));
    SPGX_CUDA(cudaMemcpyAsync(dx.as<float>(), x, size_t(n) * spgx::kMlpIn * sizeof(float), cudaMemcpyHostToDevice,
                              h->m->stream));
    h->m->infer(dx.as<float>(), n, dy.as<float>(), h->m->stream);
    SPGX_CUDA(cudaGetLastError());
    SPGX_CUDA(cudaMemcpyAsync(y, dy.as<float>(), size_t(n) * 3 * sizeof(float), cudaMemcpyDeviceToHost, h->m->stream));
    SPGX_CUDA(cudaStreamSynchronize(h->m->stream));
    return h->m->take_status();
    SPGX_GUARD_END
}

spgx_status spgx_mlp_loss_grad(spgx_mlp *h, int32_t n, const float *x, const float *y, float *loss, float *grad)
{
    SPGX_GUARD_BEGIN
    SPGX_MHANDLE(h);
    if (n <= 0 || !x || !y || !loss || !grad) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    spgx::DevBuf dx, dt;
    SPGX_TRY_STATUS(dx.alloc(size_t(n) * spgx::kMlpIn * sizeof(float)));
    SPGX_TRY_STATUS(dt.alloc(size_t(n) * 3 * sizeof(float)));
    SPGX_CUDA(cudaMemcpyAsync(dx.as<float>(), x, size_t(n) * spgx::kMlpIn * sizeof(float), cudaMemcpyHostToDevice,
                              h->m->stream));
    SPGX_CUDA(cudaMemcpyAsync(dt.as<float>(), y, size_t(n) * 3 * sizeof(float), cudaMemcpyHostToDevice, h->m->stream));
    double l = 0;
    SPGX_TRY_STATUS(h->m->loss_grad_device(dx.as<float>(), dt.as<float>(), n, &l));
    SPGX_CUDA(cudaMemcpyAsync(grad, h->m->d_g.as<float>(), spgx::kMlpParams * sizeof(float), cudaMemcpyDeviceToHost,
                              h->m->stream));
    SPGX_CUDA(cudaStreamSynchronize(h->m->stream));
    *loss = static_cast<float>(l);
    return h->m->take_status();
    SPGX_GUARD_END
}

spgx_status spgx_mlp_train(spgx_mlp *h, int32_t n, const float *x, const float *y, int32_t steps, int32_t batch,
                           float lr, uint64_t seed, float *final_loss)
{
    SPGX_GUARD_BEGIN
    SPGX_MHANDLE(h);
    if (n <= 0 || !x || !y || steps < 0 || batch <= 0 || !(lr > 0)) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    SPGX_TRY_STATUS(h->m->train(x, y, n, steps, batch, lr, seed, final_loss));
    SPGX_CUDA(cudaStreamSynchronize(h->m->stream));
    return h->m->take_status();
    SPGX_GUARD_END
}

}  // extern "C"
