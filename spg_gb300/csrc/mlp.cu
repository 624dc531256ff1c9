// Per-vertex MLP of the learned warm start: 24 -> 128 -> 128 -> 128 -> 3 with GELU, BF16
// weights, FP32 accumulation.
//
// Inference (mlp_infer_kernel) runs on the tensor cores with mma.sync m16n8k16 BF16: each warp
// owns 16 rows, the weights of all four layers are staged in shared memory as BF16 (transposed so
// each B fragment register is one 32-bit load), and the FP32 accumulator fragments of one layer
// become, after bias and GELU, the BF16 A fragments of the next without leaving registers.
//
// Training runs FP32 SIMT kernels (a tiled GEMM, GELU forward/backward, bias reductions, Adam)
// on FP32 master weights whose BF16 rounding is used in the forward pass, so the trained
// network is the one the BF16 inference kernel evaluates (straight-through for the rounding).
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

constexpr int kInferThreads = 256;  // 8 warps x 16 rows
constexpr size_t kInferSmem = size_t(128 * 32 + 128 * 128 * 2 + 8 * 128) * 2 + size_t(128 * 3 + 8) * 4;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    uint32_t r;
    memcpy(&r, &v, sizeof(r));
    return r;
}

__device__ __forceinline__ void mma_bf16(float *c, const uint32_t *a, uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One hidden layer: acc[16 n-tiles][4] = A (16 x K, as KS k-step fragments) * W (K x 128).
template <int KS>
__device__ __forceinline__ void mma_layer(float (*acc)[4], const uint32_t (*a)[4], const __nv_bfloat16 *wt, int ldk,
                                          int gid, int tid4)
{
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        const __nv_bfloat16 *row = wt + (j * 8 + gid) * ldk + tid4 * 2;
#pragma unroll
        for (int s = 0; s < KS; ++s) {
            const uint32_t b0 = *reinterpret_cast<const uint32_t *>(row + s * 16);
            const uint32_t b1 = *reinterpret_cast<const uint32_t *>(row + s * 16 + 8);
            mma_bf16(acc[j], a[s], b0, b1);
        }
    }
}

// Bias + GELU on a layer's accumulators and repacking as the next layer's A fragments.
__device__ __forceinline__ void activate(float (*acc)[4], uint32_t (*a)[4], const float *bias, int tid4)
{
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const int j0 = 2 * s, j1 = 2 * s + 1;
        const float bA0 = bias[j0 * 8 + tid4 * 2], bA1 = bias[j0 * 8 + tid4 * 2 + 1];
        const float bB0 = bias[j1 * 8 + tid4 * 2], bB1 = bias[j1 * 8 + tid4 * 2 + 1];
        a[s][0] = pack_bf16(gelu(acc[j0][0] + bA0), gelu(acc[j0][1] + bA1));
        a[s][1] = pack_bf16(gelu(acc[j0][2] + bA0), gelu(acc[j0][3] + bA1));
        a[s][2] = pack_bf16(gelu(acc[j1][0] + bB0), gelu(acc[j1][1] + bB1));
        a[s][3] = pack_bf16(gelu(acc[j1][2] + bB0), gelu(acc[j1][3] + bB1));
    }
}

__global__ void __launch_bounds__(kInferThreads) mlp_infer_kernel(MlpDevWeights W, const float *__restrict__ X, int n,
                                                                  float *__restrict__ Y)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16 *s_w1 = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
    __nv_bfloat16 *s_w2 = s_w1 + 128 * 32;
    __nv_bfloat16 *s_w3 = s_w2 + 128 * 128;
    __nv_bfloat16 *s_w4 = s_w3 + 128 * 128;
    float *s_b = reinterpret_cast<float *>(s_w4 + 8 * 128);
    {
        const uint4 *src[4] = {reinterpret_cast<const uint4 *>(W.w1t), reinterpret_cast<const uint4 *>(W.w2t),
                               reinterpret_cast<const uint4 *>(W.w3t), reinterpret_cast<const uint4 *>(W.w4t)};
        uint4 *dst[4] = {reinterpret_cast<uint4 *>(s_w1), reinterpret_cast<uint4 *>(s_w2),
                         reinterpret_cast<uint4 *>(s_w3), reinterpret_cast<uint4 *>(s_w4)};
        const int cnt[4] = {128 * 32 / 8, 128 * 128 / 8, 128 * 128 / 8, 8 * 128 / 8};
#pragma unroll
        for (int m = 0; m < 4; ++m)
            for (int i = threadIdx.x; i < cnt[m]; i += blockDim.x) dst[m][i] = __ldg(src[m] + i);
        for (int i = threadIdx.x; i < 128; i += blockDim.x) {
            s_b[i] = W.b1[i];
            s_b[128 + i] = W.b2[i];
            s_b[256 + i] = W.b3[i];
        }
        if (threadIdx.x < 8) s_b[384 + threadIdx.x] = W.b4[threadIdx.x];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gid = lane >> 2, tid4 = lane & 3;
    const int tiles = (n + 15) / 16;
    for (int t = blockIdx.x * (kInferThreads / 32) + warp; t < tiles; t += gridDim.x * (kInferThreads / 32)) {
        const int r0 = t * 16 + gid, r1 = r0 + 8;
        // Layer-1 A fragments straight from the FP32 features (k padded to 32 with zeros).
        uint32_t a[8][4];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            float v[8];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int k0 = s * 16 + q * 8 + tid4 * 2;
                v[4 * q + 0] = (r0 < n && k0 < 24) ? X[size_t(r0) * 24 + k0] : 0.f;
                v[4 * q + 1] = (r0 < n && k0 + 1 < 24) ? X[size_t(r0) * 24 + k0 + 1] : 0.f;
                v[4 * q + 2] = (r1 < n && k0 < 24) ? X[size_t(r1) * 24 + k0] : 0.f;
                v[4 * q + 3] = (r1 < n && k0 + 1 < 24) ? X[size_t(r1) * 24 + k0 + 1] : 0.f;
            }
            a[s][0] = pack_bf16(v[0], v[1]);
            a[s][1] = pack_bf16(v[2], v[3]);
            a[s][2] = pack_bf16(v[4], v[5]);
            a[s][3] = pack_bf16(v[6], v[7]);
        }
        float acc[16][4];
        mma_layer<2>(acc, a, s_w1, 32, gid, tid4);
        activate(acc, a, s_b, tid4);
        mma_layer<8>(acc, a, s_w2, 128, gid, tid4);
        activate(acc, a, s_b + 128, tid4);
        mma_layer<8>(acc, a, s_w3, 128, gid, tid4);
        activate(acc, a, s_b + 256, tid4);
        float out[4] = {0.f, 0.f, 0.f, 0.f};
        const __nv_bfloat16 *row = s_w4 + gid * 128 + tid4 * 2;
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const uint32_t b0 = *reinterpret_cast<const uint32_t *>(row + s * 16);
            const uint32_t b1 = *reinterpret_cast<const uint32_t *>(row + s * 16 + 8);
            mma_bf16(out, a[s], b0, b1);
        }
        const int c0 = tid4 * 2;
        if (c0 < 3) {
            if (r0 < n) Y[size_t(r0) * 3 + c0] = out[0] + s_b[384 + c0];
            if (r1 < n) Y[size_t(r1) * 3 + c0] = out[2] + s_b[384 + c0];
        }
        if (c0 + 1 < 3) {
            if (r0 < n) Y[size_t(r0) * 3 + c0 + 1] = out[1] + s_b[384 + c0 + 1];
            if (r1 < n) Y[size_t(r1) * 3 + c0 + 1] = out[3] + s_b[384 + c0 + 1];
        }
    }
}

// BF16 transposed copies of the FP32 master weights for the inference kernel.
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

// C[M x N] = alpha * op(A) * op(B) + beta * C, row-major, op = transpose when the flag is set.
// 64 x 64 output tile per 256-thread block, 4 x 4 outputs per thread, K chunks of 16.
__global__ void __launch_bounds__(256) gemm_f32_kernel(int M, int N, int K, const float *__restrict__ A, int lda,
                                                       bool tA, const float *__restrict__ B, int ldb, bool tB, float *C,
                                                       int ldc, float alpha, float beta)
{
    __shared__ float As[16][64 + 1];
    __shared__ float Bs[16][64 + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int i = threadIdx.x; i < 16 * 64; i += 256) {
            const int kk = i / 64, mm = i % 64;
            const int gm = m0 + mm, gk = k0 + kk;
            As[kk][mm] = (gm < M && gk < K) ? (tA ? A[size_t(gk) * lda + gm] : A[size_t(gm) * lda + gk]) : 0.f;
            const int gn = n0 + mm;
            Bs[kk][mm] = (gn < N && gk < K) ? (tB ? B[size_t(gn) * ldb + gk] : B[size_t(gk) * ldb + gn]) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            float av[4], bv[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                av[q] = As[kk][ty * 4 + q];
                bv[q] = Bs[kk][tx * 4 + q];
            }
#pragma unroll
            for (int p = 0; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[p][q] += av[p] * bv[q];
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int gm = m0 + ty * 4 + p, gn = n0 + tx * 4 + q;
            if (gm < M && gn < N) {
                float *c = C + size_t(gm) * ldc + gn;
                *c = alpha * acc[p][q] + (beta == 0.f ? 0.f : beta * *c);
            }
        }
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
                 bool tB, float *C, int ldc, float beta)
{
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    gemm_f32_kernel<<<grid, 256, 0, st>>>(M, N, K, A, lda, tA, B, ldb, tB, C, ldc, 1.f, beta);
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
    SPGX_CUDA(cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(kInferSmem)));
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
    const int tiles = (n + 15) / 16;
    const int grid = std::min(std::max(1, (tiles + 7) / 8), 2 * 152);
    mlp_infer_kernel<<<grid, kInferThreads, kInferSmem, st>>>(W, X, n, Y);
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
    gemm(stream, M, H, kMlpIn, X, kMlpIn, false, wq + kMlpOffW1, H, false, z1.as<float>(), H, 0.f);
    bias_act_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(z1.as<float>(), a1.as<float>(), wq + kMlpOffB1, M, H, true);
    gemm(stream, M, H, H, a1.as<float>(), H, false, wq + kMlpOffW2, H, false, z2.as<float>(), H, 0.f);
    bias_act_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(z2.as<float>(), a2.as<float>(), wq + kMlpOffB2, M, H, true);
    gemm(stream, M, H, H, a2.as<float>(), H, false, wq + kMlpOffW3, H, false, z3.as<float>(), H, 0.f);
    bias_act_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(z3.as<float>(), a3.as<float>(), wq + kMlpOffB3, M, H, true);
    gemm(stream, M, 3, H, a3.as<float>(), H, false, wq + kMlpOffW4, 3, false, yb.as<float>(), 3, 0.f);
    bias_act_kernel<<<blocks_for(size_t(M) * 3), 256, 0, stream>>>(yb.as<float>(), nullptr, wq + kMlpOffB4, M, 3, false);
    // loss
    SPGX_CUDA(cudaMemsetAsync(d_loss.as<double>(), 0, sizeof(double), stream));
    mse_grad_kernel<<<blocks_for(size_t(M) * 3), 256, 0, stream>>>(yb.as<float>(), T, dy.as<float>(), M,
                                                                    d_loss.as<double>());
    // backward
    gemm(stream, H, 3, M, a3.as<float>(), H, true, dy.as<float>(), 3, false, g + kMlpOffW4, 3, 0.f);
    col_sum_kernel<<<3, 256, 0, stream>>>(dy.as<float>(), g + kMlpOffB4, M, 3);
    gemm(stream, M, H, 3, dy.as<float>(), 3, false, wq + kMlpOffW4, 3, true, da.as<float>(), H, 0.f);
    gelu_back_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(da.as<float>(), z3.as<float>(), size_t(M) * H);
    gemm(stream, H, H, M, a2.as<float>(), H, true, da.as<float>(), H, false, g + kMlpOffW3, H, 0.f);
    col_sum_kernel<<<H, 256, 0, stream>>>(da.as<float>(), g + kMlpOffB3, M, H);
    gemm(stream, M, H, H, da.as<float>(), H, false, wq + kMlpOffW3, H, true, db_.as<float>(), H, 0.f);
    gelu_back_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(db_.as<float>(), z2.as<float>(), size_t(M) * H);
    gemm(stream, H, H, M, a1.as<float>(), H, true, db_.as<float>(), H, false, g + kMlpOffW2, H, 0.f);
    col_sum_kernel<<<H, 256, 0, stream>>>(db_.as<float>(), g + kMlpOffB2, M, H);
    gemm(stream, M, H, H, db_.as<float>(), H, false, wq + kMlpOffW2, H, true, da.as<float>(), H, 0.f);
    gelu_back_kernel<<<blocks_for(size_t(M) * H), 256, 0, stream>>>(da.as<float>(), z1.as<float>(), size_t(M) * H);
    gemm(stream, kMlpIn, H, M, X, kMlpIn, true, da.as<float>(), H, false, g + kMlpOffW1, H, 0.f);
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
    return SPGX_OK;
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
    return SPGX_OK;
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
    return h->m->train(x, y, n, steps, batch, lr, seed, final_loss);
    SPGX_GUARD_END
}

}  // extern "C"
