// The warm-start MLP (24 -> 128 -> 128 -> 128 -> 3, GELU): parameter layout and the handle
// behind the spgx_mlp_* C ABI.
#pragma once

#include <cuda_runtime.h>

#include <memory>

#include "devbuf.h"

namespace spgx {

constexpr int kMlpIn = 24;
constexpr int kMlpHidden = 128;
constexpr int kMlpOut = 3;
// Flat FP32 parameters, row-major W[in][out]: W1 b1 W2 b2 W3 b3 W4 b4.
constexpr int kMlpOffW1 = 0;
constexpr int kMlpOffB1 = kMlpOffW1 + kMlpIn * kMlpHidden;
constexpr int kMlpOffW2 = kMlpOffB1 + kMlpHidden;
constexpr int kMlpOffB2 = kMlpOffW2 + kMlpHidden * kMlpHidden;
constexpr int kMlpOffW3 = kMlpOffB2 + kMlpHidden;
constexpr int kMlpOffB3 = kMlpOffW3 + kMlpHidden * kMlpHidden;
constexpr int kMlpOffW4 = kMlpOffB3 + kMlpHidden;
constexpr int kMlpOffB4 = kMlpOffW4 + kMlpHidden * kMlpOut;
constexpr int kMlpParams = kMlpOffB4 + kMlpOut;

struct Mlp {
    int device{0};
    cudaStream_t stream{nullptr};
    DevBuf d_w, d_wq, d_g, d_m, d_v;         // master weights, BF16-rounded copy, grad, Adam moments
    DevBuf d_w1t, d_w2t, d_w3t, d_w4t, d_b4;  // BF16 transposed copies for inference
    DevBuf d_loss;
    DevBuf d_status;  // bit 0: a tensor-core commit (inference or training GEMM) never arrived (bounded wait)
    int num_sms{0};
    DevBuf z1, a1, z2, a2, z3, a3, yb, dy, da, db_, xb, tb, ib;
    int batch_cap{0};
    long adam_t{0};

    Mlp() = default;
    Mlp(const Mlp &) = delete;
    Mlp &operator=(const Mlp &) = delete;
    ~Mlp();

    spgx_status init(uint64_t seed, int dev);
    spgx_status set_weights(const float *w);
    spgx_status get_weights(float *w);
    spgx_status refresh();
    spgx_status ensure_batch(int M);
    spgx_status loss_grad_device(const float *X, const float *T, int M, double *loss_out);
    spgx_status train(const float *X, const float *T, int n, int steps, int batch, float lr, uint64_t seed,
                      float *final_loss);
    // Y (n x 3) = MLP(X (n x 24)) on the tensor cores (tcgen05), both device pointers (X 16-byte
    // aligned), on stream st.
    void infer(const float *X, int n, float *Y, cudaStream_t st) const;
    // SPGX_ERR_TIMEOUT (and the flag cleared) when an inference since the last call gave up
    // waiting for the tensor cores; call after synchronising the stream the inference ran on.
    spgx_status take_status();
};

}  // namespace spgx

// The opaque handle of the C ABI.
struct spgx_mlp {
    std::unique_ptr<spgx::Mlp> m;
};
