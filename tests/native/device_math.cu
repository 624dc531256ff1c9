// Test helper: runs the FP32 device math of elements.cuh (recip, arctan2) beside CUDA's own
// 1/x and atan2f on the same inputs, for the error-bound tests in tests/test_device_math.py.
#include <cuda_runtime.h>

#include "elements.cuh"

namespace {

__global__ void device_math_kernel(int n, const float *y, const float *x, float *atan_ours, float *atan_cuda,
                                   float *rcp_ours, float *rcp_cuda)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    atan_ours[i] = spgx::arctan2(y[i], x[i]);
    atan_cuda[i] = atan2f(y[i], x[i]);
    rcp_ours[i] = spgx::recip(x[i]);
    rcp_cuda[i] = 1.f / x[i];
}

}  // namespace

// out holds 4 * n floats: our atan2, atan2f, our 1/x, 1/x. Returns a cudaError_t.
extern "C" int spgx_test_device_math(int n, const float *y, const float *x, float *out)
{
    if (n <= 0) return 0;
    float *d = nullptr;
    const size_t bytes = sizeof(float) * size_t(n);
    cudaError_t e = cudaMalloc(&d, 6 * bytes);
    if (e != cudaSuccess) return int(e);
    cudaMemcpy(d, y, bytes, cudaMemcpyHostToDevice);
    cudaMemcpy(d + n, x, bytes, cudaMemcpyHostToDevice);
    device_math_kernel<<<(n + 255) / 256, 256>>>(n, d, d + n, d + 2 * n, d + 3 * n, d + 4 * n, d + 5 * n);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, d + 2 * n, 4 * bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return int(e);
}
