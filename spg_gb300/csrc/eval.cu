// Element-level evaluation on the GPU with the solver's own FP32 device code, for the
// per-element derivative parity checks (spgx_eval_vertex_blocks / spgx_eval_constraints).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "api_internal.h"
#include "devbuf.h"
#include "device_common.cuh"
#include "layout.h"

namespace spgx {

// One incidence per thread: gradient segment and Hessian block of `slot` for the element
// whose stencil positions are X[i] (S * 3 floats) with parameters prm[i] (P floats).
__global__ void eval_blocks_kernel(int type, int n, int S, int P, const float *__restrict__ X,
                                   const float *__restrict__ prm, const int *__restrict__ slots, float *grad, float *hess)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *x = X + size_t(i) * S * 3;
    const float *p = prm + size_t(i) * P;
    const int slot = slots[i];
    // Positions relative to the evaluated vertex, as the solver kernels form them.
    const V3f self = mk(x[3 * slot], x[3 * slot + 1], x[3 * slot + 2]);
    V3f r[4];
    for (int j = 0; j < S; ++j) r[j] = mk(x[3 * j] - self.x, x[3 * j + 1] - self.y, x[3 * j + 2] - self.z);
    const V3f zero = mk(0.f, 0.f, 0.f);
    Block<float> b;
    block_zero(b);
    switch (type) {
    case SPGX_ENERGY_SPRING: {
        // s = self - other = -r[other] exactly as s_hi + s_lo (error-free difference).
        const int o = 1 - slot;
        V3f sh, sl;
        two_sum(self.x, -x[3 * o], sh.x, sl.x);
        two_sum(self.y, -x[3 * o + 1], sh.y, sl.y);
        two_sum(self.z, -x[3 * o + 2], sh.z, sl.z);
        spring_block(sh, zero, sl, p[0], p[1], b);
        break;
    }
    case SPGX_ENERGY_SPRING_ANCHOR: anchor_block(mk(self.x - p[0], self.y - p[1], self.z - p[2]), zero, p[3], b); break;
    case SPGX_ENERGY_DISCRETE_BENDING:
        if (slot >= 2)
            bending_flap_block(r[0], r[1], zero, r[5 - slot], slot == 2 ? p[0] : -p[0], p[1], b);
        else
            bending_hinge_block(r[1 - slot], zero, r[2], r[3], slot == 1 ? p[0] : -p[0], p[1], b);
        break;
    case SPGX_ENERGY_MEMBRANE_STVK: {
        const float D[4] = {p[0], p[1], p[2], p[3]};
        const float Ks[6] = {p[4], 0.5f * (p[5] + p[7]), 0.5f * (p[6] + p[10]), p[8], 0.5f * (p[9] + p[11]), p[12]};
        stvk_block(r, slot, D, Ks, b);
        break;
    }
    case SPGX_ENERGY_STABLE_NEO_HOOKEAN: {
        float D[9];
        for (int k = 0; k < 9; ++k) D[k] = p[k];
        snh_block(r, slot, D, p[9], p[10], p[11], b);
        break;
    }
    default: {
        V3f q[4];
        for (int j = 0; j < 4; ++j) q[j] = j < S ? r[j] : zero;
        generic_block(type, q, slot, p, b);
        break;
    }
    }
    grad[3 * i + 0] = -b.f[0];
    grad[3 * i + 1] = -b.f[1];
    grad[3 * i + 2] = -b.f[2];
    const int m[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};
    for (int k = 0; k < 9; ++k) hess[9 * i + k] = b.h[m[k]];
}

__global__ void eval_constraints_kernel(int type, int n, int S, int P, int NC, const float *__restrict__ X,
                                        const float *__restrict__ prm, float *C, float *G)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *x = X + size_t(i) * S * 3;
    const float *p = prm + size_t(i) * P;
    V3f r[4];
    for (int j = 0; j < S; ++j) r[j] = mk(x[3 * j] - x[0], x[3 * j + 1] - x[1], x[3 * j + 2] - x[2]);
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    V3f g[16];
    switch (type) {
    case SPGX_ENERGY_SPRING: {
        const V3f s = r[0] - r[1];
        const float l = sqrtf(dot(s, s));
        c[0] = l - p[0];
        g[0] = (1.f / l) * s;
        g[1] = mk(0.f, 0.f, 0.f) - g[0];
        break;
    }
    case SPGX_ENERGY_SPRING_ANCHOR:
        anchor_constraint(mk(x[0] - p[0], x[1] - p[1], x[2] - p[2]), mk(0.f, 0.f, 0.f), c, g);
        break;
    case SPGX_ENERGY_DISCRETE_BENDING: bending_constraint(r, p[0], c, g); break;
    case SPGX_ENERGY_MEMBRANE_STVK: {
        const float D[4] = {p[0], p[1], p[2], p[3]};
        stvk_constraints(r, D, c, g);
        break;
    }
    case SPGX_ENERGY_STABLE_NEO_HOOKEAN: {
        float D[9];
        for (int k = 0; k < 9; ++k) D[k] = p[k];
        snh_constraints(r, D, p[11], c, g);
        break;
    }
    default: {  // types 6-13: per-vertex forward mode, one stencil vertex at a time
        V3f q[4];
        for (int j = 0; j < 4; ++j) q[j] = j < S ? r[j] : mk(0.f, 0.f, 0.f);
        for (int j = 0; j < S; ++j) {
            VAD<float> cv[4];
            const int nc = generic_constraints(type, q, j, p, cv);
            for (int k = 0; k < nc; ++k) {
                c[k] = cv[k].v;
                g[k * S + j] = mk(cv[k].g[0], cv[k].g[1], cv[k].g[2]);
            }
        }
        break;
    }
    }
    for (int k = 0; k < NC; ++k) {
        C[size_t(i) * NC + k] = c[k];
        for (int j = 0; j < S; ++j) {
            float *o = G + (size_t(i) * NC + k) * 3 * S + 3 * j;
            o[0] = g[k * S + j].x;
            o[1] = g[k * S + j].y;
            o[2] = g[k * S + j].z;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Allocation-free variant of the element evaluation. Its device staging lives in one
// file-scope array that every GPU loading this library holds (about 750 KB) until the process
// exits; every call shares it, so calls that overlap on a GPU race on it.
constexpr int kNoAllocMaxIncidences = 4096;
constexpr int kNoAllocMaxStencil = 4;
constexpr int kNoAllocMaxParams = 22;

struct NoAllocScratch {
    float X[kNoAllocMaxIncidences * kNoAllocMaxStencil * 3];
    float params[kNoAllocMaxIncidences * kNoAllocMaxParams];
    int slots[kNoAllocMaxIncidences];
    float grad[kNoAllocMaxIncidences * 3];
    float hess[kNoAllocMaxIncidences * 9];
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of the scratch array on the current device (the host-side symbol is only a
// stand-in, never a device address). The first lookup on a device loads this file's device
// code there, which places the array. The address is looked up on every call rather than
// cached: the lookup allocates nothing, and a cached address would go stale if the caller
// reset the device (the module, and the array with it, is then placed anew).
static spgx_status noalloc_scratch(NoAllocScratch **out)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        set_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        return SPGX_ERR_CUDA;
    }
    *out = static_cast<NoAllocScratch *>(p);
    return SPGX_OK;
}

// Converts count doubles to floats through a stack buffer and copies them to dst.
static spgx_status upload_floats(float *dst, const double *src, size_t count)
{
    float buf[1024];
    for (size_t o = 0; o < count; o += 1024) {
        const size_t m = std::min<size_t>(1024, count - o);
        for (size_t k = 0; k < m; ++k) buf[k] = static_cast<float>(src[o + k]);
        SPGX_CUDA(cudaMemcpy(dst + o, buf, m * sizeof(float), cudaMemcpyHostToDevice));
    }
    return SPGX_OK;
}

static spgx_status download_floats(double *dst, const float *src, size_t count)
{
    float buf[1024];
    for (size_t o = 0; o < count; o += 1024) {
        const size_t m = std::min<size_t>(1024, count - o);
        SPGX_CUDA(cudaMemcpy(buf, src + o, m * sizeof(float), cudaMemcpyDeviceToHost));
        for (size_t k = 0; k < m; ++k) dst[o + k] = buf[k];
    }
    return SPGX_OK;
}

}  // namespace spgx

extern "C" {

spgx_status spgx_eval_vertex_blocks(int32_t type, int32_t n, const double *X, const double *params,
                                    const int32_t *slots, double *grad, double *hess)
{
    SPGX_GUARD_BEGIN
    const int S = spgx::stencil_size(type), P = spgx::param_count(type);
    if (S == 0) {
        spgx::set_error("unsupported energy type");
        return SPGX_ERR_UNSUPPORTED_ENERGY;
    }
    if (n < 0 || (n > 0 && (!X || !params || !slots || !grad || !hess))) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    if (n == 0) return SPGX_OK;
    for (int i = 0; i < n; ++i)
        if (slots[i] < 0 || slots[i] >= S) {
            spgx::set_error("slot out of range");
            return SPGX_ERR_INVALID_ARG;
        }
    int dev = 0;
    SPGX_CUDA(cudaGetDevice(&dev));
    SPGX_TRY_STATUS(spgx::select_device(dev));
    std::vector<float> xf(size_t(n) * S * 3), pf(size_t(n) * P);
    for (size_t k = 0; k < xf.size(); ++k) xf[k] = float(X[k]);
    for (size_t k = 0; k < pf.size(); ++k) pf[k] = float(params[k]);
    std::vector<int> sl(slots, slots + n);
    spgx::DevBuf dX, dP, dS, dG, dH;
    SPGX_TRY_STATUS(dX.upload(xf));
    SPGX_TRY_STATUS(dP.upload(pf));
    SPGX_TRY_STATUS(dS.upload(sl));
    SPGX_TRY_STATUS(dG.alloc(sizeof(float) * 3 * n));
    SPGX_TRY_STATUS(dH.alloc(sizeof(float) * 9 * n));
    spgx::eval_blocks_kernel<<<(n + 127) / 128, 128>>>(type, n, S, P, dX.as<float>(), dP.as<float>(), dS.as<int>(),
                                                       dG.as<float>(), dH.as<float>());
    SPGX_CUDA(cudaGetLastError());
    std::vector<float> g(size_t(3) * n), hh(size_t(9) * n);
    SPGX_CUDA(cudaMemcpy(g.data(), dG.as<float>(), g.size() * sizeof(float), cudaMemcpyDeviceToHost));
    SPGX_CUDA(cudaMemcpy(hh.data(), dH.as<float>(), hh.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < g.size(); ++k) grad[k] = g[k];
    for (size_t k = 0; k < hh.size(); ++k) hess[k] = hh[k];
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_eval_vertex_blocks_noalloc(int32_t type, int32_t n, const double *X, const double *params,
                                            const int32_t *slots, double *grad, double *hess)
{
    SPGX_GUARD_BEGIN
    const int S = spgx::stencil_size(type), P = spgx::param_count(type);
    if (S == 0) {
        spgx::set_error("unsupported energy type");
        return SPGX_ERR_UNSUPPORTED_ENERGY;
    }
    if (n < 0 || (n > 0 && (!X || !params || !slots || !grad || !hess))) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    if (S > spgx::kNoAllocMaxStencil || P > spgx::kNoAllocMaxParams) {
        spgx::set_error("spgx_eval_vertex_blocks_noalloc: energy type " + std::to_string(type) +
                        " has more stencil vertices or parameters than the fixed scratch array holds");
        return SPGX_ERR_INVALID_ARG;
    }
    if (n > spgx::kNoAllocMaxIncidences) {
        spgx::set_error("spgx_eval_vertex_blocks_noalloc: n = " + std::to_string(n) + " exceeds the fixed capacity of " +
                        std::to_string(spgx::kNoAllocMaxIncidences) + " incidences per call");
        return SPGX_ERR_INVALID_ARG;
    }
    if (n == 0) return SPGX_OK;
    for (int i = 0; i < n; ++i)
        if (slots[i] < 0 || slots[i] >= S) {
            spgx::set_error("slot out of range");
            return SPGX_ERR_INVALID_ARG;
        }
    int dev = 0;
    SPGX_CUDA(cudaGetDevice(&dev));
    SPGX_TRY_STATUS(spgx::select_device(dev));
    spgx::NoAllocScratch *sc = nullptr;
    SPGX_TRY_STATUS(spgx::noalloc_scratch(&sc));
    SPGX_TRY_STATUS(spgx::upload_floats(sc->X, X, size_t(n) * S * 3));
    SPGX_TRY_STATUS(spgx::upload_floats(sc->params, params, size_t(n) * P));
    SPGX_CUDA(cudaMemcpy(sc->slots, slots, size_t(n) * sizeof(int), cudaMemcpyHostToDevice));
    spgx::eval_blocks_kernel<<<(n + 127) / 128, 128>>>(type, n, S, P, sc->X, sc->params, sc->slots, sc->grad,
                                                       sc->hess);
    SPGX_CUDA(cudaGetLastError());
    SPGX_TRY_STATUS(spgx::download_floats(grad, sc->grad, size_t(n) * 3));
    SPGX_TRY_STATUS(spgx::download_floats(hess, sc->hess, size_t(n) * 9));
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_eval_constraints(int32_t type, int32_t n, const double *X, const double *params, double *C,
                                  double *gradC)
{
    SPGX_GUARD_BEGIN
    const int S = spgx::stencil_size(type), P = spgx::param_count(type);
    const int NC = spgx_num_constraints(type);
    if (S == 0) {
        spgx::set_error("unsupported energy type");
        return SPGX_ERR_UNSUPPORTED_ENERGY;
    }
    if (n < 0 || (n > 0 && (!X || !params || !C || !gradC))) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    if (n == 0) return SPGX_OK;
    int dev = 0;
    SPGX_CUDA(cudaGetDevice(&dev));
    SPGX_TRY_STATUS(spgx::select_device(dev));
    std::vector<float> xf(size_t(n) * S * 3), pf(size_t(n) * P);
    for (size_t k = 0; k < xf.size(); ++k) xf[k] = float(X[k]);
    for (size_t k = 0; k < pf.size(); ++k) pf[k] = float(params[k]);
    spgx::DevBuf dX, dP, dC, dG;
    SPGX_TRY_STATUS(dX.upload(xf));
    SPGX_TRY_STATUS(dP.upload(pf));
    SPGX_TRY_STATUS(dC.alloc(sizeof(float) * NC * n));
    SPGX_TRY_STATUS(dG.alloc(sizeof(float) * NC * 3 * S * n));
    spgx::eval_constraints_kernel<<<(n + 127) / 128, 128>>>(type, n, S, P, NC, dX.as<float>(), dP.as<float>(),
                                                            dC.as<float>(), dG.as<float>());
    SPGX_CUDA(cudaGetLastError());
    std::vector<float> c(size_t(NC) * n), g(size_t(NC) * 3 * S * n);
    SPGX_CUDA(cudaMemcpy(c.data(), dC.as<float>(), c.size() * sizeof(float), cudaMemcpyDeviceToHost));
    SPGX_CUDA(cudaMemcpy(g.data(), dG.as<float>(), g.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < c.size(); ++k) C[k] = c[k];
    for (size_t k = 0; k < g.size(); ++k) gradC[k] = g[k];
    return SPGX_OK;
    SPGX_GUARD_END
}

}  // extern "C"
