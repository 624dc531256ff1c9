// Particle state management and the substep kernels shared by VBD and XPBD.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "api_internal.h"
#include "state.h"
#include "substep.cuh"

namespace spgx {

__global__ void begin_substep_kernel(float4 *pos, float4 *tgt, float4 *dold, float4 *vel, int nv, float h, float gx,
                                     float gy, float gz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) begin_substep_vertex(pos, tgt, dold, vel, i, h, gx, gy, gz);
}

__global__ void end_substep_kernel(const float4 *pos, const float4 *dold, float4 *vel, int nv, float invh)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) end_substep_vertex(pos, dold, vel, i, invh);
}

// The same update, first saving the previous velocity v_n (vel - h g) as history.
__global__ void end_substep_hist_kernel(const float4 *pos, const float4 *dold, float4 *vel, float4 *vhist, int nv,
                                        float invh, float ghx, float ghy, float ghz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 u = vel[i];
    vhist[i] = make_float4(u.x - ghx, u.y - ghy, u.z - ghz, 0.f);
    const float4 d = pos[2 * i + 1];
    const float4 o = dold[i];
    vel[i] = make_float4((d.x - o.x) * invh, (d.y - o.y) * invh, (d.z - o.z) * invh, 0.f);
}

void launch_begin_substep(const ParticleState &P, double h, const double *g, cudaStream_t st)
{
    if (P.nv == 0) return;
    begin_substep_kernel<<<(P.nv + 255) / 256, 256, 0, st>>>(P.pos(), P.tgt(), P.dold(), P.vel(), P.nv, float(h),
                                                             float(g[0]), float(g[1]), float(g[2]));
}

void launch_end_substep(const ParticleState &P, double h, cudaStream_t st, float4 *vhist, const double *g)
{
    if (P.nv == 0) return;
    if (vhist) {
        end_substep_hist_kernel<<<(P.nv + 255) / 256, 256, 0, st>>>(P.pos(), P.dold(), P.vel(), vhist, P.nv,
                                                                    float(1.0 / h), float(h * g[0]), float(h * g[1]),
                                                                    float(h * g[2]));
        return;
    }
    end_substep_kernel<<<(P.nv + 255) / 256, 256, 0, st>>>(P.pos(), P.dold(), P.vel(), P.nv, float(1.0 / h));
}

// One object's FP64 external-order state -> the device layout (base = fl(x), delta =
// fl(x - base), velocity rounded to FP32); a NULL array leaves that part unchanged.
__global__ void state_set_kernel(float4 *pos, float4 *vel, const int *ext2int, const double *x, const double *v,
                                 int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = ext2int[k];
    if (x) {
        const double px = x[3 * k], py = x[3 * k + 1], pz = x[3 * k + 2];
        const float bx = float(px), by = float(py), bz = float(pz);
        pos[2 * i] = make_float4(bx, by, bz, 0.f);
        pos[2 * i + 1] = make_float4(float(px - bx), float(py - by), float(pz - bz), 0.f);
    }
    if (v) vel[i] = make_float4(float(v[3 * k]), float(v[3 * k + 1]), float(v[3 * k + 2]), 0.f);
}

// The device layout -> one object's FP64 external-order state (x = base + delta).
__global__ void state_get_kernel(const float4 *pos, const float4 *vel, const int *ext2int, double *x, double *v, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = ext2int[k];
    if (x) {
        const float4 b = pos[2 * i], d = pos[2 * i + 1];
        x[3 * k] = double(b.x) + double(d.x);
        x[3 * k + 1] = double(b.y) + double(d.y);
        x[3 * k + 2] = double(b.z) + double(d.z);
    }
    if (v) {
        const float4 u = vel[i];
        v[3 * k] = u.x;
        v[3 * k + 1] = u.y;
        v[3 * k + 2] = u.z;
    }
}

spgx_status ParticleState::init(const SceneLayout &L)
{
    nv = L.nv;
    const size_t n = size_t(nv);
    SPGX_TRY_STATUS(d_pos.alloc(n * 2 * sizeof(float4)));
    SPGX_TRY_STATUS(d_tgt.alloc(n * sizeof(float4)));
    SPGX_TRY_STATUS(d_dold.alloc(n * sizeof(float4)));
    SPGX_TRY_STATUS(d_vel.alloc(n * sizeof(float4)));
    size_t max_obj = 1;
    for (const auto &o : L.objects) max_obj = std::max(max_obj, size_t(o.nv));
    stage_doubles = 6 * max_obj;
    SPGX_TRY_STATUS(d_stage.alloc(stage_doubles * sizeof(double)));
    SPGX_TRY_STATUS(d_ext2int.upload(L.ext2int.empty() ? std::vector<int32_t>{0} : L.ext2int));
    std::vector<float4> hp(2 * n), hv(n), tg(n);
    std::vector<float> invm(n);
    for (size_t ext = 0; ext < n; ++ext) {
        const int i = L.ext2int[ext];
        const double *x = &L.x_ext[3 * ext];
        const double *v = &L.v_ext[3 * ext];
        const float bx = float(x[0]), by = float(x[1]), bz = float(x[2]);
        hp[2 * i] = make_float4(bx, by, bz, 0.f);
        hp[2 * i + 1] = make_float4(float(x[0] - bx), float(x[1] - by), float(x[2] - bz), 0.f);
        hv[i] = make_float4(float(v[0]), float(v[1]), float(v[2]), 0.f);
        tg[i] = make_float4(hp[2 * i + 1].x, hp[2 * i + 1].y, hp[2 * i + 1].z, L.mass[i]);
        // ParticleGroup::addParticle: w = (m == 0 ? 0 : 1 / m), particleGroup.cpp:81
        invm[i] = L.mass[i] == 0.f ? 0.f : 1.f / L.mass[i];
    }
    if (n) {
        SPGX_CUDA(cudaMemcpy(pos(), hp.data(), n * 2 * sizeof(float4), cudaMemcpyHostToDevice));
        SPGX_CUDA(cudaMemcpy(vel(), hv.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
        SPGX_CUDA(cudaMemcpy(tgt(), tg.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
        SPGX_CUDA(cudaMemset(dold(), 0, n * sizeof(float4)));
    }
    SPGX_TRY_STATUS(d_invm.upload(invm));
    return SPGX_OK;
}

spgx_status ParticleState::get(const SceneLayout &L, int obj, double *x, double *v, cudaStream_t stream)
{
    if (obj < 0 || obj >= static_cast<int>(L.objects.size())) {
        set_error("invalid object index");
        return SPGX_ERR_INVALID_ARG;
    }
    const auto &O = L.objects[obj];
    const size_t n = size_t(O.nv);
    if (n == 0 || (!x && !v)) return SPGX_OK;
    double *sx = d_stage.as<double>(), *sv = sx + 3 * n;
    state_get_kernel<<<unsigned((n + 255) / 256), 256, 0, stream>>>(pos(), vel(), d_ext2int.as<int>() + O.vertex_base,
                                                                     x ? sx : nullptr, v ? sv : nullptr, int(n));
    SPGX_CUDA(cudaGetLastError());
    if (x) SPGX_CUDA(cudaMemcpyAsync(x, sx, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    if (v) SPGX_CUDA(cudaMemcpyAsync(v, sv, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, stream));
    SPGX_CUDA(cudaStreamSynchronize(stream));
    return SPGX_OK;
}

spgx_status ParticleState::set(const SceneLayout &L, int obj, const double *x, const double *v, cudaStream_t stream)
{
    if (obj < 0 || obj >= static_cast<int>(L.objects.size())) {
        set_error("invalid object index");
        return SPGX_ERR_INVALID_ARG;
    }
    const auto &O = L.objects[obj];
    const size_t n = size_t(O.nv);
    if (n == 0 || (!x && !v)) return SPGX_OK;
    double *sx = d_stage.as<double>(), *sv = sx + 3 * n;
    if (x) SPGX_CUDA(cudaMemcpyAsync(sx, x, 3 * n * sizeof(double), cudaMemcpyHostToDevice, stream));
    if (v) SPGX_CUDA(cudaMemcpyAsync(sv, v, 3 * n * sizeof(double), cudaMemcpyHostToDevice, stream));
    state_set_kernel<<<unsigned((n + 255) / 256), 256, 0, stream>>>(pos(), vel(), d_ext2int.as<int>() + O.vertex_base,
                                                                     x ? sx : nullptr, v ? sv : nullptr, int(n));
    SPGX_CUDA(cudaGetLastError());
    // The staging buffer is reused by the next call: the copies must have left the caller's
    // arrays before returning (pageable sources are copied synchronously anyway).
    SPGX_CUDA(cudaStreamSynchronize(stream));
    replaced = true;
    return SPGX_OK;
}

spgx_status ParticleState::reset(const SceneLayout &L, cudaStream_t stream)
{
    for (int o = 0; o < static_cast<int>(L.objects.size()); ++o) {
        const std::vector<double> zeros(L.objects[o].x_init.size(), 0.0);
        SPGX_TRY_STATUS(set(L, o, L.objects[o].x_init.data(), zeros.data(), stream));
    }
    return SPGX_OK;
}

}  // namespace spgx
