// Warm-start kernels and the one-ring neighbour build (see warm.h for the feature layout).
#include <algorithm>
#include <cmath>

#include "warm.h"

namespace spgx {

void build_vertex_neighbours(const SceneLayout &L, std::vector<int32_t> &off, std::vector<int32_t> &nbr,
                             std::vector<F4> &stat)
{
    const int nv = L.nv;
    std::vector<std::vector<int32_t>> ring(nv);
    auto link = [&](int a, int b) {
        if (a == b) return;
        ring[a].push_back(b);
        ring[b].push_back(a);
    };
    const ElementTables &E = L.el;
    for (const I4 &s : E.springs) link(s.x, s.y);
    for (const I4 &b : E.bend_idx) {  // hinge edge and the four triangle edges, not opp0-opp1
        link(b.x, b.y);
        link(b.x, b.z);
        link(b.y, b.z);
        link(b.x, b.w);
        link(b.y, b.w);
    }
    for (const I4 &t : E.stvk_idx) {
        link(t.x, t.y);
        link(t.y, t.z);
        link(t.x, t.z);
    }
    for (const I4 &t : E.snh_idx) {
        const int v[4] = {t.x, t.y, t.z, t.w};
        for (int a = 0; a < 4; ++a)
            for (int b = a + 1; b < 4; ++b) link(v[a], v[b]);
    }
    for (size_t e = 0; e < E.gen_idx.size(); ++e) {  // types 6-14: every pair of the stencil
        const I4 t = E.gen_idx[e];
        const int v[4] = {t.x, t.y, t.z, t.w};
        const int S = E.gen_info[e].z;
        for (int a = 0; a < S; ++a)
            for (int b = a + 1; b < S; ++b) link(v[a], v[b]);
    }
    std::vector<char> anchored(nv, 0);
    for (int32_t v : E.anchor_v) anchored[v] = 1;
    off.assign(nv + 1, 0);
    nbr.clear();
    stat.assign(nv, F4{0.f, 0.f, 0.f, 0.f});
    for (int i = 0; i < nv; ++i) {
        auto &r = ring[i];
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        int pinned = 0;
        for (int j : r) pinned += anchored[j];
        nbr.insert(nbr.end(), r.begin(), r.end());
        off[i + 1] = static_cast<int32_t>(nbr.size());
        stat[i] = F4{float(anchored[i]), r.empty() ? 0.f : float(pinned) / float(r.size()), float(r.size()) / 8.f, 0.f};
    }
}

__global__ void warm_features_kernel(const float4 *__restrict__ vel, const float4 *__restrict__ vhist,
                                     const int *__restrict__ off, const int *__restrict__ nbr,
                                     const float4 *__restrict__ stat, int nv, float a, float ghx, float ghy, float ghz,
                                     float gnx, float gny, float gnz, float *__restrict__ F)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    // After the inertial predict vel holds v_n + h g and vhist holds v_{n-1}. Every displacement
    // is h times a velocity (y - x_n = h (v_n + h g), d1 = h v_n, d2 = h v_{n-1}), so a
    // displacement over l = h^2 g0 is the velocity times a = 1 / (h g0).
    const float4 v = vel[i], p = vhist[i];
    const float d1[3] = {v.x - ghx, v.y - ghy, v.z - ghz};
    const float d2[3] = {p.x, p.y, p.z};
    float m1[3] = {0.f, 0.f, 0.f}, m2[3] = {0.f, 0.f, 0.f};
    const int b = off[i], e = off[i + 1];
    for (int k = b; k < e; ++k) {
        const int j = nbr[k];
        const float4 vj = vel[j], pj = vhist[j];
        m1[0] += vj.x - ghx;
        m1[1] += vj.y - ghy;
        m1[2] += vj.z - ghz;
        m2[0] += pj.x;
        m2[1] += pj.y;
        m2[2] += pj.z;
    }
    const float inv = e > b ? 1.f / float(e - b) : 0.f;
    float l1[3], l2[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        l1[c] = e > b ? m1[c] * inv - d1[c] : 0.f;
        l2[c] = e > b ? m2[c] * inv - d2[c] : 0.f;
    }
    const float4 s = stat[i];
    float *f = F + size_t(i) * kWarmFeatures;
    f[0] = v.x * a;
    f[1] = v.y * a;
    f[2] = v.z * a;
    f[3] = d1[0] * a;
    f[4] = d1[1] * a;
    f[5] = d1[2] * a;
    f[6] = d2[0] * a;
    f[7] = d2[1] * a;
    f[8] = d2[2] * a;
    f[9] = l1[0] * a;
    f[10] = l1[1] * a;
    f[11] = l1[2] * a;
    f[12] = l2[0] * a;
    f[13] = l2[1] * a;
    f[14] = l2[2] * a;
    f[15] = gnx;
    f[16] = gny;
    f[17] = gnz;
    f[18] = s.x;
    f[19] = s.y;
    f[20] = s.z;
    f[21] = sqrtf(d1[0] * d1[0] + d1[1] * d1[1] + d1[2] * d1[2]) * a;
    f[22] = sqrtf(l1[0] * l1[0] + l1[1] * l1[1] + l1[2] * l1[2]) * a;
    f[23] = 1.f;
}

// x_e - base = (y - base) + h (v_n - v_{n-1}) - h^2 g: the last step's acceleration carried
// over (x_e = x_n + 2 (x_n - x_{n-1}) - (x_{n-1} - x_{n-2})). vel holds v_n + h g here.
__device__ __forceinline__ float3 extrapolated_delta(float4 t, float4 v, float4 p, float h, float ghx, float ghy,
                                                     float ghz)
{
    return make_float3(t.x + h * (v.x - p.x - 2.f * ghx), t.y + h * (v.y - p.y - 2.f * ghy),
                       t.z + h * (v.z - p.z - 2.f * ghz));
}

// The learned guess: the extrapolated one plus l times the network's correction.
__global__ void warm_apply_kernel(float4 *__restrict__ pos, const float4 *__restrict__ tgt,
                                  const float4 *__restrict__ vel, const float4 *__restrict__ vhist,
                                  const float *__restrict__ out, int nv, float h, float ghx, float ghy, float ghz,
                                  float ell)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float3 e = extrapolated_delta(tgt[i], vel[i], vhist[i], h, ghx, ghy, ghz);
    const float *o = out + size_t(i) * 3;
    pos[2 * i + 1] = make_float4(e.x + ell * o[0], e.y + ell * o[1], e.z + ell * o[2], 0.f);
}

__global__ void warm_extrapolate_kernel(float4 *__restrict__ pos, const float4 *__restrict__ tgt,
                                        const float4 *__restrict__ vel, const float4 *__restrict__ vhist, int nv,
                                        float h, float ghx, float ghy, float ghz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float3 e = extrapolated_delta(tgt[i], vel[i], vhist[i], h, ghx, ghy, ghz);
    pos[2 * i + 1] = make_float4(e.x, e.y, e.z, 0.f);
}

// Chooses the start of the substep by residual. The positions hold the candidate whose squared
// residual is wres[1] (the learned guess with three_way, else the extrapolated one); wres[0]
// is y's and, with three_way, wres[2] the extrapolated guess's. Ties keep the simpler guess.
__global__ void warm_select_kernel(float4 *__restrict__ pos, const float4 *__restrict__ tgt,
                                   const float4 *__restrict__ vel, const float4 *__restrict__ vhist,
                                   const double *__restrict__ wres, int nv, bool three_way, float h, float ghx,
                                   float ghy, float ghz, int *counters)
{
    const double r0 = wres[0], r1 = wres[1], r2 = three_way ? wres[2] : INFINITY;
    const bool keep = r1 < r0 && r1 < r2;
    const bool extrap = !keep && r2 < r0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && keep) atomicAdd(counters + (three_way ? 3 : 4), 1);
    if (i == 0 && extrap) atomicAdd(counters + 4, 1);
    if (keep || i >= nv) return;
    const float4 t = tgt[i];
    if (extrap) {
        const float3 e = extrapolated_delta(t, vel[i], vhist[i], h, ghx, ghy, ghz);
        pos[2 * i + 1] = make_float4(e.x, e.y, e.z, 0.f);
    } else {
        pos[2 * i + 1] = make_float4(t.x, t.y, t.z, 0.f);
    }
}

__global__ void warm_probe_select_kernel(float4 *__restrict__ pos, const float4 *__restrict__ saved,
                                         const double *__restrict__ wres, int nv, int *counters)
{
    const bool learned = wres[1] < wres[2];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) atomicAdd(counters + (learned ? 3 : 4), 1);
    if (!learned || i >= nv) return;
    pos[2 * i] = saved[2 * i];
    pos[2 * i + 1] = saved[2 * i + 1];
}

__global__ void warm_targets_kernel(const float4 *__restrict__ pos, const float4 *__restrict__ tgt, int nv,
                                    float inv_ell, float *__restrict__ T)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 d = pos[2 * i + 1], t = tgt[i];
    T[3 * size_t(i) + 0] = (d.x - t.x) * inv_ell;
    T[3 * size_t(i) + 1] = (d.y - t.y) * inv_ell;
    T[3 * size_t(i) + 2] = (d.z - t.z) * inv_ell;
}

static int grid_for(int n) { return (n + 255) / 256; }

void launch_warm_features(const WarmStart &W, const float4 *vel, int nv, double h, const double *g, cudaStream_t st)
{
    if (nv == 0) return;
    const float a = static_cast<float>(1.0 / (h * kWarmG0));
    warm_features_kernel<<<grid_for(nv), 256, 0, st>>>(
        vel, W.vhist.as<float4>(), W.nbr_off.as<int>(), W.nbr.as<int>(), W.stat.as<float4>(), nv, a,
        float(h * g[0]), float(h * g[1]), float(h * g[2]), float(g[0] / kWarmG0), float(g[1] / kWarmG0),
        float(g[2] / kWarmG0), W.feats.as<float>());
}

__global__ void warm_smooth_kernel(const float *__restrict__ in, float *__restrict__ out, const int *__restrict__ off,
                                   const int *__restrict__ nbr, int nv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int b = off[i], e = off[i + 1];
    float m[3] = {0.f, 0.f, 0.f};
    for (int k = b; k < e; ++k) {
        const float *o = in + 3 * size_t(nbr[k]);
        m[0] += o[0];
        m[1] += o[1];
        m[2] += o[2];
    }
    const float inv = e > b ? 1.f / float(e - b) : 0.f;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float s = in[3 * size_t(i) + c];
        out[3 * size_t(i) + c] = e > b ? 0.5f * (s + m[c] * inv) : s;
    }
}

void launch_warm_smooth(const WarmStart &W, int nv, cudaStream_t st)
{
    if (nv == 0 || W.smooth <= 0) return;
    float *a = W.out.as<float>(), *b = W.out2.as<float>();
    for (int p = 0; p < W.smooth; ++p) {
        warm_smooth_kernel<<<grid_for(nv), 256, 0, st>>>(a, b, W.nbr_off.as<int>(), W.nbr.as<int>(), nv);
        std::swap(a, b);
    }
    if (a != W.out.as<float>())
        cudaMemcpyAsync(W.out.as<float>(), a, size_t(nv) * 3 * sizeof(float), cudaMemcpyDeviceToDevice, st);
}

void launch_warm_apply(const WarmStart &W, float4 *pos, const float4 *tgt, const float4 *vel, int nv, double h,
                       const double *g, cudaStream_t st)
{
    if (nv == 0) return;
    warm_apply_kernel<<<grid_for(nv), 256, 0, st>>>(pos, tgt, vel, W.vhist.as<float4>(), W.out.as<float>(), nv,
                                                    float(h), float(h * g[0]), float(h * g[1]), float(h * g[2]),
                                                    float(h * h * kWarmG0));
}

void launch_warm_extrapolate(const WarmStart &W, float4 *pos, const float4 *tgt, const float4 *vel, int nv, double h,
                             const double *g, cudaStream_t st)
{
    if (nv == 0) return;
    warm_extrapolate_kernel<<<grid_for(nv), 256, 0, st>>>(pos, tgt, vel, W.vhist.as<float4>(), nv, float(h),
                                                          float(h * g[0]), float(h * g[1]), float(h * g[2]));
}

void launch_warm_select(const WarmStart &W, float4 *pos, const float4 *tgt, const float4 *vel, int nv, double h,
                        const double *g, bool three_way, int *counters, cudaStream_t st)
{
    if (nv == 0) return;
    warm_select_kernel<<<grid_for(nv), 256, 0, st>>>(pos, tgt, vel, W.vhist.as<float4>(), W.wres.as<double>(), nv,
                                                     three_way, float(h), float(h * g[0]), float(h * g[1]),
                                                     float(h * g[2]), counters);
}

void launch_warm_probe_select(const WarmStart &W, float4 *pos, const float4 *saved, int nv, int *counters,
                              cudaStream_t st)
{
    warm_probe_select_kernel<<<grid_for(std::max(1, nv)), 256, 0, st>>>(pos, saved, W.wres.as<double>(), nv,
                                                                       counters);
}

void launch_warm_targets(const float4 *pos, const float4 *tgt, int nv, double h, float *targets, cudaStream_t st)
{
    if (nv == 0) return;
    warm_targets_kernel<<<grid_for(nv), 256, 0, st>>>(pos, tgt, nv, float(1.0 / (h * h * kWarmG0)), targets);
}

}  // namespace spgx
