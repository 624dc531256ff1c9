// Per-vertex bodies of the substep phases shared by the VBD and XPBD kernels (stand-alone
// launches in state.cu, and the persistent XPBD kernel).
#pragma once

#include <cuda_runtime.h>

namespace spgx {

// Inertial prediction shared by VBD (vbd.cpp:46-83) and XPBD (xpbd.cpp:44-74):
// v += h g; x_old = x; x += h v (and, for VBD, y = x). The base first advances to
// fl(base + delta) with the exact two-sum remainder kept as the new delta, so
// x_old = base + dold holds exactly.
__device__ __forceinline__ void begin_substep_vertex(float4 *pos, float4 *tgt, float4 *dold, float4 *vel, int i,
                                                     float h, float gx, float gy, float gz)
{
    const float4 b = pos[2 * i];
    const float4 d = pos[2 * i + 1];
    float4 v = vel[i];
    const float mass = tgt[i].w;
    float s[3], r[3];
    const float bb[3] = {b.x, b.y, b.z}, dd[3] = {d.x, d.y, d.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        s[k] = bb[k] + dd[k];
        const float t = s[k] - bb[k];
        r[k] = (bb[k] - (s[k] - t)) + (dd[k] - t);
    }
    v.x += h * gx;
    v.y += h * gy;
    v.z += h * gz;
    const float4 y = make_float4(r[0] + h * v.x, r[1] + h * v.y, r[2] + h * v.z, 0.f);
    pos[2 * i] = make_float4(s[0], s[1], s[2], b.w);
    pos[2 * i + 1] = y;
    dold[i] = make_float4(r[0], r[1], r[2], 0.f);
    tgt[i] = make_float4(y.x, y.y, y.z, mass);
    vel[i] = v;
}

// Velocity update (vbd.cpp:174-185, xpbd.cpp:111-120 -> particleGroup.cpp:65-72):
// v = (x - x_old) / h.
__device__ __forceinline__ void end_substep_vertex(const float4 *pos, const float4 *dold, float4 *vel, int i,
                                                   float invh)
{
    const float4 d = pos[2 * i + 1];
    const float4 o = dold[i];
    vel[i] = make_float4((d.x - o.x) * invh, (d.y - o.y) * invh, (d.z - o.z) * invh, 0.f);
}

}  // namespace spgx
