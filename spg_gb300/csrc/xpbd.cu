// GB300 XPBD: one colour phase per (energy slot, stencil colour), thread per stencil.
// Restates spg::solver::XPBD::step (spg/source/sim/solver/xpbd.cpp:16-131) with the block
// projection of StencilBlockEnergy::projectPosition (energy.h:117-153) and SpringEnergy's
// own projection (springEnergy.cpp:48-68). Stencils of one colour share no vertex, so every
// phase updates disjoint vertices.
#include <cuda_runtime.h>

#include <algorithm>
#include <memory>
#include <vector>

#include "api_internal.h"
#include "devbuf.h"
#include "device_common.cuh"
#include "layout.h"
#include "state.h"
#include "vbd_solver.h"

namespace spgx {

// Work item: (type << 28) | element index in the type's table (types 1..5 keep the item
// non-negative; tables are limited to 2^28 elements). Energies of types 6-13 share the tag
// kItemGeneric and index the generic element table.
constexpr int kItemShift = 28;
constexpr int kItemMask = (1 << kItemShift) - 1;
constexpr int kItemGeneric = 6;

// Position loads of the projections. Separate phase launches read positions plainly (through
// L1, which measured 14 % faster on the 513x513 cloth than L2-only loads); the dataflow
// kernel, whose CTAs read positions that other CTAs of the same launch wrote, reads them from
// L2 (ld.global.cg), never from a possibly stale L1 line.
template <bool kCoh>
__device__ __forceinline__ float4 ldp(const float4 *p)
{
    if (kCoh) return __ldcg(p);
    return *p;
}

template <bool kCoh>
__device__ __forceinline__ void add_delta(float4 *pos, int v, V3f dx)
{
    float4 d = ldp<kCoh>(pos + 2 * v + 1);
    d.x += dx.x;
    d.y += dx.y;
    d.z += dx.z;
    pos[2 * v + 1] = d;
}

// A = gradC^T W gradC + compliance / h^2 + 1e-10 I; dlambda = -A^-1 C; dx_j = w_j gradC_j dlambda.
template <int S, int NC, bool kCoh>
__device__ __forceinline__ void project_block(float4 *pos, const int *idx, const float *w, const float *C,
                                              const V3f *grad, const float *cmp, float invh2)
{
    float A[NC][NC];
#pragma unroll
    for (int r = 0; r < NC; ++r)
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int j = 0; j < S; ++j) acc += w[j] * dot(grad[r * S + j], grad[c * S + j]);
            A[r][c] = acc + cmp[r * NC + c] * invh2 + (r == c ? 1e-10f : 0.f);
        }
    float dl[NC];
    if (NC == 1) {
        dl[0] = -C[0] / A[0][0];
    } else if (NC == 4) {
        // Gaussian elimination (A is symmetric positive definite plus the compliance).
        float M[NC][NC + 1];
#pragma unroll
        for (int r = 0; r < NC; ++r) {
#pragma unroll
            for (int c = 0; c < NC; ++c) M[r][c] = A[r][c];
            M[r][NC] = -C[r];
        }
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const float ip = 1.f / M[k][k];
#pragma unroll
            for (int r = k + 1; r < NC; ++r) {
                const float f = M[r][k] * ip;
#pragma unroll
                for (int c = k; c <= NC; ++c) M[r][c] -= f * M[k][c];
            }
        }
#pragma unroll
        for (int k = NC - 1; k >= 0; --k) {
            float acc = M[k][NC];
#pragma unroll
            for (int c = k + 1; c < NC; ++c) acc -= M[k][c] * dl[c];
            dl[k] = acc / M[k][k];
        }
    } else if (NC == 2) {
        const float det = A[0][0] * A[1][1] - A[0][1] * A[1][0];
        dl[0] = -(A[1][1] * C[0] - A[0][1] * C[1]) / det;
        dl[1] = -(-A[1][0] * C[0] + A[0][0] * C[1]) / det;
    } else {
        const float c00 = A[1][1] * A[2][2] - A[1][2] * A[2][1];
        const float c01 = A[1][2] * A[2][0] - A[1][0] * A[2][2];
        const float c02 = A[1][0] * A[2][1] - A[1][1] * A[2][0];
        const float det = A[0][0] * c00 + A[0][1] * c01 + A[0][2] * c02;
        const float id = 1.f / det;
        const float I00 = c00 * id, I01 = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) * id,
                    I02 = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) * id;
        const float I10 = c01 * id, I11 = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) * id,
                    I12 = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) * id;
        const float I20 = c02 * id, I21 = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) * id,
                    I22 = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) * id;
        dl[0] = -(I00 * C[0] + I01 * C[1] + I02 * C[2]);
        dl[1] = -(I10 * C[0] + I11 * C[1] + I12 * C[2]);
        dl[2] = -(I20 * C[0] + I21 * C[1] + I22 * C[2]);
    }
#pragma unroll
    for (int j = 0; j < S; ++j) {
        V3f dx = mk(0.f, 0.f, 0.f);
#pragma unroll
        for (int c = 0; c < NC; ++c) dx = dx + (w[j] * dl[c]) * grad[c * S + j];
        add_delta<kCoh>(pos, idx[j], dx);
    }
}

// StencilBlockEnergy::projectPosition (energy.h:117-153) for the energies of types 6-13: the
// constraint gradients with respect to each stencil vertex come from the per-vertex
// forward-mode evaluation, one vertex at a time.
template <int S, int NC, bool kCoh>
__device__ __forceinline__ void xpbd_generic_project(float4 *pos, const int *idx, const float *w, int type,
                                                     const V3f *p, const float *prm, float invh2)
{
    float C[NC];
    V3f g[NC * S];
#pragma unroll
    for (int j = 0; j < S; ++j) {
        VAD<float> c[4];
        generic_constraints(type, p, j, prm, c);
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            g[k * S + j] = mk(c[k].g[0], c[k].g[1], c[k].g[2]);
            if (j == 0) C[k] = c[k].v;
        }
    }
    float cmp[NC * NC];
#pragma unroll
    for (int r = 0; r < NC; ++r)
#pragma unroll
        for (int c = 0; c < NC; ++c) cmp[r * NC + c] = r == c ? generic_compliance(type, prm, r) : 0.f;
    project_block<S, NC, kCoh>(pos, idx, w, C, g, cmp, invh2);
}

template <bool kCoh>
__device__ __noinline__ void xpbd_generic(const DevTables &T, float4 *pos, const float *__restrict__ invm, int e,
                                          float invh2)
{
    const int4 ix = __ldg(T.gen_idx + e);
    const int4 info = __ldg(T.gen_info + e);
    const int type = info.x, S = info.z;
    const float *prm = T.gen_prm + info.y;
    const int idx[4] = {ix.x, ix.y, ix.z, ix.w};
    const V3f b0 = v3(ldp<kCoh>(pos + 2 * ix.x)), d0 = v3(ldp<kCoh>(pos + 2 * ix.x + 1));
    V3f p[4];
    float w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        p[j] = (j == 0 || j >= S) ? mk(0.f, 0.f, 0.f) : (v3(ldp<kCoh>(pos + 2 * idx[j])) - b0) + (v3(ldp<kCoh>(pos + 2 * idx[j] + 1)) - d0);
        w[j] = j < S ? __ldg(invm + idx[j]) : 0.f;
    }
    switch (type) {
    case SPGX_ENERGY_STVK:
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: xpbd_generic_project<4, 2, kCoh>(pos, idx, w, type, p, prm, invh2); break;
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN: xpbd_generic_project<3, 3, kCoh>(pos, idx, w, type, p, prm, invh2); break;
    case SPGX_ENERGY_MEMBRANE_CHOI: xpbd_generic_project<3, 4, kCoh>(pos, idx, w, type, p, prm, invh2); break;
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING: xpbd_generic_project<4, 1, kCoh>(pos, idx, w, type, p, prm, invh2); break;
    case SPGX_ENERGY_QUADRATIC_BENDING: xpbd_generic_project<4, 3, kCoh>(pos, idx, w, type, p, prm, invh2); break;
    default: xpbd_generic_project<2, 1, kCoh>(pos, idx, w, type, p, prm, invh2); break;  // continuum springs
    }
}

// Projects the constraints of one work item (one stencil).
// Type paths a kernel instance carries, beyond springs, bending and anchors: the register
// budget of a kernel is that of its heaviest path, so scenes without the heavy types run a
// lighter instance.
constexpr int kPathGeneric = 1, kPathStvk = 2, kPathSnh = 4;

template <int kPaths, bool kCoh>
__device__ __forceinline__ void project_item(const DevTables &T, float4 *pos, const float *__restrict__ invm, int item,
                                             float invh2)
{
    const int type = (item >> kItemShift) & 7;
    const int e = item & kItemMask;
    if ((kPaths & kPathGeneric) && type == kItemGeneric) {
        xpbd_generic<kCoh>(T, pos, invm, e, invh2);
        return;
    }
    if (!(kPaths & kPathStvk) && type == SPGX_ENERGY_MEMBRANE_STVK) return;
    if (!(kPaths & kPathSnh) && type == SPGX_ENERGY_STABLE_NEO_HOOKEAN) return;
    switch (type) {
    case SPGX_ENERGY_SPRING: {
        // SpringEnergy::projectPosition, springEnergy.cpp:48-68
        const int4 s = __ldg(T.springs + e);
        const float w0 = __ldg(invm + s.x), w1 = __ldg(invm + s.y);
        const float wSum = w0 + w1;
        if (wSum < 1e-6f) return;
        const V3f b0 = v3(ldp<kCoh>(pos + 2 * s.x)), d0 = v3(ldp<kCoh>(pos + 2 * s.x + 1));
        const V3f b1 = v3(ldp<kCoh>(pos + 2 * s.y)), d1 = v3(ldp<kCoh>(pos + 2 * s.y + 1));
        const V3f n = (b1 - b0) + (d1 - d0);
        const float d = sqrtf(dot(n, n));
        if (d < 1e-6f) return;
        const float alpha = __ldg(T.spring_cmp + e) * invh2;
        const float sc = (d - __int_as_float(s.z)) / (d * (wSum + alpha));
        const V3f corr = sc * n;
        add_delta<kCoh>(pos, s.x, w0 * corr);
        add_delta<kCoh>(pos, s.y, mk(0.f, 0.f, 0.f) - w1 * corr);
        break;
    }
    case SPGX_ENERGY_DISCRETE_BENDING: {
        const int4 st = __ldg(T.bend_idx + e);
        const float4 pr = __ldg(T.bend_prm + e);
        const int idx[4] = {st.x, st.y, st.z, st.w};
        const V3f b0 = v3(ldp<kCoh>(pos + 2 * st.x)), d0 = v3(ldp<kCoh>(pos + 2 * st.x + 1));
        V3f p[4];
        float w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            p[j] = j == 0 ? mk(0.f, 0.f, 0.f) : (v3(ldp<kCoh>(pos + 2 * idx[j])) - b0) + (v3(ldp<kCoh>(pos + 2 * idx[j] + 1)) - d0);
            w[j] = __ldg(invm + idx[j]);
        }
        float C[1];
        V3f g[4];
        bending_constraint(p, pr.x, C, g);
        const float cmp[1] = {pr.z};
        project_block<4, 1, kCoh>(pos, idx, w, C, g, cmp, invh2);
        break;
    }
    case SPGX_ENERGY_MEMBRANE_STVK: {
        if (!(kPaths & kPathStvk)) break;
        const int4 st = __ldg(T.stvk_idx + e);
        const float4 D4 = __ldg(T.stvk_D + e);
        const float4 Ca = __ldg(T.stvk_Ca + e), Cb = __ldg(T.stvk_Cb + e);
        const float Cc = __ldg(T.stvk_Cc + e);
        const int idx[3] = {st.x, st.y, st.z};
        const V3f b0 = v3(ldp<kCoh>(pos + 2 * st.x)), d0 = v3(ldp<kCoh>(pos + 2 * st.x + 1));
        V3f p[3];
        float w[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            p[j] = j == 0 ? mk(0.f, 0.f, 0.f) : (v3(ldp<kCoh>(pos + 2 * idx[j])) - b0) + (v3(ldp<kCoh>(pos + 2 * idx[j] + 1)) - d0);
            w[j] = __ldg(invm + idx[j]);
        }
        const float D[4] = {D4.x, D4.y, D4.z, D4.w};
        float C[3];
        V3f g[9];
        stvk_constraints(p, D, C, g);
        const float cmp[9] = {Ca.x, Ca.y, Ca.z, Ca.w, Cb.x, Cb.y, Cb.z, Cb.w, Cc};
        project_block<3, 3, kCoh>(pos, idx, w, C, g, cmp, invh2);
        break;
    }
    default: {
        if (!(kPaths & kPathSnh)) break;
        const int4 st = __ldg(T.snh_idx + e);
        const float4 a = __ldg(T.snh_p0 + e), b = __ldg(T.snh_p1 + e), c = __ldg(T.snh_p2 + e);
        const float2 cm = __ldg(T.snh_cmp + e);
        const int idx[4] = {st.x, st.y, st.z, st.w};
        const V3f b0 = v3(ldp<kCoh>(pos + 2 * st.x)), d0 = v3(ldp<kCoh>(pos + 2 * st.x + 1));
        V3f p[4];
        float w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            p[j] = j == 0 ? mk(0.f, 0.f, 0.f) : (v3(ldp<kCoh>(pos + 2 * idx[j])) - b0) + (v3(ldp<kCoh>(pos + 2 * idx[j] + 1)) - d0);
            w[j] = __ldg(invm + idx[j]);
        }
        const float D[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x};
        float C[2];
        V3f g[8];
        snh_constraints(p, D, c.w, C, g);
        const float cmp[4] = {cm.x, 0.f, 0.f, cm.y};
        project_block<4, 2, kCoh>(pos, idx, w, C, g, cmp, invh2);
        break;
    }
    }
}

// Anchors are projected by their own kernel because their stencil is a single vertex that is
// not part of the element record (StencilBlockEnergy::projectPosition with the anchor
// constraint, springAnchorEnergy.cpp:8-19).
template <bool kCoh>
__device__ __forceinline__ void project_anchor(const DevTables &T, const int *__restrict__ anchor_v, float4 *pos,
                                               const float *__restrict__ invm, int item, float invh2)
{
    const int e = item & kItemMask;
    const float4 a = __ldg(T.anchors + e);
    const int v = __ldg(anchor_v + e);
    const V3f xa = (v3(ldp<kCoh>(pos + 2 * v)) - mk(a.x, a.y, a.z)) + v3(ldp<kCoh>(pos + 2 * v + 1));
    float C[1];
    V3f g[1];
    anchor_constraint(xa, mk(0.f, 0.f, 0.f), C, g);
    const float w[1] = {__ldg(invm + v)};
    const int idx[1] = {v};
    const float cmp[1] = {__ldg(T.anchor_cmp + e).x};
    project_block<1, 1, kCoh>(pos, idx, w, C, g, cmp, invh2);
}

// Work item t of a phase: item0 + t when the phase covers consecutive elements of one type
// (item0 >= 0), else the phase's item list.
__device__ __forceinline__ int phase_item(const int *__restrict__ items, int item0, int t)
{
    return item0 >= 0 ? item0 + t : __ldg(items + t);
}

template <int kPaths>
__global__ void __launch_bounds__(256) xpbd_phase_kernel(const DevTables T, float4 *pos, const float *__restrict__ invm,
                                                         const int *__restrict__ items, int item0, int n, float invh2)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) project_item<kPaths, false>(T, pos, invm, phase_item(items, item0, t), invh2);
}

__global__ void xpbd_anchor_kernel(const DevTables T, const int *__restrict__ anchor_v, float4 *pos,
                                   const float *__restrict__ invm, const int *__restrict__ items, int item0, int n,
                                   float invh2)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) project_anchor<false>(T, anchor_v, pos, invm, phase_item(items, item0, t), invh2);
}

// ---------------------------------------------------------------------------------------
// Dataflow XPBD: every substep of a step in one persistent cooperative launch, with no
// barrier between projection phases or substeps.
//
// Each phase's work items are cut into chunks of kXpbdChunk consecutive items (one CTA task,
// one thread per item). A task is (substep, chunk), handed out in (substep, phase, chunk)
// order by an atomic ticket. Per vertex, the chunks that touch it form a chain in phase order;
// a chunk waits for the previous chunk of the chain of each of its vertices to have finished
// this substep and, for the vertices whose chain it starts, for the chain's last chunk to have
// finished the previous substep. That is the order of the reference's phase loop
// (xpbd.cpp:79-106): every read of a vertex sees the writes of all earlier phases and none of
// the later ones. The chain's first chunk also runs the vertex's inertial prediction
// (xpbd.cpp:44-74) before its projections, and its last chunk the velocity update
// (xpbd.cpp:111-120) after them. Every wait is on a smaller ticket, held by a co-resident CTA,
// so waits end; each is still bounded, and a wait that gives up aborts the launch with status
// bit 1, as in the VBD dataflow kernel.
constexpr int kXpbdChunk = 128;
constexpr int kXpbdMaxPolls = 1 << 21;

struct XpbdFlowView {
    const int4 *chunk;   // per chunk: {first item, items, first dependency, dependencies}
    const int4 *chunkv;  // per chunk: {first predicted vertex, count, first velocity vertex, count}
    const int *deps;     // chunk id, bit 31 set when it is awaited for the same substep
    const int *verts;    // the predicted and velocity-updated vertex lists
    int *epoch;          // per chunk: substeps completed (monotonic over launches)
    int *ticket;         // [0] next task, [1] abort flag (zeroed before a launch)
};

// Inertial prediction and velocity update with L2-coherent loads (the vertex's previous
// updates come from other CTAs of the same launch); the arithmetic of begin_substep_vertex and
// end_substep_vertex (substep.cuh).
__device__ __forceinline__ void xpbd_predict_vertex(float4 *pos, float4 *tgt, float4 *dold, float4 *vel, int i,
                                                    float h, float gx, float gy, float gz)
{
    const float4 b = __ldcg(pos + 2 * i);
    const float4 d = __ldcg(pos + 2 * i + 1);
    float4 v = __ldcg(vel + i);
    const float mass = __ldcg(tgt + i).w;
    float sx[3], r[3];
    const float bb[3] = {b.x, b.y, b.z}, dd[3] = {d.x, d.y, d.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        sx[k] = bb[k] + dd[k];
        const float t = sx[k] - bb[k];
        r[k] = (bb[k] - (sx[k] - t)) + (dd[k] - t);
    }
    v.x += h * gx;
    v.y += h * gy;
    v.z += h * gz;
    const float4 y = make_float4(r[0] + h * v.x, r[1] + h * v.y, r[2] + h * v.z, 0.f);
    pos[2 * i] = make_float4(sx[0], sx[1], sx[2], b.w);
    pos[2 * i + 1] = y;
    dold[i] = make_float4(r[0], r[1], r[2], 0.f);
    tgt[i] = make_float4(y.x, y.y, y.z, mass);
    vel[i] = v;
}

__device__ __forceinline__ void xpbd_velocity_vertex(const float4 *pos, const float4 *dold, float4 *vel, int i,
                                                     float invh)
{
    const float4 d = __ldcg(pos + 2 * i + 1);
    const float4 o = __ldcg(dold + i);
    vel[i] = make_float4((d.x - o.x) * invh, (d.y - o.y) * invh, (d.z - o.z) * invh, 0.f);
}

// Between two substeps of the phase launches: the velocity update of the one that ended and the
// inertial prediction of the next, in one pass (each touches one vertex only).
__global__ void xpbd_between_substeps_kernel(float4 *pos, float4 *tgt, float4 *dold, float4 *vel, int nv, float invh,
                                             float h, float gx, float gy, float gz)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    xpbd_velocity_vertex(pos, dold, vel, i, invh);
    xpbd_predict_vertex(pos, tgt, dold, vel, i, h, gx, gy, gz);
}

template <int kPaths>
__global__ void __launch_bounds__(kXpbdChunk) xpbd_flow_kernel(const DevTables T, float4 *pos, float4 *tgt,
                                                               float4 *dold, float4 *vel,
                                                               const float *__restrict__ invm,
                                                               const int *__restrict__ items,
                                                               const int *__restrict__ anchor_v,
                                                               const XpbdFlowView F, int n_chunks, int substeps,
                                                               int epoch_base, float h, float invh, float invh2,
                                                               float gx, float gy, float gz, unsigned int *status)
{
    __shared__ int s_task, s_fail;
    const int total = substeps * n_chunks;
    for (;;) {
        if (threadIdx.x == 0) s_task = ld_relaxed_gpu(F.ticket + 1) ? total : atomicAdd(F.ticket, 1);
        __syncthreads();
        const int task = s_task;
        if (task >= total) break;
        const int s = task / n_chunks;
        const int c = task - s * n_chunks;
        const int4 ch = __ldg(F.chunk + c);
        // Wait for the chunks this one follows (warp 0, one dependency per lane).
        if (threadIdx.x < 32) {
            bool ok = true;
            for (int j = threadIdx.x; j < ch.w && ok; j += 32) {
                const int pk = __ldg(F.deps + ch.z + j);
                const int u = pk & 0x7fffffff;
                const int need = epoch_base + s + (pk < 0 ? 1 : 0);
                int polls = 0;
                while (ld_acquire_gpu(F.epoch + u) < need) {
                    if (++polls > kXpbdMaxPolls || ld_relaxed_gpu(F.ticket + 1)) {
                        ok = false;
                        break;
                    }
                    __nanosleep(64);
                }
            }
            ok = __all_sync(0xffffffffu, ok);
            if (threadIdx.x == 0) s_fail = !ok;
        }
        __syncthreads();
        if (s_fail) {
            if (threadIdx.x == 0) {
                atomicExch(F.ticket + 1, 1);
                atomicOr(status, 2u);
            }
            break;
        }
        const int4 cv = __ldg(F.chunkv + c);
        for (int i = threadIdx.x; i < cv.y; i += blockDim.x)
            xpbd_predict_vertex(pos, tgt, dold, vel, __ldg(F.verts + cv.x + i), h, gx, gy, gz);
        if (cv.y) __syncthreads();
        if (threadIdx.x < ch.y) {
            const int item = __ldg(items + ch.x + threadIdx.x);
            if (((item >> kItemShift) & 7) == SPGX_ENERGY_SPRING_ANCHOR)
                project_anchor<true>(T, anchor_v, pos, invm, item, invh2);
            else
                project_item<kPaths, true>(T, pos, invm, item, invh2);
        }
        if (cv.w) {
            __syncthreads();
            for (int i = threadIdx.x; i < cv.w; i += blockDim.x)
                xpbd_velocity_vertex(pos, dold, vel, __ldg(F.verts + cv.z + i), invh);
        }
        __syncthreads();  // every write of the task is done; the release below covers them
        if (threadIdx.x == 0) st_release_gpu(F.epoch + c, epoch_base + s + 1);
    }
}

// ---------------------------------------------------------------------------------------
// Synchronised XPBD: every substep of a step in one persistent cooperative launch, one CTA
// per SM, with a counting grid barrier after the prediction and after every
// projection phase instead of a kernel boundary (about 6 us per graph node on the 513^2
// cloth, whose substep has 28 phases). The phases, their work items and the per-item
// arithmetic are those of the phase launches (with L2-coherent loads), so the result is the
// same bit for bit. The velocity update of substep s-1 (xpbd.cpp:111-120) and the prediction
// of substep s (xpbd.cpp:44-74) touch one vertex each and run in one pass.
constexpr int kXpbdSyncThreads = 512;
constexpr int kXpbdSyncTimeout = 1;

struct XpbdSyncView {
    const int4 *phase;  // per phase: {first item, items, anchors, item0 (phase_item)}
    int n_phases;
    int *arrive;        // the grid barrier's counter (zeroed before each launch)
    int *status;        // kXpbdSyncTimeout when a barrier wait gave up
};

template <int kPaths>
__global__ void __launch_bounds__(kXpbdSyncThreads) xpbd_sync_kernel(const DevTables T, float4 *pos, float4 *tgt,
                                                                     float4 *dold, float4 *vel,
                                                                     const float *__restrict__ invm,
                                                                     const int *__restrict__ items,
                                                                     const int *__restrict__ anchor_v,
                                                                     const XpbdSyncView Y, int nv, int substeps,
                                                                     float h, float invh, float invh2, float gx,
                                                                     float gy, float gz)
{
    const int TT = gridDim.x * blockDim.x;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    int gen = 0;
    // Each CTA takes an equal contiguous share of a phase's items (all SMs work on every
    // phase); a thread's first item of the next phase, and the phase's table entry, are read
    // before the barrier that precedes it (the tables are read-only), so that after the barrier
    // only the element record and the positions remain on the dependency chain.
    auto share = [&](const int4 &ph, int &first, int &end) {
        const int per = (ph.y + int(gridDim.x) - 1) / int(gridDim.x);
        first = min(ph.y, int(blockIdx.x) * per);
        end = min(ph.y, first + per);
    };
    auto first_item = [&](const int4 &ph) {
        int f, e;
        share(ph, f, e);
        return f + int(threadIdx.x) < e ? phase_item(items + ph.x, ph.w, f + threadIdx.x) : -1;
    };
    for (int s = 0; s < substeps; ++s) {
        for (int i = g; i < nv; i += TT) {
            if (s > 0) xpbd_velocity_vertex(pos, dold, vel, i, invh);
            xpbd_predict_vertex(pos, tgt, dold, vel, i, h, gx, gy, gz);
        }
        int4 ph = Y.n_phases > 0 ? __ldg(Y.phase) : make_int4(0, 0, 0, 0);
        int item = first_item(ph);
        if (!grid_counter_sync(Y.arrive, Y.status, gen, kXpbdMaxPolls, kXpbdSyncTimeout)) return;
        for (int p = 0; p < Y.n_phases; ++p) {
            int f, e;
            share(ph, f, e);
            for (int t = f + threadIdx.x; t < e; t += blockDim.x) {
                const int it = t == f + int(threadIdx.x) ? item : phase_item(items + ph.x, ph.w, t);
                if (ph.z)
                    project_anchor<true>(T, anchor_v, pos, invm, it, invh2);
                else
                    project_item<kPaths, true>(T, pos, invm, it, invh2);
            }
            if (p + 1 < Y.n_phases) {
                ph = __ldg(Y.phase + p + 1);
                item = first_item(ph);
            }
            if (!grid_counter_sync(Y.arrive, Y.status, gen, kXpbdMaxPolls, kXpbdSyncTimeout)) return;
        }
    }
    for (int i = g; i < nv; i += TT) xpbd_velocity_vertex(pos, dold, vel, i, invh);
}

struct XpbdPhase {
    int offset;
    int count;
    bool anchors;
    int item0;  // the first item when the phase's items are consecutive elements of one type, else -1
};

struct XpbdSolver {
    SceneLayout L;
    spgx_xpbd_params P{};
    double h_sub{0.01};
    int device{0};
    int block{128};
    cudaStream_t stream{nullptr};
    cudaEvent_t ev0{nullptr}, ev1{nullptr};
    cudaGraphExec_t graph_exec{nullptr};
    bool graph_valid{false};
    ParticleState X;
    ElementBuffers EB;
    DevBuf d_items, d_anchor_v;
    DevTables T{};
    std::vector<XpbdPhase> phases;
    int paths{0};  // kPath* bits of the scene's energy types
    // Dataflow kernel (kernel 2): chunk tables, per-chunk substep counters, the ticket.
    DevBuf fx_chunk, fx_chunkv, fx_deps, fx_verts, fx_epoch, fx_ticket, d_status;
    XpbdFlowView FV{};
    int n_chunks{0};
    int flow_grid{0};
    int flow_epoch{0};
    std::vector<int32_t> items_host;
    // Synchronised kernel (kernel 3): the phase table, the barrier counter and status.
    DevBuf sy_phase, sy_sync;
    int sync_grid{0};
    bool stall_next{false};  // test hook: the next synchronised launch starts with an unreachable counter

    ~XpbdSolver()
    {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }

    static spgx_status check_params(const spgx_xpbd_params *p)
    {
        if (!p || !(p->dt > 0) || p->substeps < 1 || p->kernel < 0 || p->kernel > 3 ||
            (p->block_size != 0 && (p->block_size % 32 != 0 || p->block_size < 32 || p->block_size > 256))) {
            set_error("invalid XPBD parameters");
            return SPGX_ERR_INVALID_ARG;
        }
        return SPGX_OK;
    }

    spgx_status init(const spgx_scene_desc *scene, const spgx_xpbd_params *params)
    {
        std::string err;
        const spgx_status st = build_scene_layout(scene, true, L, err);
        if (st != SPGX_OK) {
            set_error(err);
            return st;
        }
        for (const auto &O : L.objects)
            for (int t : O.energy_types)
                if (t == SPGX_ENERGY_STATIC_LOAD) {  // the reference throws too (staticLoadEnergy.cpp:8-15)
                    set_error("Constraint-based load energy not implemented");
                    return SPGX_ERR_UNSUPPORTED_ENERGY;
                }
        SPGX_TRY_STATUS(check_params(params));
        P = *params;
        h_sub = P.dt / P.substeps;
        // One warp per block by default: a phase's few tens of thousands of stencils then spread
        // over every SM (513^2 cloth: 3.48 ms per step, against 3.55, 3.64 and 3.76 ms with 64,
        // 128 and 256 threads).
        block = P.block_size ? P.block_size : 32;
        SPGX_TRY_STATUS(select_device(P.device));
        device = P.device;
        SPGX_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        SPGX_CUDA(cudaEventCreate(&ev0));
        SPGX_CUDA(cudaEventCreate(&ev1));
        SPGX_TRY_STATUS(X.init(L));
        const size_t cap = size_t(1) << kItemShift;
        if (L.el.anchors.size() >= cap || L.el.springs.size() >= cap || L.el.bend_idx.size() >= cap ||
            L.el.stvk_idx.size() >= cap || L.el.snh_idx.size() >= cap || L.el.gen_idx.size() >= cap) {
            set_error("XPBD supports at most 2^28 stencils per energy type");
            return SPGX_ERR_INVALID_ARG;
        }
        // Phases: energy slot k, colour c (xpbd.cpp:84-95), over all objects at once. Anchors
        // run in their own phases so the generic kernel never branches to them.
        int max_e = 0;
        for (const auto &O : L.objects) max_e = std::max<int>(max_e, static_cast<int>(O.energy_types.size()));
        std::vector<int32_t> items;
        for (int k = 0; k < max_e; ++k) {
            int max_c = 0;
            for (const auto &O : L.objects)
                if (k < static_cast<int>(O.stencil_colors.size()))
                    for (int c : O.stencil_colors[k]) max_c = std::max(max_c, c + 1);
            for (int c = 0; c < max_c; ++c) {
                for (int anch = 0; anch < 2; ++anch) {
                    XpbdPhase ph{static_cast<int>(items.size()), 0, anch == 1, -1};
                    for (size_t o = 0; o < L.objects.size(); ++o) {
                        const auto &O = L.objects[o];
                        if (k >= static_cast<int>(O.stencil_colors.size())) continue;
                        const int type = O.energy_types[k];
                        if ((type == SPGX_ENERGY_SPRING_ANCHOR) != (anch == 1)) continue;
                        const auto &cols = O.stencil_colors[k];
                        for (int s = 0; s < static_cast<int>(cols.size()); ++s)
                            if (cols[s] == c)
                                items.push_back(((is_generic_type(type) ? kItemGeneric : type) << kItemShift) |
                                                (L.elem_base[o][k] + s));
                    }
                    ph.count = static_cast<int>(items.size()) - ph.offset;
                    if (ph.count > 0) phases.push_back(ph);
                }
            }
        }
        renumber_in_phase_order(items);
        SPGX_TRY_STATUS(EB.upload(el, T));
        SPGX_TRY_STATUS(EB.upload_generic(L, T));
        if (!el.gen_idx.empty()) {  // this handle's order of the generic elements (parameters stay put)
            SPGX_TRY_STATUS(EB.gen_idx.upload(el.gen_idx));
            SPGX_TRY_STATUS(EB.gen_info.upload(el.gen_info));
            T.gen_idx = EB.gen_idx.as<int4>();
            T.gen_info = EB.gen_info.as<int4>();
        }
        SPGX_TRY_STATUS(d_anchor_v.upload(el.anchor_v));
        SPGX_TRY_STATUS(d_items.upload(items));
        items_host = items;
        SPGX_TRY_STATUS(setup_paths());
        SPGX_TRY_STATUS(setup_sync());
        return setup_flow();
    }

    spgx_status setup_sync()
    {
        std::vector<I4> tab;
        for (const auto &ph : phases) tab.push_back(I4{ph.offset, ph.count, ph.anchors ? 1 : 0, ph.item0});
        if (tab.empty()) tab.push_back(I4{0, 0, 0, 0});
        SPGX_TRY_STATUS(sy_phase.upload(tab));
        SPGX_TRY_STATUS(sy_sync.alloc(2 * sizeof(int)));
        SPGX_CUDA(cudaMemset(sy_sync.as<void>(), 0, 2 * sizeof(int)));
        int sms = 0, per_sm = 0;
        SPGX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        SPGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sync_fn(), kXpbdSyncThreads, 0));
        if (per_sm < 1) {
            set_error("the synchronised XPBD kernel does not fit on an SM");
            return SPGX_ERR_CUDA;
        }
        sync_grid = sms;  // one CTA per SM: fewer barrier participants
        return SPGX_OK;
    }

    const void *sync_fn() const
    {
        switch (paths) {
        case 0: return reinterpret_cast<const void *>(xpbd_sync_kernel<0>);
        case 1: return reinterpret_cast<const void *>(xpbd_sync_kernel<1>);
        case 2: return reinterpret_cast<const void *>(xpbd_sync_kernel<2>);
        case 3: return reinterpret_cast<const void *>(xpbd_sync_kernel<3>);
        case 4: return reinterpret_cast<const void *>(xpbd_sync_kernel<4>);
        case 5: return reinterpret_cast<const void *>(xpbd_sync_kernel<5>);
        case 6: return reinterpret_cast<const void *>(xpbd_sync_kernel<6>);
        default: return reinterpret_cast<const void *>(xpbd_sync_kernel<7>);
        }
    }

    // Every substep of one step in one cooperative launch with grid barriers between phases.
    spgx_status launch_sync(cudaStream_t st)
    {
        SPGX_CUDA(cudaMemsetAsync(sy_sync.as<void>(), 0, 2 * sizeof(int), st));
        if (stall_next) {  // a counter no barrier reaches: every wait runs out its bounded polls
            SPGX_CUDA(cudaMemsetAsync(sy_sync.as<void>(), 0x80, sizeof(int), st));
            stall_next = false;
        }
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(static_cast<unsigned>(sync_grid));
        cfg.blockDim = dim3(kXpbdSyncThreads);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        float h = static_cast<float>(h_sub);
        float gx = static_cast<float>(P.gravity[0]), gy = static_cast<float>(P.gravity[1]),
              gz = static_cast<float>(P.gravity[2]);
        DevTables Tt = T;
        float4 *pos = X.pos(), *tgt = X.tgt(), *dold = X.dold(), *vel = X.vel();
        const float *invm = X.invm();
        const int *items = d_items.as<int>(), *av = d_anchor_v.as<int>();
        XpbdSyncView Y{sy_phase.as<int4>(), static_cast<int>(phases.size()), sy_sync.as<int>(), sy_sync.as<int>() + 1};
        int nv = L.nv, ns = P.substeps;
        float invh = static_cast<float>(1.0 / h_sub), invh2 = static_cast<float>(1.0 / (h_sub * h_sub));
        void *args[] = {&Tt, &pos, &tgt, &dold, &vel, &invm, &items, &av, &Y, &nv, &ns, &h, &invh, &invh2, &gx, &gy, &gz};
        SPGX_CUDA(cudaLaunchKernelExC(&cfg, sync_fn(), args));
        return SPGX_OK;
    }

    // This handle's element tables: each energy type's elements renumbered in the order the
    // phases visit them, so that a phase of one type covers consecutive elements. Its kernels
    // then take element first + t without reading a work-item list, and its record loads are
    // coalesced. The projections and their order per vertex are unchanged.
    ElementTables el;

    void renumber_in_phase_order(std::vector<int32_t> &items)
    {
        const ElementTables &E = L.el;
        el = E;
        std::vector<int32_t> next(8, 0);
        for (auto &it : items) {
            const int type = (it >> kItemShift) & 7;
            const int e = it & kItemMask;
            const int n = next[type]++;
            switch (type) {
            case SPGX_ENERGY_SPRING_ANCHOR:
                el.anchors[n] = E.anchors[e];
                el.anchor_v[n] = E.anchor_v[e];
                el.anchor_cmp[n] = E.anchor_cmp[e];
                break;
            case SPGX_ENERGY_SPRING:
                el.springs[n] = E.springs[e];
                el.spring_cmp[n] = E.spring_cmp[e];
                break;
            case SPGX_ENERGY_DISCRETE_BENDING:
                el.bend_idx[n] = E.bend_idx[e];
                el.bend_prm[n] = E.bend_prm[e];
                break;
            case SPGX_ENERGY_MEMBRANE_STVK:
                el.stvk_idx[n] = E.stvk_idx[e];
                el.stvk_D[n] = E.stvk_D[e];
                el.stvk_Ka[n] = E.stvk_Ka[e];
                el.stvk_Kb[n] = E.stvk_Kb[e];
                el.stvk_Ca[n] = E.stvk_Ca[e];
                el.stvk_Cb[n] = E.stvk_Cb[e];
                el.stvk_Cc[n] = E.stvk_Cc[e];
                break;
            case kItemGeneric:
                el.gen_idx[n] = E.gen_idx[e];
                el.gen_info[n] = E.gen_info[e];
                break;
            default:
                el.snh_idx[n] = E.snh_idx[e];
                el.snh_p0[n] = E.snh_p0[e];
                el.snh_p1[n] = E.snh_p1[e];
                el.snh_p2[n] = E.snh_p2[e];
                el.snh_cmp[n] = E.snh_cmp[e];
                break;
            }
            it = (type << kItemShift) | n;
        }
        // A phase whose items are one type's consecutive elements runs without its item list.
        for (auto &ph : phases) {
            ph.item0 = items[ph.offset];
            for (int t = 1; t < ph.count && ph.item0 >= 0; ++t)
                if (items[ph.offset + t] != ph.item0 + t) ph.item0 = -1;
        }
    }

    // Vertices of one work item (internal indices, this handle's element order).
    int item_vertices(int item, int *v) const
    {
        const int type = (item >> kItemShift) & 7;
        const int e = item & kItemMask;
        const ElementTables &E = el;
        switch (type) {
        case SPGX_ENERGY_SPRING_ANCHOR: v[0] = E.anchor_v[e]; return 1;
        case SPGX_ENERGY_SPRING: v[0] = E.springs[e].x, v[1] = E.springs[e].y; return 2;
        case SPGX_ENERGY_DISCRETE_BENDING: {
            const I4 &q = E.bend_idx[e];
            v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
            return 4;
        }
        case SPGX_ENERGY_MEMBRANE_STVK: {
            const I4 &q = E.stvk_idx[e];
            v[0] = q.x, v[1] = q.y, v[2] = q.z;
            return 3;
        }
        case kItemGeneric: {
            const I4 &q = E.gen_idx[e];
            const int n = E.gen_info[e].z;
            const int all[4] = {q.x, q.y, q.z, q.w};
            for (int j = 0; j < n; ++j) v[j] = all[j];
            return n;
        }
        default: {
            const I4 &q = E.snh_idx[e];
            v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
            return 4;
        }
        }
    }

    // Chunks of the dataflow kernel and the chain dependencies between them: per vertex, the
    // chunks that touch it in phase order. A chunk waits for its predecessor on every chain
    // (same substep) and, where it starts a chain, for the chain's last chunk (previous
    // substep). Vertices no chunk touches are predicted and updated by chunk 0, which then also
    // waits for its own previous substep.
    spgx_status setup_flow()
    {
        std::vector<I4> chunk;
        std::vector<std::vector<int32_t>> cdeps, cpred;
        std::vector<int32_t> last(std::max(1, L.nv), -1), first(std::max(1, L.nv), -1);
        int vv[4];
        for (const auto &ph : phases)
            for (int o = 0; o < ph.count; o += kXpbdChunk) {
                const int c = static_cast<int>(chunk.size());
                const int n = std::min(kXpbdChunk, ph.count - o);
                chunk.push_back(I4{ph.offset + o, n, 0, 0});
                cdeps.emplace_back();
                cpred.emplace_back();
                for (int i = 0; i < n; ++i) {
                    const int k = item_vertices(items_host[ph.offset + o + i], vv);
                    for (int j = 0; j < k; ++j) {
                        const int v = vv[j];
                        if (last[v] >= 0 && last[v] != c) {
                            cdeps[c].push_back(static_cast<int32_t>(uint32_t(last[v]) | 0x80000000u));
                        } else if (last[v] < 0) {
                            first[v] = c;
                            cpred[c].push_back(v);
                        }
                        last[v] = c;
                    }
                }
            }
        n_chunks = static_cast<int>(chunk.size());
        if (n_chunks == 0) return SPGX_OK;
        std::vector<std::vector<int32_t>> cend(n_chunks);
        for (int v = 0; v < L.nv; ++v) {
            if (last[v] >= 0) {
                cend[last[v]].push_back(v);
                cdeps[first[v]].push_back(last[v]);  // the chain's last chunk, previous substep
            } else {
                cpred[0].push_back(v);
                cend[0].push_back(v);
                cdeps[0].push_back(0);
            }
        }
        std::vector<int32_t> deps, verts;
        std::vector<I4> chunkv(n_chunks);
        for (int c = 0; c < n_chunks; ++c) {
            auto &d = cdeps[c];
            std::sort(d.begin(), d.end());
            d.erase(std::unique(d.begin(), d.end()), d.end());
            chunk[c].z = static_cast<int32_t>(deps.size());
            chunk[c].w = static_cast<int32_t>(d.size());
            deps.insert(deps.end(), d.begin(), d.end());
            chunkv[c].x = static_cast<int32_t>(verts.size());
            chunkv[c].y = static_cast<int32_t>(cpred[c].size());
            verts.insert(verts.end(), cpred[c].begin(), cpred[c].end());
            chunkv[c].z = static_cast<int32_t>(verts.size());
            chunkv[c].w = static_cast<int32_t>(cend[c].size());
            verts.insert(verts.end(), cend[c].begin(), cend[c].end());
        }
        if (deps.empty()) deps.push_back(0);
        if (verts.empty()) verts.push_back(0);
        SPGX_TRY_STATUS(fx_chunk.upload(chunk));
        SPGX_TRY_STATUS(fx_chunkv.upload(chunkv));
        SPGX_TRY_STATUS(fx_deps.upload(deps));
        SPGX_TRY_STATUS(fx_verts.upload(verts));
        SPGX_TRY_STATUS(fx_epoch.alloc(size_t(n_chunks) * sizeof(int)));
        SPGX_TRY_STATUS(fx_ticket.alloc(2 * sizeof(int)));
        FV = XpbdFlowView{fx_chunk.as<int4>(), fx_chunkv.as<int4>(), fx_deps.as<int>(), fx_verts.as<int>(),
                          fx_epoch.as<int>(), fx_ticket.as<int>()};
        SPGX_TRY_STATUS(d_status.alloc(sizeof(unsigned int)));
        SPGX_CUDA(cudaMemset(d_status.as<void>(), 0, sizeof(unsigned int)));
        int sms = 0, per_sm = 0;
        SPGX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        SPGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, flow_fn(), kXpbdChunk, 0));
        flow_grid = std::max(1, per_sm * sms);
        return reset_flow();
    }

    const void *flow_fn() const
    {
        switch (paths) {
        case 0: return reinterpret_cast<const void *>(xpbd_flow_kernel<0>);
        case 1: return reinterpret_cast<const void *>(xpbd_flow_kernel<1>);
        case 2: return reinterpret_cast<const void *>(xpbd_flow_kernel<2>);
        case 3: return reinterpret_cast<const void *>(xpbd_flow_kernel<3>);
        case 4: return reinterpret_cast<const void *>(xpbd_flow_kernel<4>);
        case 5: return reinterpret_cast<const void *>(xpbd_flow_kernel<5>);
        case 6: return reinterpret_cast<const void *>(xpbd_flow_kernel<6>);
        default: return reinterpret_cast<const void *>(xpbd_flow_kernel<7>);
        }
    }

    spgx_status reset_flow()
    {
        if (n_chunks == 0) return SPGX_OK;
        SPGX_CUDA(cudaMemsetAsync(fx_epoch.as<int>(), 0, size_t(n_chunks) * sizeof(int), stream));
        SPGX_CUDA(cudaStreamSynchronize(stream));
        flow_epoch = 0;
        return SPGX_OK;
    }

    // Every substep of one step in one cooperative launch (one resident wave of CTAs).
    spgx_status launch_flow(cudaStream_t st)
    {
        SPGX_CUDA(cudaMemsetAsync(FV.ticket, 0, 2 * sizeof(int), st));
        cudaLaunchConfig_t cfg{};
        const long long tasks = static_cast<long long>(P.substeps) * n_chunks;
        cfg.gridDim = dim3(static_cast<unsigned>(std::min<long long>(tasks, flow_grid)));
        cfg.blockDim = dim3(kXpbdChunk);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        float h = static_cast<float>(h_sub);
        float gx = static_cast<float>(P.gravity[0]), gy = static_cast<float>(P.gravity[1]),
              gz = static_cast<float>(P.gravity[2]);
        DevTables Tt = T;
        float4 *pos = X.pos(), *tgt = X.tgt(), *dold = X.dold(), *vel = X.vel();
        const float *invm = X.invm();
        const int *items = d_items.as<int>(), *av = d_anchor_v.as<int>();
        unsigned int *status = d_status.as<unsigned int>();
        int nc = n_chunks, ns = P.substeps, base = flow_epoch;
        float invh = static_cast<float>(1.0 / h_sub), invh2 = static_cast<float>(1.0 / (h_sub * h_sub));
        void *args[] = {&Tt, &pos, &tgt, &dold, &vel, &invm, &items, &av, &FV, &nc, &ns, &base, &h, &invh, &invh2,
                        &gx, &gy, &gz, &status};
        SPGX_CUDA(cudaLaunchKernelExC(&cfg, flow_fn(), args));
        flow_epoch += P.substeps;
        return SPGX_OK;
    }

    // The kernel instance carries only the type paths the scene needs.
    spgx_status setup_paths()
    {
        paths = (L.el.gen_idx.empty() ? 0 : kPathGeneric) | (L.el.stvk_idx.empty() ? 0 : kPathStvk) |
                (L.el.snh_idx.empty() ? 0 : kPathSnh);
        return SPGX_OK;
    }

    void launch_phase(int grid, cudaStream_t st, const int *items, int item0, int n, float invh2)
    {
        switch (paths) {
        case 0: xpbd_phase_kernel<0><<<grid, block, 0, st>>>(T, X.pos(), X.invm(), items, item0, n, invh2); break;
        case 1: xpbd_phase_kernel<1><<<grid, block, 0, st>>>(T, X.pos(), X.invm(), items, item0, n, invh2); break;
        case 2: xpbd_phase_kernel<2><<<grid, block, 0, st>>>(T, X.pos(), X.invm(), items, item0, n, invh2); break;
        case 3: xpbd_phase_kernel<3><<<grid, block, 0, st>>>(T, X.pos(), X.invm(), items, item0, n, invh2); break;
        case 4: xpbd_phase_kernel<4><<<grid, block, 0, st>>>(T, X.pos(), X.invm(), items, item0, n, invh2); break;
        case 5: xpbd_phase_kernel<5><<<grid, block, 0, st>>>(T, X.pos(), X.invm(), items, item0, n, invh2); break;
        case 6: xpbd_phase_kernel<6><<<grid, block, 0, st>>>(T, X.pos(), X.invm(), items, item0, n, invh2); break;
        default: xpbd_phase_kernel<7><<<grid, block, 0, st>>>(T, X.pos(), X.invm(), items, item0, n, invh2); break;
        }
    }

    void launch_phases(cudaStream_t st)
    {
        const float invh2 = static_cast<float>(1.0 / (h_sub * h_sub));
        for (const auto &ph : phases) {
            const int grid = (ph.count + block - 1) / block;
            if (ph.anchors)
                xpbd_anchor_kernel<<<grid, block, 0, st>>>(T, d_anchor_v.as<int>(), X.pos(), X.invm(),
                                                           d_items.as<int>() + ph.offset, ph.item0, ph.count, invh2);
            else
                launch_phase(grid, st, d_items.as<int>() + ph.offset, ph.item0, ph.count, invh2);
        }
    }

    void launch_step(cudaStream_t st)
    {
        launch_begin_substep(X, h_sub, P.gravity, st);
        for (int s = 0; s < P.substeps; ++s) {
            launch_phases(st);
            if (s + 1 < P.substeps && L.nv > 0)
                xpbd_between_substeps_kernel<<<(L.nv + 255) / 256, 256, 0, st>>>(
                    X.pos(), X.tgt(), X.dold(), X.vel(), L.nv, static_cast<float>(1.0 / h_sub), static_cast<float>(h_sub),
                    static_cast<float>(P.gravity[0]), static_cast<float>(P.gravity[1]),
                    static_cast<float>(P.gravity[2]));
        }
        launch_end_substep(X, h_sub, st);
    }

    spgx_status build_graph()
    {
        if (graph_exec) {
            cudaGraphExecDestroy(graph_exec);
            graph_exec = nullptr;
        }
        cudaGraph_t g = nullptr;
        SPGX_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        launch_step(stream);
        const cudaError_t ce = cudaStreamEndCapture(stream, &g);
        if (ce != cudaSuccess) {
            set_error(std::string("graph capture failed: ") + cudaGetErrorString(ce));
            return SPGX_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(&graph_exec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            set_error(std::string("graph instantiation failed: ") + cudaGetErrorString(ie));
            return SPGX_ERR_CUDA;
        }
        graph_valid = true;
        return SPGX_OK;
    }

    spgx_status step(spgx_step_stats *stats)
    {
        SPGX_TRY_STATUS(X.upload_if_dirty(stream));
        X.mark_device_advanced();
        SPGX_CUDA(cudaEventRecord(ev0, stream));
        const bool flow = P.kernel == 2 && n_chunks > 0;
        const bool sync = P.kernel == 3 && L.nv > 0;
        if (flow) {
            SPGX_TRY_STATUS(launch_flow(stream));
        } else if (sync) {
            SPGX_TRY_STATUS(launch_sync(stream));
        } else if (P.use_graph) {
            if (!graph_valid) SPGX_TRY_STATUS(build_graph());
            SPGX_CUDA(cudaGraphLaunch(graph_exec, stream));
        } else {
            launch_step(stream);
        }
        SPGX_CUDA(cudaEventRecord(ev1, stream));
        SPGX_CUDA(cudaGetLastError());
        SPGX_CUDA(cudaStreamSynchronize(stream));
        if (flow) {
            unsigned int hs = 0;
            SPGX_CUDA(cudaMemcpy(&hs, d_status.as<void>(), sizeof(hs), cudaMemcpyDeviceToHost));
            if (hs & 2u) {
                SPGX_CUDA(cudaMemset(d_status.as<void>(), 0, sizeof(unsigned int)));
                SPGX_TRY_STATUS(reset_flow());
                set_error("an XPBD dataflow wait gave up (bounded poll); the step did not complete");
                return SPGX_ERR_TIMEOUT;
            }
        }
        if (sync) {
            int hs[2] = {0, 0};
            SPGX_CUDA(cudaMemcpy(hs, sy_sync.as<void>(), sizeof(hs), cudaMemcpyDeviceToHost));
            if (hs[1] == kXpbdSyncTimeout) {
                set_error("an XPBD grid barrier wait gave up (bounded poll); the step did not complete");
                return SPGX_ERR_TIMEOUT;
            }
        }

        float ms = 0.f;
        SPGX_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        if (stats) {
            *stats = spgx_step_stats{};
            stats->iterations = P.substeps;
            stats->converged = 1;
            stats->device_ms = ms;
        }
        return SPGX_OK;
    }
};

}  // namespace spgx

using spgx::XpbdSolver;

struct spgx_xpbd {
    std::unique_ptr<XpbdSolver> s;
};

#define SPGX_XHANDLE(h)                                \
    if (!(h)) {                                        \
        spgx::set_error("NULL solver handle");         \
        return SPGX_ERR_INVALID_ARG;                   \
    }                                                  \
    SPGX_CUDA(cudaSetDevice((h)->s->device))

extern "C" {

spgx_status spgx_xpbd_create(const spgx_scene_desc *scene, const spgx_xpbd_params *params, spgx_xpbd **out)
{
    SPGX_GUARD_BEGIN
    if (!out) {
        spgx::set_error("out is NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    *out = nullptr;
    spgx_xpbd_params p;
    if (params)
        p = *params;
    else
        spgx_xpbd_params_default(&p);
    auto h = std::make_unique<spgx_xpbd>();
    h->s = std::make_unique<XpbdSolver>();
    SPGX_TRY_STATUS(h->s->init(scene, &p));
    *out = h.release();
    spgx::clear_error();
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_xpbd_destroy(spgx_xpbd *h)
{
    SPGX_GUARD_BEGIN
    if (h) {
        cudaSetDevice(h->s->device);
        delete h;
    }
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_xpbd_set_params(spgx_xpbd *h, const spgx_xpbd_params *params)
{
    SPGX_GUARD_BEGIN
    SPGX_XHANDLE(h);
    SPGX_TRY_STATUS(XpbdSolver::check_params(params));
    if (params->device != h->s->device) {
        spgx::set_error("the device of a solver cannot change");
        return SPGX_ERR_INVALID_ARG;
    }
    h->s->P = *params;
    h->s->h_sub = params->dt / params->substeps;
    h->s->block = params->block_size ? params->block_size : 128;
    h->s->graph_valid = false;
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_xpbd_step(spgx_xpbd *h, spgx_step_stats *stats)
{
    SPGX_GUARD_BEGIN
    SPGX_XHANDLE(h);
    return h->s->step(stats);
    SPGX_GUARD_END
}

spgx_status spgx_xpbd_get_state(spgx_xpbd *h, int32_t object, double *x, double *v)
{
    SPGX_GUARD_BEGIN
    SPGX_XHANDLE(h);
    return h->s->X.get(h->s->L, object, x, v, h->s->stream);
    SPGX_GUARD_END
}

spgx_status spgx_xpbd_set_state(spgx_xpbd *h, int32_t object, const double *x, const double *v)
{
    SPGX_GUARD_BEGIN
    SPGX_XHANDLE(h);
    return h->s->X.set(h->s->L, object, x, v, h->s->stream);
    SPGX_GUARD_END
}

spgx_status spgx_xpbd_reset(spgx_xpbd *h)
{
    SPGX_GUARD_BEGIN
    SPGX_XHANDLE(h);
    return h->s->X.reset(h->s->L, h->s->stream);
    SPGX_GUARD_END
}

spgx_status spgx_xpbd_test_stall(spgx_xpbd *h)
{
    SPGX_GUARD_BEGIN
    SPGX_XHANDLE(h);
    auto &s = *h->s;
    if (s.P.kernel == 3 && s.L.nv > 0) {
        s.stall_next = true;
        return SPGX_OK;
    }
    if (s.P.kernel != 2 || s.n_chunks == 0) {
        spgx::set_error("the handle does not run the dataflow or the synchronised kernel");
        return SPGX_ERR_INVALID_ARG;
    }
    // The last chunk in ticket order ends every chain it is on, and the first chunk of each of
    // those chains waits for it at the start of a substep: with a counter no substep reaches,
    // those waits run out their bounded polls.
    const int never = -(1 << 30);
    SPGX_CUDA(cudaMemcpyAsync(s.fx_epoch.as<int>() + s.n_chunks - 1, &never, sizeof(int), cudaMemcpyHostToDevice,
                              s.stream));
    SPGX_CUDA(cudaStreamSynchronize(s.stream));
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_xpbd_get_stencil_colors(spgx_xpbd *h, int32_t object, int32_t energy, int32_t *colors)
{
    SPGX_GUARD_BEGIN
    if (!h || !colors || object < 0 || object >= static_cast<int>(h->s->L.objects.size())) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    const auto &O = h->s->L.objects[object];
    if (energy < 0 || energy >= static_cast<int>(O.stencil_colors.size())) {
        spgx::set_error("invalid energy index");
        return SPGX_ERR_INVALID_ARG;
    }
    std::copy(O.stencil_colors[energy].begin(), O.stencil_colors[energy].end(), colors);
    return SPGX_OK;
    SPGX_GUARD_END
}

}  // extern "C"
