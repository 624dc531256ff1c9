// Device-side views of the solver state and element tables, and the per-vertex incidence
// accumulation shared by the VBD colour kernel and the residual kernel.
//
// State layout (internal, colour-major vertex order):
//   pos[2 v]     base position of the current step (x_n, FP32), w unused
//   pos[2 v + 1] delta from the base (x = base + delta), w unused
//   tgt[v]       inertial target as a delta from the base (y - base), w = mass
//   dold[v]      delta of x_old (the position at the start of the substep)
//   vel[v]       velocity
// Element evaluation subtracts bases and deltas separately, relative to the vertex being
// solved, so FP32 resolves the within-step motion far below the ulp of absolute positions.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "elements.cuh"
#include "generic.cuh"

namespace spgx {

struct DevTables {
    const float4 *anchors;
    const int4 *springs;
    const float *spring_cmp;
    const int4 *bend_idx;
    const float4 *bend_prm;
    const int4 *stvk_idx;
    const float4 *stvk_D;
    const float4 *stvk_Ka;
    const float4 *stvk_Kb;
    const float4 *stvk_Ca;
    const float4 *stvk_Cb;
    const float *stvk_Cc;
    const int4 *snh_idx;
    const float4 *snh_p0;
    const float4 *snh_p1;
    const float4 *snh_p2;
    const float2 *snh_cmp;
    const float2 *anchor_cmp;
    // Energies of types 6-14: per internal vertex gen_off[v]..gen_off[v+1] in gen_adj
    // ((element << 2) | slot); per element its vertices (gen_idx, -1 padded) and
    // {type, parameter offset, stencil size, 0} (gen_info); parameters in gen_prm.
    // gen_off is null when the scene has none.
    const int *gen_off;
    const int *gen_adj;
    const int4 *gen_idx;
    const int4 *gen_info;
    const float *gen_prm;
};

constexpr int kCounters = 8;

struct DevState {
    float4 *pos;
    float4 *tgt;
    float4 *dold;
    float4 *vel;
    const int4 *hdr;
    const int *adj;
    int *counters;          // [0] FP64 fallback solves, [1] det-guard skips, [3] learned guesses kept,
                            // [4] extrapolated guesses kept (kCounters ints; [2] is status)
    unsigned int *status;   // bit 0: non-finite update, bit 1: a bounded wait gave up
    // Dynamic anchors (interactive picking): n_pick one-stencil spring anchors, each pulling
    // internal vertex pick_v[q] towards pick_a[q].xyz with stiffness pick_a[q].w.
    int n_pick;
    const int *pick_v;
    const float4 *pick_a;
};

// Adds the dynamic anchors of vertex v (base b, delta d) to a force and Hessian diagonal:
// f -= k (x - a), H += k I, as SpringAnchorEnergy does for the energy appended last.
__device__ __forceinline__ void add_picks(const DevState &S, int v, float4 b, float4 d, float &f0, float &f1,
                                          float &f2, float &hd)
{
    for (int q = 0; q < S.n_pick; ++q)
        if (__ldg(S.pick_v + q) == v) {
            const float4 a = __ldg(S.pick_a + q);
            f0 -= a.w * ((b.x - a.x) + d.x);
            f1 -= a.w * ((b.y - a.y) + d.y);
            f2 -= a.w * ((b.z - a.z) + d.z);
            hd += a.w;
        }
}

typedef Vec3<float> V3f;

__device__ __forceinline__ V3f v3(float4 a) { return mk(a.x, a.y, a.z); }

// Position of vertex j relative to the vertex whose base/delta are (bs, ds).
__device__ __forceinline__ V3f rel_pos(const float4 *__restrict__ pos, int j, V3f bs, V3f ds)
{
    const float4 b = __ldg(pos + 2 * j);
    const float4 d = __ldg(pos + 2 * j + 1);
    return mk((b.x - bs.x) + (d.x - ds.x), (b.y - bs.y) + (d.y - ds.y), (b.z - bs.z) + (d.z - ds.z));
}

// The same as hi + lo, where lo is the rounding remainder of adding the base and delta
// differences (an error-free sum), for the spring stretch.
__device__ __forceinline__ V3f rel_pos2(const float4 *__restrict__ pos, int j, V3f bs, V3f ds, V3f &lo)
{
    const float4 b = __ldg(pos + 2 * j);
    const float4 d = __ldg(pos + 2 * j + 1);
    V3f hi;
    two_sum(b.x - bs.x, d.x - ds.x, hi.x, lo.x);
    two_sum(b.y - bs.y, d.y - ds.y, hi.y, lo.y);
    two_sum(b.z - bs.z, d.z - ds.z, hi.z, lo.z);
    return hi;
}

__device__ __forceinline__ int warp_max(int v) { return __reduce_max_sync(0xffffffffu, v); }

// Waits until the previous kernel on the stream has completed and its writes are visible
// (programmatic dependent launch); a no-op when the kernel was launched without it.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
// Lets the next kernel on the stream start launching once every CTA of this grid has called it
// or exited (the next kernel still waits in wait_prior_grid for this grid's completion).
__device__ __forceinline__ void allow_next_grid() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// GPU-scope acquire load / release store of a 32-bit counter (inter-CTA signalling).
__device__ __forceinline__ int ld_acquire_gpu(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int *p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_gpu(const int *p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Release add to a grid barrier's counter: the arriving CTA's writes (its threads' writes
// before the CTA barrier) are released with it.
__device__ __forceinline__ void red_add_release_gpu(int *p, int v)
{
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier number gen (counted from 0 within a cooperative launch): every CTA adds 1 to
// *arrive (zeroed before the launch) and waits until gridDim.x (gen + 1) arrivals have been
// counted; the acquire and the CTA barrier that follows make every CTA's earlier writes
// visible to all threads of this one. The wait is bounded (max_polls sleeps of 32 ns plus an
// L2 round trip each): one that runs out sets *status to timeout_code and the barrier returns
// false in every thread of this CTA.
__device__ __forceinline__ bool grid_counter_sync(int *arrive, int *status, int &gen, int max_polls, int timeout_code)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        red_add_release_gpu(arrive, 1);
        const int target = (gen + 1) * int(gridDim.x);
        int polls = 0, ok = 1;
        while (ld_acquire_gpu(arrive) < target) {
            if (++polls > max_polls) {
                atomicExch(status, timeout_code);
                ok = 0;
                break;
            }
            __nanosleep(32);
        }
        s_ok = ok;
    }
    ++gen;
    __syncthreads();
    return s_ok != 0;
}


// Walks the vertex's class-sorted incidence list with G lanes per vertex (lane-strided) and
// accumulates the force and Hessian block of every incident element into acc; with kGeneric
// also the vertex's incidences of energy types 6-14 (T.gen_off must then be set).
// Loop trip counts are warp-uniform (max over the warp), so all 32 lanes stay converged.
template <int G, bool kGeneric = false>
__device__ __forceinline__ void accumulate_incidences(const DevTables &T, const float4 *__restrict__ pos,
                                                      const int *__restrict__ adj, int4 h, int lane, V3f bs, V3f ds,
                                                      Block<float> &acc, int v)
{
    int off = h.x;
    const V3f zero = mk(0.f, 0.f, 0.f);
    // Anchors
    {
        const int n = h.y & 0xffff;
        const int rounds = warp_max((n + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < n) {
                const int e = __ldg(adj + off + i) >> 2;
                const float4 a = __ldg(T.anchors + e);
                const V3f xa = mk((bs.x - a.x) + ds.x, (bs.y - a.y) + ds.y, (bs.z - a.z) + ds.z);
                anchor_block(xa, zero, a.w, acc);
            }
        }
        off += n;
    }
    // Springs
    {
        const int n = (h.y >> 16) & 0xffff;
        const int rounds = warp_max((n + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < n) {
                const int ent = __ldg(adj + off + i);
                const int4 s = __ldg(T.springs + (ent >> 2));
                const int o = (ent & 3) ? s.x : s.y;
                V3f lo;
                const V3f po = rel_pos2(pos, o, bs, ds, lo);
                spring_block(zero, po, mk(-lo.x, -lo.y, -lo.z), __int_as_float(s.z), __int_as_float(s.w), acc);
            }
        }
        off += n;
    }
    // Bending, flap vertices (slots 2, 3)
    {
        const int n = h.z & 0xffff;
        const int rounds = warp_max((n + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < n) {
                const int ent = __ldg(adj + off + i);
                const int e = ent >> 2;
                const int slot = ent & 3;
                const int4 st = __ldg(T.bend_idx + e);
                const float4 pr = __ldg(T.bend_prm + e);
                const V3f p0 = rel_pos(pos, st.x, bs, ds);
                const V3f p1 = rel_pos(pos, st.y, bs, ds);
                const V3f po = rel_pos(pos, slot == 2 ? st.w : st.z, bs, ds);
                bending_flap_block(p0, p1, zero, po, slot == 2 ? pr.x : -pr.x, pr.y, acc);
            }
        }
        off += n;
    }
    // Bending, hinge vertices (slots 0, 1)
    {
        const int n = (h.z >> 16) & 0xffff;
        const int rounds = warp_max((n + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < n) {
                const int ent = __ldg(adj + off + i);
                const int e = ent >> 2;
                const int slot = ent & 3;
                const int4 st = __ldg(T.bend_idx + e);
                const float4 pr = __ldg(T.bend_prm + e);
                const V3f po = rel_pos(pos, slot == 1 ? st.x : st.y, bs, ds);
                const V3f pa = rel_pos(pos, st.z, bs, ds);
                const V3f pb = rel_pos(pos, st.w, bs, ds);
                bending_hinge_block(po, zero, pa, pb, slot == 1 ? pr.x : -pr.x, pr.y, acc);
            }
        }
        off += n;
    }
    // StVK membrane
    {
        const int n = h.w & 0xffff;
        const int rounds = warp_max((n + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < n) {
                const int ent = __ldg(adj + off + i);
                const int e = ent >> 2;
                const int slot = ent & 3;
                const int4 st = __ldg(T.stvk_idx + e);
                const float4 D4 = __ldg(T.stvk_D + e);
                const float4 Ka = __ldg(T.stvk_Ka + e);
                const float4 Kb = __ldg(T.stvk_Kb + e);
                V3f p[3];
                p[0] = slot == 0 ? zero : rel_pos(pos, st.x, bs, ds);
                p[1] = slot == 1 ? zero : rel_pos(pos, st.y, bs, ds);
                p[2] = slot == 2 ? zero : rel_pos(pos, st.z, bs, ds);
                const float D[4] = {D4.x, D4.y, D4.z, D4.w};
                const float Ks[6] = {Ka.x, Ka.y, Ka.z, Ka.w, Kb.x, Kb.y};
                stvk_block(p, slot, D, Ks, acc);
            }
        }
        off += n;
    }
    // Stable Neo-Hookean
    {
        const int n = (h.w >> 16) & 0xffff;
        const int rounds = warp_max((n + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < n) {
                const int ent = __ldg(adj + off + i);
                const int e = ent >> 2;
                const int slot = ent & 3;
                const int4 st = __ldg(T.snh_idx + e);
                const float4 a = __ldg(T.snh_p0 + e);
                const float4 b = __ldg(T.snh_p1 + e);
                const float4 c = __ldg(T.snh_p2 + e);
                V3f p[4];
                p[0] = slot == 0 ? zero : rel_pos(pos, st.x, bs, ds);
                p[1] = slot == 1 ? zero : rel_pos(pos, st.y, bs, ds);
                p[2] = slot == 2 ? zero : rel_pos(pos, st.z, bs, ds);
                p[3] = slot == 3 ? zero : rel_pos(pos, st.w, bs, ds);
                const float D[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x};
                snh_block(p, slot, D, c.y, c.z, c.w, acc);
            }
        }
    }
    // Energies of types 6-14 (v < 0: inactive lane of a partial group). A separate kernel
    // instantiation, so scenes without them keep the lean register budget.
    if (kGeneric) {
        int b = 0, n = 0;
        if (v >= 0) {
            b = __ldg(T.gen_off + v);
            n = __ldg(T.gen_off + v + 1) - b;
        }
        const int rounds = warp_max((n + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < n) {
                const int ent = __ldg(T.gen_adj + b + i);
                const int e = ent >> 2;
                const int slot = ent & 3;
                const int4 ix = __ldg(T.gen_idx + e);
                const int4 info = __ldg(T.gen_info + e);
                const int iv[4] = {ix.x, ix.y, ix.z, ix.w};
                V3f p[4];
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    p[j] = (j >= info.z || j == slot) ? zero : rel_pos(pos, iv[j], bs, ds);
                generic_block(info.x, p, slot, T.gen_prm + info.y, acc);
            }
        }
    }
}

// Sum of the 9 block entries over the G lanes of a vertex group (xor butterfly; every lane
// ends with the total).
template <int G>
__device__ __forceinline__ void group_reduce(Block<float> &acc)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 3; ++k) acc.f[k] += __shfl_xor_sync(0xffffffffu, acc.f[k], o);
#pragma unroll
        for (int k = 0; k < 6; ++k) acc.h[k] += __shfl_xor_sync(0xffffffffu, acc.h[k], o);
    }
}

// Three lanes per vertex (lanes 3g, 3g + 1, 3g + 2 of a warp): the first lane of each group
// ends with the total (the others, and the two idle lanes 30 and 31, with partial sums).
template <>
__device__ __forceinline__ void group_reduce<3>(Block<float> &acc)
{
#pragma unroll
    for (int k = 0; k < 3; ++k)
        acc.f[k] += __shfl_down_sync(0xffffffffu, acc.f[k], 1) + __shfl_down_sync(0xffffffffu, acc.f[k], 2);
#pragma unroll
    for (int k = 0; k < 6; ++k)
        acc.h[k] += __shfl_down_sync(0xffffffffu, acc.h[k], 1) + __shfl_down_sync(0xffffffffu, acc.h[k], 2);
}

}  // namespace spgx
