// Shared-memory tile kernel of the VBD colour phase (one CTA per tile of same-colour
// vertices; tile records are built by build_tiles, layout.h).
//
// 1. The CTA gathers the base/delta positions of its vertices and halo into shared memory.
// 2. It streams the tile's incidence records (coalesced, class by class) and adds each
//    record's force and Hessian block to a per-vertex accumulator in shared memory.
// 3. One thread per tile vertex adds the inertia term, solves the 3x3 system and writes the
//    new delta (or, for the residual, reduces |r|^2 in FP64).
#pragma once

#include "device_common.cuh"
#include "layout.h"

namespace spgx {

constexpr int kTileThreads = 128;

struct TileView {
    const int4 *hdr;
    const int *halo;
    const int4 *rec_anchor;
    const int4 *rec_spring;
    const int4 *rec_flap;
    const int4 *rec_hinge;
    const int4 *rec_stvk;
    const int4 *rec_snh;
};

// Dynamic shared memory: base[max_local], delta[max_local], acc[9][tile_vertices].
struct TileSmem {
    float4 *base;
    float4 *delta;
    float *acc;
    int stride;  // tile_vertices
    __device__ float &a(int k, int v) { return acc[k * stride + v]; }
};

__device__ __forceinline__ TileSmem tile_smem(int max_local, int tile_vertices)
{
    extern __shared__ float4 tile_dyn[];
    TileSmem sm;
    sm.base = tile_dyn;
    sm.delta = tile_dyn + max_local;
    sm.acc = reinterpret_cast<float *>(tile_dyn + 2 * max_local);
    sm.stride = tile_vertices;
    return sm;
}

inline size_t tile_smem_bytes(int max_local, int tile_vertices)
{
    return size_t(2 * max_local) * 16 + size_t(9 * tile_vertices) * 4;
}

// Position of local vertex j relative to local vertex s.
__device__ __forceinline__ V3f tile_rel(const TileSmem &sm, int j, int s)
{
    const float4 bj = sm.base[j], dj = sm.delta[j], bs = sm.base[s], ds = sm.delta[s];
    return mk((bj.x - bs.x) + (dj.x - ds.x), (bj.y - bs.y) + (dj.y - ds.y), (bj.z - bs.z) + (dj.z - ds.z));
}

__device__ __forceinline__ void tile_add(TileSmem &sm, int v, const Block<float> &b)
{
    atomicAdd(&sm.a(0, v), b.f[0]);
    atomicAdd(&sm.a(1, v), b.f[1]);
    atomicAdd(&sm.a(2, v), b.f[2]);
    atomicAdd(&sm.a(3, v), b.h[0]);
    atomicAdd(&sm.a(4, v), b.h[1]);
    atomicAdd(&sm.a(5, v), b.h[2]);
    atomicAdd(&sm.a(6, v), b.h[3]);
    atomicAdd(&sm.a(7, v), b.h[4]);
    atomicAdd(&sm.a(8, v), b.h[5]);
}

// Loads the tile's positions into shared memory, zeroes the accumulators and adds every
// incidence record. Returns the tile header's first entry {vstart, nvt, halo_off, n_halo}.
__device__ __forceinline__ int4 tile_accumulate(const TileView &V, const float4 *__restrict__ pos, int tile,
                                                TileSmem &sm)
{
    const int4 h0 = __ldg(V.hdr + 4 * tile);
    const int4 h1 = __ldg(V.hdr + 4 * tile + 1);
    const int4 h2 = __ldg(V.hdr + 4 * tile + 2);
    const int4 h3 = __ldg(V.hdr + 4 * tile + 3);
    const int nvt = h0.y, nl = h0.y + h0.w;
    for (int i = threadIdx.x; i < nl; i += blockDim.x) {
        const int g = i < nvt ? h0.x + i : __ldg(V.halo + h0.z + i - nvt);
        sm.base[i] = __ldg(pos + 2 * g);
        sm.delta[i] = __ldg(pos + 2 * g + 1);
    }
    for (int i = threadIdx.x; i < 9 * sm.stride; i += blockDim.x) sm.acc[i] = 0.f;
    __syncthreads();
    const V3f zero = mk(0.f, 0.f, 0.f);
    // Anchors: {self, k}, {ax, ay, az}
    for (int r = threadIdx.x; r < h2.z; r += blockDim.x) {
        const int4 a = __ldg(V.rec_anchor + 2 * (h1.x + r));
        const int4 p = __ldg(V.rec_anchor + 2 * (h1.x + r) + 1);
        const int s = a.x;
        const float4 b = sm.base[s], d = sm.delta[s];
        const V3f xa = mk((b.x - __int_as_float(p.x)) + d.x, (b.y - __int_as_float(p.y)) + d.y,
                          (b.z - __int_as_float(p.z)) + d.z);
        Block<float> blk;
        block_zero(blk);
        anchor_block(xa, zero, __int_as_float(a.y), blk);
        tile_add(sm, s, blk);
    }
    // Springs: {self | other << 16, L0, k}
    for (int r = threadIdx.x; r < h2.w; r += blockDim.x) {
        const int4 q = __ldg(V.rec_spring + h1.y + r);
        const int s = q.x & 0xffff;
        Block<float> blk;
        block_zero(blk);
        spring_block(zero, tile_rel(sm, q.x >> 16, s), __int_as_float(q.y), __int_as_float(q.z), blk);
        tile_add(sm, s, blk);
    }
    // Bending flaps: {self | p0 << 16, p1 | other flap << 16, signed theta0, k}
    for (int r = threadIdx.x; r < h3.x; r += blockDim.x) {
        const int4 q = __ldg(V.rec_flap + h1.z + r);
        const int s = q.x & 0xffff;
        Block<float> blk;
        block_zero(blk);
        bending_flap_block(tile_rel(sm, q.x >> 16, s), tile_rel(sm, q.y & 0xffff, s), zero, tile_rel(sm, q.y >> 16, s),
                           __int_as_float(q.z), __int_as_float(q.w), blk);
        tile_add(sm, s, blk);
    }
    // Bending hinges: {self | other hinge << 16, p2 | p3 << 16, signed theta0, k}
    for (int r = threadIdx.x; r < h3.y; r += blockDim.x) {
        const int4 q = __ldg(V.rec_hinge + h1.w + r);
        const int s = q.x & 0xffff;
        Block<float> blk;
        block_zero(blk);
        bending_hinge_block(tile_rel(sm, q.x >> 16, s), zero, tile_rel(sm, q.y & 0xffff, s), tile_rel(sm, q.y >> 16, s),
                            __int_as_float(q.z), __int_as_float(q.w), blk);
        tile_add(sm, s, blk);
    }
    // StVK: {i0 | i1 << 16, i2 | slot << 16, D0, D1}, {D2, D3, K00, K01}, {K02, K11, K12, K22}
    for (int r = threadIdx.x; r < h3.z; r += blockDim.x) {
        const int4 a = __ldg(V.rec_stvk + 3 * (h2.x + r));
        const int4 b = __ldg(V.rec_stvk + 3 * (h2.x + r) + 1);
        const int4 c = __ldg(V.rec_stvk + 3 * (h2.x + r) + 2);
        const int i0 = a.x & 0xffff, i1 = a.x >> 16, i2 = a.y & 0xffff, slot = a.y >> 16;
        const int s = slot == 0 ? i0 : (slot == 1 ? i1 : i2);
        V3f p[3];
        p[0] = tile_rel(sm, i0, s);
        p[1] = tile_rel(sm, i1, s);
        p[2] = tile_rel(sm, i2, s);
        const float D[4] = {__int_as_float(a.z), __int_as_float(a.w), __int_as_float(b.x), __int_as_float(b.y)};
        const float Ks[6] = {__int_as_float(b.z), __int_as_float(b.w), __int_as_float(c.x),
                             __int_as_float(c.y), __int_as_float(c.z), __int_as_float(c.w)};
        Block<float> blk;
        block_zero(blk);
        stvk_block(p, slot, D, Ks, blk);
        tile_add(sm, s, blk);
    }
    // SNH: {i0 | i1 << 16, i2 | i3 << 16, slot, D0}, {D1..D4}, {D5..D8}, {lambda, mu, alpha}
    for (int r = threadIdx.x; r < h3.w; r += blockDim.x) {
        const int4 a = __ldg(V.rec_snh + 4 * (h2.y + r));
        const int4 b = __ldg(V.rec_snh + 4 * (h2.y + r) + 1);
        const int4 c = __ldg(V.rec_snh + 4 * (h2.y + r) + 2);
        const int4 d = __ldg(V.rec_snh + 4 * (h2.y + r) + 3);
        const int i0 = a.x & 0xffff, i1 = a.x >> 16, i2 = a.y & 0xffff, i3 = a.y >> 16;
        const int slot = a.z;
        const int s = slot == 0 ? i0 : (slot == 1 ? i1 : (slot == 2 ? i2 : i3));
        V3f p[4];
        p[0] = tile_rel(sm, i0, s);
        p[1] = tile_rel(sm, i1, s);
        p[2] = tile_rel(sm, i2, s);
        p[3] = tile_rel(sm, i3, s);
        const float D[9] = {__int_as_float(a.w), __int_as_float(b.x), __int_as_float(b.y),
                            __int_as_float(b.z), __int_as_float(b.w), __int_as_float(c.x),
                            __int_as_float(c.y), __int_as_float(c.z), __int_as_float(c.w)};
        Block<float> blk;
        block_zero(blk);
        snh_block(p, slot, D, __int_as_float(d.x), __int_as_float(d.y), __int_as_float(d.z), blk);
        tile_add(sm, s, blk);
    }
    __syncthreads();
    return h0;
}

}  // namespace spgx
