// Shared-memory tile kernel of the VBD colour phase: one CTA per tile of same-colour vertices
// (tiles and records are built by build_tiles, layout.h), G lanes per vertex.
//
// 1. The CTA stages its tile's record block and the base/delta positions of its vertices and
//    halo into shared memory with asynchronous 16-byte copies (cp.async), so the whole tile
//    costs one header load, one halo-index load and one wave of copies of latency.
// 2. The G lanes of each vertex walk its records class by class (warp-uniform trip counts)
//    and accumulate the force and Hessian block in registers.
// 3. A shuffle reduction over the G lanes, then lane 0 adds the inertia term, solves the 3x3
//    system and writes the new delta (or, for the residual, reduces |r|^2 in FP64).
#pragma once

#include "device_common.cuh"
#include "layout.h"

namespace spgx {

constexpr int kTileThreads = 256;  // maximum threads per tile CTA (tile vertices x lanes)
// Tile sizes (vertices per tile) the launch autotuner tries when none is requested; the first
// is the tiling a solver starts with.
constexpr int kTileCandidates[2] = {32, 64};

struct TileView {
    const int4 *hdr;      // 2 per tile
    const int *halo;
    const int4 *records;
    const int *vrec;      // per internal vertex: record offset inside its tile's block
    int max_records;      // 16-byte record units of the largest tile
    // Energies of types 6-14 (null when the scene has none): per internal vertex the range of
    // its generic incidences (their count is the vertex's number of generic records), and the
    // FP32 parameter table the records point into.
    const int *gen_off;
    const float *gen_prm;
};

// Tables of the dataflow kernel (vbd_flow_kernel).
struct FlowView {
    const int2 *fhdr;  // per tile: {first entry in nbrp, number of entries}
    const int *nbrp;   // neighbour tiles (self included): tile id, with bit 31 set when that
                       // tile's colour is lower than the owner's (its current sweep is awaited)
    int *epoch;        // per tile: sweeps completed (monotonic over launches)
    int *ticket;       // [0] next task, [1] abort flag (both zeroed before a launch)
};

// Positions (base + delta) of the local vertices and the record block; the dataflow kernel
// also keeps the next task's local-vertex indices (4 B each).
inline size_t tile_smem_bytes(int max_local, int max_records)
{
    return size_t(2 * max_local) * 16 + size_t(max_records) * 16 + size_t(max_local) * 4;
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

struct TileCtx {
    const float4 *sb;
    const float4 *sd;
    const int4 *rec;
    V3f bs, ds;  // base and delta of the lane's vertex
    __device__ __forceinline__ V3f rel(int j) const
    {
        const float4 b = sb[j], d = sd[j];
        return mk((b.x - bs.x) + (d.x - ds.x), (b.y - bs.y) + (d.y - ds.y), (b.z - bs.z) + (d.z - ds.z));
    }
};

// Per-thread data of the tile vertex the thread works on, fetched while the staging copies fly.
struct TileVertex {
    int4 hv;     // incidence header
    int roff;    // record offset inside the tile's block
    int ngen;    // generic (type 6-14) records after the six classes
    float4 tg;   // inertial target (y - base, mass)
};

// Generic incidences of internal vertex v (0 when the scene has none).
__device__ __forceinline__ int tile_generic_count(const TileView &V, int v)
{
    return V.gen_off ? __ldg(V.gen_off + v + 1) - __ldg(V.gen_off + v) : 0;
}

// Stages the tile into shared memory. The tile's records and halo indices never change, so
// they are fetched before waiting for the previous colour; the positions after. The header
// and record offset of the thread's vertex (G threads per vertex) are loaded before the wait
// and its inertial target after it, all while the copies are in flight. Returns
// {vstart, nvt, halo_off, n_halo}.
template <int G>
__device__ __forceinline__ int4 tile_stage(const TileView &V, const DevState &S, int tile, float4 *sb, float4 *sd,
                                           int4 *srec, TileVertex &tv)
{
    const float4 *__restrict__ pos = S.pos;
    const int4 h0 = __ldg(V.hdr + 2 * tile);
    const int4 h1 = __ldg(V.hdr + 2 * tile + 1);
    for (int i = threadIdx.x; i < h1.y; i += blockDim.x) cp_async16(srec + i, V.records + h1.x + i);
    const int nvt = h0.y, nl = h0.y + h0.w;
    const int lv = threadIdx.x / G;
    tv.hv = make_int4(0, 0, 0, 0);
    tv.roff = 0;
    tv.ngen = 0;
    tv.tg = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lv < nvt) {
        tv.hv = __ldg(S.hdr + h0.x + lv);
        tv.roff = __ldg(V.vrec + h0.x + lv);
        tv.ngen = tile_generic_count(V, h0.x + lv);
    }
    constexpr int kMaxHaloPerThread = 8;
    int gidx[kMaxHaloPerThread];
#pragma unroll
    for (int k = 0; k < kMaxHaloPerThread; ++k) {
        const int i = threadIdx.x + k * blockDim.x;
        gidx[k] = i < nvt ? h0.x + i : (i < nl ? __ldg(V.halo + h0.z + i - nvt) : -1);
    }
    wait_prior_grid();
#pragma unroll
    for (int k = 0; k < kMaxHaloPerThread; ++k) {
        const int i = threadIdx.x + k * blockDim.x;
        if (gidx[k] >= 0) {
            cp_async16(sb + i, pos + 2 * gidx[k]);
            cp_async16(sd + i, pos + 2 * gidx[k] + 1);
        }
    }
    for (int i = threadIdx.x + kMaxHaloPerThread * blockDim.x; i < nl; i += blockDim.x) {
        const int g = i < nvt ? h0.x + i : __ldg(V.halo + h0.z + i - nvt);
        cp_async16(sb + i, pos + 2 * g);
        cp_async16(sd + i, pos + 2 * g + 1);
    }
    if (lv < nvt) tv.tg = S.tgt[h0.x + lv];
    cp_async_wait_all();
    __syncthreads();
    return h0;
}

// Accumulates every incidence of one vertex from its staged records (G lanes, lane-strided);
// with kGeneric also its ngen records of energy types 6-14 (parameters in gen_prm).
template <int G, bool kGeneric = false>
__device__ __forceinline__ void tile_vertex_accumulate(const TileCtx &cx, int4 h, int roff, int lane,
                                                       Block<float> &acc, int ngen = 0,
                                                       const float *__restrict__ gen_prm = nullptr)
{
    const V3f zero = mk(0.f, 0.f, 0.f);
    int off = roff;
    {  // anchors: {ax, ay, az, k}
        const int n = h.y & 0xffff;
        const int rounds = warp_max((n + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < n) {
                const int4 q = cx.rec[off + i];
                const V3f xa = mk((cx.bs.x - __int_as_float(q.x)) + cx.ds.x, (cx.bs.y - __int_as_float(q.y)) + cx.ds.y,
                                  (cx.bs.z - __int_as_float(q.z)) + cx.ds.z);
                anchor_block(xa, zero, __int_as_float(q.w), acc);
            }
        }
        off += n;
    }
    // Springs, bending flaps and bending hinges take two incidences per round where both exist,
    // so their arithmetic forms two independent dependency chains, and one incidence in the
    // last round otherwise (6 incidences over 2 lanes: a pair round, then a single round).
    {  // springs: {other, L0, k}
        const int n = (h.y >> 16) & 0xffff;
        const int rounds = warp_max((n + 2 * G - 1) / (2 * G));
        for (int r = 0; r < rounds; ++r) {
            const int i0 = 2 * r * G + lane, i1 = i0 + G;
            if (i1 < n) {
                const int4 q0 = cx.rec[off + i0];
                const int4 q1 = cx.rec[off + i1];
                spring_block(zero, cx.rel(q0.x), __int_as_float(q0.y), __int_as_float(q0.z), acc);
                spring_block(zero, cx.rel(q1.x), __int_as_float(q1.y), __int_as_float(q1.z), acc);
            } else if (i0 < n) {
                const int4 q0 = cx.rec[off + i0];
                spring_block(zero, cx.rel(q0.x), __int_as_float(q0.y), __int_as_float(q0.z), acc);
            }
        }
        off += n;
    }
    {  // bending flaps: {p0 | p1 << 16, other flap, signed theta0, k}
        const int n = h.z & 0xffff;
        const int rounds = warp_max((n + 2 * G - 1) / (2 * G));
        for (int r = 0; r < rounds; ++r) {
            const int i0 = 2 * r * G + lane, i1 = i0 + G;
            if (i1 < n) {
                const int4 q0 = cx.rec[off + i0];
                const int4 q1 = cx.rec[off + i1];
                bending_flap_block(cx.rel(q0.x & 0xffff), cx.rel(q0.x >> 16), zero, cx.rel(q0.y), __int_as_float(q0.z),
                                   __int_as_float(q0.w), acc);
                bending_flap_block(cx.rel(q1.x & 0xffff), cx.rel(q1.x >> 16), zero, cx.rel(q1.y), __int_as_float(q1.z),
                                   __int_as_float(q1.w), acc);
            } else if (i0 < n) {
                const int4 q0 = cx.rec[off + i0];
                bending_flap_block(cx.rel(q0.x & 0xffff), cx.rel(q0.x >> 16), zero, cx.rel(q0.y), __int_as_float(q0.z),
                                   __int_as_float(q0.w), acc);
            }
        }
        off += n;
    }
    {  // bending hinges: {other hinge, p2 | p3 << 16, signed theta0, k}
        const int n = (h.z >> 16) & 0xffff;
        const int rounds = warp_max((n + 2 * G - 1) / (2 * G));
        for (int r = 0; r < rounds; ++r) {
            const int i0 = 2 * r * G + lane, i1 = i0 + G;
            if (i1 < n) {
                const int4 q0 = cx.rec[off + i0];
                const int4 q1 = cx.rec[off + i1];
                bending_hinge_block(cx.rel(q0.x), zero, cx.rel(q0.y & 0xffff), cx.rel(q0.y >> 16), __int_as_float(q0.z),
                                    __int_as_float(q0.w), acc);
                bending_hinge_block(cx.rel(q1.x), zero, cx.rel(q1.y & 0xffff), cx.rel(q1.y >> 16), __int_as_float(q1.z),
                                    __int_as_float(q1.w), acc);
            } else if (i0 < n) {
                const int4 q0 = cx.rec[off + i0];
                bending_hinge_block(cx.rel(q0.x), zero, cx.rel(q0.y & 0xffff), cx.rel(q0.y >> 16), __int_as_float(q0.z),
                                    __int_as_float(q0.w), acc);
            }
        }
        off += n;
    }
    {  // StVK: {i0 | i1 << 16, i2 | slot << 16, D0, D1}, {D2, D3, K00, K01}, {K02, K11, K12, K22}
        const int n = h.w & 0xffff;
        const int rounds = warp_max((n + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < n) {
                const int4 a = cx.rec[off + 3 * i], b = cx.rec[off + 3 * i + 1], c = cx.rec[off + 3 * i + 2];
                V3f p[3];
                p[0] = cx.rel(a.x & 0xffff);
                p[1] = cx.rel(a.x >> 16);
                p[2] = cx.rel(a.y & 0xffff);
                const float D[4] = {__int_as_float(a.z), __int_as_float(a.w), __int_as_float(b.x), __int_as_float(b.y)};
                const float Ks[6] = {__int_as_float(b.z), __int_as_float(b.w), __int_as_float(c.x),
                                     __int_as_float(c.y), __int_as_float(c.z), __int_as_float(c.w)};
                stvk_block(p, a.y >> 16, D, Ks, acc);
            }
        }
        off += 3 * n;
    }
    {  // SNH: {i0 | i1 << 16, i2 | i3 << 16, slot, D0}, {D1..D4}, {D5..D8}, {lambda, mu, alpha}
        const int n = (h.w >> 16) & 0xffff;
        const int rounds = warp_max((n + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < n) {
                const int4 a = cx.rec[off + 4 * i], b = cx.rec[off + 4 * i + 1];
                const int4 c = cx.rec[off + 4 * i + 2], d = cx.rec[off + 4 * i + 3];
                V3f p[4];
                p[0] = cx.rel(a.x & 0xffff);
                p[1] = cx.rel(a.x >> 16);
                p[2] = cx.rel(a.y & 0xffff);
                p[3] = cx.rel(a.y >> 16);
                const float D[9] = {__int_as_float(a.w), __int_as_float(b.x), __int_as_float(b.y),
                                    __int_as_float(b.z), __int_as_float(b.w), __int_as_float(c.x),
                                    __int_as_float(c.y), __int_as_float(c.z), __int_as_float(c.w)};
                snh_block(p, a.z, D, __int_as_float(d.x), __int_as_float(d.y), __int_as_float(d.z), acc);
            }
        }
        off += 4 * n;
    }
    if (kGeneric) {  // {v0 | v1 << 16, v2 | v3 << 16, type | slot << 8 | size << 16, parameter offset}
        const int rounds = warp_max((ngen + G - 1) / G);
        for (int r = 0; r < rounds; ++r) {
            const int i = r * G + lane;
            if (i < ngen) {
                const int4 q = cx.rec[off + i];
                const int type = q.z & 0xff, slot = (q.z >> 8) & 0xff, S = (q.z >> 16) & 0xff;
                const int lj[4] = {q.x & 0xffff, q.x >> 16, q.y & 0xffff, q.y >> 16};
                V3f p[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) p[j] = (j >= S || j == slot) ? zero : cx.rel(lj[j]);
                generic_block(type, p, slot, gen_prm + q.w, acc);
            }
        }
    }
}

}  // namespace spgx
