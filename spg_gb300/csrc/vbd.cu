// GB300 Vertex Block Descent: colour kernels, substep kernels, FP64 residual reduction and
// the spgx_vbd_* C ABI. Restates spg::solver::VBD::step (spg/source/sim/solver/vbd.cpp:12-195)
// as: one inertial-prediction launch, `iterations` x (one launch per colour), one velocity
// launch per substep, replayed as a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "api_internal.h"
#include "devbuf.h"
#include "device_common.cuh"
#include "layout.h"
#include "state.h"
#include "mlp.h"
#include "vbd_solver.h"

namespace spgx {

// ---------------------------------------------------------------------------------------
// Kernels

// Per-vertex 3x3 solve and position update, l_vertexDescent's tail (vbd.cpp:139-146):
// H = m/h^2 I + sum of blocks, f = -m/h^2 (x - y) + sum of forces, x += H^-1 f when
// det(H) > 1e-10. The solve runs in FP32 on the max-norm-scaled block unless its Frobenius
// condition estimate exceeds the fallback threshold, in which case it is redone in FP64.
__device__ __forceinline__ void solve_and_update(const DevState &S, int v, const Block<float> &acc, float4 d4,
                                                 float4 tg, float invdt2, float fb2)
{
    const float c = tg.w * invdt2;
    float f0 = acc.f[0] - c * (d4.x - tg.x);
    float f1 = acc.f[1] - c * (d4.y - tg.y);
    float f2 = acc.f[2] - c * (d4.z - tg.z);
    float hd = c;
    if (S.n_pick) add_picks(S, v, S.pos[2 * v], d4, f0, f1, f2, hd);
    const float h0 = acc.h[0] + hd, h1 = acc.h[1], h2 = acc.h[2];
    const float h3 = acc.h[3] + hd, h4 = acc.h[4], h5 = acc.h[5] + hd;
    const float s = fmaxf(fmaxf(fmaxf(fabsf(h0), fabsf(h1)), fmaxf(fabsf(h2), fabsf(h3))), fmaxf(fabsf(h4), fabsf(h5)));
    float dx = 0.f, dy = 0.f, dz = 0.f;
    bool apply = false;
    bool fp32_ok = false;
    if (s > 0.f && s < INFINITY) {
        const float is = 1.f / s;
        const float a = h0 * is, b = h1 * is, cc = h2 * is, d = h3 * is, e = h4 * is, f = h5 * is;
        const float A00 = d * f - e * e, A01 = cc * e - b * f, A02 = b * e - cc * d;
        const float A11 = a * f - cc * cc, A12 = b * cc - a * e, A22 = a * d - b * b;
        const float det = a * A00 + b * A01 + cc * A02;
        const float nH2 = a * a + d * d + f * f + 2.f * (b * b + cc * cc + e * e);
        const float nA2 = A00 * A00 + A11 * A11 + A22 * A22 + 2.f * (A01 * A01 + A02 * A02 + A12 * A12);
        if (det > 0.f && nH2 * nA2 <= fb2 * det * det) {
            fp32_ok = true;
            if (det * s * s * s > 1e-10f) {
                const float inv = is / det;
                dx = (A00 * f0 + A01 * f1 + A02 * f2) * inv;
                dy = (A01 * f0 + A11 * f1 + A12 * f2) * inv;
                dz = (A02 * f0 + A12 * f1 + A22 * f2) * inv;
                apply = true;
            }
        }
    }
    if (!fp32_ok) {
        atomicAdd(S.counters + 0, 1);
        const double a = h0, b = h1, cc = h2, d = h3, e = h4, f = h5;
        const double A00 = d * f - e * e, A01 = cc * e - b * f, A02 = b * e - cc * d;
        const double A11 = a * f - cc * cc, A12 = b * cc - a * e, A22 = a * d - b * b;
        const double det = a * A00 + b * A01 + cc * A02;
        if (det > 1e-10) {
            const double inv = 1.0 / det;
            dx = static_cast<float>((A00 * f0 + A01 * f1 + A02 * f2) * inv);
            dy = static_cast<float>((A01 * f0 + A11 * f1 + A12 * f2) * inv);
            dz = static_cast<float>((A02 * f0 + A12 * f1 + A22 * f2) * inv);
            apply = true;
        }
    }
    if (!apply) {
        atomicAdd(S.counters + 1, 1);
        return;
    }
    const float nx = d4.x + dx, ny = d4.y + dy, nz = d4.z + dz;
    if (isfinite(nx) && isfinite(ny) && isfinite(nz)) {
        S.pos[2 * v + 1] = make_float4(nx, ny, nz, d4.w);
    } else {
        atomicOr(S.status, 1u);
    }
}

// One colour phase: G lanes per vertex over the vertices [cstart, cend) of one colour.
template <int G, bool kGeneric>
__global__ void __launch_bounds__(256) vbd_color_kernel(const DevTables T, const DevState S, int cstart, int cend,
                                                        float invdt2, float fb2)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & (G - 1);
    const int v = cstart + t / G;
    const bool active = v < cend;
    int4 h = make_int4(0, 0, 0, 0);
    V3f bs = mk(0.f, 0.f, 0.f), ds = bs;
    if (active) h = __ldg(S.hdr + v);
    wait_prior_grid();
    if (active) {
        bs = v3(__ldg(S.pos + 2 * v));
        ds = v3(__ldg(S.pos + 2 * v + 1));
    }
    Block<float> acc;
    block_zero(acc);
    accumulate_incidences<G, kGeneric>(T, S.pos, S.adj, h, lane, bs, ds, acc, active ? v : -1);
    group_reduce<G>(acc);
    allow_next_grid();
    if (active && lane == 0) solve_and_update(S, v, acc, S.pos[2 * v + 1], S.tgt[v], invdt2, fb2);
}

// One colour phase with the shared-memory tile kernel: one CTA per tile of the colour,
// G lanes per tile vertex (blockDim = tile_vertices * G).
template <int G, bool kGeneric>
__global__ void __launch_bounds__(kTileThreads) vbd_tile_kernel(const TileView V, const DevState S, int tile0,
                                                                int max_local, float invdt2, float fb2)
{
    extern __shared__ float4 dyn[];
    float4 *sb = dyn;
    float4 *sd = dyn + max_local;
    int4 *srec = reinterpret_cast<int4 *>(dyn + 2 * max_local);
    TileVertex tv;
    const int4 h0 = tile_stage<G>(V, S, tile0 + blockIdx.x, sb, sd, srec, tv);
    const int lv = threadIdx.x / G;
    const int lane = threadIdx.x & (G - 1);
    const bool active = lv < h0.y;
    TileCtx cx{sb, sd, srec, mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f)};
    if (active) {
        cx.bs = v3(sb[lv]);
        cx.ds = v3(sd[lv]);
    }
    Block<float> acc;
    block_zero(acc);
    tile_vertex_accumulate<G, kGeneric>(cx, tv.hv, tv.roff, lane, acc, tv.ngen, V.gen_prm);
    group_reduce<G>(acc);
    allow_next_grid();
    if (active && lane == 0) solve_and_update(S, h0.x + lv, acc, sd[lv], tv.tg, invdt2, fb2);
}

// Dataflow sweeps: a persistent kernel that runs `iterations` colour sweeps with no barrier
// between colours. Every (iteration, tile) is one task, handed out in (iteration, colour,
// tile) order by an atomic ticket. Tile T of colour c at iteration k may start when every
// neighbour tile U (the tiles owning T's halo, and T itself) has finished iteration k if U's
// colour is lower than c, and iteration k - 1 otherwise: exactly the reads Gauss-Seidel over
// colours prescribes. Higher-colour neighbours cannot overwrite T's inputs early, because
// they in turn wait for T. Each task waits only on tasks with smaller tickets, all held by
// co-resident CTAs (cooperative launch), so the waits always end; each is still bounded, and
// a wait that gives up sets the abort flag and status bit 1 so that every CTA leaves. A CTA
// takes its next ticket while it polls for the current one: the smallest unfinished ticket is
// then always running (a CTA holding it unstarted would be running a smaller unfinished one),
// so progress is kept.
constexpr int kFlowMaxPolls = 1 << 21;  // each poll an L2 round trip (a few hundred ns): about a second per wait
constexpr int kFlowPollMax = 64;       // neighbour-list entries prefetched per task (the rest are read directly)

template <int G, bool kGeneric>
__global__ void __launch_bounds__(kTileThreads) vbd_flow_kernel(const TileView V, const DevState S,
                                                                const FlowView F, int n_tiles, int iterations,
                                                                int epoch_base, int max_local, float invdt2,
                                                                float fb2)
{
    // Shared memory: base and delta positions of the local vertices, the record block, and the
    // global indices of the next task's local vertices (fetched while the current one runs).
    extern __shared__ float4 dyn[];
    float4 *sb = dyn;
    float4 *sd = dyn + max_local;
    int4 *srec = reinterpret_cast<int4 *>(dyn + 2 * max_local);
    // The next task's tile header, neighbour-list range and packed neighbour list, copied while
    // the current task stages and computes, so that no global round trip is spent on them
    // between two tasks.
    __shared__ int4 s_hdr[2];
    __shared__ int2 s_fh;
    __shared__ int s_poll[kFlowPollMax];
    __shared__ int s_next, s_fail;
    // Completion of the record block's bulk copy (one phase per task).
    __shared__ __align__(8) unsigned long long s_rec_bar;
    const uint32_t rec_bar = static_cast<uint32_t>(__cvta_generic_to_shared(&s_rec_bar));
    uint32_t rec_phase = 0;
    const int total = iterations * n_tiles;
    const int lv = threadIdx.x / G;
    const int lane = threadIdx.x & (G - 1);
    int *sidx = reinterpret_cast<int *>(srec + V.max_records);

    // Thread 0: the header and neighbour-list range of task t, async (waited with the staging).
    auto prefetch_header = [&](int t) {
        if (threadIdx.x == 0 && t < total) {
            const int tile = t % n_tiles;
            cp_async16(s_hdr, V.hdr + 2 * tile);
            cp_async16(s_hdr + 1, V.hdr + 2 * tile + 1);
            cp_async8(&s_fh, F.fhdr + tile);
        }
    };
    // Warp 0: the first kFlowPollMax entries of task t's neighbour list, async, as one group
    // (each lane later reads only the entries it copied). Needs s_fh.
    auto prefetch_poll = [&](int t) {
        if (threadIdx.x < 32 && t < total) {
            const int2 fh = s_fh;
            const int n = min(fh.y, kFlowPollMax);
            for (int j = threadIdx.x; j < n; j += 32) cp_async4(s_poll + j, F.nbrp + fh.x + j);
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        }
    };
    // Static data of a task, fetched while the previous task finishes or its dependencies are
    // polled: its record block and the indices of its local vertices (both into shared memory,
    // async), and the header, record offset and inertial target of the thread's vertex. The
    // target y is fixed for the whole step. The tile header comes from the prefetch.
    auto fetch_static = [&](int4 &h0, int4 &h1, int4 &hv, int &roff, int &ngen, float4 &tg) {
        h0 = s_hdr[0];
        h1 = s_hdr[1];
        const int nvt = h0.y, nl = h0.y + h0.w;
        // The record block (contiguous, 16-byte aligned, a multiple of 16 bytes) in one bulk copy
        // by the tensor memory accelerator, completed on s_rec_bar: one instruction instead of a
        // 16-byte copy per record. The block's previous contents were last read before the
        // barrier that preceded this call; the proxy fence orders those reads before the copy.
        if (threadIdx.x == 0 && h1.y > 0) {
            const uint32_t bytes = static_cast<uint32_t>(h1.y) * 16u;
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(rec_bar), "r"(bytes)
                         : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                    static_cast<uint32_t>(__cvta_generic_to_shared(srec))),
                "l"(V.records + h1.x), "r"(bytes), "r"(rec_bar)
                : "memory");
        }
        for (int i = threadIdx.x; i < nl; i += blockDim.x) {
            if (i < nvt)
                sidx[i] = h0.x + i;
            else
                cp_async4(sidx + i, V.halo + h0.z + i - nvt);
        }
        hv = make_int4(0, 0, 0, 0);
        roff = 0;
        ngen = 0;
        tg = make_float4(0.f, 0.f, 0.f, 0.f);
        if (lv < nvt) {
            hv = __ldg(S.hdr + h0.x + lv);
            roff = __ldg(V.vrec + h0.x + lv);
            if (kGeneric) ngen = tile_generic_count(V, h0.x + lv);
            tg = S.tgt[h0.x + lv];
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    if (threadIdx.x == 0) {
        s_next = ld_relaxed_gpu(F.ticket + 1) ? total : atomicAdd(F.ticket, 1);
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(rec_bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    int task = s_next;
    // Bounded wait for the record block of the task fetched last (its bulk copy has arrived
    // once the mbarrier phase completes); false when the polls ran out.
    auto wait_records = [&](int n_rec) -> bool {
        if (n_rec <= 0) return true;
        for (int i = 0; i < kFlowMaxPolls; ++i) {
            uint32_t done;
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}\n"
                : "=r"(done)
                : "r"(rec_bar), "r"(rec_phase)
                : "memory");
            if (done) return true;
            __nanosleep(32);
        }
        return false;
    };
    prefetch_header(task);
    cp_async_wait_all();
    __syncthreads();
    prefetch_poll(task);
    int4 h0, h1, hv;
    int roff, ngen;
    float4 tg;
    if (task < total) fetch_static(h0, h1, hv, roff, ngen, tg);
    while (task < total) {
        const int k = task / n_tiles;
        const int tile = task - k * n_tiles;
        // Wait for the tiles this sweep reads (warp 0 polls, one neighbour per lane). Thread 0
        // also takes the next ticket, so that the next task's header can be prefetched while
        // this one runs; a task still waits only on tasks with smaller tickets.
        if (threadIdx.x < 32) {
            int ticket = total;
            if (threadIdx.x == 0) ticket = ld_relaxed_gpu(F.ticket + 1) ? total : atomicAdd(F.ticket, 1);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // this lane's neighbour entries
            const int2 fh = s_fh;
            bool ok = true;
            for (int j = threadIdx.x; j < fh.y && ok; j += 32) {
                const int pk = j < kFlowPollMax ? s_poll[j] : __ldg(F.nbrp + fh.x + j);
                const int u = pk & 0x7fffffff;
                const int need = epoch_base + k + (pk < 0 ? 1 : 0);
                int polls = 0;
                while (ld_acquire_gpu(F.epoch + u) < need) {
                    if (++polls > kFlowMaxPolls || ld_relaxed_gpu(F.ticket + 1)) {
                        ok = false;
                        break;
                    }
                    // No sleep between polls: a dependency is seen one L2 round trip after its
                    // release (a 128 ns sleep cost 1.3 % of the step on the 513^2 cloth).
                }
            }
            ok = __all_sync(0xffffffffu, ok);
            if (threadIdx.x == 0) {
                s_fail = !ok;
                s_next = ticket;
            }
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");  // this thread's index and record copies
        __syncthreads();  // every thread's index and record copies, the poll result and s_next
        if (s_fail) {
            if (threadIdx.x == 0) {
                atomicExch(F.ticket + 1, 1);
                atomicOr(S.status, 2u);
            }
            wait_records(h1.y);  // the record copy in flight lands before the CTA leaves
            break;
        }
        prefetch_header(s_next);
        // Stage the current positions of the local vertices.
        const int nl = h0.y + h0.w;
        for (int i = threadIdx.x; i < nl; i += blockDim.x) {
            const int g = sidx[i];
            cp_async16(sb + i, S.pos + 2 * g);
            cp_async16(sd + i, S.pos + 2 * g + 1);
        }
        const bool active = lv < h0.y;
        cp_async_wait_all();
        const bool rec_ok = wait_records(h1.y);
        if (h1.y > 0) rec_phase ^= 1u;
        if (!__syncthreads_and(rec_ok)) {  // the staging, the records and the next task's header
            if (threadIdx.x == 0) {
                atomicExch(F.ticket + 1, 1);
                atomicOr(S.status, 2u);
            }
            break;
        }
        prefetch_poll(s_next);
        TileCtx cx{sb, sd, srec, mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f)};
        if (active) {
            cx.bs = v3(sb[lv]);
            cx.ds = v3(sd[lv]);
        }
        Block<float> acc;
        block_zero(acc);
        tile_vertex_accumulate<G, kGeneric>(cx, hv, roff, lane, acc, ngen, V.gen_prm);
        group_reduce<G>(acc);
        if (active && lane == 0) solve_and_update(S, h0.x + lv, acc, sd[lv], tg, invdt2, fb2);
        __syncthreads();  // every position of the tile is written and the staging consumed
        // The release is cumulative: the CTA's position writes, ordered before it by the barrier,
        // are visible to any CTA that acquires this epoch.
        if (threadIdx.x == 0) st_release_gpu(F.epoch + tile, epoch_base + k + 1);
        task = s_next;
        if (task < total) fetch_static(h0, h1, hv, roff, ngen, tg);
    }
}

// Block-wide FP64 sum into *out (one atomic per block).
__device__ __forceinline__ void block_sum_atomic(double v, double *out)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ double part[32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) part[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < (blockDim.x + 31) / 32; ++k) s += part[k];
        atomicAdd(out, s);
    }
}

// Residual with the tile layout: every tile of every colour (positions are not modified).
template <int G, bool kGeneric>
__global__ void __launch_bounds__(kTileThreads) residual_tile_kernel(const TileView V, const DevState S,
                                                                     int max_local, float invdt2, double *out)
{
    extern __shared__ float4 dyn[];
    float4 *sb = dyn;
    float4 *sd = dyn + max_local;
    int4 *srec = reinterpret_cast<int4 *>(dyn + 2 * max_local);
    TileVertex tv;
    const int4 h0 = tile_stage<G>(V, S, blockIdx.x, sb, sd, srec, tv);
    const int lv = threadIdx.x / G;
    const int lane = threadIdx.x & (G - 1);
    const bool active = lv < h0.y;
    TileCtx cx{sb, sd, srec, mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 0.f)};
    if (active) {
        cx.bs = v3(sb[lv]);
        cx.ds = v3(sd[lv]);
    }
    Block<float> acc;
    block_zero(acc);
    tile_vertex_accumulate<G, kGeneric>(cx, tv.hv, tv.roff, lane, acc, tv.ngen, V.gen_prm);
    group_reduce<G>(acc);
    double r2 = 0.0;
    if (active && lane == 0) {
        const float4 tg = tv.tg;
        if (S.n_pick) {
            float hd = 0.f;
            add_picks(S, h0.x + lv, sb[lv], sd[lv], acc.f[0], acc.f[1], acc.f[2], hd);
        }
        const double c = double(tg.w) * invdt2;
        const double rx = c * (double(cx.ds.x) - tg.x) - acc.f[0];
        const double ry = c * (double(cx.ds.y) - tg.y) - acc.f[1];
        const double rz = c * (double(cx.ds.z) - tg.z) - acc.f[2];
        r2 = rx * rx + ry * ry + rz * rz;
    }
    block_sum_atomic(r2, out);
}

// ||M/h^2 (x - y) + grad E(x)||^2 with per-vertex FP32 forces and an FP64 reduction.
template <int G, bool kGeneric>
__global__ void __launch_bounds__(256) residual_kernel(const DevTables T, const DevState S, int nv, float invdt2,
                                                       double *out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & (G - 1);
    const int v = t / G;
    const bool active = v < nv;
    int4 h = make_int4(0, 0, 0, 0);
    V3f bs = mk(0.f, 0.f, 0.f), ds = bs;
    if (active) {
        h = __ldg(S.hdr + v);
        bs = v3(__ldg(S.pos + 2 * v));
        ds = v3(__ldg(S.pos + 2 * v + 1));
    }
    Block<float> acc;
    block_zero(acc);
    accumulate_incidences<G, kGeneric>(T, S.pos, S.adj, h, lane, bs, ds, acc, active ? v : -1);
    group_reduce<G>(acc);
    double r2 = 0.0;
    if (active && lane == 0) {
        const float4 tg = S.tgt[v];
        if (S.n_pick) {
            float hd = 0.f;
            add_picks(S, v, S.pos[2 * v], S.pos[2 * v + 1], acc.f[0], acc.f[1], acc.f[2], hd);
        }
        const double c = double(tg.w) * invdt2;
        const double rx = c * (double(ds.x) - tg.x) - acc.f[0];
        const double ry = c * (double(ds.y) - tg.y) - acc.f[1];
        const double rz = c * (double(ds.z) - tg.z) - acc.f[2];
        r2 = rx * rx + ry * ry + rz * rz;
    }
    block_sum_atomic(r2, out);
}

// ---------------------------------------------------------------------------------------
// Launch helpers

static int ceil_div(long long a, long long b) { return static_cast<int>((a + b - 1) / b); }

// Launches a tile kernel with programmatic dependent launch: its static prologue (tile header,
// record copies, halo indices) overlaps the tail of the previous kernel, and it waits
// (griddepcontrol.wait) before copying positions, which it reads through L2 only.
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kernel)(KArgs...), int grid, int block, size_t smem, cudaStream_t st, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

template <bool kGeneric>
static void launch_lanes(int lanes, int grid, int block, cudaStream_t st, const DevTables &T, const DevState &S,
                         int cs, int ce, float invdt2, float fb2)
{
    switch (lanes) {
    case 1: vbd_color_kernel<1, kGeneric><<<grid, block, 0, st>>>(T, S, cs, ce, invdt2, fb2); break;
    case 2: vbd_color_kernel<2, kGeneric><<<grid, block, 0, st>>>(T, S, cs, ce, invdt2, fb2); break;
    case 4: vbd_color_kernel<4, kGeneric><<<grid, block, 0, st>>>(T, S, cs, ce, invdt2, fb2); break;
    case 8: vbd_color_kernel<8, kGeneric><<<grid, block, 0, st>>>(T, S, cs, ce, invdt2, fb2); break;
    case 16: vbd_color_kernel<16, kGeneric><<<grid, block, 0, st>>>(T, S, cs, ce, invdt2, fb2); break;
    default: vbd_color_kernel<32, kGeneric><<<grid, block, 0, st>>>(T, S, cs, ce, invdt2, fb2); break;
    }
}

template <bool kGeneric>
static void launch_residual_lanes(int lanes, int grid, int block, cudaStream_t st, const DevTables &T,
                                  const DevState &S, int nv, float invdt2, double *out)
{
    switch (lanes) {
    case 1: residual_kernel<1, kGeneric><<<grid, block, 0, st>>>(T, S, nv, invdt2, out); break;
    case 2: residual_kernel<2, kGeneric><<<grid, block, 0, st>>>(T, S, nv, invdt2, out); break;
    case 4: residual_kernel<4, kGeneric><<<grid, block, 0, st>>>(T, S, nv, invdt2, out); break;
    case 8: residual_kernel<8, kGeneric><<<grid, block, 0, st>>>(T, S, nv, invdt2, out); break;
    case 16: residual_kernel<16, kGeneric><<<grid, block, 0, st>>>(T, S, nv, invdt2, out); break;
    default: residual_kernel<32, kGeneric><<<grid, block, 0, st>>>(T, S, nv, invdt2, out); break;
    }
}

template <bool kGen>
static void launch_tile(const VbdSolver &s, int t0, int t1, int threads, cudaStream_t st, float invdt2, float fb2)
{
    switch (s.lanes) {
    case 1: launch_pdl(vbd_tile_kernel<1, kGen>, t1 - t0, threads, s.tile_smem, st, s.TV, s.S, t0, s.TL.max_local, invdt2, fb2); break;
    case 2: launch_pdl(vbd_tile_kernel<2, kGen>, t1 - t0, threads, s.tile_smem, st, s.TV, s.S, t0, s.TL.max_local, invdt2, fb2); break;
    case 4: launch_pdl(vbd_tile_kernel<4, kGen>, t1 - t0, threads, s.tile_smem, st, s.TV, s.S, t0, s.TL.max_local, invdt2, fb2); break;
    default: launch_pdl(vbd_tile_kernel<8, kGen>, t1 - t0, threads, s.tile_smem, st, s.TV, s.S, t0, s.TL.max_local, invdt2, fb2); break;
    }
}

template <bool kGen>
static cudaError_t launch_flow_kernel(const VbdSolver &s, const cudaLaunchConfig_t &cfg, int n_tiles, int n, int base,
                                      float invdt2, float fb2)
{
    switch (s.lanes) {
    case 1: return cudaLaunchKernelEx(&cfg, vbd_flow_kernel<1, kGen>, s.TV, s.S, s.FV, n_tiles, n, base, s.TL.max_local, invdt2, fb2);
    case 2: return cudaLaunchKernelEx(&cfg, vbd_flow_kernel<2, kGen>, s.TV, s.S, s.FV, n_tiles, n, base, s.TL.max_local, invdt2, fb2);
    case 4: return cudaLaunchKernelEx(&cfg, vbd_flow_kernel<4, kGen>, s.TV, s.S, s.FV, n_tiles, n, base, s.TL.max_local, invdt2, fb2);
    default: return cudaLaunchKernelEx(&cfg, vbd_flow_kernel<8, kGen>, s.TV, s.S, s.FV, n_tiles, n, base, s.TL.max_local, invdt2, fb2);
    }
}

template <bool kGen>
static void launch_residual_tile(const VbdSolver &s, int nt, int threads, cudaStream_t st, float invdt2, double *out)
{
    switch (s.lanes) {
    case 1: residual_tile_kernel<1, kGen><<<nt, threads, s.tile_smem, st>>>(s.TV, s.S, s.TL.max_local, invdt2, out); break;
    case 2: residual_tile_kernel<2, kGen><<<nt, threads, s.tile_smem, st>>>(s.TV, s.S, s.TL.max_local, invdt2, out); break;
    case 4: residual_tile_kernel<4, kGen><<<nt, threads, s.tile_smem, st>>>(s.TV, s.S, s.TL.max_local, invdt2, out); break;
    default: residual_tile_kernel<8, kGen><<<nt, threads, s.tile_smem, st>>>(s.TV, s.S, s.TL.max_local, invdt2, out); break;
    }
}

static void launch_color(const VbdSolver &s, int c, cudaStream_t st)
{
    if (s.kernel == 2) {
        const int t0 = s.TL.color_tiles[c], t1 = s.TL.color_tiles[c + 1];
        if (t1 <= t0) return;
        const float invdt2 = static_cast<float>(1.0 / (s.h_sub * s.h_sub));
        const float fb2 = static_cast<float>(s.P.fallback_condition * s.P.fallback_condition);
        const int threads = s.TL.tile_vertices * s.lanes;
        if (s.TV.gen_off)
            launch_tile<true>(s, t0, t1, threads, st, invdt2, fb2);
        else
            launch_tile<false>(s, t0, t1, threads, st, invdt2, fb2);
        return;
    }
    const int cs = s.L.color_start[c], ce = s.L.color_start[c + 1];
    if (ce <= cs) return;
    const int grid = ceil_div(static_cast<long long>(ce - cs) * s.lanes, s.block);
    const float invdt2 = static_cast<float>(1.0 / (s.h_sub * s.h_sub));
    const float fb2 = static_cast<float>(s.P.fallback_condition * s.P.fallback_condition);
    // Launched without programmatic overlap: this kernel reads neighbour positions through the
    // read-only data path, which must not run while the previous colour still writes them.
    if (s.T.gen_off) {
        launch_lanes<true>(s.lanes, grid, s.block, st, s.T, s.S, cs, ce, invdt2, fb2);
        return;
    }
    launch_lanes<false>(s.lanes, grid, s.block, st, s.T, s.S, cs, ce, invdt2, fb2);
}

// n sweeps of the dataflow kernel in one cooperative launch (one resident wave of CTAs).
static void launch_flow(const VbdSolver &s, int n, cudaStream_t st)
{
    const int n_tiles = s.TL.color_tiles.back();
    if (n <= 0 || n_tiles <= 0) return;
    cudaMemsetAsync(s.FV.ticket, 0, 2 * sizeof(int), st);
    const int li = s.lanes == 1 ? 0 : s.lanes == 2 ? 1 : s.lanes == 4 ? 2 : 3;
    const long long tasks = static_cast<long long>(n) * n_tiles;
    const int grid = static_cast<int>(std::min<long long>(tasks, static_cast<long long>(s.flow_blocks_per_sm[li]) *
                                                                     s.num_sms));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(s.TL.tile_vertices * s.lanes);
    cfg.dynamicSmemBytes = s.tile_smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const float invdt2 = static_cast<float>(1.0 / (s.h_sub * s.h_sub));
    const float fb2 = static_cast<float>(s.P.fallback_condition * s.P.fallback_condition);
    const int base = s.flow_epoch;
    cudaError_t e = cudaErrorInvalidConfiguration;  // warp 0 polls with full-warp votes: >= 32 threads
    if (cfg.blockDim.x >= 32) {
        e = s.TV.gen_off ? launch_flow_kernel<true>(s, cfg, n_tiles, n, base, invdt2, fb2)
                         : launch_flow_kernel<false>(s, cfg, n_tiles, n, base, invdt2, fb2);
    }
    // The counters only advance when the sweeps were enqueued; a failed launch is reported by
    // the caller's error check.
    if (e == cudaSuccess)
        s.flow_epoch += n;
    else
        s.flow_launch_error = e;
}

static void launch_iterations(const VbdSolver &s, int n, cudaStream_t st)
{
    if (n <= 0) return;
    if (s.kernel == 3) {
        launch_flow(s, n, st);
        return;
    }
    for (int it = 0; it < n; ++it)
        for (int c = 0; c < s.L.n_colors; ++c) launch_color(s, c, st);
}

static void launch_begin(const VbdSolver &s, cudaStream_t st) { launch_begin_substep(s.X, s.h_sub, s.P.gravity, st); }

static void launch_end(const VbdSolver &s, cudaStream_t st)
{
    launch_end_substep(s.X, s.h_sub, st, s.W.history ? s.W.vhist.as<float4>() : nullptr, s.P.gravity);
}

// Adds ||r(x)||^2 of the current positions to *out (default: the handle's residual slot).
static void launch_residual(const VbdSolver &s, cudaStream_t st, double *out = nullptr)
{
    if (s.L.nv == 0) return;
    const float invdt2 = static_cast<float>(1.0 / (s.h_sub * s.h_sub));
    if (!out) out = s.d_resid.as<double>();
    if (s.kernel >= 2) {
        const int nt = s.TL.color_tiles.back();
        const int threads = s.TL.tile_vertices * s.lanes;
        if (nt > 0) {
            if (s.TV.gen_off)
                launch_residual_tile<true>(s, nt, threads, st, invdt2, out);
            else
                launch_residual_tile<false>(s, nt, threads, st, invdt2, out);
        }
        return;
    }
    const int grid = ceil_div(static_cast<long long>(s.L.nv) * s.lanes, s.block);
    if (s.T.gen_off)
        launch_residual_lanes<true>(s.lanes, grid, s.block, st, s.T, s.S, s.L.nv, invdt2, out);
    else
        launch_residual_lanes<false>(s.lanes, grid, s.block, st, s.T, s.S, s.L.nv, invdt2, out);
}

// ---------------------------------------------------------------------------------------
// Solver methods

spgx_status ElementBuffers::upload_generic(const SceneLayout &L, DevTables &T)
{
    if (L.gen_off.empty()) return SPGX_OK;
    SPGX_TRY_STATUS(gen_off.upload(L.gen_off));
    SPGX_TRY_STATUS(gen_adj.upload(L.gen_adj));
    SPGX_TRY_STATUS(gen_idx.upload(L.el.gen_idx));
    SPGX_TRY_STATUS(gen_info.upload(L.el.gen_info));
    SPGX_TRY_STATUS(gen_prm.upload(L.el.gen_prm));
    T.gen_off = gen_off.as<int>();
    T.gen_adj = gen_adj.as<int>();
    T.gen_idx = gen_idx.as<int4>();
    T.gen_info = gen_info.as<int4>();
    T.gen_prm = gen_prm.as<float>();
    return SPGX_OK;
}

spgx_status ElementBuffers::upload(const ElementTables &E, DevTables &T)
{
    SPGX_TRY_STATUS(anchors.upload(E.anchors));
    SPGX_TRY_STATUS(anchor_cmp.upload(E.anchor_cmp));
    SPGX_TRY_STATUS(springs.upload(E.springs));
    SPGX_TRY_STATUS(spring_cmp.upload(E.spring_cmp));
    SPGX_TRY_STATUS(bend_idx.upload(E.bend_idx));
    SPGX_TRY_STATUS(bend_prm.upload(E.bend_prm));
    SPGX_TRY_STATUS(stvk_idx.upload(E.stvk_idx));
    SPGX_TRY_STATUS(stvk_D.upload(E.stvk_D));
    SPGX_TRY_STATUS(stvk_Ka.upload(E.stvk_Ka));
    SPGX_TRY_STATUS(stvk_Kb.upload(E.stvk_Kb));
    SPGX_TRY_STATUS(stvk_Ca.upload(E.stvk_Ca));
    SPGX_TRY_STATUS(stvk_Cb.upload(E.stvk_Cb));
    SPGX_TRY_STATUS(stvk_Cc.upload(E.stvk_Cc));
    SPGX_TRY_STATUS(snh_idx.upload(E.snh_idx));
    SPGX_TRY_STATUS(snh_p0.upload(E.snh_p0));
    SPGX_TRY_STATUS(snh_p1.upload(E.snh_p1));
    SPGX_TRY_STATUS(snh_p2.upload(E.snh_p2));
    SPGX_TRY_STATUS(snh_cmp.upload(E.snh_cmp));
    T = DevTables{};
    T.anchors = anchors.as<float4>();
    T.anchor_cmp = anchor_cmp.as<float2>();
    T.springs = springs.as<int4>();
    T.spring_cmp = spring_cmp.as<float>();
    T.bend_idx = bend_idx.as<int4>();
    T.bend_prm = bend_prm.as<float4>();
    T.stvk_idx = stvk_idx.as<int4>();
    T.stvk_D = stvk_D.as<float4>();
    T.stvk_Ka = stvk_Ka.as<float4>();
    T.stvk_Kb = stvk_Kb.as<float4>();
    T.stvk_Ca = stvk_Ca.as<float4>();
    T.stvk_Cb = stvk_Cb.as<float4>();
    T.stvk_Cc = stvk_Cc.as<float>();
    T.snh_idx = snh_idx.as<int4>();
    T.snh_p0 = snh_p0.as<float4>();
    T.snh_p1 = snh_p1.as<float4>();
    T.snh_p2 = snh_p2.as<float4>();
    T.snh_cmp = snh_cmp.as<float2>();
    return SPGX_OK;
}

spgx_status VbdSolver::init(const spgx_scene_desc *scene, const spgx_vbd_params *params)
{
    std::string err;
    const spgx_status st = build_scene_layout(scene, false, L, err);
    if (st != SPGX_OK) {
        set_error(err);
        return st;
    }
    SPGX_TRY_STATUS(check_params(params));
    P = *params;
    h_sub = P.dt / P.substeps;
    SPGX_TRY_STATUS(select_device(P.device));
    device = P.device;
    SPGX_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    SPGX_CUDA(cudaEventCreate(&ev0));
    SPGX_CUDA(cudaEventCreate(&ev1));
    SPGX_TRY_STATUS(X.init(L));
    SPGX_TRY_STATUS(EB.upload(L.el, T));
    SPGX_TRY_STATUS(EB.upload_generic(L, T));
    SPGX_TRY_STATUS(d_hdr.upload(L.hdr));
    SPGX_TRY_STATUS(d_adj.upload(L.adj));
    SPGX_TRY_STATUS(d_counters.alloc(kCounters * sizeof(int)));
    SPGX_TRY_STATUS(d_resid.alloc(2 * sizeof(double)));
    SPGX_TRY_STATUS(d_backup.alloc(size_t(L.nv) * 2 * sizeof(float4)));
    SPGX_TRY_STATUS(h_counters.alloc(kCounters * sizeof(int) + 4 * sizeof(double)));
    SPGX_CUDA(cudaMemset(d_counters.as<int>(), 0, kCounters * sizeof(int)));
    S = DevState{};
    S.pos = X.pos();
    S.tgt = X.tgt();
    S.dold = X.dold();
    S.vel = X.vel();
    S.hdr = d_hdr.as<int4>();
    S.adj = d_adj.as<int>();
    S.counters = d_counters.as<int>();
    S.status = reinterpret_cast<unsigned int *>(d_counters.as<int>() + 2);
    SPGX_TRY_STATUS(d_pick_v.alloc(SPGX_MAX_PICKS * sizeof(int)));
    SPGX_TRY_STATUS(d_pick_a.alloc(SPGX_MAX_PICKS * sizeof(float4)));
    S.n_pick = 0;
    S.pick_v = d_pick_v.as<int>();
    S.pick_a = d_pick_a.as<float4>();
    SPGX_TRY_STATUS(setup_tiles(P.tile_vertices ? P.tile_vertices : kTileCandidates[0]));
    SPGX_TRY_STATUS(setup_flow());
    SPGX_TRY_STATUS(configure_launch());
    return SPGX_OK;
}

spgx_status VbdSolver::setup_tiles(int tv)
{
    std::string err;
    const spgx_status st = build_tiles(L, tv, TL, err);
    if (st != SPGX_OK) {
        set_error(err);
        return st;
    }
    SPGX_TRY_STATUS(tb_hdr.upload(TL.hdr));
    SPGX_TRY_STATUS(tb_halo.upload(TL.halo));
    SPGX_TRY_STATUS(tb_records.upload(TL.records));
    SPGX_TRY_STATUS(tb_vrec.upload(TL.vrec));
    TV.hdr = tb_hdr.as<int4>();
    TV.halo = tb_halo.as<int>();
    TV.records = tb_records.as<int4>();
    TV.vrec = tb_vrec.as<int>();
    TV.gen_off = T.gen_off;
    TV.gen_prm = T.gen_prm;
    TV.max_records = std::max(1, TL.max_records);
    tile_smem = tile_smem_bytes(std::max(1, TL.max_local), std::max(1, TL.max_records));
    // The opt-in limit is declared once for every tile kernel, whatever this scene needs: the
    // attribute is process-wide, so a per-scene value would break a larger scene's live
    // handle, and the residual kernel's 256 B of static shared memory would not fit a dynamic
    // block just under the 48 KB default.
    int optin = 0;
    SPGX_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    const int cap = optin - 512;  // room for the kernels' static shared memory (304 bytes at most)
    if (tile_smem > size_t(cap)) {
        set_error("a tile needs more shared memory than the device offers; lower tile_vertices");
        return SPGX_ERR_INVALID_ARG;
    }
    {
        // Each kernel may take the opt-in limit less its own static shared memory.
        auto raise = [optin](const void *fn) -> cudaError_t {
            cudaFuncAttributes a{};
            const cudaError_t e = cudaFuncGetAttributes(&a, fn);
            if (e != cudaSuccess) return e;
            return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        optin - static_cast<int>(a.sharedSizeBytes));
        };
        const void *fns[] = {
            reinterpret_cast<const void *>(vbd_tile_kernel<1, false>), reinterpret_cast<const void *>(vbd_tile_kernel<2, false>),
            reinterpret_cast<const void *>(vbd_tile_kernel<4, false>), reinterpret_cast<const void *>(vbd_tile_kernel<8, false>),
            reinterpret_cast<const void *>(vbd_flow_kernel<1, false>), reinterpret_cast<const void *>(vbd_flow_kernel<2, false>),
            reinterpret_cast<const void *>(vbd_flow_kernel<4, false>), reinterpret_cast<const void *>(vbd_flow_kernel<8, false>),
            reinterpret_cast<const void *>(residual_tile_kernel<1, false>), reinterpret_cast<const void *>(residual_tile_kernel<2, false>),
            reinterpret_cast<const void *>(residual_tile_kernel<4, false>), reinterpret_cast<const void *>(residual_tile_kernel<8, false>),
            reinterpret_cast<const void *>(vbd_tile_kernel<1, true>), reinterpret_cast<const void *>(vbd_tile_kernel<2, true>),
            reinterpret_cast<const void *>(vbd_tile_kernel<4, true>), reinterpret_cast<const void *>(vbd_tile_kernel<8, true>),
            reinterpret_cast<const void *>(vbd_flow_kernel<1, true>), reinterpret_cast<const void *>(vbd_flow_kernel<2, true>),
            reinterpret_cast<const void *>(vbd_flow_kernel<4, true>), reinterpret_cast<const void *>(vbd_flow_kernel<8, true>),
            reinterpret_cast<const void *>(residual_tile_kernel<1, true>), reinterpret_cast<const void *>(residual_tile_kernel<2, true>),
            reinterpret_cast<const void *>(residual_tile_kernel<4, true>), reinterpret_cast<const void *>(residual_tile_kernel<8, true>)};
        for (const void *fn : fns) SPGX_CUDA(raise(fn));
    }
    return SPGX_OK;
}

// Dataflow tables: each tile's colour and its neighbour tiles (the owners of its halo
// vertices, and itself), the per-tile sweep counters and the resident CTAs per SM.
spgx_status VbdSolver::setup_flow()
{
    const int n_tiles = TL.color_tiles.empty() ? 0 : TL.color_tiles.back();
    std::vector<int32_t> color(std::max(1, n_tiles), 0), tile_of(std::max(1, L.nv), -1);
    for (int c = 0; c < L.n_colors; ++c)
        for (int t = TL.color_tiles[c]; t < TL.color_tiles[c + 1]; ++t) {
            color[t] = c;
            const I4 h = TL.hdr[2 * t];
            for (int i = 0; i < h.y; ++i) tile_of[h.x + i] = t;
        }
    std::vector<int32_t> nbr;
    std::vector<I2> fhdr(std::max(1, n_tiles), I2{0, 0});
    std::vector<int32_t> tmp;
    for (int t = 0; t < n_tiles; ++t) {
        const I4 h = TL.hdr[2 * t];
        tmp.assign(1, t);
        for (int i = 0; i < h.w; ++i) tmp.push_back(tile_of[TL.halo[h.z + i]]);
        std::sort(tmp.begin(), tmp.end());
        tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
        if (!tmp.empty() && tmp.front() < 0) {
            set_error("internal: a halo vertex belongs to no tile");
            return SPGX_ERR_INVALID_ARG;
        }
        fhdr[t] = I2{static_cast<int32_t>(nbr.size()), static_cast<int32_t>(tmp.size())};
        for (int u : tmp) nbr.push_back(color[u] < color[t] ? static_cast<int32_t>(uint32_t(u) | 0x80000000u) : u);
    }
    if (nbr.empty()) nbr.push_back(0);
    SPGX_TRY_STATUS(fl_fhdr.upload(fhdr));
    SPGX_TRY_STATUS(fl_nbrp.upload(nbr));
    SPGX_TRY_STATUS(fl_epoch.alloc(size_t(std::max(1, n_tiles)) * sizeof(int)));
    SPGX_TRY_STATUS(fl_ticket.alloc(2 * sizeof(int)));
    FV = FlowView{fl_fhdr.as<int2>(), fl_nbrp.as<int>(), fl_epoch.as<int>(), fl_ticket.as<int>()};
    SPGX_CUDA(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
    const int T = TL.tile_vertices;
    const bool gen = TV.gen_off != nullptr;
    const void *fns[4] = {gen ? reinterpret_cast<const void *>(vbd_flow_kernel<1, true>)
                              : reinterpret_cast<const void *>(vbd_flow_kernel<1, false>),
                          gen ? reinterpret_cast<const void *>(vbd_flow_kernel<2, true>)
                              : reinterpret_cast<const void *>(vbd_flow_kernel<2, false>),
                          gen ? reinterpret_cast<const void *>(vbd_flow_kernel<4, true>)
                              : reinterpret_cast<const void *>(vbd_flow_kernel<4, false>),
                          gen ? reinterpret_cast<const void *>(vbd_flow_kernel<8, true>)
                              : reinterpret_cast<const void *>(vbd_flow_kernel<8, false>)};
    const int gs[4] = {1, 2, 4, 8};
    for (int i = 0; i < 4; ++i) {
        flow_blocks_per_sm[i] = 0;
        if (T * gs[i] > kTileThreads) continue;
        SPGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&flow_blocks_per_sm[i], fns[i], T * gs[i], tile_smem));
    }
    return reset_flow();
}

spgx_status VbdSolver::take_flow_launch_error()
{
    const cudaError_t e = flow_launch_error;
    flow_launch_error = cudaSuccess;
    if (e == cudaSuccess) return SPGX_OK;
    set_error(std::string("dataflow kernel launch: ") + cudaGetErrorString(e));
    return SPGX_ERR_CUDA;
}

spgx_status VbdSolver::reset_flow()
{
    const int n_tiles = TL.color_tiles.empty() ? 0 : TL.color_tiles.back();
    SPGX_CUDA(cudaMemsetAsync(fl_epoch.as<int>(), 0, size_t(std::max(1, n_tiles)) * sizeof(int), stream));
    SPGX_CUDA(cudaStreamSynchronize(stream));
    flow_epoch = 0;
    return SPGX_OK;
}

spgx_status VbdSolver::check_params(const spgx_vbd_params *p)
{
    if (!p || !(p->dt > 0) || p->substeps < 1 || p->iterations < 0 || p->max_iterations < 0 ||
        (p->tolerance > 0 && p->check_interval < 1) || !(p->fallback_condition > 0)) {
        set_error("invalid VBD parameters");
        return SPGX_ERR_INVALID_ARG;
    }
    const int g = p->lanes_per_vertex;
    if (!(g == 0 || g == 1 || g == 2 || g == 4 || g == 8 || g == 16 || g == 32)) {
        set_error("lanes_per_vertex must be 0, 1, 2, 4, 8, 16 or 32");
        return SPGX_ERR_INVALID_ARG;
    }
    if (p->kernel < 0 || p->kernel > 3 || p->tile_vertices < 0 || p->tile_vertices > kTileMaxVerts) {
        set_error("kernel must be 0, 1, 2 or 3 and tile_vertices in [0, 128]");
        return SPGX_ERR_INVALID_ARG;
    }
    if (p->block_size != 0 && (p->block_size % 32 != 0 || p->block_size < 32 || p->block_size > 256)) {
        set_error("block_size must be 0 or a multiple of 32 in [32, 256]");
        return SPGX_ERR_INVALID_ARG;
    }
    return SPGX_OK;
}

spgx_status VbdSolver::set_params(const spgx_vbd_params *params)
{
    SPGX_TRY_STATUS(check_params(params));
    const bool relaunch = params->lanes_per_vertex != P.lanes_per_vertex || params->block_size != P.block_size ||
                          params->kernel != P.kernel;
    if (params->tile_vertices != P.tile_vertices) {
        set_error("tile_vertices is fixed when the solver is created");
        return SPGX_ERR_INVALID_ARG;
    }
    if (params->device != P.device) {
        set_error("the device of a solver cannot change");
        return SPGX_ERR_INVALID_ARG;
    }
    P = *params;
    h_sub = P.dt / P.substeps;
    graph_valid = false;
    if (relaunch) SPGX_TRY_STATUS(configure_launch());
    return SPGX_OK;
}

// Picks the kernel and its launch shape. Explicit parameters win; otherwise every candidate
// is timed on two sweeps of this scene and the fastest kept: the lanes kernel with lanes up to
// twice the mean vertex degree and blocks of 64/128/256 threads, and the tile and dataflow
// kernels with 1/2/4/8 lanes per vertex on tiles of each size in kTileCandidates (or the
// requested size). The scene is re-tiled for each tile size tried and left tiled for the pick;
// the positions are restored afterwards.
spgx_status VbdSolver::configure_launch()
{
    graph_valid = false;
    struct Cand {
        int kernel, lanes, block, tile;
    };
    const bool want_lanes = P.kernel == 0 || P.kernel == 1;
    const bool want_tiles = P.kernel == 0 || P.kernel == 2;
    const bool want_flow = P.kernel == 0 || P.kernel == 3;
    std::vector<int> tile_sizes;
    if (P.tile_vertices)
        tile_sizes.push_back(P.tile_vertices);
    else if (want_tiles || want_flow)
        tile_sizes.assign(std::begin(kTileCandidates), std::end(kTileCandidates));
    // Candidates of one tile size; the flow candidates read the occupancy of the current tiling.
    auto tile_cands = [&](int T, std::vector<Cand> &out) {
        if (want_tiles)
            for (int g : {1, 2, 4, 8})
                if (T * g <= kTileThreads && (P.lanes_per_vertex == 0 || P.lanes_per_vertex == g))
                    out.push_back({2, g, T * g, T});
        if (want_flow)
            for (int g : {1, 2, 4, 8}) {
                const int li = g == 1 ? 0 : g == 2 ? 1 : g == 4 ? 2 : 3;
                if (T * g <= kTileThreads && T * g >= 32 && flow_blocks_per_sm[li] > 0 &&
                    (P.lanes_per_vertex == 0 || P.lanes_per_vertex == g))
                    out.push_back({3, g, T * g, T});
            }
    };
    auto retile = [&](int T) -> spgx_status {
        if (TL.tile_vertices == T) return SPGX_OK;
        SPGX_TRY_STATUS(setup_tiles(T));
        return setup_flow();
    };
    std::vector<Cand> lane_cands;
    if (want_lanes) {
        std::vector<int> blocks;
        if (P.block_size)
            blocks.push_back(P.block_size);
        else
            blocks = {64, 128, 256};
        std::vector<int> lane_opts;
        if (P.lanes_per_vertex)
            lane_opts.push_back(P.lanes_per_vertex);
        else
            for (int g : {1, 2, 4, 8, 16, 32})
                if (g == 1 || g <= 2 * std::max(1.0, L.mean_degree)) lane_opts.push_back(g);
        for (int g : lane_opts)
            for (int b : blocks) lane_cands.push_back({1, g, b, 0});
    }
    // A single candidate (or an empty scene) needs no timing.
    if (tile_sizes.size() <= 1) {
        std::vector<Cand> all = lane_cands;
        if (!tile_sizes.empty()) {
            SPGX_TRY_STATUS(retile(tile_sizes[0]));
            tile_cands(tile_sizes[0], all);
        }
        if (all.empty()) {
            set_error("no kernel variant fits the requested launch parameters");
            return SPGX_ERR_INVALID_ARG;
        }
        if (all.size() == 1 || L.nv == 0) {
            kernel = all[0].kernel;
            lanes = all[0].lanes;
            block = all[0].block;
            return SPGX_OK;
        }
    }
    SPGX_TRY_STATUS(X.upload_if_dirty(stream));
    SPGX_CUDA(cudaMemcpyAsync(d_backup.as<void>(), S.pos, size_t(L.nv) * 2 * sizeof(float4),
                              cudaMemcpyDeviceToDevice, stream));
    float best = 1e30f;
    Cand pick{};
    bool have_pick = false;
    auto time_all = [&](const std::vector<Cand> &cs) -> spgx_status {
        for (const auto &c : cs) {
            kernel = c.kernel;
            lanes = c.lanes;
            block = c.block;
            launch_iterations(*this, 1, stream);
            SPGX_CUDA(cudaEventRecord(ev0, stream));
            launch_iterations(*this, 2, stream);
            SPGX_CUDA(cudaEventRecord(ev1, stream));
            SPGX_CUDA(cudaEventSynchronize(ev1));
            float ms = 0.f;
            SPGX_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
            if (!have_pick || ms < best) {
                best = ms;
                pick = c;
                have_pick = true;
            }
            SPGX_CUDA(cudaMemcpyAsync(S.pos, d_backup.as<void>(), size_t(L.nv) * 2 * sizeof(float4),
                                      cudaMemcpyDeviceToDevice, stream));
        }
        // A dataflow sweep that gave up leaves its tiles' epochs behind: check before the
        // next tiling replaces them.
        int *hc = h_counters.as<int>();
        SPGX_CUDA(cudaMemcpyAsync(hc, d_counters.as<int>(), kCounters * sizeof(int), cudaMemcpyDeviceToHost, stream));
        SPGX_CUDA(cudaMemsetAsync(d_counters.as<int>(), 0, kCounters * sizeof(int), stream));
        SPGX_CUDA(cudaStreamSynchronize(stream));
        SPGX_CUDA(cudaGetLastError());
        SPGX_TRY_STATUS(take_flow_launch_error());
        if (hc[2] & 2u) {
            SPGX_TRY_STATUS(reset_flow());
            set_error("a dataflow sweep gave up waiting for a neighbour tile while timing launch shapes");
            return SPGX_ERR_TIMEOUT;
        }
        return SPGX_OK;
    };
    SPGX_TRY_STATUS(time_all(lane_cands));
    for (int T : tile_sizes) {
        SPGX_TRY_STATUS(retile(T));
        std::vector<Cand> tc;
        tile_cands(T, tc);
        SPGX_TRY_STATUS(time_all(tc));
    }
    if (!have_pick) {
        set_error("no kernel variant fits the requested launch parameters");
        return SPGX_ERR_INVALID_ARG;
    }
    if (pick.tile) SPGX_TRY_STATUS(retile(pick.tile));
    kernel = pick.kernel;
    lanes = pick.lanes;
    block = pick.block;
    return SPGX_OK;
}

spgx_status VbdSolver::set_picks(int n, const int32_t *object, const int32_t *vertex, const double *target,
                                 const double *k)
{
    if (n < 0 || n > SPGX_MAX_PICKS || (n > 0 && (!object || !vertex || !target || !k))) {
        set_error("picks: 0 to SPGX_MAX_PICKS anchors with object, vertex, target and stiffness");
        return SPGX_ERR_INVALID_ARG;
    }
    int vi[SPGX_MAX_PICKS];
    float4 a[SPGX_MAX_PICKS];
    for (int q = 0; q < n; ++q) {
        if (object[q] < 0 || object[q] >= static_cast<int>(L.objects.size()) || vertex[q] < 0 ||
            vertex[q] >= L.objects[object[q]].nv) {
            set_error("pick " + std::to_string(q) + " names no vertex of the scene");
            return SPGX_ERR_INVALID_ARG;
        }
        vi[q] = L.ext2int[L.objects[object[q]].vertex_base + vertex[q]];
        a[q] = make_float4(float(target[3 * q]), float(target[3 * q + 1]), float(target[3 * q + 2]), float(k[q]));
    }
    if (n > 0) {
        SPGX_CUDA(cudaMemcpyAsync(d_pick_v.as<int>(), vi, n * sizeof(int), cudaMemcpyHostToDevice, stream));
        SPGX_CUDA(cudaMemcpyAsync(d_pick_a.as<float4>(), a, n * sizeof(float4), cudaMemcpyHostToDevice, stream));
        SPGX_CUDA(cudaStreamSynchronize(stream));
    }
    // The count is a kernel argument (captured in the step graph); the slots are read live.
    if (S.n_pick != n) graph_valid = false;
    S.n_pick = n;
    return SPGX_OK;
}

spgx_status VbdSolver::build_graph()
{
    if (graph_exec) {
        cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    SPGX_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < P.substeps; ++s) {
        launch_begin(*this, stream);
        if (W.mode != kWarmInertial) launch_warm(stream);
        launch_iterations(*this, P.iterations - warm_probe_sweeps(), stream);
        launch_end(*this, stream);
    }
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

spgx_status VbdSolver::profile_sweeps(int iterations, double *color_ms)
{
    SPGX_TRY_STATUS(X.upload_if_dirty(stream));
    X.mark_device_advanced();
    const int nc = L.n_colors;
    if (kernel == 3) {  // no per-colour launches: the whole sweep goes to color_ms[0]
        SPGX_CUDA(cudaEventRecord(ev0, stream));
        launch_iterations(*this, iterations, stream);
        SPGX_CUDA(cudaEventRecord(ev1, stream));
        SPGX_CUDA(cudaGetLastError());
        SPGX_CUDA(cudaEventSynchronize(ev1));
        float ms = 0.f;
        SPGX_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        for (int c = 0; c < nc; ++c) color_ms[c] = 0.0;
        if (nc > 0) color_ms[0] = ms / std::max(1, iterations);
        return SPGX_OK;
    }
    std::vector<cudaEvent_t> ev(size_t(nc) * iterations * 2, nullptr);
    for (auto &e : ev) SPGX_CUDA(cudaEventCreate(&e));
    for (int it = 0; it < iterations; ++it)
        for (int c = 0; c < nc; ++c) {
            SPGX_CUDA(cudaEventRecord(ev[2 * (size_t(it) * nc + c)], stream));
            launch_color(*this, c, stream);
            SPGX_CUDA(cudaEventRecord(ev[2 * (size_t(it) * nc + c) + 1], stream));
        }
    SPGX_CUDA(cudaGetLastError());
    SPGX_CUDA(cudaStreamSynchronize(stream));
    for (int c = 0; c < nc; ++c) {
        double acc = 0;
        for (int it = 0; it < iterations; ++it) {
            float ms = 0.f;
            SPGX_CUDA(cudaEventElapsedTime(&ms, ev[2 * (size_t(it) * nc + c)], ev[2 * (size_t(it) * nc + c) + 1]));
            acc += ms;
        }
        color_ms[c] = acc / iterations;
    }
    for (auto &e : ev) cudaEventDestroy(e);
    return SPGX_OK;
}

spgx_status VbdSolver::residual_norm(double *out)
{
    SPGX_CUDA(cudaMemsetAsync(d_resid.as<double>(), 0, sizeof(double), stream));
    launch_residual(*this, stream);
    SPGX_CUDA(cudaGetLastError());
    double *hr = reinterpret_cast<double *>(h_counters.as<int>() + kCounters);
    SPGX_CUDA(cudaMemcpyAsync(hr, d_resid.as<double>(), sizeof(double), cudaMemcpyDeviceToHost, stream));
    SPGX_CUDA(cudaStreamSynchronize(stream));
    *out = std::sqrt(*hr);
    return SPGX_OK;
}

// Initial guess of one substep, after the inertial predict, all on the stream with no host
// round trip. wres[0] = ||r(y)||^2.
// Extrapolated mode: wres[1] = ||r(x_e)||^2, and the substep starts from the better of y and x_e.
// Learned mode: the residual of a guess right after the jump weighs its high-frequency error
// (per-vertex noise stretches the stiff springs) far above its smooth error, which the sweeps
// remove first; the learned guess x_e + l MLP has much lower error overall but a higher
// initial residual. So each of x_w and x_e first runs kWarmProbeSweeps sweeps: wres[1] and
// wres[2] are the residuals after them, and the substep continues from the better state (the
// other probe's sweeps are spent). Returns the sweeps the probes ran.
int VbdSolver::launch_warm(cudaStream_t st)
{
    double *wres = W.wres.as<double>();
    cudaMemsetAsync(wres, 0, 3 * sizeof(double), st);
    launch_residual(*this, st, wres);
    launch_warm_extrapolate(W, X.pos(), X.tgt(), X.vel(), L.nv, h_sub, P.gravity, st);
    if (W.mode != kWarmLearned) {
        launch_residual(*this, st, wres + 1);
        launch_warm_select(W, X.pos(), X.tgt(), X.vel(), L.nv, h_sub, P.gravity, false, d_counters.as<int>(), st);
        return 0;
    }
    const int probe = warm_probe_sweeps();
    launch_warm_features(W, X.vel(), L.nv, h_sub, P.gravity, st);
    W.mlp->infer(W.feats.as<float>(), L.nv, W.out.as<float>(), st);
    launch_warm_smooth(W, L.nv, st);
    launch_warm_apply(W, X.pos(), X.tgt(), X.vel(), L.nv, h_sub, P.gravity, st);
    launch_iterations(*this, probe, st);
    launch_residual(*this, st, wres + 1);
    cudaMemcpyAsync(d_backup.as<void>(), X.pos(), size_t(L.nv) * 2 * sizeof(float4), cudaMemcpyDeviceToDevice, st);
    launch_warm_extrapolate(W, X.pos(), X.tgt(), X.vel(), L.nv, h_sub, P.gravity, st);
    launch_iterations(*this, probe, st);
    launch_residual(*this, st, wres + 2);
    launch_warm_probe_select(W, X.pos(), d_backup.as<float4>(), L.nv, d_counters.as<int>(), st);
    return 2 * probe;
}

// Uploads positions/velocities set from the host; a replaced state restarts the displacement
// history at constant velocity.
spgx_status VbdSolver::upload_state()
{
    const bool replaced = X.take_replaced();
    if (replaced && W.history)
        SPGX_CUDA(cudaMemcpyAsync(W.vhist.as<void>(), X.vel(), size_t(L.nv) * sizeof(float4),
                                  cudaMemcpyDeviceToDevice, stream));
    return SPGX_OK;
}

spgx_status VbdSolver::enable_history()
{
    if (W.history) return SPGX_OK;
    std::vector<int32_t> off, nbr;
    std::vector<F4> stat;
    build_vertex_neighbours(L, off, nbr, stat);
    if (nbr.empty()) nbr.push_back(0);
    SPGX_TRY_STATUS(W.nbr_off.upload(off));
    SPGX_TRY_STATUS(W.nbr.upload(nbr));
    SPGX_TRY_STATUS(W.stat.upload(stat));
    const size_t n = size_t(std::max(1, L.nv));
    SPGX_TRY_STATUS(W.vhist.alloc(n * sizeof(float4)));
    SPGX_TRY_STATUS(W.feats.alloc(n * kWarmFeatures * sizeof(float)));
    SPGX_TRY_STATUS(W.out.alloc(n * 3 * sizeof(float)));
    SPGX_TRY_STATUS(W.out2.alloc(n * 3 * sizeof(float)));
    SPGX_TRY_STATUS(W.wres.alloc(3 * sizeof(double)));
    // No earlier motion is known: take the previous step's displacement equal to the current
    // velocity's (constant-velocity history).
    SPGX_TRY_STATUS(X.upload_if_dirty(stream));
    SPGX_CUDA(cudaMemcpyAsync(W.vhist.as<void>(), X.vel(), size_t(L.nv) * sizeof(float4), cudaMemcpyDeviceToDevice,
                              stream));
    SPGX_CUDA(cudaStreamSynchronize(stream));
    W.history = true;
    graph_valid = false;
    return SPGX_OK;
}

spgx_status VbdSolver::set_warm_start(const Mlp *mlp, int mode)
{
    if (mode < kWarmInertial || mode > kWarmExtrapolate) {
        set_error("warm-start mode must be 0 (inertial), 1 (learned) or 2 (extrapolated)");
        return SPGX_ERR_INVALID_ARG;
    }
    if (mode == kWarmLearned && !mlp) {
        set_error("the learned warm start needs an MLP handle");
        return SPGX_ERR_INVALID_ARG;
    }
    if (mlp && mlp->device != device) {
        set_error("the MLP handle lives on another device than the solver");
        return SPGX_ERR_INVALID_ARG;
    }
    SPGX_TRY_STATUS(enable_history());
    W.mlp = mlp;
    W.mode = mode;
    graph_valid = false;
    return SPGX_OK;
}

spgx_status VbdSolver::step(spgx_step_stats *stats, float *features, float *targets)
{
    const bool record = features || targets;
    if (record && (P.substeps != 1 || !W.history)) {
        set_error("recording needs one substep and the displacement history (spgx_vbd_set_warm_start)");
        return SPGX_ERR_INVALID_ARG;
    }
    SPGX_TRY_STATUS(upload_state());
    X.mark_device_advanced();
    if (flow_epoch > (1 << 30)) SPGX_TRY_STATUS(reset_flow());  // keep the sweep counters far from overflow
    spgx_step_stats st{};
    SPGX_CUDA(cudaMemsetAsync(d_counters.as<int>(), 0, kCounters * sizeof(int), stream));
    SPGX_CUDA(cudaEventRecord(ev0, stream));
    double *hw = reinterpret_cast<double *>(h_counters.as<int>() + kCounters);  // 4 doubles of pinned scratch
    if (P.tolerance <= 0 && !record) {
        if (P.use_graph && kernel != 3) {
            if (!graph_valid) SPGX_TRY_STATUS(build_graph());
            SPGX_CUDA(cudaGraphLaunch(graph_exec, stream));
        } else {
            for (int s = 0; s < P.substeps; ++s) {
                launch_begin(*this, stream);
                if (W.mode != kWarmInertial) launch_warm(stream);
                launch_iterations(*this, P.iterations - warm_probe_sweeps(), stream);
                launch_end(*this, stream);
            }
        }
        // The probe of the guess that was not kept adds its sweeps.
        st.iterations = (P.iterations + warm_probe_sweeps()) * P.substeps;
        st.converged = 1;
    } else {
        st.converged = 1;
        for (int s = 0; s < P.substeps; ++s) {
            launch_begin(*this, stream);
            double r0 = 0, r = 0;
            int probe = 0;  // sweeps already applied to the state the substep continues from
            if (W.mode != kWarmInertial) {
                launch_warm(stream);
                SPGX_CUDA(cudaMemcpyAsync(hw, W.wres.as<double>(), 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                          stream));
                SPGX_CUDA(cudaStreamSynchronize(stream));
                const bool learned = W.mode == kWarmLearned;
                r0 = std::sqrt(hw[0]);
                st.residual_warm = std::sqrt(hw[1]);
                st.residual_extrapolated = std::sqrt(learned ? hw[2] : hw[1]);
                r = std::sqrt(learned ? std::min(hw[1], hw[2]) : std::min(hw[0], hw[1]));
                probe = warm_probe_sweeps();
                st.iterations += probe;  // the probe that was not kept
            } else {
                if (P.tolerance > 0) SPGX_TRY_STATUS(residual_norm(&r0));
                r = r0;
            }
            // Features depend on the velocities and the history only; the learned guess has
            // computed them already.
            if (record && W.mode != kWarmLearned) launch_warm_features(W, X.vel(), L.nv, h_sub, P.gravity, stream);
            if (P.tolerance > 0) {
                // Sweeps run in chunks of check_interval between residual checks. Once two
                // checks give a decay rate, the next chunk is cut to the sweeps that rate needs to
                // reach the tolerance (5 % margin, at least kMinCheckChunk): a check costs about
                // one sweep, and a full last chunk would overshoot by half an interval on average.
                constexpr int kMinCheckChunk = 10;
                int it = probe, it_prev = -1;
                double r_prev = 0.0;
                while (it < P.max_iterations && r > P.tolerance * r0) {
                    int chunk = std::min(P.check_interval, P.max_iterations - it);
                    if (it_prev >= 0 && r < r_prev && r > 0.0) {
                        const double rate = std::log(r / r_prev) / double(it - it_prev);  // per sweep, < 0
                        const double need = std::log(P.tolerance * r0 / r) / rate;
                        if (std::isfinite(need) && need > 0.0)
                            chunk = std::min(chunk, std::max(kMinCheckChunk, static_cast<int>(std::ceil(1.05 * need))));
                    }
                    r_prev = r;
                    it_prev = it;
                    launch_iterations(*this, chunk, stream);
                    it += chunk;
                    SPGX_TRY_STATUS(residual_norm(&r));
                }
                if (r > P.tolerance * r0) st.converged = 0;
                st.iterations += it;
                st.residual_initial = r0;
                st.residual_final = r;
            } else {
                launch_iterations(*this, P.iterations - probe, stream);
                st.iterations += P.iterations;
            }
            if (record) launch_warm_targets(X.pos(), X.tgt(), L.nv, h_sub, W.out.as<float>(), stream);
            launch_end(*this, stream);
        }
    }
    SPGX_CUDA(cudaEventRecord(ev1, stream));
    SPGX_CUDA(cudaGetLastError());
    SPGX_TRY_STATUS(take_flow_launch_error());
    int *hc = h_counters.as<int>();
    SPGX_CUDA(cudaMemcpyAsync(hc, d_counters.as<int>(), kCounters * sizeof(int), cudaMemcpyDeviceToHost, stream));
    if (features)
        SPGX_CUDA(cudaMemcpyAsync(features, W.feats.as<float>(), size_t(L.nv) * kWarmFeatures * sizeof(float),
                                  cudaMemcpyDeviceToHost, stream));
    if (targets)
        SPGX_CUDA(cudaMemcpyAsync(targets, W.out.as<float>(), size_t(L.nv) * 3 * sizeof(float),
                                  cudaMemcpyDeviceToHost, stream));
    SPGX_CUDA(cudaStreamSynchronize(stream));
    float ms = 0.f;
    SPGX_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    st.device_ms = ms;
    st.fallback_solves = hc[0];
    st.skipped_solves = hc[1];
    st.warm_accepted = hc[3];
    st.extrapolated_accepted = hc[4];
    if (stats) *stats = st;
    if (hc[2] & 2u) {
        SPGX_TRY_STATUS(reset_flow());
        set_error("a dataflow sweep gave up waiting for a neighbour tile; the step is incomplete");
        return SPGX_ERR_TIMEOUT;
    }
    if (hc[2] & 1u) {
        set_error("a vertex update produced a non-finite position; the update was not stored");
        return SPGX_ERR_NONFINITE;
    }
    return SPGX_OK;
}

VbdSolver::~VbdSolver()
{
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
}

}  // namespace spgx

// =======================================================================================
// C ABI

using spgx::VbdSolver;

struct spgx_vbd {
    std::unique_ptr<VbdSolver> s;
};

extern "C" {

spgx_status spgx_vbd_create(const spgx_scene_desc *scene, const spgx_vbd_params *params, spgx_vbd **out)
{
    SPGX_GUARD_BEGIN
    if (!out) {
        spgx::set_error("out is NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    *out = nullptr;
    spgx_vbd_params p;
    if (params)
        p = *params;
    else
        spgx_vbd_params_default(&p);
    auto h = std::make_unique<spgx_vbd>();
    h->s = std::make_unique<VbdSolver>();
    SPGX_TRY_STATUS(h->s->init(scene, &p));
    *out = h.release();
    spgx::clear_error();
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_vbd_destroy(spgx_vbd *h)
{
    SPGX_GUARD_BEGIN
    if (h) {
        cudaSetDevice(h->s->device);
        delete h;
    }
    return SPGX_OK;
    SPGX_GUARD_END
}

#define SPGX_HANDLE(h)                                 \
    if (!(h)) {                                        \
        spgx::set_error("NULL solver handle");         \
        return SPGX_ERR_INVALID_ARG;                   \
    }                                                  \
    SPGX_CUDA(cudaSetDevice((h)->s->device))

spgx_status spgx_vbd_set_params(spgx_vbd *h, const spgx_vbd_params *params)
{
    SPGX_GUARD_BEGIN
    SPGX_HANDLE(h);
    return h->s->set_params(params);
    SPGX_GUARD_END
}

spgx_status spgx_vbd_step(spgx_vbd *h, spgx_step_stats *stats)
{
    SPGX_GUARD_BEGIN
    SPGX_HANDLE(h);
    return h->s->step(stats);
    SPGX_GUARD_END
}

spgx_status spgx_vbd_get_state(spgx_vbd *h, int32_t object, double *x, double *v)
{
    SPGX_GUARD_BEGIN
    SPGX_HANDLE(h);
    return h->s->X.get(h->s->L, object, x, v, h->s->stream);
    SPGX_GUARD_END
}

spgx_status spgx_vbd_set_state(spgx_vbd *h, int32_t object, const double *x, const double *v)
{
    SPGX_GUARD_BEGIN
    SPGX_HANDLE(h);
    return h->s->X.set(h->s->L, object, x, v, h->s->stream);
    SPGX_GUARD_END
}

spgx_status spgx_vbd_reset(spgx_vbd *h)
{
    SPGX_GUARD_BEGIN
    SPGX_HANDLE(h);
    return h->s->X.reset(h->s->L, h->s->stream);
    SPGX_GUARD_END
}

spgx_status spgx_vbd_residual(spgx_vbd *h, double *norm)
{
    SPGX_GUARD_BEGIN
    SPGX_HANDLE(h);
    if (!norm) {
        spgx::set_error("norm is NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    SPGX_TRY_STATUS(h->s->upload_state());
    return h->s->residual_norm(norm);
    SPGX_GUARD_END
}

spgx_status spgx_vbd_set_warm_start(spgx_vbd *h, const spgx_mlp *mlp, int32_t mode)
{
    SPGX_GUARD_BEGIN
    SPGX_HANDLE(h);
    return h->s->set_warm_start(mlp ? mlp->m.get() : nullptr, mode);
    SPGX_GUARD_END
}

spgx_status spgx_vbd_get_vertex_order(spgx_vbd *h, int32_t *ext_of_internal)
{
    SPGX_GUARD_BEGIN
    SPGX_HANDLE(h);
    if (!ext_of_internal) {
        spgx::set_error("ext_of_internal is NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    const auto &L = h->s->L;
    std::copy(L.int2ext.begin(), L.int2ext.end(), ext_of_internal);
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_vbd_step_record(spgx_vbd *h, float *features, float *targets, spgx_step_stats *stats)
{
    SPGX_GUARD_BEGIN
    SPGX_HANDLE(h);
    if (!features || !targets) {
        spgx::set_error("features and targets must not be NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    return h->s->step(stats, features, targets);
    SPGX_GUARD_END
}

spgx_status spgx_vbd_num_colors(spgx_vbd *h, int32_t object, int32_t *n)
{
    SPGX_GUARD_BEGIN
    if (!h || !n || object < -1 || object >= static_cast<int>(h->s->L.objects.size())) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    *n = object < 0 ? h->s->L.n_colors : h->s->L.objects[object].n_colors;
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_vbd_get_colors(spgx_vbd *h, int32_t object, int32_t *colors)
{
    SPGX_GUARD_BEGIN
    if (!h || !colors || object < 0 || object >= static_cast<int>(h->s->L.objects.size())) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    const auto &c = h->s->L.objects[object].colors;
    std::copy(c.begin(), c.end(), colors);
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_vbd_get_adjacency(spgx_vbd *h, int32_t object, int32_t *counts, int32_t *entries, int64_t *total)
{
    SPGX_GUARD_BEGIN
    if (!h || !total || object < 0 || object >= static_cast<int>(h->s->L.objects.size())) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    const auto &O = h->s->L.objects[object];
    *total = static_cast<int64_t>(O.adj_entries.size() / 2);
    if (counts) std::copy(O.adj_counts.begin(), O.adj_counts.end(), counts);
    if (entries) std::copy(O.adj_entries.begin(), O.adj_entries.end(), entries);
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_vbd_set_picks(spgx_vbd *h, int32_t n, const int32_t *object, const int32_t *vertex,
                               const double *target, const double *stiffness)
{
    SPGX_GUARD_BEGIN
    if (!h) {
        spgx::set_error("NULL solver handle");
        return SPGX_ERR_INVALID_ARG;
    }
    SPGX_CUDA(cudaSetDevice(h->s->device));
    return h->s->set_picks(n, object, vertex, target, stiffness);
    SPGX_GUARD_END
}

spgx_status spgx_vbd_set_warm_start_smoothing(spgx_vbd *h, int32_t passes)
{
    SPGX_GUARD_BEGIN
    if (!h || passes < 0 || passes > 64) {
        spgx::set_error("smoothing passes must be in [0, 64]");
        return SPGX_ERR_INVALID_ARG;
    }
    h->s->W.smooth = passes;
    h->s->graph_valid = false;
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_vbd_test_stall_tile(spgx_vbd *h, int32_t tile)
{
    SPGX_GUARD_BEGIN
    if (!h) {
        spgx::set_error("NULL solver handle");
        return SPGX_ERR_INVALID_ARG;
    }
    auto &s = *h->s;
    const int n_tiles = s.TL.color_tiles.empty() ? 0 : s.TL.color_tiles.back();
    if (s.kernel != 3 || tile < 0 || tile >= n_tiles) {
        spgx::set_error("the handle does not run the dataflow kernel, or no such tile");
        return SPGX_ERR_INVALID_ARG;
    }
    SPGX_CUDA(cudaSetDevice(s.device));
    // A sweep counter no sweep ever reaches: every task that reads this tile waits until its
    // bounded poll gives up.
    const int never = -(1 << 30);
    SPGX_CUDA(cudaMemcpyAsync(s.fl_epoch.as<int>() + tile, &never, sizeof(int), cudaMemcpyHostToDevice, s.stream));
    SPGX_CUDA(cudaStreamSynchronize(s.stream));
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_vbd_get_launch(spgx_vbd *h, int32_t *kernel, int32_t *lanes_per_vertex, int32_t *block_size)
{
    SPGX_GUARD_BEGIN
    if (!h) {
        spgx::set_error("NULL solver handle");
        return SPGX_ERR_INVALID_ARG;
    }
    if (kernel) *kernel = h->s->kernel;
    if (lanes_per_vertex) *lanes_per_vertex = h->s->lanes;
    if (block_size) *block_size = h->s->block;
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_vbd_profile_sweeps(spgx_vbd *h, int32_t iterations, double *color_ms)
{
    SPGX_GUARD_BEGIN
    SPGX_HANDLE(h);
    if (iterations < 1 || !color_ms) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    return h->s->profile_sweeps(iterations, color_ms);
    SPGX_GUARD_END
}

}  // extern "C"
