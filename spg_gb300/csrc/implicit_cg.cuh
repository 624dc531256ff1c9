// The global solvers' conjugate gradients (Eigen::ConjugateGradient with the diagonal
// preconditioner, as ImplicitEulerBase::solveLinearSystem calls it, implicitEulerBase.cpp:
// 225-240) as one persistent cooperative launch per solve, in double-float arithmetic.
//
// Why this shape on GB300:
// - FP64 runs at about 1/64 of the FP32 rate, so the vector updates (x += alpha p,
//   r -= alpha Ap, z = D^-1 r, p = z + beta p and the three dot products) are done on FP32
//   hi/lo pairs (48 significant bits) with error-free products and sums. Only the block
//   partial sums and the scalars alpha, beta are FP64.
// - The matrix is symmetric (a Hessian), so only its upper blocks and the diagonal are stored:
//   1.84 M instead of 3.42 M blocks on the 513^2 cloth. Row i reads its lower blocks (i, j),
//   j < i, as the transposes of the stored (j, i). The rows are in reverse Cuthill-McKee
//   order, so block (j, i) was read by row j a few hundred rows earlier and is still in L2.
// - One launch holds the whole solve, one block of 1024 threads per SM, each block owning an
//   equal contiguous range of rows in every phase. Two grid barriers per iteration: after the
//   product with its dot products (a reduction), and after the vector update. A barrier is a
//   counter every block adds to (release) and polls (acquire) until all blocks have arrived;
//   after a reduction each block sums every block's partials itself, in the same fixed order,
//   so alpha, beta and the stopping decision are identical everywhere without a second round
//   trip, and the solve is deterministic. Every wait is bounded; a wait that runs out sets a
//   status the host reports.
//
// Stopping rule and iteration count are those of the FP64 path: |r|^2 < tol^2 |b|^2 after an
// update, or max_its updates.

constexpr int kCgThreads = 1024;
constexpr int kCgMaxPolls = 1 << 21;  // with 32 ns sleeps and an L2 round trip: about a second per wait

// Symmetric block matrix in double-float: for row i the upper blocks (i, j), j >= i, diagonal
// first, and references to the stored transposes of its lower blocks. A block is one 80-byte
// record, entries q = 0..8 (row-major) as {hi, lo} pairs and 8 bytes of padding, read with five
// 16-byte loads (three or four 32-byte sectors, also for the scattered transposed reads).
struct CgSymDf {
    const int *urow;     // upper blocks of row i: [urow[i], urow[i+1]), nv + 1 entries
    const int *ucol;     // their block columns
    const float4 *ublk;  // upper block k at ublk[5 k .. 5 k + 4]
    const int *lrow;     // lower blocks of row i: [lrow[i], lrow[i+1])
    const int2 *lent;    // {column j, upper position of block (j, i)}
    int nnzu;
};
constexpr int kCgBlockFloat4 = 5;

// The solve's vectors: one 24-byte record per row (vertex), {x.hi, x.lo}, {y.hi, y.lo},
// {z.hi, z.lo}: the vector pass streams twelve of them per row and iteration.
struct CgDfVecs {
    const double *b;     // right-hand side (FP64, 3 per row)
    const double *dinv;  // diagonal preconditioner 1 / A_ii (FP64, 3 per row)
    double *x;           // the solution, written in FP64 at the end
    float2 *x2, *r2, *p2, *Ap2, *d2;  // Ap2 holds s = A p (kept by recurrence)
    float2 *u2, *w2;                   // u = D^-1 r and w = A u
    double *part;        // per barrier parity and block: {p.Ap, r.r, r.z, out of range}
    int nv;
};

struct CgSync {
    int arrive;  // arrivals at all barriers so far
    int status;  // 0, kCgTimeout or kCgOutOfRange
};
constexpr int kCgTimeout = 1;
constexpr int kCgOutOfRange = 2;

// (h, l) with |l| <= ulp(h) / 2 from an unnormalised pair (fast two-sum; |h| >= |l|).
__device__ __forceinline__ float2 df_norm(float h, float l)
{
    const float s = __fadd_rn(h, l);
    return make_float2(s, __fsub_rn(l, __fsub_rn(s, h)));
}
// a * b + c, normalised.
__device__ __forceinline__ float2 df_madd(float2 a, float2 b, float2 c)
{
    float h = c.x, l = c.y;
    df_fma(h, l, a, b);
    return df_norm(h, l);
}
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ bool df_out_of_range(float2 a) { return !(fabsf(a.x) <= 0x1p60f); }

// One row's three double-float values.
struct DF3 {
    float2 v[3];
};
// Vectors written within the launch are read with plain (coherent) loads: after a grid
// barrier's acquire and the CTA barrier that follows it, they see every block's writes, and the
// neighbours a block gathers (rows a few hundred apart in reverse Cuthill-McKee order) mostly
// hit its L1. The read-only path (__ldg) is kept for the matrix, which the launch never writes.
__device__ __forceinline__ DF3 ld_row(const float2 *P, int i)
{
    const float2 *q = P + 3 * size_t(i);
    return {{q[0], q[1], q[2]}};
}
__device__ __forceinline__ void st_row(float2 *P, int i, const DF3 &r)
{
    float2 *q = P + 3 * size_t(i);
    q[0] = r.v[0];
    q[1] = r.v[1];
    q[2] = r.v[2];
}
__device__ __forceinline__ bool df3_out_of_range(const DF3 &r)
{
    return df_out_of_range(r.v[0]) || df_out_of_range(r.v[1]) || df_out_of_range(r.v[2]);
}
// Scalars shared through global memory within the launch are read past the L1.
template <typename T>
__device__ __forceinline__ T vload(const T *p)
{
    return *(volatile const T *)p;
}

// Sums of four per-thread values over the block (three double-float, one flag), written by
// lane 0 of warp 0 to part[4 * blockIdx.x ...]: warp sums, then warp 0 sums the warps', all
// in double-float (FP32 pipes); only the three results are formed in FP64. Fixed order.
__device__ __forceinline__ void cg_block_partials(float2 a, float2 b, float2 c, bool bad, double *part)
{
    auto warp_sum = [](float2 &v) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            df_add(v.x, v.y, __shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
    };
    warp_sum(a);
    warp_sum(b);
    warp_sum(c);
    const bool any_bad = __any_sync(0xffffffffu, bad);
    __shared__ float2 s_w[kCgThreads / 32][3];
    __shared__ int s_bad[kCgThreads / 32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        s_w[w][0] = a;
        s_w[w][1] = b;
        s_w[w][2] = c;
        s_bad[w] = any_bad;
    }
    __syncthreads();
    if (w == 0) {
        const bool in = lane < kCgThreads / 32;
        float2 x = in ? s_w[lane][0] : make_float2(0.f, 0.f), y = in ? s_w[lane][1] : make_float2(0.f, 0.f),
               z = in ? s_w[lane][2] : make_float2(0.f, 0.f);
        warp_sum(x);
        warp_sum(y);
        warp_sum(z);
        const bool nb = __any_sync(0xffffffffu, in && s_bad[lane]);
        if (lane == 0) {
            part[4 * blockIdx.x] = double(x.x) + double(x.y);
            part[4 * blockIdx.x + 1] = double(y.x) + double(y.y);
            part[4 * blockIdx.x + 2] = double(z.x) + double(z.y);
            part[4 * blockIdx.x + 3] = nb ? 1.0 : 0.0;
        }
    }
}

// Grid barrier number gen of the CG launch (grid_counter_sync on the solve's counter).
__device__ __forceinline__ void cg_grid_sync(CgSync *s, int &gen)
{
    grid_counter_sync(&s->arrive, &s->status, gen, kCgMaxPolls, kCgTimeout);
}

__device__ __forceinline__ int cg_status(const CgSync *s) { return vload(&s->status); }

// Every block's sums of the four partials of barrier gen over all blocks (fixed order, so the
// same in every block), into tot[4] in shared memory: the block's partials are written, the
// grid barrier passed, and warp 0 adds. The partials alternate between two buffers by barrier
// parity: a block can be at most one barrier ahead of another while that one still reads.
__device__ __forceinline__ void cg_allreduce(const CgDfVecs &V, CgSync *S, int &gen, float2 a, float2 b, float2 c,
                                             bool bad, double *tot)
{
    double *part = V.part + size_t(gen & 1) * 4 * gridDim.x;
    cg_block_partials(a, b, c, bad, part);
    cg_grid_sync(S, gen);
    if (threadIdx.x < 32) {
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        for (int k = threadIdx.x; k < gridDim.x; k += 32)
#pragma unroll
            for (int q = 0; q < 4; ++q) s[q] += __ldcg(part + 4 * k + q);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int q = 0; q < 4; ++q) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
        if (threadIdx.x == 0)
#pragma unroll
            for (int q = 0; q < 4; ++q) tot[q] = s[q];
    }
    __syncthreads();
}

// (h, l)[r] += row r of the block at bp (of its transpose with kT) times x, in double-float.
template <bool kT>
__device__ __forceinline__ void cg_block_product(const float4 *bp, const DF3 &x, float h[3], float l[3])
{
    const float4 q0 = __ldg(bp), q1 = __ldg(bp + 1), q2 = __ldg(bp + 2), q3 = __ldg(bp + 3), q4 = __ldg(bp + 4);
    const float2 e[9] = {make_float2(q0.x, q0.y), make_float2(q0.z, q0.w), make_float2(q1.x, q1.y),
                         make_float2(q1.z, q1.w), make_float2(q2.x, q2.y), make_float2(q2.z, q2.w),
                         make_float2(q3.x, q3.y), make_float2(q3.z, q3.w), make_float2(q4.x, q4.y)};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) df_fma(h[r], l[r], kT ? e[3 * c + r] : e[3 * r + c], x.v[c]);
}

// The whole CG solve, with LANES lanes per block row in the product. The grid must be
// co-resident (cooperative launch). *wide is set by the split when the matrix is out of
// double-float range; the solve then reports kCgOutOfRange at once, as it does when the
// right-hand side or an iterate leaves the range, and the host runs the FP64 path.
template <int LANES>
__global__ void __launch_bounds__(kCgThreads, 1) implicit_cg_df_kernel(CgSymDf A, CgDfVecs V, CgSync *S, CgControl *C,
                                                                        const int *wide, double tol, int max_its)
{
    const int nv = V.nv;
    const int r0 = int(static_cast<long long>(blockIdx.x) * nv / gridDim.x);
    const int r1 = int(static_cast<long long>(blockIdx.x + 1) * nv / gridDim.x);
    const bool reporter = blockIdx.x == 0 && threadIdx.x == 0;
    if (vload(wide)) {
        if (reporter) {
            S->status = kCgOutOfRange;
            C->done = 1;
        }
        return;
    }
    __shared__ double s_tot[4];
    __shared__ float2 s_scalar;  // alpha or beta in double-float, for the vector phases
    int gen = 0;

    // The iteration in the Chronopoulos-Gear form of preconditioned CG (the same iterates as
    // Eigen's CG in exact arithmetic): with u = D^-1 r, w = A u, gamma = r.u, delta = u.w,
    //   beta = gamma / gamma_prev, alpha = gamma / (delta - beta gamma / alpha_prev),
    //   p = u + beta p, s = w + beta s (s = A p by recurrence), x += alpha p, r -= alpha s,
    // so the product and all three dot products (with r.r for the stopping test) need one
    // grid reduction per iteration instead of two. The stopping test (|r|^2 < tol^2 |b|^2 after
    // an update, or max_its updates) and the iteration count are those of the FP64 path.

    // Start (x = 0, p = s = 0): r = b, u = D^-1 r. r.u and r.r are summed where r and u are
    // formed (here and in the vector pass) and reduced with the next product's u.w.
    bool bad = false;
    float2 ru_part = make_float2(0.f, 0.f), rr_part = ru_part;
    {
        const DF3 zero3{{make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)}};
        for (int i = r0 + threadIdx.x; i < r1; i += kCgThreads) {
            DF3 r, d, u;
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                bool o1, o2;
                r.v[c] = split_df(V.b[3 * size_t(i) + c], o1);
                d.v[c] = split_df(V.dinv[3 * size_t(i) + c], o2);
                u.v[c] = df_madd(d.v[c], r.v[c], make_float2(0.f, 0.f));
                ru_part = df_madd(r.v[c], u.v[c], ru_part);
                rr_part = df_madd(r.v[c], r.v[c], rr_part);
                bad |= o1 | o2;
            }
            st_row(V.x2, i, zero3);
            st_row(V.r2, i, r);
            st_row(V.d2, i, d);
            st_row(V.u2, i, u);
            st_row(V.p2, i, zero3);
            st_row(V.Ap2, i, zero3);
        }
        cg_grid_sync(S, gen);  // u complete before the product gathers it
    }
    __shared__ double s_alpha;
    double rr0 = 0.0, thr2 = 0.0, rr_last = 0.0, gamma_prev = 0.0, alpha_prev = 1.0;
    int its = 0;
    bool out_of_range = false;

    for (int k = 0; !cg_status(S); ++k) {
        // w = A u (upper blocks, then the transposes of the lower ones); u.w.
        {
            float2 uw = make_float2(0.f, 0.f);
            const int w = threadIdx.x >> 5, lane = threadIdx.x & (LANES - 1);
            for (int base = r0 + w * (32 / LANES); base < r1; base += kCgThreads / LANES) {
                const int i = base + (threadIdx.x & 31) / LANES;
                float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
                if (i < r1) {
                    const int u0 = __ldg(A.urow + i), nu = __ldg(A.urow + i + 1) - u0;
                    const int w0 = __ldg(A.lrow + i), nl = __ldg(A.lrow + i + 1) - w0;
                    // Upper blocks: row r of block (i, c) times u_c. The next trip's column is
                    // fetched before this trip's values are used.
                    int cn = lane < nu ? __ldg(A.ucol + u0 + lane) : 0;
                    for (int t = lane; t < nu; t += LANES) {
                        const int kk = u0 + t, c = cn;
                        if (t + LANES < nu) cn = __ldg(A.ucol + kk + LANES);
                        cg_block_product<false>(A.ublk + kCgBlockFloat4 * size_t(kk), ld_row(V.u2, c), h, l);
                    }
                    // Lower blocks: block (i, c) is the transpose of the stored (c, i).
                    int2 en = lane < nl ? __ldg(A.lent + w0 + lane) : make_int2(0, 0);
                    for (int t = lane; t < nl; t += LANES) {
                        const int2 e = en;
                        if (t + LANES < nl) en = __ldg(A.lent + w0 + t + LANES);
                        cg_block_product<true>(A.ublk + kCgBlockFloat4 * size_t(e.y), ld_row(V.u2, e.x), h, l);
                    }
                }
#pragma unroll
                for (int o = LANES / 2; o > 0; o >>= 1)
#pragma unroll
                    for (int r = 0; r < 3; ++r)
                        df_add(h[r], l[r], __shfl_xor_sync(0xffffffffu, h[r], o), __shfl_xor_sync(0xffffffffu, l[r], o));
                if (i < r1 && lane == 0) {
                    const DF3 wi{{df_norm(h[0], l[0]), df_norm(h[1], l[1]), df_norm(h[2], l[2])}};
                    st_row(V.w2, i, wi);
                    const DF3 ui = ld_row(V.u2, i);
#pragma unroll
                    for (int r = 0; r < 3; ++r) uw = df_madd(ui.v[r], wi.v[r], uw);
                    bad |= df3_out_of_range(wi);
                }
            }
            cg_allreduce(V, S, gen, ru_part, rr_part, uw, bad, s_tot);
        }
        if (cg_status(S)) break;
        const double gamma = s_tot[0], rr = s_tot[1], delta = s_tot[2];
        if (s_tot[3] != 0.0) {
            out_of_range = true;
            break;
        }
        if (k == 0) {
            // Eigen's start: nothing to do for b = 0; otherwise iterate while |r|^2 >= thr2.
            rr0 = rr_last = rr;
            thr2 = fmax(tol * tol * rr0, 1e-300);
            if (rr0 == 0.0 || rr0 < thr2 || max_its <= 0) break;
        } else {
            ++its;
            if (rr < thr2 || its >= max_its) {
                rr_last = rr;
                break;
            }
        }
        if (threadIdx.x == 0) {
            bool o;
            const double beta = k == 0 ? 0.0 : gamma / gamma_prev;
            const double alpha = gamma / (delta - beta * gamma / alpha_prev);
            s_scalar = split_df(beta, o);
            s_alpha = alpha;
        }
        __syncthreads();
        const double alpha_d = s_alpha;
        const float2 beta = s_scalar;
        alpha_prev = alpha_d;
        gamma_prev = gamma;

        // p = u + beta p; s = w + beta s; x += alpha p; r -= alpha s; u = D^-1 r.
        {
            bool o;
            const float2 alpha = split_df(alpha_d, o);
            const float2 nalpha = df_neg(alpha);
            bad = o || df_out_of_range(beta);
            ru_part = rr_part = make_float2(0.f, 0.f);
            float2 *__restrict__ xv = V.x2, *__restrict__ rv = V.r2, *__restrict__ pv = V.p2,
                                 *__restrict__ sv = V.Ap2, *__restrict__ uv = V.u2;
            const float2 *__restrict__ wv = V.w2, *__restrict__ dv = V.d2;
            for (int i = r0 + threadIdx.x; i < r1; i += kCgThreads) {
                DF3 p = ld_row(pv, i), sr = ld_row(sv, i), x = ld_row(xv, i), r = ld_row(rv, i);
                const DF3 u = ld_row(uv, i), wi = ld_row(wv, i), d = ld_row(dv, i);
                DF3 un;
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    p.v[c] = df_madd(beta, p.v[c], u.v[c]);
                    sr.v[c] = df_madd(beta, sr.v[c], wi.v[c]);
                    x.v[c] = df_madd(alpha, p.v[c], x.v[c]);
                    r.v[c] = df_madd(nalpha, sr.v[c], r.v[c]);
                    un.v[c] = df_madd(d.v[c], r.v[c], make_float2(0.f, 0.f));
                    ru_part = df_madd(r.v[c], un.v[c], ru_part);
                    rr_part = df_madd(r.v[c], r.v[c], rr_part);
                }
                st_row(pv, i, p);
                st_row(sv, i, sr);
                st_row(xv, i, x);
                st_row(rv, i, r);
                st_row(uv, i, un);
                bad |= df3_out_of_range(r) || df3_out_of_range(p);
            }
            cg_grid_sync(S, gen);  // u complete before the next product
        }
    }
    if (reporter) {
        C->rr0 = rr0;
        C->rr = rr_last;
        C->thr2 = thr2;
        C->its = its;
        C->max_its = max_its;
        C->done = 1;
        if (out_of_range) atomicExch(&S->status, kCgOutOfRange);
    }
    if (out_of_range || cg_status(S)) return;
    for (int i = r0 + threadIdx.x; i < r1; i += kCgThreads) {
        const DF3 x = ld_row(V.x2, i);
#pragma unroll
        for (int c = 0; c < 3; ++c) V.x[3 * size_t(i) + c] = double(x.v[c].x) + double(x.v[c].y);
    }
}
