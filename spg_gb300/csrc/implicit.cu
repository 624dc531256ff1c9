// GB300 global solvers of SPG: the implicit Euler family, BDF2, static and quasi-static Newton
// and symplectic Euler (spg/source/sim/solver/), on ImplicitEulerBase's system assembly and
// linear solve (implicitEulerBase.cpp:102-240):
//
//   f = M g - grad E(x) (getSystemForce); K = -hess E(x) (getSystemStiffnessMatrix, full
//   element Hessians, no definiteness projection); linear systems alpha M - beta K solved by
//   conjugate gradients with the diagonal preconditioner (Eigen::ConjugateGradient: relative
//   tolerance 1e-5, 300 iterations, zero initial guess).
//
// Per substep of step h (each method's step(), restated operation by operation):
//   NewtonDx (implicitEulerNewtonDx.cpp:31-55): x0 = x; x += v h; solve (M/h^2 - K) dx = f;
//     x += dx; v = (x - x0) / h.
//   NewtonDv (implicitEulerNewtonDv.cpp:31-60): x += v h; solve (M - h^2 K) dv = h f;
//     v = v0 + dv; x = x0 + v h.
//   NewtonRobust (implicitEulerNewtonRobust.cpp:33-126): Newton iterations on
//     (M - h^2 K) dv = h f - M (v_i - v0) with a halving line search on the residual norm,
//     up to 5 iterations and 5 line-search steps; a failed substep restores x0, v0 and scales
//     the step by 0.75, more than 5 successes in a row grow it back (the step persists).
//   BaraffWitkin (implicitEulerBaraffWitkin.cpp:31-52): solve (M - h^2 K) dv = h (f + h K v0);
//     v = v0 + dv; x += v h.
//   BDF2 (bdf2.cpp:31-74): solve (M - 4/9 h^2 K) dv = 1/3 M (v0 - v-1)
//     + 2/3 h (f + 1/3 K (x0 - x-1 + 2 h v0)); v = v0 + dv; x = 4/3 x0 - 1/3 x-1 + 2/3 v h.
//   StaticNewton (staticNewton.cpp:30-45): solve K dx = -f; x += dx.
//   QuasiStaticNewton (quasiStaticNewton.cpp:32-49): solve (M - h^2 K) dx = h^2 f; x += dx.
//   QuasiStaticNewtonRobust (quasiStaticNewtonRobust.cpp:33-136): Newton iterations on
//     (M/h^2 - K) dx = f - M v / h, v = (x - x0) / h, with the same line search and step
//     control (threshold 1e-2).
//   SimplecticEuler (simplecticEuler.cpp:11-62): v += h g; v += h W (-grad E); x += v h.
//
// Layout: the global matrix is block-sparse with 3x3 blocks (BSR) over the vertex adjacency of
// all stencils; one thread per element computes the element's gradient and Hessian blocks by
// forward-mode differentiation over vertex pairs (6 seeded coordinates) and adds them with
// atomics. State, assembly, parameters and the CG are FP64: a flat cloth at rest has no
// transverse stiffness, and FP32 rounding of 1 - L0 / |x1 - x0| would add some of the order of
// the M / h^2 term and change the solution. These solvers are off the VBD hot path, so FP64's
// lower rate is acceptable here.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "api_internal.h"
#include "devbuf.h"
#include "device_common.cuh"
#include "layout.h"
#include "state.h"

namespace spgx {

struct ImplicitTables {
    const int4 *idx;     // per element: internal vertex ids (-1 padded)
    const int4 *info;    // per element: {type, param offset, stencil size, 0}
    const double *prm;   // parameters in the spgx.h layouts
    const int *eblk;     // per element: S x S block positions in the BSR values (row-major)
    const int *row_ptr;  // BSR rows (internal vertices)
    const int *col;      // BSR block columns
    double *val;         // BSR values, 9 per block (row-major)
    const int *diag;     // per vertex: position of its diagonal block
    int *wide;           // set when the CG's matrix leaves the double-float range
    int nnzb;            // number of blocks
};

// Double-float form of an FP64 value: a = hi + lo with hi = fl32(a) and lo = fl32(a - hi),
// 48 significant bits. GB300 runs FP64 at about 1/64 of its FP32 rate, so the CG runs on the
// FP32 pipes in this form. A value above 2^60 in magnitude, or not finite, reports out of
// range: the solve then runs in FP64.
__device__ __forceinline__ float2 split_df(double a, bool &out_of_range)
{
    out_of_range = !(fabs(a) <= 0x1p60);
    const float hi = __double2float_rn(a);
    return make_float2(hi, __double2float_rn(a - double(hi)));
}

// Sets *wide once per warp if any lane of the warp saw an out-of-range value.
__device__ __forceinline__ void flag_wide(bool bad, int *wide)
{
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(wide, 1);
}

// Vectors over the vertices: 3 doubles per vertex.
__device__ __forceinline__ void atomic_block(double *val, int blk, const double H[9])
{
    double *b = val + size_t(blk) * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) atomicAdd(b + k, H[k]);
}

__device__ __forceinline__ void atomic_force(double *f, int v, double gx, double gy, double gz)
{
    atomicAdd(f + 3 * v, -gx);
    atomicAdd(f + 3 * v + 1, -gy);
    atomicAdd(f + 3 * v + 2, -gz);
}

// First-order forward mode with the three coordinates of one vertex as tangents: the
// Hessian of an energy whose gradient has a closed form is the derivative of that gradient.
struct D3 {
    double v, d[3];
};
__device__ __forceinline__ D3 operator+(D3 a, D3 b)
{
    return {a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}};
}
__device__ __forceinline__ D3 operator-(D3 a, D3 b)
{
    return {a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}};
}
__device__ __forceinline__ D3 operator-(D3 a) { return {-a.v, {-a.d[0], -a.d[1], -a.d[2]}}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b)
{
    return {a.v * b.v, {a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1], a.d[2] * b.v + a.v * b.d[2]}};
}
__device__ __forceinline__ D3 recip(D3 a)
{
    const double r = 1.0 / a.v, s = -r * r;
    return {r, {s * a.d[0], s * a.d[1], s * a.d[2]}};
}
__device__ __forceinline__ D3 sq_root(D3 a)
{
    const double r = sqrt(a.v), s = 0.5 / r;
    return {r, {s * a.d[0], s * a.d[1], s * a.d[2]}};
}

template <typename T>
__device__ __forceinline__ T comp(const Vec3<T> &v, int r)
{
    return r == 0 ? v.x : (r == 1 ? v.y : v.z);
}

// Gradient of the dihedral angle of DiscreteBendingEnergy (discreteBendingEnergy.cpp; hinge
// x0-x1, flaps x2 and x3) with respect to x1, x2 and x3, from e = x1 - x0, a = x2 - x0,
// b = x3 - x0, Na = e x a, Nb = e x b:
//   dtheta/dx1 = (a.e) Na / (|e| |Na|^2) - (b.e) Nb / (|e| |Nb|^2),
//   dtheta/dx2 = -|e| Na / |Na|^2,   dtheta/dx3 = |e| Nb / |Nb|^2,
// and dtheta/dx0 = -(the sum of the three).
template <typename T>
__device__ __forceinline__ void dihedral_gradient(Vec3<T> e, Vec3<T> a, Vec3<T> b, Vec3<T> g[3])
{
    const Vec3<T> Na = cross(e, a), Nb = cross(e, b);
    const T L = sq_root(dot(e, e));
    const T iL = recip(L);
    const T ina = recip(dot(Na, Na)), inb = recip(dot(Nb, Nb));
    g[0] = (dot(a, e) * iL * ina) * Na - (dot(b, e) * iL * inb) * Nb;
    g[1] = (-(L * ina)) * Na;
    g[2] = (L * inb) * Nb;
}

// DiscreteBendingEnergy, E = 1/2 k (theta - theta0)^2 (prm = [theta0, k]): gradient
// k C grad theta and Hessian k (grad theta grad theta^T + C hess theta), C = theta - theta0,
// theta = atan2(-|e| Na.b, -Na.Nb) (the reference's atan2 of the normals, simplified).
// hess theta is the forward-mode derivative of the closed-form gradient, one seeded vertex
// (x1, x2, x3) at a time; column x0 follows from translation invariance.
template <bool kHess>
__device__ void assemble_bending(const ImplicitTables &T, const double *__restrict__ x, double *force, int e,
                                 int4 ix, const double *prm)
{
    const int iv[4] = {ix.x, ix.y, ix.z, ix.w};
    const int *eb = T.eblk + size_t(e) * 16;
    const double *x0 = x + 3 * size_t(iv[0]);
    Vec3<double> p[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const double *xj = x + 3 * size_t(iv[j + 1]);
        p[j] = mk(xj[0] - x0[0], xj[1] - x0[1], xj[2] - x0[2]);
    }
    const Vec3<double> Na = cross(p[0], p[1]), Nb = cross(p[0], p[2]);
    const double th = atan2(-sqrt(dot(p[0], p[0])) * dot(Na, p[2]), -dot(Na, Nb));
    const double k = prm[1], C = th - prm[0];
    Vec3<double> g[4];
    dihedral_gradient<double>(p[0], p[1], p[2], g + 1);
    g[0] = mk(-(g[1].x + g[2].x + g[3].x), -(g[1].y + g[2].y + g[3].y), -(g[1].z + g[2].z + g[3].z));
#pragma unroll
    for (int a = 0; a < 4; ++a) atomic_force(force, iv[a], k * C * g[a].x, k * C * g[a].y, k * C * g[a].z);
    if (!kHess) return;
    double D00[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) D00[q] = 0.0;
#pragma unroll
    for (int sv = 1; sv < 4; ++sv) {
        Vec3<D3> q[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double t = j + 1 == sv ? 1.0 : 0.0;
            q[j] = mk(D3{p[j].x, {t, 0.0, 0.0}}, D3{p[j].y, {0.0, t, 0.0}}, D3{p[j].z, {0.0, 0.0, t}});
        }
        Vec3<D3> dg[3];
        dihedral_gradient<D3>(q[0], q[1], q[2], dg);
        // J_a[r][c] = d g_a[r] / d x_sv[c] for a = 1..3; a = 0 is minus their sum.
        double H[9], Ht[9];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const double J = a == 0 ? -(comp(dg[0], r).d[c] + comp(dg[1], r).d[c] + comp(dg[2], r).d[c])
                                            : comp(dg[a - 1], r).d[c];
                    if (a == 0) D00[3 * r + c] -= J;
                    H[3 * r + c] = k * (comp(g[a], r) * comp(g[sv], c) + C * J);
                    Ht[3 * c + r] = H[3 * r + c];
                }
            atomic_block(T.val, eb[a * 4 + sv], H);
            if (a == 0) atomic_block(T.val, eb[sv * 4], Ht);
        }
    }
    double H[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) H[3 * r + c] = k * (comp(g[0], r) * comp(g[0], c) + C * D00[3 * r + c]);
    atomic_block(T.val, eb[0], H);
}

// SpringEnergy, E = 1/2 k (|x0 - x1| - L0)^2 (prm = [L0, k]): with d = x0 - x1, l = |d|,
// grad_0 = k (l - L0) d / l = -grad_1 and H_00 = H_11 = -H_01 = -H_10
// = k ((1 - L0 / l) I + L0 d d^T / l^3).
template <bool kHess>
__device__ void assemble_spring(const ImplicitTables &T, const double *__restrict__ x, double *force, int e, int4 ix,
                                const double *prm)
{
    const double *xa = x + 3 * size_t(ix.x), *xb = x + 3 * size_t(ix.y);
    const double d[3] = {xa[0] - xb[0], xa[1] - xb[1], xa[2] - xb[2]};
    const double l = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double L0 = prm[0], k = prm[1], il = 1.0 / l;
    const double s = k * (l - L0) * il;
    atomic_force(force, ix.x, s * d[0], s * d[1], s * d[2]);
    atomic_force(force, ix.y, -s * d[0], -s * d[1], -s * d[2]);
    if (!kHess) return;
    const double dg = k * (1.0 - L0 * il), o = k * L0 * il * il * il;
    double H[9], Hn[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            H[3 * r + c] = (r == c ? dg : 0.0) + o * d[r] * d[c];
            Hn[3 * r + c] = -H[3 * r + c];
        }
    const int *eb = T.eblk + size_t(e) * 16;
    atomic_block(T.val, eb[0], H);
    atomic_block(T.val, eb[1], Hn);
    atomic_block(T.val, eb[2], Hn);
    atomic_block(T.val, eb[3], H);
}

// Gradient and Hessian blocks of one element at the positions x (FP64, 3 per vertex), added to
// the forces (f -= grad) and, with kHess, to the matrix (val += hess). Positions enter
// relative to the element's first vertex (the energies are translation invariant).
template <int S, bool kHess>
__device__ void assemble_element(const ImplicitTables &T, const double *__restrict__ x, double *force, int e,
                                 int4 ix, int4 info)
{
    const int iv[4] = {ix.x, ix.y, ix.z, ix.w};
    const double *prm = T.prm + info.y;
    const int type = info.x;
    const int *eb = T.eblk + size_t(e) * 16;
    const double *x0 = x + 3 * size_t(iv[0]);
    Vec3<double> p[S];
#pragma unroll
    for (int j = 0; j < S; ++j) {
        const double *xj = x + 3 * size_t(iv[j]);
        p[j] = mk(xj[0] - x0[0], xj[1] - x0[1], xj[2] - x0[2]);
    }
    if (type == SPGX_ENERGY_QUADRATIC_BENDING) {
        // C = sum_s c_s x_s (linear): grad_a = k c_a C, hess_ab = k c_a c_b I.
        Vec3<double> C = mk(0.0, 0.0, 0.0);
#pragma unroll
        for (int s = 0; s < S; ++s) C = C + prm[s] * p[s];
        const double k = prm[4];
#pragma unroll
        for (int a = 0; a < S; ++a) {
            atomic_force(force, iv[a], k * prm[a] * C.x, k * prm[a] * C.y, k * prm[a] * C.z);
            if (kHess)
#pragma unroll
                for (int b = 0; b < S; ++b) {
                    const double s = k * prm[a] * prm[b];
                    const double H[9] = {s, 0.0, 0.0, 0.0, s, 0.0, 0.0, 0.0, s};
                    atomic_block(T.val, eb[a * S + b], H);
                }
        }
        return;
    }
    // Vertex pairs (a, b), a < b: 6 seeded coordinates give blocks (a,a), (a,b), (b,b). The
    // diagonal block and gradient of a vertex are taken from one pair only: (a, a+1), and for
    // the last vertex (S-2, S-1).
#pragma unroll
    for (int a = 0; a < S; ++a)
#pragma unroll
        for (int b = a + 1; b < S; ++b) {
            const bool diag_a = b == a + 1;
            const bool diag_b = a == S - 2 && b == S - 1;
            if (!kHess && !diag_a && !diag_b) continue;
            V3A<double, 6> q[S];
            seed_positions<double, S, 6>(p, a, q, b);
            const VAD<double, 6> E = energy_ad(type, q, prm);
            if (kHess) {
                double Hab[9], Hba[9];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        Hab[3 * r + c] = E.h[hidx<6>(r, 3 + c)];
                        Hba[3 * c + r] = Hab[3 * r + c];
                    }
                atomic_block(T.val, eb[a * S + b], Hab);
                atomic_block(T.val, eb[b * S + a], Hba);
            }
            if (diag_a) {
                if (kHess) {
                    double H[9];
#pragma unroll
                    for (int r = 0; r < 3; ++r)
#pragma unroll
                        for (int c = 0; c < 3; ++c) H[3 * r + c] = E.h[r <= c ? hidx<6>(r, c) : hidx<6>(c, r)];
                    atomic_block(T.val, eb[a * S + a], H);
                }
                atomic_force(force, iv[a], E.g[0], E.g[1], E.g[2]);
            }
            if (diag_b) {
                if (kHess) {
                    double H[9];
#pragma unroll
                    for (int r = 0; r < 3; ++r)
#pragma unroll
                        for (int c = 0; c < 3; ++c)
                            H[3 * r + c] = E.h[r <= c ? hidx<6>(3 + r, 3 + c) : hidx<6>(3 + c, 3 + r)];
                    atomic_block(T.val, eb[b * S + b], H);
                }
                atomic_force(force, iv[b], E.g[3], E.g[4], E.g[5]);
            }
        }
}

template <bool kHess>
__global__ void __launch_bounds__(128) implicit_assemble_kernel(ImplicitTables T, const double *__restrict__ x,
                                                                double *force, int n_elem)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_elem) return;
    const int4 ix = __ldg(T.idx + e);
    const int4 info = __ldg(T.info + e);
    const double *prm = T.prm + info.y;
    switch (info.z) {
    case 1: {
        const int v = ix.x;
        if (info.x == SPGX_ENERGY_STATIC_LOAD) {  // E = -k d . x: force k d, no Hessian
            atomic_force(force, v, -prm[0] * prm[1], -prm[0] * prm[2], -prm[0] * prm[3]);
            return;
        }
        // Anchor: 1/2 k |x - a|^2.
        const double *xv = x + 3 * size_t(v);
        const double k = prm[3];
        atomic_force(force, v, k * (xv[0] - prm[0]), k * (xv[1] - prm[1]), k * (xv[2] - prm[2]));
        if (kHess) {
            const double H[9] = {k, 0.0, 0.0, 0.0, k, 0.0, 0.0, 0.0, k};
            atomic_block(T.val, T.eblk[size_t(e) * 16], H);
        }
        return;
    }
    case 2:
        if (info.x == SPGX_ENERGY_SPRING)
            assemble_spring<kHess>(T, x, force, e, ix, prm);
        else
            assemble_element<2, kHess>(T, x, force, e, ix, info);
        break;
    case 3: assemble_element<3, kHess>(T, x, force, e, ix, info); break;
    default:
        if (info.x == SPGX_ENERGY_DISCRETE_BENDING)
            assemble_bending<kHess>(T, x, force, e, ix, prm);
        else
            assemble_element<4, kHess>(T, x, force, e, ix, info);
        break;
    }
}

// The system matrix alpha M + beta H (H = hess E = -K, assembled into val) and the diagonal
// preconditioner 1 / A_ii (Eigen's DiagonalPreconditioner: 1 where A_ii is 0). One thread per
// block row.
__global__ void implicit_lhs_kernel(ImplicitTables T, const double *mass, int nv, double alpha, double beta,
                                    double *dinv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    if (beta != 1.0)
        for (int k = T.row_ptr[i]; k < T.row_ptr[i + 1]; ++k)
            for (int q = 0; q < 9; ++q) T.val[size_t(k) * 9 + q] *= beta;
    double *b = T.val + size_t(T.diag[i]) * 9;
    const double m = alpha * mass[i];
    b[0] += m;
    b[4] += m;
    b[8] += m;
    dinv[3 * i] = b[0] != 0.0 ? 1.0 / b[0] : 1.0;
    dinv[3 * i + 1] = b[4] != 0.0 ? 1.0 / b[4] : 1.0;
    dinv[3 * i + 2] = b[8] != 0.0 ? 1.0 / b[8] : 1.0;
}

// The CG's symmetric double-float matrix: the 9 entries of every upper block (ufull: its
// position in the full pattern) as split_df pairs, one 80-byte record per block (10 pairs, the
// last zero). A nonzero diagonal below 2^-60 in magnitude (a row whose scale nears FP32's
// underflow) also selects the FP64 solve.
__global__ void implicit_split_kernel(ImplicitTables T, float2 *ublk, const int *ufull, int nnzu, int nv)
{
    bool bad = false;
    const size_t n_values = 10 * size_t(nnzu);
    for (size_t o = blockIdx.x * size_t(blockDim.x) + threadIdx.x; o < n_values; o += size_t(gridDim.x) * blockDim.x) {
        const size_t k = o / 10, q = o - k * 10;
        bool out = false;
        ublk[o] = q < 9 ? split_df(T.val[size_t(__ldg(ufull + k)) * 9 + q], out) : make_float2(0.f, 0.f);
        bad |= out;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x) {
        const double *d = T.val + size_t(T.diag[i]) * 9;
        for (int q = 0; q < 9; q += 4)
            if (d[q] != 0.0 && fabs(d[q]) < 0x1p-60) bad = true;
    }
    flag_wide(bad, T.wide);
}

// Block-wide FP64 sums of a and b into *oa and *ob (one atomic each per block; ob may be
// NULL). Each kernel calls this once: the shared partials are not reused within a launch.
__device__ __forceinline__ void block_reduce_add2(double a, double b, double *oa, double *ob)
{
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    __shared__ double part[2][32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        part[0][w] = a;
        part[1][w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0.0, sb = 0.0;
        for (int k = 0; k < (blockDim.x + 31) / 32; ++k) {
            sa += part[0][k];
            sb += part[1][k];
        }
        atomicAdd(oa, sa);
        if (ob) atomicAdd(ob, sb);
    }
}

__device__ __forceinline__ void block_reduce_add(double v, double *out)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ double part1[32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) part1[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < (blockDim.x + 31) / 32; ++k) s += part1[k];
        atomicAdd(out, s);
    }
}

// Device-side control of one CG solve: the iteration loop runs as captured graphs of several
// iterations with no host round trip per iteration; once done is set every later kernel of
// the graph returns at once.
struct CgControl {
    int done;        // converged (|r|^2 < thr2) or out of iterations
    int its;         // iterations taken
    int max_its;
    int pad;
    double thr2;     // tol^2 |b|^2
    double rr0;      // |b|^2
    double rr;       // |r|^2 when done was set
};

__device__ __forceinline__ bool cg_done(const CgControl *c) { return c && *(volatile const int *)&c->done; }

// Ap = A p in FP64 with LANES lanes per block row: the lanes of a row read consecutive 3x3
// blocks, and a shuffle reduction sums their partial products. With dots, dots[0] += p . Ap.
// This is the product of the FP64 CG (the fallback when the system leaves the double-float
// range) and of the methods' K v terms. Small systems are latency bound and take 8 lanes per
// row; large ones 1, where the FP64 pipe binds.
constexpr int kSpmvLanesSmall = 8;
constexpr int kSpmvSmallRows = 65536;
constexpr int kSplitBlocks = 152 * 8;  // grid-stride split of the system matrix

// s += a x in double-float: the head product's rounding error comes back exactly from an
// FMA, the heads are summed by Knuth's two-sum, and the tails and errors gather in sl.
// The _rn intrinsics keep the compiler from contracting the products into the sums.
__device__ __forceinline__ void df_fma(float &sh, float &sl, float2 a, float2 x)
{
    const float ph = __fmul_rn(a.x, x.x);
    const float pl = fmaf(a.x, x.y, fmaf(a.y, x.x, fmaf(a.x, x.x, -ph)));
    const float s = __fadd_rn(sh, ph);
    const float bb = __fsub_rn(s, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(e, pl));
}

// (sh, sl) += (bh, bl) in double-float (two-sum of the heads).
__device__ __forceinline__ void df_add(float &sh, float &sl, float bh, float bl)
{
    const float s = __fadd_rn(sh, bh);
    const float bb = __fsub_rn(s, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(e, bl));
}

template <int LANES>
__global__ void implicit_spmv_kernel(ImplicitTables T, const double *__restrict__ p, double *Ap, int nv, double *dots,
                                     const CgControl *ctl = nullptr)
{
    if (cg_done(ctl)) return;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / LANES;
    const int lane = t & (LANES - 1);
    double y0 = 0.0, y1 = 0.0, y2 = 0.0;
    if (i < nv) {
        const int k1 = __ldg(T.row_ptr + i + 1);
        for (int k = __ldg(T.row_ptr + i) + lane; k < k1; k += LANES) {
            const double *bl = T.val + size_t(k) * 9;
            const double *x = p + 3 * size_t(__ldg(T.col + k));
            const double x0 = x[0], x1 = x[1], x2 = x[2];
            y0 += bl[0] * x0 + bl[1] * x1 + bl[2] * x2;
            y1 += bl[3] * x0 + bl[4] * x1 + bl[5] * x2;
            y2 += bl[6] * x0 + bl[7] * x1 + bl[8] * x2;
        }
    }
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) {
        y0 += __shfl_xor_sync(0xffffffffu, y0, o);
        y1 += __shfl_xor_sync(0xffffffffu, y1, o);
        y2 += __shfl_xor_sync(0xffffffffu, y2, o);
    }
    double pap = 0.0;
    if (i < nv && lane == 0) {
        Ap[3 * i] = y0;
        Ap[3 * i + 1] = y1;
        Ap[3 * i + 2] = y2;
        pap = p[3 * i] * y0 + p[3 * i + 1] * y1 + p[3 * i + 2] * y2;
    }
    if (dots) block_reduce_add(pap, dots);
}

// One FP64 product on the stream, with the lane count for the system's size.
static void launch_spmv(const ImplicitTables &T, const double *p, double *Ap, int nv, double *dots,
                        const CgControl *ctl, cudaStream_t st)
{
    if (nv < kSpmvSmallRows)
        implicit_spmv_kernel<kSpmvLanesSmall>
            <<<(nv * kSpmvLanesSmall + 255) / 256, 256, 0, st>>>(T, p, Ap, nv, dots, ctl);
    else
        implicit_spmv_kernel<1><<<(nv + 255) / 256, 256, 0, st>>>(T, p, Ap, nv, dots, ctl);
}

// FP64 CG start with x = 0: r = b, z = D^-1 r, p = z; dots[1] += r.r, dots[2] += r.z.
__global__ void implicit_cg_init_kernel(const double *b, const double *dinv, double *x, double *r, double *z,
                                       double *p, int n, double *dots)
{
    double rr = 0.0, rz = 0.0;
#pragma unroll 4
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double ri = b[i], zi = ri * dinv[i];
        x[i] = 0.0;
        r[i] = ri;
        z[i] = zi;
        p[i] = zi;
        rr += ri * ri;
        rz += ri * zi;
    }
    block_reduce_add2(rr, rz, dots + 1, dots + 2);
}
// Eigen's start: nothing to do for b = 0; otherwise iterate while |r|^2 >= tol^2 |b|^2.
__global__ void implicit_cg_control_kernel(CgControl *c, const double *dots, double tol, int max_its)
{
    const double rr0 = dots[1];
    c->rr0 = rr0;
    c->rr = rr0;
    c->thr2 = fmax(tol * tol * rr0, 1e-300);
    c->its = 0;
    c->max_its = max_its;
    c->done = (rr0 == 0.0 || rr0 < c->thr2 || max_its <= 0) ? 1 : 0;
}

// x += alpha p; r -= alpha Ap; z = D^-1 r; dots[1] += r.r, dots[2] += r.z (alpha = rz / pAp).
__global__ void implicit_cg_update_kernel(double *x, double *r, double *z, const double *p, const double *Ap,
                                         const double *dinv, int n, const double *prev, double *dots,
                                         CgControl *ctl)
{
    if (cg_done(ctl)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) ++ctl->its;  // read by the direction kernel
    __shared__ double s_alpha;
    if (threadIdx.x == 0) s_alpha = prev[2] / prev[0];
    __syncthreads();
    const double alpha = s_alpha;
    double rr = 0.0, rz = 0.0;
#pragma unroll 4
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double ri = r[i] - alpha * Ap[i];
        r[i] = ri;
        const double zi = ri * dinv[i];
        z[i] = zi;
        rr += ri * ri;
        rz += ri * zi;
    }
    block_reduce_add2(rr, rz, dots + 1, dots + 2);
}
// The iteration's stopping test (Eigen: |r|^2 < thr2 after the update, or the iteration
// limit), then p = z + beta p with beta = rz_new / rz_old. Every block takes the same
// decision: its inputs were written by earlier kernels.
__global__ void implicit_cg_direction_kernel(double *p, const double *z, int n, const double *prev, const double *cur,
                                            CgControl *ctl)
{
    if (cg_done(ctl)) return;
    const double rr = cur[1];
    const bool stop = rr < ctl->thr2 || ctl->its >= ctl->max_its;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (stop) {
            ctl->rr = rr;
            ctl->done = 1;
        }
    }
    if (stop) return;
    __shared__ double s_beta;
    if (threadIdx.x == 0) s_beta = cur[2] / prev[2];
    __syncthreads();
    const double beta = s_beta;
#pragma unroll 4
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = z[i] + beta * p[i];
}

#include "implicit_cg.cuh"

// ---- vector steps of the methods (n = 3 V degrees of freedom; mass per vertex) ------------

// f = M g (getSystemForce's gravity term), or 0.
__global__ void force_init_kernel(double *f, const double *mass, int n, double gx, double gy, double gz, bool gravity)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double g = i % 3 == 0 ? gx : (i % 3 == 1 ? gy : gz);
    f[i] = gravity ? g * mass[i / 3] : 0.0;
}

// y = y + x s (integrateVelocities with x = v, s = h; updatePositionsFromDx with s = 1).
__global__ void axpy_kernel(double *y, const double *x, double s, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = y[i] + x[i] * s;
}

// out = a + b s.
__global__ void lincomb_kernel(double *out, const double *a, const double *b, double s, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] + b[i] * s;
}

// out = (a - b) s (computeIntegratedVelocities).
__global__ void diffscale_kernel(double *out, const double *a, const double *b, double s, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (a[i] - b[i]) * s;
}

// out = s a.
__global__ void scale_kernel(double *out, const double *a, double s, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = s * a[i];
}

// Baraff-Witkin: b = h (f + h (K v0)), K v0 = -u with u = H v0.
__global__ void bw_rhs_kernel(double *b, const double *f, const double *u, double h, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = h * (f[i] + h * -u[i]);
}

// BDF2: w = x0 - x_-1 + 2 h v0.
__global__ void bdf2_w_kernel(double *w, const double *x0, const double *xm1, const double *v0, double h2, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) w[i] = (x0[i] - xm1[i]) + h2 * v0[i];
}

// BDF2: b = 1/3 M (v0 - v_-1) + 2/3 h (f + 1/3 K w), K w = -u with u = H w.
__global__ void bdf2_rhs_kernel(double *b, const double *mass, const double *v0, const double *vm1, const double *f,
                                const double *u, double h, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    b[i] = (1.0 / 3.0 * mass[i / 3]) * (v0[i] - vm1[i]) + (2.0 / 3.0 * h) * (f[i] + 1.0 / 3.0 * -u[i]);
}

// BDF2: x = 4/3 x0 - 1/3 x_-1 + 2/3 v h; then x_-1 = x0, v_-1 = v0.
__global__ void bdf2_update_kernel(double *x, double *xm1, double *vm1, const double *x0, const double *v0,
                                   const double *v, double h, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = (4.0 / 3.0 * x0[i] - 1.0 / 3.0 * xm1[i]) + 2.0 / 3.0 * v[i] * h;
    xm1[i] = x0[i];
    vm1[i] = v0[i];
}

// NewtonRobust: r = h f - M (v - v0); b = r when given; norm2 += |r|^2.
__global__ void robust_rhs_kernel(double *b, const double *f, const double *v, const double *v0, const double *mass,
                                  double h, int n, double *norm2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    if (i < n) {
        const double r = h * f[i] - mass[i / 3] * (v[i] - v0[i]);
        if (b) b[i] = r;
        s = r * r;
    }
    block_reduce_add(s, norm2);
}

// QuasiStaticNewtonRobust: r = f - (M / h) v; b = r when given; norm2 += |r|^2.
__global__ void qs_rhs_kernel(double *b, const double *f, const double *v, const double *mass, double invdt, int n,
                              double *norm2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double s = 0.0;
    if (i < n) {
        const double r = f[i] - (invdt * mass[i / 3]) * v[i];
        if (b) b[i] = r;
        s = r * r;
    }
    block_reduce_add(s, norm2);
}

// SimplecticEuler: v += h g, then v += h W f_internal (W: inverse masses, 0 for massless).
__global__ void symplectic_kernel(double *v, const double *f, const double *mass, double h, double dgx, double dgy,
                                  double dgz, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dg = i % 3 == 0 ? dgx : (i % 3 == 1 ? dgy : dgz);
    const double m = mass[i / 3];
    const double w = m == 0.0 ? 0.0 : 1.0 / m;
    v[i] = (v[i] + dg) + w * f[i] * h;
}

static int grid_of(int n, int t = 256) { return (n + t - 1) / t; }
// The CG's vector kernels loop over several entries per thread, so their FP64 block
// reductions (a shuffle tree per thread) are paid once per few entries: 4 blocks of 256 per SM.
static int cg_grid(int n) { return std::max(1, std::min(grid_of(n), 152 * 4)); }

// Reverse Cuthill-McKee order of a graph given by adjacency lists (each sorted, the vertex
// itself included): per component, breadth-first from a pseudo-peripheral vertex (George and
// Liu's search: restart from a minimum-degree vertex of the last level while that deepens the
// level structure), neighbours taken in increasing degree; the whole order is then reversed.
// Returns each vertex's position. Vertices that share a block of the system matrix get
// positions a few hundred apart on a cloth, which is what the symmetric product's transposed
// reads need to find their blocks in L2.
static std::vector<int32_t> rcm_positions(const std::vector<std::vector<int32_t>> &adj)
{
    const int n = static_cast<int>(adj.size());
    auto deg = [&](int v) { return static_cast<int>(adj[v].size()); };
    auto lighter = [&](int a, int b) { return deg(a) < deg(b) || (deg(a) == deg(b) && a < b); };
    std::vector<int32_t> mark(n, -1), order, cur, next;
    std::vector<char> placed(n, 0);
    order.reserve(n);
    int stamp = 0;
    // Depth of the level structure rooted at s, and a minimum-degree vertex of its last level.
    auto levels = [&](int s, int &far) {
        ++stamp;
        cur.assign(1, s);
        mark[s] = stamp;
        int depth = 0;
        for (;;) {
            next.clear();
            for (int v : cur)
                for (int u : adj[v])
                    if (mark[u] != stamp) {
                        mark[u] = stamp;
                        next.push_back(u);
                    }
            if (next.empty()) break;
            cur.swap(next);
            ++depth;
        }
        far = *std::min_element(cur.begin(), cur.end(), lighter);
        return depth;
    };
    for (int s = 0; s < n; ++s) {
        if (placed[s]) continue;
        int root = s, far = s;
        int depth = levels(root, far);
        for (int tries = 0; tries < 8; ++tries) {
            int far2 = far;
            const int d2 = levels(far, far2);
            if (d2 <= depth) break;
            root = far;
            depth = d2;
            far = far2;
        }
        const size_t first = order.size();
        order.push_back(root);
        placed[root] = 1;
        std::vector<int32_t> nbrs;
        for (size_t q = first; q < order.size(); ++q) {
            nbrs.clear();
            for (int u : adj[order[q]])
                if (!placed[u]) nbrs.push_back(u);
            std::sort(nbrs.begin(), nbrs.end(), lighter);
            for (int u : nbrs) {
                placed[u] = 1;
                order.push_back(u);
            }
        }
    }
    std::vector<int32_t> pos(n);
    for (int k = 0; k < n; ++k) pos[order[k]] = n - 1 - k;
    return pos;
}

struct ImplicitSolver {
    SceneLayout L;
    spgx_implicit_params P{};
    int device{0};
    cudaStream_t stream{nullptr};
    cudaEvent_t ev0{nullptr}, ev1{nullptr};
    DevBuf d_idx, d_info, d_prm, d_eblk, d_row, d_col, d_val, d_diag, d_mass;
    DevBuf d_x, d_v, d_x0, d_v0, d_vi, d_xm1, d_vm1, d_f, d_b, d_u, d_w;
    DevBuf d_dx, d_r, d_z, d_p, d_Ap, d_dinv, d_dots, d_ctl;
    DevBuf d_wide;  // the matrix is out of double-float range
    // The double-float CG: symmetric matrix, vectors, block partials and barrier state.
    DevBuf d_urow, d_ucol, d_uval, d_ufull, d_lrow, d_lent;
    DevBuf d_x2, d_r2, d_p2, d_Ap2, d_d2, d_u2, d_w2, d_part, d_sync;
    HostBuf h_dots, h_ctl, h_sync;
    CgSymDf SD{};
    int cg_lanes{4}, cg_blocks{0};
    bool stall_next{false};  // test hook: the next double-float solve's barrier waits run out
    std::vector<int32_t> row_of;  // the CG's row of each vertex (scene order over all objects)
    cudaGraphExec_t cg_graph{nullptr};
    ImplicitTables T{};
    int n_elem{0}, nnzb{0};
    // Step control of the robust methods (m_currentDt, m_consecutiveSuccessfulSteps) and the
    // BDF2 history (m_xMinusOne / m_vMinusOne initialised).
    double current_dt{-1.0};
    int successes{0};
    bool history{false};

    ~ImplicitSolver()
    {
        if (cg_graph) cudaGraphExecDestroy(cg_graph);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) {
            cudaStreamSynchronize(stream);
            cudaStreamDestroy(stream);
        }
    }

    static spgx_status check_params(const spgx_implicit_params *p)
    {
        if (!p || !(p->dt > 0) || p->substeps < 1 || !(p->cg_threshold >= 0) || p->cg_max_iterations < 0 ||
            p->method < SPGX_IMPLICIT_NEWTON_DX || p->method > SPGX_SYMPLECTIC_EULER || p->cg_precision < 0 ||
            p->cg_precision > 1) {
            set_error("invalid implicit solver parameters");
            return SPGX_ERR_INVALID_ARG;
        }
        return SPGX_OK;
    }

    // BaseSolver::setDt / setNumSubsteps / setGravity between steps: the next step reads the
    // new values. The step size and BDF2's history carry over; method and device are fixed.
    spgx_status set_params(const spgx_implicit_params *p)
    {
        SPGX_TRY_STATUS(check_params(p));
        if (p->method != P.method || p->device != P.device) {
            set_error("method and device are fixed when the solver is created");
            return SPGX_ERR_INVALID_ARG;
        }
        P = *p;
        return SPGX_OK;
    }

    int n3() const { return 3 * L.nv; }
    double *vec(DevBuf &b) { return b.as<double>(); }

    spgx_status init(const spgx_scene_desc *scene, const spgx_implicit_params *params)
    {
        std::string err;
        SPGX_TRY_STATUS(check_params(params));
        const spgx_status st = build_scene_layout(scene, false, L, err);
        if (st != SPGX_OK) {
            set_error(err);
            return st;
        }
        P = *params;
        SPGX_TRY_STATUS(select_device(P.device));
        device = P.device;
        SPGX_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        SPGX_CUDA(cudaEventCreate(&ev0));
        SPGX_CUDA(cudaEventCreate(&ev1));
        // Element list over every energy and the vertex adjacency (scene vertex ids: object
        // base + vertex), then the rows in reverse Cuthill-McKee order of that adjacency.
        const int nv = L.nv;
        std::vector<I4> idx, info;
        std::vector<double> prm, mass(std::max(1, nv), 0.0);
        std::vector<std::vector<int32_t>> nb(nv);
        for (int v = 0; v < nv; ++v) nb[v].push_back(v);
        for (int o = 0; o < scene->n_objects; ++o) {
            const auto &ob = scene->objects[o];
            const int vb = L.objects[o].vertex_base;
            for (int e = 0; e < ob.n_energies; ++e) {
                const auto &E = ob.energies[e];
                const int S = stencil_size(E.type), Pc = param_count(E.type);
                for (int s = 0; s < E.n_stencils; ++s) {
                    int iv[4] = {-1, -1, -1, -1};
                    for (int k = 0; k < S; ++k) iv[k] = vb + E.stencils[int64_t(s) * S + k];
                    idx.push_back({iv[0], iv[1], iv[2], iv[3]});
                    info.push_back({E.type, static_cast<int32_t>(prm.size()), S, 0});
                    for (int k = 0; k < Pc; ++k) prm.push_back(E.params[int64_t(s) * Pc + k]);
                    for (int a = 0; a < S; ++a)
                        for (int b = 0; b < S; ++b)
                            if (a != b) nb[iv[a]].push_back(iv[b]);
                }
            }
        }
        for (auto &r : nb) {
            std::sort(r.begin(), r.end());
            r.erase(std::unique(r.begin(), r.end()), r.end());
        }
        row_of = rcm_positions(nb);
        for (int o = 0; o < scene->n_objects; ++o) {
            const int vb = L.objects[o].vertex_base;
            for (int k = 0; k < scene->objects[o].n_vertices; ++k) mass[row_of[vb + k]] = scene->objects[o].mass[k];
        }
        for (auto &e : idx) {
            int *iv[4] = {&e.x, &e.y, &e.z, &e.w};
            for (int *v : iv)
                if (*v >= 0) *v = row_of[*v];
        }
        {
            std::vector<std::vector<int32_t>> by_row(nv);
            for (int v = 0; v < nv; ++v) {
                auto &r = by_row[row_of[v]];
                for (int u : nb[v]) r.push_back(row_of[u]);
                std::sort(r.begin(), r.end());
            }
            nb.swap(by_row);
        }
        n_elem = static_cast<int>(idx.size());
        std::vector<int32_t> row(nv + 1, 0), col, diag(nv);
        for (int v = 0; v < nv; ++v) {
            for (int c : nb[v]) {
                if (c == v) diag[v] = static_cast<int32_t>(col.size());
                col.push_back(c);
            }
            row[v + 1] = static_cast<int32_t>(col.size());
        }
        nnzb = static_cast<int>(col.size());
        std::vector<int32_t> eblk(size_t(std::max(1, n_elem)) * 16, 0);
        for (int e = 0; e < n_elem; ++e) {
            const int iv[4] = {idx[e].x, idx[e].y, idx[e].z, idx[e].w};
            const int S = info[e].z;
            for (int a = 0; a < S; ++a)
                for (int b = 0; b < S; ++b) {
                    const auto first = col.begin() + row[iv[a]], last = col.begin() + row[iv[a] + 1];
                    eblk[size_t(e) * 16 + a * S + b] = static_cast<int32_t>(std::lower_bound(first, last, iv[b]) - col.begin());
                }
        }
        if (idx.empty()) {
            idx.push_back({0, -1, -1, -1});
            info.push_back({0, 0, 0, 0});
        }
        if (prm.empty()) prm.push_back(0.0);
        if (col.empty()) col.push_back(0);
        SPGX_TRY_STATUS(d_idx.upload(idx));
        SPGX_TRY_STATUS(d_info.upload(info));
        SPGX_TRY_STATUS(d_prm.upload(prm));
        SPGX_TRY_STATUS(d_eblk.upload(eblk));
        SPGX_TRY_STATUS(d_row.upload(row));
        SPGX_TRY_STATUS(d_col.upload(col));
        SPGX_TRY_STATUS(d_diag.upload(diag.empty() ? std::vector<int32_t>{0} : diag));
        SPGX_TRY_STATUS(d_mass.upload(mass));
        SPGX_TRY_STATUS(d_val.alloc(size_t(std::max(1, nnzb)) * 9 * sizeof(double)));
        // The CG's symmetric pattern: row i's upper blocks are the tail of its full row from the
        // diagonal on; its lower block (i, j) is read as the transpose of the stored (j, i).
        {
            std::vector<int32_t> urow(nv + 1, 0), ucol, ufull, lrow(nv + 1, 0), lent;
            for (int i = 0; i < nv; ++i) {
                for (int f = diag[i]; f < row[i + 1]; ++f) {
                    ucol.push_back(col[f]);
                    ufull.push_back(f);
                }
                urow[i + 1] = static_cast<int32_t>(ucol.size());
            }
            for (int i = 0; i < nv; ++i) {
                for (int f = row[i]; f < diag[i]; ++f) {
                    const int j = col[f];
                    const int fji = static_cast<int>(std::lower_bound(col.begin() + row[j], col.begin() + row[j + 1], i) -
                                                     col.begin());
                    lent.push_back(j);
                    lent.push_back(urow[j] + (fji - diag[j]));
                }
                lrow[i + 1] = static_cast<int32_t>(lent.size() / 2);
            }
            SD.nnzu = static_cast<int>(ucol.size());
            if (ucol.empty()) {
                ucol.push_back(0);
                ufull.push_back(0);
            }
            if (lent.empty()) lent.assign(2, 0);
            SPGX_TRY_STATUS(d_urow.upload(urow));
            SPGX_TRY_STATUS(d_ucol.upload(ucol));
            SPGX_TRY_STATUS(d_ufull.upload(ufull));
            SPGX_TRY_STATUS(d_lrow.upload(lrow));
            SPGX_TRY_STATUS(d_lent.upload(lent));
            SPGX_TRY_STATUS(d_uval.alloc(size_t(std::max(1, SD.nnzu)) * kCgBlockFloat4 * sizeof(float4)));
            SD.urow = d_urow.as<int>();
            SD.ucol = d_ucol.as<int>();
            SD.ublk = d_uval.as<float4>();
            SD.lrow = d_lrow.as<int>();
            SD.lent = d_lent.as<int2>();
        }
        const size_t vb = size_t(std::max(1, nv)) * 3 * sizeof(double);
        for (DevBuf *b : {&d_x, &d_v, &d_x0, &d_v0, &d_vi, &d_xm1, &d_vm1, &d_f, &d_b, &d_u, &d_w, &d_dx, &d_r, &d_z,
                          &d_p, &d_Ap, &d_dinv})
            SPGX_TRY_STATUS(b->alloc(vb));
        for (DevBuf *b : {&d_x2, &d_r2, &d_p2, &d_Ap2, &d_d2, &d_u2, &d_w2})
            SPGX_TRY_STATUS(b->alloc(size_t(std::max(1, nv)) * 3 * sizeof(float2)));
        SPGX_TRY_STATUS(d_wide.alloc(sizeof(int)));
        SPGX_TRY_STATUS(d_sync.alloc(sizeof(CgSync)));
        SPGX_TRY_STATUS(h_sync.alloc(sizeof(CgSync)));
        // The CG's launch shape: one lane per row on large systems (the fewest dependent
        // memory round trips per warp), 8 on small ones (latency bound, few rows to spread); as
        // many co-resident blocks as fit and the rows need (one per SM).
        {
            cg_lanes = nv < kSpmvSmallRows ? 8 : 4;
            int per_sm = 0, sms = 0;
            SPGX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &per_sm, cg_lanes == 8 ? implicit_cg_df_kernel<8> : implicit_cg_df_kernel<4>, kCgThreads, 0));
            SPGX_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
            const long long need = (std::max<long long>(3LL * nv, 1LL * nv * cg_lanes) + kCgThreads - 1) / kCgThreads;
            cg_blocks = static_cast<int>(std::max(1LL, std::min<long long>(need, 1LL * std::max(1, per_sm) * sms)));
            SPGX_TRY_STATUS(d_part.alloc(size_t(cg_blocks) * 2 * 4 * sizeof(double)));
        }
        SPGX_TRY_STATUS(d_dots.alloc(size_t(8) * sizeof(double)));
        SPGX_TRY_STATUS(h_dots.alloc(size_t(8) * sizeof(double)));
        SPGX_TRY_STATUS(d_ctl.alloc(sizeof(CgControl)));
        SPGX_TRY_STATUS(h_ctl.alloc(sizeof(CgControl)));
        T = ImplicitTables{d_idx.as<int4>(), d_info.as<int4>(), d_prm.as<double>(), d_eblk.as<int>(), d_row.as<int>(),
                           d_col.as<int>(), d_val.as<double>(), d_diag.as<int>(), d_wide.as<int>(), nnzb};
        std::vector<double> x(3 * size_t(std::max(1, nv)), 0.0), v(x.size(), 0.0);
        for (int i = 0; i < nv; ++i) {
            const int k = row_of[i];
            for (int a = 0; a < 3; ++a) {
                x[3 * size_t(k) + a] = L.x_ext[3 * size_t(i) + a];
                v[3 * size_t(k) + a] = L.v_ext[3 * size_t(i) + a];
            }
        }
        SPGX_CUDA(cudaMemcpy(vec(d_x), x.data(), x.size() * sizeof(double), cudaMemcpyHostToDevice));
        SPGX_CUDA(cudaMemcpy(vec(d_v), v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
        return SPGX_OK;
    }

    // getSystemForce at x into d_f (gravity included unless told otherwise) and, with hessian,
    // getSystemStiffnessMatrix as H = -K into the BSR values.
    void assemble(const double *x, bool hessian, bool gravity = true)
    {
        const int n = n3();
        force_init_kernel<<<grid_of(n), 256, 0, stream>>>(vec(d_f), vec(d_mass), n, P.gravity[0], P.gravity[1],
                                                          P.gravity[2], gravity);
        if (hessian) cudaMemsetAsync(d_val.as<double>(), 0, size_t(std::max(1, nnzb)) * 9 * sizeof(double), stream);
        if (n_elem > 0) {
            if (hessian)
                implicit_assemble_kernel<true><<<grid_of(n_elem, 128), 128, 0, stream>>>(T, x, vec(d_f), n_elem);
            else
                implicit_assemble_kernel<false><<<grid_of(n_elem, 128), 128, 0, stream>>>(T, x, vec(d_f), n_elem);
        }
    }

    // Reads the scalar accumulated at d_dots[7] (after the stream's work) and clears it.
    spgx_status take_norm(double &out)
    {
        double *hd = h_dots.as<double>();
        SPGX_CUDA(cudaMemcpyAsync(hd + 7, d_dots.as<double>() + 7, sizeof(double), cudaMemcpyDeviceToHost, stream));
        SPGX_CUDA(cudaMemsetAsync(d_dots.as<double>() + 7, 0, sizeof(double), stream));
        SPGX_CUDA(cudaStreamSynchronize(stream));
        out = std::sqrt(hd[7]);
        return SPGX_OK;
    }

    // The FP64 CG's iterations as one graph of kCgChunk iterations (two parities of the
    // dot-product slots per pair of iterations), replayed until the device-side control says
    // done.
    static constexpr int kCgChunk = 32;
    spgx_status build_cg_graph()
    {
        const int nv = L.nv, n = n3();
        double *A = d_dots.as<double>(), *B = A + 3;
        CgControl *ctl = d_ctl.as<CgControl>();
        cudaGraph_t g = nullptr;
        SPGX_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        for (int it = 0; it < kCgChunk; ++it) {
            double *prev = it % 2 == 0 ? A : B, *cur = it % 2 == 0 ? B : A;
            cudaMemsetAsync(prev, 0, sizeof(double), stream);
            launch_spmv(T, vec(d_p), vec(d_Ap), nv, prev, ctl, stream);
            cudaMemsetAsync(cur, 0, 3 * sizeof(double), stream);
            implicit_cg_update_kernel<<<cg_grid(n), 256, 0, stream>>>(vec(d_dx), vec(d_r), vec(d_z), vec(d_p),
                                                                     vec(d_Ap), vec(d_dinv), n, prev, cur, ctl);
            implicit_cg_direction_kernel<<<cg_grid(n), 256, 0, stream>>>(vec(d_p), vec(d_z), n, prev, cur, ctl);
        }
        const cudaError_t ce = cudaStreamEndCapture(stream, &g);
        if (ce != cudaSuccess) {
            set_error(std::string("CG graph capture failed: ") + cudaGetErrorString(ce));
            return SPGX_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(&cg_graph, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            set_error(std::string("CG graph instantiation failed: ") + cudaGetErrorString(ie));
            return SPGX_ERR_CUDA;
        }
        return SPGX_OK;
    }

    // One CG solve of (alpha M + beta H) d_dx = d_b (ImplicitEulerBase::solveLinearSystem,
    // implicitEulerBase.cpp:227-239) with Eigen::ConjugateGradient's stopping rule
    // |r|^2 < tol^2 |b|^2. The BSR holds H on entry. The solve runs in double-float as one
    // cooperative launch; when the system leaves that range it runs again in FP64.
    spgx_status cg(double alpha, double beta, int &iterations, double &rel_residual)
    {
        const int nv = L.nv;
        implicit_lhs_kernel<<<grid_of(nv), 256, 0, stream>>>(T, vec(d_mass), nv, alpha, beta, vec(d_dinv));
        if (P.cg_precision == 1) return cg_fp64(iterations, rel_residual);
        SPGX_CUDA(cudaMemsetAsync(T.wide, 0, sizeof(int), stream));
        implicit_split_kernel<<<kSplitBlocks, 256, 0, stream>>>(T, d_uval.as<float2>(), d_ufull.as<int>(), SD.nnzu, nv);
        SPGX_CUDA(cudaMemsetAsync(d_sync.as<void>(), 0, sizeof(CgSync), stream));
        if (stall_next) {  // test hook: a barrier counter no barrier completes from
            SPGX_CUDA(cudaMemsetAsync(d_sync.as<void>(), 0x80, sizeof(int), stream));
            stall_next = false;
        }
        SPGX_CUDA(cudaGetLastError());
        CgDfVecs V{vec(d_b), vec(d_dinv), vec(d_dx), d_x2.as<float2>(), d_r2.as<float2>(), d_p2.as<float2>(),
                   d_Ap2.as<float2>(), d_d2.as<float2>(), d_u2.as<float2>(), d_w2.as<float2>(), d_part.as<double>(), nv};
        CgSync *sync = d_sync.as<CgSync>();
        CgControl *ctl = d_ctl.as<CgControl>();
        const int *wide = T.wide;
        const double tol = P.cg_threshold;
        int max_its = P.cg_max_iterations;
        void *args[] = {&SD, &V, &sync, &ctl, &wide, const_cast<double *>(&tol), &max_its};
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(cg_blocks);
        cfg.blockDim = dim3(kCgThreads);
        cfg.stream = stream;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        SPGX_CUDA(cudaLaunchKernelExC(&cfg,
                                      cg_lanes == 8 ? reinterpret_cast<const void *>(implicit_cg_df_kernel<8>)
                                                    : reinterpret_cast<const void *>(implicit_cg_df_kernel<4>),
                                      args));
        SPGX_CUDA(cudaMemcpyAsync(h_ctl.as<void>(), ctl, sizeof(CgControl), cudaMemcpyDeviceToHost, stream));
        SPGX_CUDA(cudaMemcpyAsync(h_sync.as<void>(), sync, sizeof(CgSync), cudaMemcpyDeviceToHost, stream));
        SPGX_CUDA(cudaStreamSynchronize(stream));
        const CgControl *hc = h_ctl.as<CgControl>();
        const int status = h_sync.as<CgSync>()->status;
        if (status == kCgTimeout) {
            set_error("a grid barrier of the CG solve gave up waiting");
            return SPGX_ERR_TIMEOUT;
        }
        if (status == kCgOutOfRange) return cg_fp64(iterations, rel_residual);
        fp64_products = false;
        iterations = hc->its;
        rel_residual = hc->rr0 > 0.0 ? std::sqrt(hc->rr / hc->rr0) : 0.0;
        return SPGX_OK;
    }

    // The FP64 CG on the full pattern, for systems outside the double-float range; the system
    // matrix and preconditioner are already in place.
    spgx_status cg_fp64(int &iterations, double &rel_residual)
    {
        const int n = n3();
        double *dots = d_dots.as<double>();  // two sets of {pAp, rr, rz}: [0..2] and [3..5]
        SPGX_CUDA(cudaMemsetAsync(dots, 0, 6 * sizeof(double), stream));
        implicit_cg_init_kernel<<<cg_grid(n), 256, 0, stream>>>(vec(d_b), vec(d_dinv), vec(d_dx), vec(d_r), vec(d_z),
                                                                vec(d_p), n, dots);
        implicit_cg_control_kernel<<<1, 1, 0, stream>>>(d_ctl.as<CgControl>(), dots, P.cg_threshold,
                                                        P.cg_max_iterations);
        SPGX_CUDA(cudaGetLastError());
        if (!cg_graph) SPGX_TRY_STATUS(build_cg_graph());
        const CgControl *hc = h_ctl.as<CgControl>();
        const int max_launches = P.cg_max_iterations / kCgChunk + 2;
        for (int k = 0; k < max_launches; ++k) {
            SPGX_CUDA(cudaGraphLaunch(cg_graph, stream));
            SPGX_CUDA(cudaMemcpyAsync(h_ctl.as<void>(), d_ctl.as<void>(), sizeof(CgControl), cudaMemcpyDeviceToHost,
                                      stream));
            SPGX_CUDA(cudaStreamSynchronize(stream));
            if (hc->done) break;
        }
        if (!hc->done) {
            set_error("internal: the CG control did not finish");
            return SPGX_ERR_CUDA;
        }
        fp64_products = true;
        iterations = hc->its;
        rel_residual = hc->rr0 > 0.0 ? std::sqrt(hc->rr / hc->rr0) : 0.0;
        return SPGX_OK;
    }

    bool fp64_products{false};  // the last solve ran in FP64 (out of double-float range)

    struct Tally {
        int cg_iterations = 0, newton_iterations = 0, failed = 0, fp64_solves = 0;
        bool converged = true;
        double first_residual = -1.0, last_residual = 0.0;
    };

    spgx_status solve(double alpha, double beta, Tally &t)
    {
        int its = 0;
        double rel = 0.0;
        SPGX_TRY_STATUS(cg(alpha, beta, its, rel));
        t.cg_iterations += its;
        t.fp64_solves += fp64_products ? 1 : 0;
        t.last_residual = rel;
        if (rel > P.cg_threshold) t.converged = false;
        return SPGX_OK;
    }

    // One substep of a method without step control.
    spgx_status substep(double h, Tally &t)
    {
        const int n = n3(), g = grid_of(n);
        double *x = vec(d_x), *v = vec(d_v), *x0 = vec(d_x0), *v0 = vec(d_v0), *f = vec(d_f), *b = vec(d_b);
        const size_t bytes = size_t(n) * sizeof(double);
        switch (P.method) {
        case SPGX_IMPLICIT_NEWTON_DX: {
            SPGX_CUDA(cudaMemcpyAsync(x0, x, bytes, cudaMemcpyDeviceToDevice, stream));
            axpy_kernel<<<g, 256, 0, stream>>>(x, v, h, n);
            assemble(x, true);
            SPGX_CUDA(cudaMemcpyAsync(b, f, bytes, cudaMemcpyDeviceToDevice, stream));
            const double invdt = 1. / h;
            SPGX_TRY_STATUS(solve(invdt * invdt, 1.0, t));
            axpy_kernel<<<g, 256, 0, stream>>>(x, vec(d_dx), 1.0, n);
            diffscale_kernel<<<g, 256, 0, stream>>>(v, x, x0, invdt, n);
            break;
        }
        case SPGX_IMPLICIT_NEWTON_DV: {
            SPGX_CUDA(cudaMemcpyAsync(x0, x, bytes, cudaMemcpyDeviceToDevice, stream));
            SPGX_CUDA(cudaMemcpyAsync(v0, v, bytes, cudaMemcpyDeviceToDevice, stream));
            axpy_kernel<<<g, 256, 0, stream>>>(x, v, h, n);
            assemble(x, true);
            scale_kernel<<<g, 256, 0, stream>>>(b, f, h, n);
            SPGX_TRY_STATUS(solve(1.0, h * h, t));
            lincomb_kernel<<<g, 256, 0, stream>>>(v, v0, vec(d_dx), 1.0, n);
            lincomb_kernel<<<g, 256, 0, stream>>>(x, x0, v, h, n);
            break;
        }
        case SPGX_IMPLICIT_BARAFF_WITKIN: {
            SPGX_CUDA(cudaMemcpyAsync(v0, v, bytes, cudaMemcpyDeviceToDevice, stream));
            assemble(x, true);
            launch_spmv(T, v0, vec(d_u), L.nv, nullptr, nullptr, stream);
            bw_rhs_kernel<<<g, 256, 0, stream>>>(b, f, vec(d_u), h, n);
            SPGX_TRY_STATUS(solve(1.0, h * h, t));
            lincomb_kernel<<<g, 256, 0, stream>>>(v, v0, vec(d_dx), 1.0, n);
            axpy_kernel<<<g, 256, 0, stream>>>(x, v, h, n);
            break;
        }
        case SPGX_IMPLICIT_BDF2: {
            SPGX_CUDA(cudaMemcpyAsync(x0, x, bytes, cudaMemcpyDeviceToDevice, stream));
            SPGX_CUDA(cudaMemcpyAsync(v0, v, bytes, cudaMemcpyDeviceToDevice, stream));
            if (!history) {
                SPGX_CUDA(cudaMemcpyAsync(vec(d_xm1), x, bytes, cudaMemcpyDeviceToDevice, stream));
                SPGX_CUDA(cudaMemcpyAsync(vec(d_vm1), v, bytes, cudaMemcpyDeviceToDevice, stream));
                history = true;
            }
            assemble(x, true);
            bdf2_w_kernel<<<g, 256, 0, stream>>>(vec(d_w), x0, vec(d_xm1), v0, 2 * h, n);
            launch_spmv(T, vec(d_w), vec(d_u), L.nv, nullptr, nullptr, stream);
            bdf2_rhs_kernel<<<g, 256, 0, stream>>>(b, vec(d_mass), v0, vec(d_vm1), f, vec(d_u), h, n);
            SPGX_TRY_STATUS(solve(1.0, 4.0 / 9.0 * (h * h), t));
            lincomb_kernel<<<g, 256, 0, stream>>>(v, v0, vec(d_dx), 1.0, n);
            bdf2_update_kernel<<<g, 256, 0, stream>>>(x, vec(d_xm1), vec(d_vm1), x0, v0, v, h, n);
            break;
        }
        case SPGX_STATIC_NEWTON: {
            assemble(x, true);
            scale_kernel<<<g, 256, 0, stream>>>(b, f, -1.0, n);
            SPGX_TRY_STATUS(solve(0.0, -1.0, t));
            axpy_kernel<<<g, 256, 0, stream>>>(x, vec(d_dx), 1.0, n);
            break;
        }
        case SPGX_QUASI_STATIC_NEWTON: {
            assemble(x, true);
            const double dtdt = h * h;
            scale_kernel<<<g, 256, 0, stream>>>(b, f, dtdt, n);
            SPGX_TRY_STATUS(solve(1.0, dtdt, t));
            axpy_kernel<<<g, 256, 0, stream>>>(x, vec(d_dx), 1.0, n);
            break;
        }
        case SPGX_SYMPLECTIC_EULER: {
            assemble(x, false, false);
            symplectic_kernel<<<g, 256, 0, stream>>>(v, f, vec(d_mass), h, h * P.gravity[0], h * P.gravity[1],
                                                     h * P.gravity[2], n);
            axpy_kernel<<<g, 256, 0, stream>>>(x, v, h, n);
            break;
        }
        default: break;
        }
        SPGX_CUDA(cudaGetLastError());
        return SPGX_OK;
    }

    double begin_controlled(double &max_dt)
    {
        max_dt = P.dt / P.substeps;
        if (current_dt == -1. || current_dt > max_dt) current_dt = max_dt;
        return current_dt;
    }

    void end_controlled(bool ok, double max_dt, Tally &t)
    {
        if (!ok) {
            current_dt *= 0.75;
            successes = 0;
            ++t.failed;
            t.converged = false;
        } else {
            ++successes;
            if (successes > 5 && current_dt < max_dt) current_dt /= 0.75;
        }
    }

    // ImplicitEulerNewtonRobust substep (implicitEulerNewtonRobust.cpp:33-126).
    spgx_status newton_robust(Tally &t)
    {
        const double threshold = 1e-5;
        const int n = n3(), g = grid_of(n);
        const size_t bytes = size_t(n) * sizeof(double);
        double *x = vec(d_x), *v = vec(d_v), *x0 = vec(d_x0), *v0 = vec(d_v0), *vi = vec(d_vi);
        double *norm2 = d_dots.as<double>() + 7;
        double max_dt;
        const double dt = begin_controlled(max_dt);
        bool ok = true;
        SPGX_CUDA(cudaMemcpyAsync(x0, x, bytes, cudaMemcpyDeviceToDevice, stream));
        SPGX_CUDA(cudaMemcpyAsync(v0, v, bytes, cudaMemcpyDeviceToDevice, stream));
        SPGX_CUDA(cudaMemsetAsync(norm2, 0, sizeof(double), stream));
        axpy_kernel<<<g, 256, 0, stream>>>(x, v, dt, n);
        SPGX_CUDA(cudaMemcpyAsync(vi, v0, bytes, cudaMemcpyDeviceToDevice, stream));
        int it = 0;
        double res = 0.0;
        do {
            assemble(x, true);
            robust_rhs_kernel<<<g, 256, 0, stream>>>(vec(d_b), vec(d_f), vi, v0, vec(d_mass), dt, n, norm2);
            double r0;
            SPGX_TRY_STATUS(take_norm(r0));
            if (t.first_residual < 0) t.first_residual = r0;
            SPGX_TRY_STATUS(solve(1.0, dt * dt, t));
            res = r0;
            int ls = 0;
            double alpha = 1.;
            while (res >= r0 && ls < 5) {
                lincomb_kernel<<<g, 256, 0, stream>>>(v, vi, vec(d_dx), alpha, n);
                lincomb_kernel<<<g, 256, 0, stream>>>(x, x0, v, dt, n);
                assemble(x, false);
                robust_rhs_kernel<<<g, 256, 0, stream>>>(nullptr, vec(d_f), v, v0, vec(d_mass), dt, n, norm2);
                SPGX_TRY_STATUS(take_norm(res));
                if (res < r0) SPGX_CUDA(cudaMemcpyAsync(vi, v, bytes, cudaMemcpyDeviceToDevice, stream));
                alpha *= 0.5;
                ++ls;
            }
            if (res >= r0 && res > threshold) ok = false;
            ++it;
        } while (res > threshold && ok && it < 5);
        t.newton_iterations += it;
        t.last_residual = res;
        if (res > threshold) ok = false;
        if (!ok) {
            SPGX_CUDA(cudaMemcpyAsync(x, x0, bytes, cudaMemcpyDeviceToDevice, stream));
            SPGX_CUDA(cudaMemcpyAsync(v, v0, bytes, cudaMemcpyDeviceToDevice, stream));
        }
        end_controlled(ok, max_dt, t);
        SPGX_CUDA(cudaGetLastError());
        return SPGX_OK;
    }

    // QuasiStaticNewtonRobust substep (quasiStaticNewtonRobust.cpp:33-136).
    spgx_status quasi_static_robust(Tally &t)
    {
        const double threshold = 1e-2;
        const int n = n3(), g = grid_of(n);
        const size_t bytes = size_t(n) * sizeof(double);
        double *x = vec(d_x), *v = vec(d_v), *x0 = vec(d_x0), *xi = vec(d_vi);
        double *norm2 = d_dots.as<double>() + 7;
        double max_dt;
        const double dt = begin_controlled(max_dt);
        const double invdt = 1 / dt;
        const double invdt2 = invdt * invdt;
        bool ok = true;
        SPGX_CUDA(cudaMemcpyAsync(x0, x, bytes, cudaMemcpyDeviceToDevice, stream));
        SPGX_CUDA(cudaMemcpyAsync(xi, x0, bytes, cudaMemcpyDeviceToDevice, stream));
        SPGX_CUDA(cudaMemsetAsync(norm2, 0, sizeof(double), stream));
        int it = 0;
        double res = 0.0;
        do {
            assemble(x, true);
            diffscale_kernel<<<g, 256, 0, stream>>>(v, x, x0, invdt, n);
            qs_rhs_kernel<<<g, 256, 0, stream>>>(vec(d_b), vec(d_f), v, vec(d_mass), invdt, n, norm2);
            double r0;
            SPGX_TRY_STATUS(take_norm(r0));
            if (t.first_residual < 0) t.first_residual = r0;
            SPGX_TRY_STATUS(solve(invdt2, 1.0, t));
            res = r0;
            int ls = 0;
            double alpha = 1.;
            while (res >= r0 && ls < 5) {
                lincomb_kernel<<<g, 256, 0, stream>>>(x, xi, vec(d_dx), alpha, n);
                diffscale_kernel<<<g, 256, 0, stream>>>(v, x, x0, invdt, n);
                assemble(x, false);
                qs_rhs_kernel<<<g, 256, 0, stream>>>(nullptr, vec(d_f), v, vec(d_mass), invdt, n, norm2);
                SPGX_TRY_STATUS(take_norm(res));
                if (res < r0) SPGX_CUDA(cudaMemcpyAsync(xi, x, bytes, cudaMemcpyDeviceToDevice, stream));
                alpha *= 0.5;
                ++ls;
            }
            if (res >= r0 && res > threshold) ok = false;
            ++it;
        } while (res > threshold && ok && it < 5);
        t.newton_iterations += it;
        t.last_residual = res;
        if (res > threshold) ok = false;
        if (!ok) SPGX_CUDA(cudaMemcpyAsync(x, x0, bytes, cudaMemcpyDeviceToDevice, stream));
        end_controlled(ok, max_dt, t);
        SPGX_CUDA(cudaGetLastError());
        return SPGX_OK;
    }

    spgx_status step(spgx_step_stats *stats)
    {
        Tally t;
        const int nv = L.nv;
        const double h = P.dt / P.substeps;
        SPGX_CUDA(cudaEventRecord(ev0, stream));
        for (int s = 0; s < P.substeps && nv > 0; ++s) {
            if (P.method == SPGX_IMPLICIT_NEWTON_ROBUST)
                SPGX_TRY_STATUS(newton_robust(t));
            else if (P.method == SPGX_QUASI_STATIC_NEWTON_ROBUST)
                SPGX_TRY_STATUS(quasi_static_robust(t));
            else
                SPGX_TRY_STATUS(substep(h, t));
        }
        SPGX_CUDA(cudaEventRecord(ev1, stream));
        SPGX_CUDA(cudaGetLastError());
        SPGX_CUDA(cudaStreamSynchronize(stream));
        float ms = 0.f;
        SPGX_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
        spgx_step_stats st{};
        st.iterations = t.cg_iterations;
        st.fallback_solves = t.newton_iterations;
        st.skipped_solves = t.failed;
        st.converged = t.converged ? 1 : 0;
        st.residual_initial = t.first_residual < 0 ? 0.0 : t.first_residual;
        st.residual_final = t.last_residual;
        st.device_ms = ms;
        st.warm_accepted = t.fp64_solves;
        if (stats) *stats = st;
        return SPGX_OK;
    }

    // State in the external order of one object.
    spgx_status get(int obj, double *x, double *v)
    {
        if (obj < 0 || obj >= static_cast<int>(L.objects.size())) {
            set_error("invalid object index");
            return SPGX_ERR_INVALID_ARG;
        }
        const size_t n = 3 * size_t(std::max(1, L.nv));
        std::vector<double> hx(n), hv(n);
        SPGX_CUDA(cudaMemcpyAsync(hx.data(), vec(d_x), n * sizeof(double), cudaMemcpyDeviceToHost, stream));
        SPGX_CUDA(cudaMemcpyAsync(hv.data(), vec(d_v), n * sizeof(double), cudaMemcpyDeviceToHost, stream));
        SPGX_CUDA(cudaStreamSynchronize(stream));
        const auto &O = L.objects[obj];
        for (int k = 0; k < O.nv; ++k) {
            const size_t i = size_t(row_of[O.vertex_base + k]);
            for (int a = 0; a < 3; ++a) {
                if (x) x[3 * k + a] = hx[3 * i + a];
                if (v) v[3 * k + a] = hv[3 * i + a];
            }
        }
        return SPGX_OK;
    }

    spgx_status set(int obj, const double *x, const double *v)
    {
        if (obj < 0 || obj >= static_cast<int>(L.objects.size())) {
            set_error("invalid object index");
            return SPGX_ERR_INVALID_ARG;
        }
        const size_t n = 3 * size_t(std::max(1, L.nv));
        std::vector<double> hx(n), hv(n);
        SPGX_CUDA(cudaMemcpyAsync(hx.data(), vec(d_x), n * sizeof(double), cudaMemcpyDeviceToHost, stream));
        SPGX_CUDA(cudaMemcpyAsync(hv.data(), vec(d_v), n * sizeof(double), cudaMemcpyDeviceToHost, stream));
        SPGX_CUDA(cudaStreamSynchronize(stream));
        const auto &O = L.objects[obj];
        for (int k = 0; k < O.nv; ++k) {
            const size_t i = size_t(row_of[O.vertex_base + k]);
            for (int a = 0; a < 3; ++a) {
                if (x) hx[3 * i + a] = x[3 * k + a];
                if (v) hv[3 * i + a] = v[3 * k + a];
            }
        }
        SPGX_CUDA(cudaMemcpyAsync(vec(d_x), hx.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream));
        SPGX_CUDA(cudaMemcpyAsync(vec(d_v), hv.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream));
        SPGX_CUDA(cudaStreamSynchronize(stream));
        return SPGX_OK;
    }

    // BaseSolver::reset: initial positions, zero velocities; the robust methods' step control
    // and BDF2's history start over (NewtonRobust::reset, BDF2::reset).
    spgx_status reset()
    {
        for (int o = 0; o < static_cast<int>(L.objects.size()); ++o) {
            const std::vector<double> zeros(L.objects[o].x_init.size(), 0.0);
            SPGX_TRY_STATUS(set(o, L.objects[o].x_init.data(), zeros.data()));
        }
        current_dt = -1.0;
        successes = 0;
        history = false;
        return SPGX_OK;
    }
};

}  // namespace spgx

// =======================================================================================
// C ABI

struct spgx_implicit {
    std::unique_ptr<spgx::ImplicitSolver> s;
};

extern "C" {

void spgx_implicit_params_default(spgx_implicit_params *p)
{
    if (!p) return;
    *p = spgx_implicit_params{};
    p->dt = 0.01;
    p->substeps = 1;
    p->gravity[0] = 0.0;
    p->gravity[1] = -9.8;
    p->gravity[2] = 0.0;
    p->cg_threshold = 1e-5;
    p->cg_max_iterations = 300;
    p->device = 0;
    p->method = SPGX_IMPLICIT_NEWTON_DX;
    p->cg_precision = 0;
}

spgx_status spgx_implicit_create(const spgx_scene_desc *scene, const spgx_implicit_params *params, spgx_implicit **out)
{
    SPGX_GUARD_BEGIN
    if (!out) {
        spgx::set_error("out is NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    *out = nullptr;
    auto h = std::make_unique<spgx_implicit>();
    h->s = std::make_unique<spgx::ImplicitSolver>();
    SPGX_TRY_STATUS(h->s->init(scene, params));
    *out = h.release();
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_implicit_destroy(spgx_implicit *h)
{
    SPGX_GUARD_BEGIN
    if (h) {
        cudaSetDevice(h->s->device);
        delete h;
    }
    return SPGX_OK;
    SPGX_GUARD_END
}

#define SPGX_IHANDLE(h)                                \
    if (!(h)) {                                        \
        spgx::set_error("NULL implicit solver handle"); \
        return SPGX_ERR_INVALID_ARG;                   \
    }                                                  \
    SPGX_CUDA(cudaSetDevice((h)->s->device))

spgx_status spgx_implicit_step(spgx_implicit *h, spgx_step_stats *stats)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    return h->s->step(stats);
    SPGX_GUARD_END
}

spgx_status spgx_implicit_get_state(spgx_implicit *h, int32_t object, double *x, double *v)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    return h->s->get(object, x, v);
    SPGX_GUARD_END
}

spgx_status spgx_implicit_set_state(spgx_implicit *h, int32_t object, const double *x, const double *v)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    return h->s->set(object, x, v);
    SPGX_GUARD_END
}

spgx_status spgx_implicit_reset(spgx_implicit *h)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    return h->s->reset();
    SPGX_GUARD_END
}

spgx_status spgx_implicit_set_params(spgx_implicit *h, const spgx_implicit_params *params)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    return h->s->set_params(params);
    SPGX_GUARD_END
}

spgx_status spgx_implicit_get_step_size(spgx_implicit *h, double *dt)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    if (!dt) {
        spgx::set_error("dt is NULL");
        return SPGX_ERR_INVALID_ARG;
    }
    *dt = h->s->current_dt;
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_implicit_test_stall(spgx_implicit *h)
{
    SPGX_GUARD_BEGIN
    SPGX_IHANDLE(h);
    h->s->stall_next = true;
    return SPGX_OK;
    SPGX_GUARD_END
}

}  // extern "C"
