// Per-vertex blocks of the energies outside the closed-form five (types 6-14 of spgx.h), by
// forward-mode differentiation restricted to the three coordinates of the vertex being
// solved: every quantity carries its value, its gradient and its symmetric 3x3 Hessian with
// respect to that vertex. This is what the reference's TinyAD evaluation of the full element
// yields for the vertex's gradient segment and diagonal Hessian block (energy.h:240-258,
// 336-362), at a fraction of the cost (10 components instead of 1 + 3S + (3S)^2).
//
// Energies (parameter layouts in spgx.h), each E = 1/2 C^T K C over its constraints C unless
// stated (energy.h:336-347, K the diagonal effective stiffness):
//   STVK (tet)        E = 1/2 lambda tr(G)^2 + mu tr(G^T G), G = 1/2 (F^T F - I)  stvkEnergy.cpp:37-60
//   SSNH              C = [det F - 1, tr(F^T F) - 3]         stableSquaredNeoHookeanEnergy.cpp:9-31
//   BW membrane       C = [|F0| - 1, |F1| - 1, F0 . F1]       membraneBaraffWitkinEnergy.cpp:9-26
//   Choi membrane     C = [|F0|-1, |F1|-1, |(F0+F1)/sqrt2|-1, |(F0-F1)/sqrt2|-1]  membraneChoiEnergy.cpp:9-29
//   BW bending        C = theta - theta0 with the norms held constant  baraffWitkinBendingEnergy.cpp:9-38
//   quadratic bending C = sum_s c_s x_s (linear; closed form)            quadraticBendingEnergy.cpp:9-30
//   spring continuum  C = |x0 - x1| / L0 - 1                             springContinuumEnergy.cpp:8-17
//   spring squared    C = |x0 - x1|^2 / L0^2 - 1                         springSquaredContinuumEnergy.cpp:8-17
//   static load       E = -k d . x (gradient -k d, zero Hessian)         staticLoadEnergy.cpp:17-23
#pragma once

#include "elements.cuh"
#include "spgx.h"

namespace spgx {

// One out-of-line copy per scalar type: every kernel that evaluates these energies calls the
// same function instead of inlining all of them.
#ifdef __CUDA_ARCH__
#define SPGX_GENERIC_NOINLINE __noinline__
#else
#define SPGX_GENERIC_NOINLINE
#endif

// Value, gradient and symmetric Hessian with respect to K seeded coordinates (K = 3: the
// vertex being solved; K = 6: a pair of stencil vertices, for off-diagonal Hessian blocks).
// The Hessian holds the upper triangle row by row (for K = 3: xx, xy, xz, yy, yz, zz).
template <typename T, int K = 3>
struct VAD {
    static constexpr int kH = K * (K + 1) / 2;
    T v, g[K], h[kH];
};

template <int K>
SPGX_HD constexpr int hidx(int i, int j)
{
    return i * K - i * (i - 1) / 2 + (j - i);
}

template <typename T, int K = 3>
SPGX_HD VAD<T, K> vconst(T x)
{
    VAD<T, K> r;
    r.v = x;
#pragma unroll
    for (int i = 0; i < K; ++i) r.g[i] = T(0);
#pragma unroll
    for (int i = 0; i < VAD<T, K>::kH; ++i) r.h[i] = T(0);
    return r;
}

template <typename T, int K>
SPGX_HD VAD<T, K> operator+(const VAD<T, K> &a, const VAD<T, K> &b)
{
    VAD<T, K> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.g[i] = a.g[i] + b.g[i];
#pragma unroll
    for (int i = 0; i < VAD<T, K>::kH; ++i) r.h[i] = a.h[i] + b.h[i];
    return r;
}

template <typename T, int K>
SPGX_HD VAD<T, K> operator-(const VAD<T, K> &a, const VAD<T, K> &b)
{
    VAD<T, K> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.g[i] = a.g[i] - b.g[i];
#pragma unroll
    for (int i = 0; i < VAD<T, K>::kH; ++i) r.h[i] = a.h[i] - b.h[i];
    return r;
}

template <typename T, int K>
SPGX_HD VAD<T, K> operator-(const VAD<T, K> &a)
{
    VAD<T, K> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.g[i] = -a.g[i];
#pragma unroll
    for (int i = 0; i < VAD<T, K>::kH; ++i) r.h[i] = -a.h[i];
    return r;
}

template <typename T, int K>
SPGX_HD VAD<T, K> operator*(T s, const VAD<T, K> &a)
{
    VAD<T, K> r;
    r.v = s * a.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.g[i] = s * a.g[i];
#pragma unroll
    for (int i = 0; i < VAD<T, K>::kH; ++i) r.h[i] = s * a.h[i];
    return r;
}

template <typename T, int K>
SPGX_HD VAD<T, K> operator+(const VAD<T, K> &a, T s)
{
    VAD<T, K> r = a;
    r.v = a.v + s;
    return r;
}

template <typename T, int K>
SPGX_HD VAD<T, K> operator*(const VAD<T, K> &a, const VAD<T, K> &b)
{
    VAD<T, K> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < K; ++i) r.g[i] = a.v * b.g[i] + b.v * a.g[i];
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
        for (int j = i; j < K; ++j) {
            const int k = hidx<K>(i, j);
            r.h[k] = a.v * b.h[k] + b.v * a.h[k] + a.g[i] * b.g[j] + a.g[j] * b.g[i];
        }
    return r;
}

// f(a) for a scalar function with derivatives d1 = f'(a.v), d2 = f''(a.v).
template <typename T, int K>
SPGX_HD VAD<T, K> chain(const VAD<T, K> &a, T f, T d1, T d2)
{
    VAD<T, K> r;
    r.v = f;
#pragma unroll
    for (int i = 0; i < K; ++i) r.g[i] = d1 * a.g[i];
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
        for (int j = i; j < K; ++j) {
            const int k = hidx<K>(i, j);
            r.h[k] = d1 * a.h[k] + d2 * a.g[i] * a.g[j];
        }
    return r;
}

template <typename T, int K>
SPGX_HD VAD<T, K> vsqrt(const VAD<T, K> &a)
{
    const T s = sqrt(a.v);
    const T d1 = T(0.5) / s;
    return chain(a, s, d1, -d1 / (T(2) * a.v));
}

template <typename T, int K>
SPGX_HD VAD<T, K> vrecip(const VAD<T, K> &a)
{
    const T r = T(1) / a.v;
    return chain(a, r, -r * r, T(2) * r * r * r);
}

// atan2(y, x) through its partial derivatives: d/dy = x / q, d/dx = -y / q (q = x^2 + y^2).
template <typename T, int K>
SPGX_HD VAD<T, K> vatan2(const VAD<T, K> &y, const VAD<T, K> &x)
{
    const T q = x.v * x.v + y.v * y.v;
    const T iq = T(1) / q;
    const T ay = x.v * iq, ax = -y.v * iq;       // first partials
    const T iq2 = iq * iq;
    const T ayy = -T(2) * x.v * y.v * iq2;        // d2/dy2
    const T axx = T(2) * x.v * y.v * iq2;         // d2/dx2
    const T axy = (y.v * y.v - x.v * x.v) * iq2;  // d2/dxdy
    VAD<T, K> r;
    r.v = atan2(y.v, x.v);
#pragma unroll
    for (int i = 0; i < K; ++i) r.g[i] = ay * y.g[i] + ax * x.g[i];
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
        for (int j = i; j < K; ++j) {
            const int k = hidx<K>(i, j);
            r.h[k] = ay * y.h[k] + ax * x.h[k] + ayy * y.g[i] * y.g[j] + axx * x.g[i] * x.g[j] +
                     axy * (x.g[i] * y.g[j] + y.g[i] * x.g[j]);
        }
    return r;
}

template <typename T, int K = 3>
struct V3A {
    VAD<T, K> x, y, z;
};

template <typename T, int K>
SPGX_HD V3A<T, K> vsub(const V3A<T, K> &a, const V3A<T, K> &b)
{
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T, int K>
SPGX_HD V3A<T, K> vadd(const V3A<T, K> &a, const V3A<T, K> &b)
{
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename T, int K>
SPGX_HD V3A<T, K> vscale(T s, const V3A<T, K> &a)
{
    return {s * a.x, s * a.y, s * a.z};
}
template <typename T, int K>
SPGX_HD VAD<T, K> vdot(const V3A<T, K> &a, const V3A<T, K> &b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T, int K>
SPGX_HD V3A<T, K> vcross(const V3A<T, K> &a, const V3A<T, K> &b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T, int K>
SPGX_HD VAD<T, K> vnorm(const V3A<T, K> &a)
{
    return vsqrt(vdot(a, a));
}

// Positions as differentiable vectors: vertex `a` carries seeds 0..2 and, with K = 6, vertex
// `b` seeds 3..5; the others are constants. Positions may be relative to any point (the
// energies are translation invariant).
template <typename T, int S, int K = 3>
SPGX_HD void seed_positions(const Vec3<T> *p, int a, V3A<T, K> *q, int b = -1)
{
#pragma unroll
    for (int j = 0; j < S; ++j) {
        q[j].x = vconst<T, K>(p[j].x);
        q[j].y = vconst<T, K>(p[j].y);
        q[j].z = vconst<T, K>(p[j].z);
        if (j == a) {
            q[j].x.g[0] = T(1);
            q[j].y.g[1] = T(1);
            q[j].z.g[2] = T(1);
        }
        if (K == 6 && j == b) {
            q[j].x.g[K == 6 ? 3 : 0] = T(1);
            q[j].y.g[K == 6 ? 4 : 0] = T(1);
            q[j].z.g[K == 6 ? 5 : 0] = T(1);
        }
    }
}

template <typename T>
SPGX_HD void add_vad(Block<T> &b, const VAD<T> &E)
{
#pragma unroll
    for (int i = 0; i < 3; ++i) b.f[i] -= E.g[i];
#pragma unroll
    for (int i = 0; i < 6; ++i) b.h[i] += E.h[i];
}

// F columns f_c = sum_j d_j D[j][c] over the edge vectors d_j = x_{j+1} - x_0 (Dinv row-major, n x n).
template <typename T, int N, int K>
SPGX_HD void deformation_columns(const V3A<T, K> *q, const T *D, V3A<T, K> *f)
{
    V3A<T, K> d[N];
#pragma unroll
    for (int j = 0; j < N; ++j) d[j] = vsub(q[j + 1], q[0]);
#pragma unroll
    for (int c = 0; c < N; ++c) {
        f[c] = vscale(D[c], d[0]);
#pragma unroll
        for (int j = 1; j < N; ++j) f[c] = vadd(f[c], vscale(D[j * N + c], d[j]));
    }
}

template <typename T, int K>
SPGX_HD VAD<T, K> half_k_sq(T k, const VAD<T, K> &c)
{
    return (T(0.5) * k) * (c * c);
}

// ---------------------------------------------------------------------------------------
// Element energies on seeded positions (all types but the quadratic bending and the static
// load, whose derivatives are closed-form and linear). Types 1-5 (used by the implicit
// solver's assembly; the VBD kernels keep their closed forms):
//   SPRING            1/2 k (|x0 - x1| - L0)^2                        springEnergy.cpp:70-99
//   ANCHOR            1/2 k |x - a|^2 (q[0] is x - a)                  springAnchorEnergy.cpp:21-26
//   DISCRETE_BENDING  1/2 k (theta - theta0)^2, normalized normals     discreteBendingEnergy.cpp:9-30
//   MEMBRANE_STVK     1/2 C^T K C, C = [G00, G11, 2 G01]               membraneStvkEnergy.cpp:9-28
//   SNH               1/2 lambda (J - alpha)^2 + 1/2 mu (tr F^T F - 3)  stableNeoHookeanEnergy.cpp:33-61

template <typename T, int K>
SPGX_HD VAD<T, K> stvk_tet_energy(const V3A<T, K> *q, const T *prm)
{
    V3A<T, K> f[3];
    deformation_columns<T, 3>(q, prm, f);
    VAD<T, K> tr = vconst<T, K>(T(0)), sq = vconst<T, K>(T(0));
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            VAD<T, K> G = T(0.5) * vdot(f[a], f[c]);
            if (a == c) G = G + T(-0.5);
            if (a == c) tr = tr + G;
            sq = sq + G * G;
        }
    return (T(0.5) * prm[9]) * (tr * tr) + prm[10] * sq;
}

template <typename T, int K>
SPGX_HD VAD<T, K> ssnh_energy(const V3A<T, K> *q, const T *prm)
{
    V3A<T, K> f[3];
    deformation_columns<T, 3>(q, prm, f);
    const VAD<T, K> J = vdot(f[0], vcross(f[1], f[2])) + T(-1);
    const VAD<T, K> I = vdot(f[0], f[0]) + vdot(f[1], f[1]) + vdot(f[2], f[2]) + T(-3);
    return half_k_sq(prm[9], J) + half_k_sq(prm[10], I);
}

template <typename T, int K>
SPGX_HD VAD<T, K> bw_membrane_energy(const V3A<T, K> *q, const T *prm, bool choi)
{
    V3A<T, K> f[2];
    deformation_columns<T, 2>(q, prm, f);
    VAD<T, K> E = half_k_sq(prm[4], vnorm(f[0]) + T(-1)) + half_k_sq(prm[5], vnorm(f[1]) + T(-1));
    if (!choi) return E + half_k_sq(prm[6], vdot(f[0], f[1]));
    const T s = T(0.70710678118654752440);
    E = E + half_k_sq(prm[6], vnorm(vscale(s, vadd(f[0], f[1]))) + T(-1));
    return E + half_k_sq(prm[7], vnorm(vscale(s, vsub(f[0], f[1]))) + T(-1));
}

template <typename T, int K>
SPGX_HD VAD<T, K> bw_bending_energy(const V3A<T, K> *q, const T *prm)
{
    const V3A<T, K> e0 = vsub(q[1], q[0]), e3 = vsub(q[2], q[1]), e4 = vsub(q[3], q[1]);
    // The norms are held constant (their values only), as the reference does with .val.
    const T e0i = T(1) / sqrt(vdot(e0, e0).v);
    const V3A<T, K> n1 = vcross(e0, e3);
    const V3A<T, K> n2 = vscale(T(-1), vcross(e0, e4));
    const T n1i = T(1) / sqrt(vdot(n1, n1).v);
    const T n2i = T(1) / sqrt(vdot(n2, n2).v);
    const V3A<T, K> a = vscale(n1i, n1), c = vscale(n2i, n2);
    const VAD<T, K> th = vatan2(vdot(vcross(a, c), vscale(e0i, e0)), vdot(a, c));
    return half_k_sq(prm[1], th + (-prm[0]));
}

template <typename T, int K>
SPGX_HD VAD<T, K> continuum_spring_energy(const V3A<T, K> *q, const T *prm, bool squared)
{
    const V3A<T, K> d = vsub(q[0], q[1]);
    const T L0 = prm[0];
    const VAD<T, K> C = squared ? (T(1) / (L0 * L0)) * vdot(d, d) + T(-1) : (T(1) / L0) * vnorm(d) + T(-1);
    return half_k_sq(prm[1], C);
}

template <typename T, int K>
SPGX_HD VAD<T, K> spring_energy_ad(const V3A<T, K> *q, const T *prm)
{
    return half_k_sq(prm[1], vnorm(vsub(q[0], q[1])) + (-prm[0]));
}

template <typename T, int K>
SPGX_HD VAD<T, K> anchor_energy_ad(const V3A<T, K> *q, const T *prm)
{
    return (T(0.5) * prm[3]) * vdot(q[0], q[0]);
}

template <typename T, int K>
SPGX_HD V3A<T, K> vnormalized(const V3A<T, K> &a)
{
    const VAD<T, K> inv = vrecip(vnorm(a));
    return {a.x * inv, a.y * inv, a.z * inv};
}

template <typename T, int K>
SPGX_HD VAD<T, K> discrete_bending_energy_ad(const V3A<T, K> *q, const T *prm)
{
    const V3A<T, K> e0 = vsub(q[1], q[0]), e3 = vsub(q[2], q[1]), e4 = vsub(q[3], q[1]);
    const V3A<T, K> n1 = vnormalized(vcross(e0, e3));
    const V3A<T, K> n2 = vscale(T(-1), vnormalized(vcross(e0, e4)));
    const VAD<T, K> th = vatan2(vdot(vcross(n1, n2), vnormalized(e0)), vdot(n1, n2));
    return half_k_sq(prm[1], th + (-prm[0]));
}

template <typename T, int K>
SPGX_HD VAD<T, K> membrane_stvk_energy_ad(const V3A<T, K> *q, const T *prm)
{
    V3A<T, K> f[2];
    deformation_columns<T, 2>(q, prm, f);
    VAD<T, K> C[3];
    C[0] = T(0.5) * (vdot(f[0], f[0]) + T(-1));
    C[1] = T(0.5) * (vdot(f[1], f[1]) + T(-1));
    C[2] = vdot(f[0], f[1]);
    const T *Km = prm + 4;
    VAD<T, K> e = vconst<T, K>(T(0));
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const VAD<T, K> kc = Km[3 * i] * C[0] + Km[3 * i + 1] * C[1] + Km[3 * i + 2] * C[2];
        e = e + C[i] * kc;
    }
    return T(0.5) * e;
}

template <typename T, int K>
SPGX_HD VAD<T, K> snh_energy_ad(const V3A<T, K> *q, const T *prm)
{
    V3A<T, K> f[3];
    deformation_columns<T, 3>(q, prm, f);
    const VAD<T, K> J = vdot(f[0], vcross(f[1], f[2])) + (-prm[11]);
    const VAD<T, K> tr = vdot(f[0], f[0]) + vdot(f[1], f[1]) + vdot(f[2], f[2]) + T(-3);
    return (T(0.5) * prm[9]) * (J * J) + (T(0.5) * prm[10]) * tr;
}

// The energy of one element of `type` at seeded positions q (types 1-10, 12, 13).
template <typename T, int K>
SPGX_HD VAD<T, K> energy_ad(int type, const V3A<T, K> *q, const T *prm)
{
    switch (type) {
    case SPGX_ENERGY_SPRING: return spring_energy_ad(q, prm);
    case SPGX_ENERGY_SPRING_ANCHOR: return anchor_energy_ad(q, prm);
    case SPGX_ENERGY_DISCRETE_BENDING: return discrete_bending_energy_ad(q, prm);
    case SPGX_ENERGY_MEMBRANE_STVK: return membrane_stvk_energy_ad(q, prm);
    case SPGX_ENERGY_STABLE_NEO_HOOKEAN: return snh_energy_ad(q, prm);
    case SPGX_ENERGY_STVK: return stvk_tet_energy(q, prm);
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: return ssnh_energy(q, prm);
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN: return bw_membrane_energy(q, prm, false);
    case SPGX_ENERGY_MEMBRANE_CHOI: return bw_membrane_energy(q, prm, true);
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING: return bw_bending_energy(q, prm);
    case SPGX_ENERGY_SPRING_CONTINUUM: return continuum_spring_energy(q, prm, false);
    case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM: return continuum_spring_energy(q, prm, true);
    default: return vconst<T, K>(T(0));
    }
}

// Per-vertex forward-mode block (K = 3, the vertex at `slot`) of an energy whose function is
// given as a callable on seeded positions.
template <typename T, int S, typename Fn>
SPGX_HD void vertex_energy_block(Fn fn, const Vec3<T> *p, int slot, Block<T> &b)
{
    V3A<T> q[S];
    seed_positions<T, S>(p, slot, q);
    add_vad(b, fn(q));
}

// Linear constraint C = sum_s c_s x_s: gradient k c_slot C, Hessian k c_slot^2 I.
template <typename T>
SPGX_HD void quadratic_bending_block(const Vec3<T> *p, int slot, const T *prm, Block<T> &b)
{
    Vec3<T> C = mk(T(0), T(0), T(0));
#pragma unroll
    for (int s = 0; s < 4; ++s) C = C + prm[s] * p[s];
    const T cs = prm[slot];
    const T k = prm[4];
    sub_force(b, C, k * cs);
    add_diag(b, k * cs * cs);
}

template <typename T>
SPGX_HD void static_load_block(const T *prm, Block<T> &b)
{
    // E = -k d.x: the force is k d, the Hessian zero.
    const Vec3<T> d = mk(prm[1], prm[2], prm[3]);
    sub_force(b, d, -prm[0]);
}

// Constraints of types 6-13 (the reference's dConstraints lambdas, cited above; the StVK tet's
// is [tr G, sqrt(2 tr(G G))], stvkEnergy.cpp:9-35, with the second set to 0 when its value
// is 0), differentiated with respect to the vertex at `slot`. Returns their number (0 for the
// static load, which has no constraint form: staticLoadEnergy.cpp:8-15).
template <typename T>
SPGX_HD SPGX_GENERIC_NOINLINE int generic_constraints(int type, const Vec3<T> *p, int slot, const T *prm, VAD<T> *C)
{
    switch (type) {
    case SPGX_ENERGY_STVK: {
        V3A<T> q[4], f[3];
        seed_positions<T, 4>(p, slot, q);
        deformation_columns<T, 3>(q, prm, f);
        VAD<T> tr = vconst(T(0)), sq = vconst(T(0));
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                VAD<T> G = T(0.5) * vdot(f[a], f[c]);
                if (a == c) G = G + T(-0.5);
                if (a == c) tr = tr + G;
                sq = sq + G * G;
            }
        C[0] = tr;
        C[1] = sq.v == T(0) ? vconst(T(0)) : vsqrt(T(2) * sq);
        return 2;
    }
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: {
        V3A<T> q[4], f[3];
        seed_positions<T, 4>(p, slot, q);
        deformation_columns<T, 3>(q, prm, f);
        C[0] = vdot(f[0], vcross(f[1], f[2])) + T(-1);
        C[1] = vdot(f[0], f[0]) + vdot(f[1], f[1]) + vdot(f[2], f[2]) + T(-3);
        return 2;
    }
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN:
    case SPGX_ENERGY_MEMBRANE_CHOI: {
        V3A<T> q[3], f[2];
        seed_positions<T, 3>(p, slot, q);
        deformation_columns<T, 2>(q, prm, f);
        C[0] = vnorm(f[0]) + T(-1);
        C[1] = vnorm(f[1]) + T(-1);
        if (type == SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN) {
            C[2] = vdot(f[0], f[1]);
            return 3;
        }
        const T s = T(0.70710678118654752440);
        C[2] = vnorm(vscale(s, vadd(f[0], f[1]))) + T(-1);
        C[3] = vnorm(vscale(s, vsub(f[0], f[1]))) + T(-1);
        return 4;
    }
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING: {
        V3A<T> q[4];
        seed_positions<T, 4>(p, slot, q);
        const V3A<T> e0 = vsub(q[1], q[0]), e3 = vsub(q[2], q[1]), e4 = vsub(q[3], q[1]);
        const T e0i = T(1) / sqrt(vdot(e0, e0).v);
        const V3A<T> n1 = vcross(e0, e3);
        const V3A<T> n2 = vscale(T(-1), vcross(e0, e4));
        const T n1i = T(1) / sqrt(vdot(n1, n1).v);
        const T n2i = T(1) / sqrt(vdot(n2, n2).v);
        const V3A<T> a = vscale(n1i, n1), c = vscale(n2i, n2);
        C[0] = vatan2(vdot(vcross(a, c), vscale(e0i, e0)), vdot(a, c)) + (-prm[0]);
        return 1;
    }
    case SPGX_ENERGY_QUADRATIC_BENDING: {
        V3A<T> q[4];
        seed_positions<T, 4>(p, slot, q);
        V3A<T> s = vscale(prm[0], q[0]);
#pragma unroll
        for (int j = 1; j < 4; ++j) s = vadd(s, vscale(prm[j], q[j]));
        C[0] = s.x;
        C[1] = s.y;
        C[2] = s.z;
        return 3;
    }
    case SPGX_ENERGY_SPRING_CONTINUUM:
    case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM: {
        V3A<T> q[2];
        seed_positions<T, 2>(p, slot, q);
        const V3A<T> d = vsub(q[0], q[1]);
        const T L0 = prm[0];
        C[0] = type == SPGX_ENERGY_SPRING_SQUARED_CONTINUUM ? (T(1) / (L0 * L0)) * vdot(d, d) + T(-1)
                                                            : (T(1) / L0) * vnorm(d) + T(-1);
        return 1;
    }
    default: return 0;
    }
}

// Effective compliance diagonal of a type-6..13 element (parameter layouts in spgx.h).
template <typename T>
SPGX_HD T generic_compliance(int type, const T *prm, int c)
{
    switch (type) {
    case SPGX_ENERGY_STVK:
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: return prm[11 + c];
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN: return prm[7 + c];
    case SPGX_ENERGY_MEMBRANE_CHOI: return prm[8 + c];
    case SPGX_ENERGY_QUADRATIC_BENDING: return prm[5];
    default: return prm[2];  // Baraff-Witkin bending, continuum springs
    }
}

// The block of one incidence of a type-6..14 energy at stencil positions p (relative to the
// solved vertex, p[slot] = 0).
template <typename T>
SPGX_HD SPGX_GENERIC_NOINLINE void generic_block(int type, const Vec3<T> *p, int slot, const T *prm, Block<T> &b)
{
    using Q = V3A<T>;
    switch (type) {
    case SPGX_ENERGY_STVK:
        vertex_energy_block<T, 4>([prm](const Q *q) { return stvk_tet_energy(q, prm); }, p, slot, b);
        break;
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN:
        vertex_energy_block<T, 4>([prm](const Q *q) { return ssnh_energy(q, prm); }, p, slot, b);
        break;
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING:
        vertex_energy_block<T, 4>([prm](const Q *q) { return bw_bending_energy(q, prm); }, p, slot, b);
        break;
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN:
        vertex_energy_block<T, 3>([prm](const Q *q) { return bw_membrane_energy(q, prm, false); }, p, slot, b);
        break;
    case SPGX_ENERGY_MEMBRANE_CHOI:
        vertex_energy_block<T, 3>([prm](const Q *q) { return bw_membrane_energy(q, prm, true); }, p, slot, b);
        break;
    case SPGX_ENERGY_QUADRATIC_BENDING: quadratic_bending_block(p, slot, prm, b); break;
    case SPGX_ENERGY_SPRING_CONTINUUM:
        vertex_energy_block<T, 2>([prm](const Q *q) { return continuum_spring_energy(q, prm, false); }, p, slot, b);
        break;
    case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM:
        vertex_energy_block<T, 2>([prm](const Q *q) { return continuum_spring_energy(q, prm, true); }, p, slot, b);
        break;
    case SPGX_ENERGY_STATIC_LOAD: static_load_block(prm, b); break;
    default: break;
    }
}

}  // namespace spgx
