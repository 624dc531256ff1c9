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

// Value, gradient and Hessian (xx, xy, xz, yy, yz, zz) with respect to one vertex.
template <typename T>
struct VAD {
    T v, g[3], h[6];
};

template <typename T>
SPGX_HD VAD<T> vconst(T x)
{
    VAD<T> r;
    r.v = x;
#pragma unroll
    for (int i = 0; i < 3; ++i) r.g[i] = T(0);
#pragma unroll
    for (int i = 0; i < 6; ++i) r.h[i] = T(0);
    return r;
}

template <typename T>
SPGX_HD VAD<T> operator+(const VAD<T> &a, const VAD<T> &b)
{
    VAD<T> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < 3; ++i) r.g[i] = a.g[i] + b.g[i];
#pragma unroll
    for (int i = 0; i < 6; ++i) r.h[i] = a.h[i] + b.h[i];
    return r;
}

template <typename T>
SPGX_HD VAD<T> operator-(const VAD<T> &a, const VAD<T> &b)
{
    VAD<T> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < 3; ++i) r.g[i] = a.g[i] - b.g[i];
#pragma unroll
    for (int i = 0; i < 6; ++i) r.h[i] = a.h[i] - b.h[i];
    return r;
}

template <typename T>
SPGX_HD VAD<T> operator-(const VAD<T> &a)
{
    VAD<T> r;
    r.v = -a.v;
#pragma unroll
    for (int i = 0; i < 3; ++i) r.g[i] = -a.g[i];
#pragma unroll
    for (int i = 0; i < 6; ++i) r.h[i] = -a.h[i];
    return r;
}

template <typename T>
SPGX_HD VAD<T> operator*(T s, const VAD<T> &a)
{
    VAD<T> r;
    r.v = s * a.v;
#pragma unroll
    for (int i = 0; i < 3; ++i) r.g[i] = s * a.g[i];
#pragma unroll
    for (int i = 0; i < 6; ++i) r.h[i] = s * a.h[i];
    return r;
}

template <typename T>
SPGX_HD VAD<T> operator+(const VAD<T> &a, T s)
{
    VAD<T> r = a;
    r.v = a.v + s;
    return r;
}

template <typename T>
SPGX_HD VAD<T> operator*(const VAD<T> &a, const VAD<T> &b)
{
    VAD<T> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < 3; ++i) r.g[i] = a.v * b.g[i] + b.v * a.g[i];
    const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int k = 0; k < 6; ++k)
        r.h[k] = a.v * b.h[k] + b.v * a.h[k] + a.g[I[k]] * b.g[J[k]] + a.g[J[k]] * b.g[I[k]];
    return r;
}

// f(a) for a scalar function with derivatives d1 = f'(a.v), d2 = f''(a.v).
template <typename T>
SPGX_HD VAD<T> chain(const VAD<T> &a, T f, T d1, T d2)
{
    VAD<T> r;
    r.v = f;
#pragma unroll
    for (int i = 0; i < 3; ++i) r.g[i] = d1 * a.g[i];
    const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int k = 0; k < 6; ++k) r.h[k] = d1 * a.h[k] + d2 * a.g[I[k]] * a.g[J[k]];
    return r;
}

template <typename T>
SPGX_HD VAD<T> vsqrt(const VAD<T> &a)
{
    const T s = sqrt(a.v);
    const T d1 = T(0.5) / s;
    return chain(a, s, d1, -d1 / (T(2) * a.v));
}

template <typename T>
SPGX_HD VAD<T> vrecip(const VAD<T> &a)
{
    const T r = T(1) / a.v;
    return chain(a, r, -r * r, T(2) * r * r * r);
}

// atan2(y, x) through its partial derivatives: d/dy = x / q, d/dx = -y / q (q = x^2 + y^2).
template <typename T>
SPGX_HD VAD<T> vatan2(const VAD<T> &y, const VAD<T> &x)
{
    const T q = x.v * x.v + y.v * y.v;
    const T iq = T(1) / q;
    const T ay = x.v * iq, ax = -y.v * iq;                // first partials
    const T iq2 = iq * iq;
    const T ayy = -T(2) * x.v * y.v * iq2;                 // d2/dy2
    const T axx = T(2) * x.v * y.v * iq2;                  // d2/dx2
    const T axy = (y.v * y.v - x.v * x.v) * iq2;           // d2/dxdy
    VAD<T> r;
    r.v = atan2(y.v, x.v);
#pragma unroll
    for (int i = 0; i < 3; ++i) r.g[i] = ay * y.g[i] + ax * x.g[i];
    const int I[6] = {0, 0, 0, 1, 1, 2}, J[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int k = 0; k < 6; ++k)
        r.h[k] = ay * y.h[k] + ax * x.h[k] + ayy * y.g[I[k]] * y.g[J[k]] + axx * x.g[I[k]] * x.g[J[k]] +
                 axy * (x.g[I[k]] * y.g[J[k]] + y.g[I[k]] * x.g[J[k]]);
    return r;
}

template <typename T>
struct V3A {
    VAD<T> x, y, z;
};

template <typename T>
SPGX_HD V3A<T> vsub(const V3A<T> &a, const V3A<T> &b)
{
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
SPGX_HD V3A<T> vadd(const V3A<T> &a, const V3A<T> &b)
{
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename T>
SPGX_HD V3A<T> vscale(T s, const V3A<T> &a)
{
    return {s * a.x, s * a.y, s * a.z};
}
template <typename T>
SPGX_HD VAD<T> vdot(const V3A<T> &a, const V3A<T> &b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
SPGX_HD V3A<T> vcross(const V3A<T> &a, const V3A<T> &b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T>
SPGX_HD VAD<T> vnorm(const V3A<T> &a)
{
    return vsqrt(vdot(a, a));
}

// Positions as differentiable vectors: the vertex at `slot` is the variable (at the origin:
// positions are relative to it), the others constants.
template <typename T, int S>
SPGX_HD void seed_positions(const Vec3<T> *p, int slot, V3A<T> *q)
{
#pragma unroll
    for (int j = 0; j < S; ++j) {
        q[j].x = vconst(p[j].x);
        q[j].y = vconst(p[j].y);
        q[j].z = vconst(p[j].z);
        if (j == slot) {
            q[j].x.g[0] = T(1);
            q[j].y.g[1] = T(1);
            q[j].z.g[2] = T(1);
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
template <typename T, int N>
SPGX_HD void deformation_columns(const V3A<T> *q, const T *D, V3A<T> *f)
{
    V3A<T> d[N];
#pragma unroll
    for (int j = 0; j < N; ++j) d[j] = vsub(q[j + 1], q[0]);
#pragma unroll
    for (int c = 0; c < N; ++c) {
        f[c] = vscale(D[c], d[0]);
#pragma unroll
        for (int j = 1; j < N; ++j) f[c] = vadd(f[c], vscale(D[j * N + c], d[j]));
    }
}

template <typename T>
SPGX_HD VAD<T> half_k_sq(T k, const VAD<T> &c)
{
    return (T(0.5) * k) * (c * c);
}

template <typename T>
SPGX_HD void stvk_tet_generic(const Vec3<T> *p, int slot, const T *prm, Block<T> &b)
{
    V3A<T> q[4], f[3];
    seed_positions<T, 4>(p, slot, q);
    deformation_columns<T, 3>(q, prm, f);
    const T lambda = prm[9], mu = prm[10];
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
    add_vad(b, (T(0.5) * lambda) * (tr * tr) + mu * sq);
}

template <typename T>
SPGX_HD void ssnh_generic(const Vec3<T> *p, int slot, const T *prm, Block<T> &b)
{
    V3A<T> q[4], f[3];
    seed_positions<T, 4>(p, slot, q);
    deformation_columns<T, 3>(q, prm, f);
    const VAD<T> J = vdot(f[0], vcross(f[1], f[2])) + T(-1);
    const VAD<T> I = vdot(f[0], f[0]) + vdot(f[1], f[1]) + vdot(f[2], f[2]) + T(-3);
    add_vad(b, half_k_sq(prm[9], J) + half_k_sq(prm[10], I));
}

template <typename T>
SPGX_HD void bw_membrane_generic(const Vec3<T> *p, int slot, const T *prm, Block<T> &b, bool choi)
{
    V3A<T> q[3], f[2];
    seed_positions<T, 3>(p, slot, q);
    deformation_columns<T, 2>(q, prm, f);
    VAD<T> E = half_k_sq(prm[4], vnorm(f[0]) + T(-1)) + half_k_sq(prm[5], vnorm(f[1]) + T(-1));
    if (!choi) {
        E = E + half_k_sq(prm[6], vdot(f[0], f[1]));
    } else {
        const T s = T(0.70710678118654752440);
        E = E + half_k_sq(prm[6], vnorm(vscale(s, vadd(f[0], f[1]))) + T(-1));
        E = E + half_k_sq(prm[7], vnorm(vscale(s, vsub(f[0], f[1]))) + T(-1));
    }
    add_vad(b, E);
}

template <typename T>
SPGX_HD void bw_bending_generic(const Vec3<T> *p, int slot, const T *prm, Block<T> &b)
{
    V3A<T> q[4];
    seed_positions<T, 4>(p, slot, q);
    const V3A<T> e0 = vsub(q[1], q[0]), e3 = vsub(q[2], q[1]), e4 = vsub(q[3], q[1]);
    // The norms are held constant (their values only), as the reference does with .val.
    const T e0i = T(1) / sqrt(vdot(e0, e0).v);
    const V3A<T> n1 = vcross(e0, e3);
    const V3A<T> n2 = vscale(T(-1), vcross(e0, e4));
    const T n1i = T(1) / sqrt(vdot(n1, n1).v);
    const T n2i = T(1) / sqrt(vdot(n2, n2).v);
    const V3A<T> a = vscale(n1i, n1), c = vscale(n2i, n2);
    const VAD<T> th = vatan2(vdot(vcross(a, c), vscale(e0i, e0)), vdot(a, c));
    add_vad(b, half_k_sq(prm[1], th + (-prm[0])));
}

template <typename T>
SPGX_HD void continuum_spring_generic(const Vec3<T> *p, int slot, const T *prm, Block<T> &b, bool squared)
{
    V3A<T> q[2];
    seed_positions<T, 2>(p, slot, q);
    const V3A<T> d = vsub(q[0], q[1]);
    const T L0 = prm[0];
    const VAD<T> C = squared ? (T(1) / (L0 * L0)) * vdot(d, d) + T(-1) : (T(1) / L0) * vnorm(d) + T(-1);
    add_vad(b, half_k_sq(prm[1], C));
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
SPGX_HD int generic_constraints(int type, const Vec3<T> *p, int slot, const T *prm, VAD<T> *C)
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
SPGX_HD void generic_block(int type, const Vec3<T> *p, int slot, const T *prm, Block<T> &b)
{
    switch (type) {
    case SPGX_ENERGY_STVK: stvk_tet_generic(p, slot, prm, b); break;
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: ssnh_generic(p, slot, prm, b); break;
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN: bw_membrane_generic(p, slot, prm, b, false); break;
    case SPGX_ENERGY_MEMBRANE_CHOI: bw_membrane_generic(p, slot, prm, b, true); break;
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING: bw_bending_generic(p, slot, prm, b); break;
    case SPGX_ENERGY_QUADRATIC_BENDING: quadratic_bending_block(p, slot, prm, b); break;
    case SPGX_ENERGY_SPRING_CONTINUUM: continuum_spring_generic(p, slot, prm, b, false); break;
    case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM: continuum_spring_generic(p, slot, prm, b, true); break;
    case SPGX_ENERGY_STATIC_LOAD: static_load_block(prm, b); break;
    default: break;
    }
}

}  // namespace spgx
