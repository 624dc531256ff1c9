// ORACLE — test infrastructure only. Nothing in the shipped library links this file.
//
// FP64 restatement of the five particle energies on SPG's VBD/XPBD hot path, written as
// scalar-generic functions so they can be evaluated on double or on the forward-mode AD
// scalar of ad.h (the reference evaluates them on TinyAD scalars). Parameter packing per
// stencil (the reference's precomputed per-stencil data, in the order the C ABI uses):
//   SPRING   [L0, k, compliance]                       springEnergy.cpp:33-46
//   ANCHOR   [ax, ay, az, k, compliance]               springAnchorEnergy.cpp:29-39
//   BENDING  [theta0, k_eff, compliance_eff]           discreteBendingEnergy.cpp:33-72
//   STVK     [Dinv(2x2 row-major), K(3x3), Cmp(3x3)]   membraneStvkEnergy.cpp:31-71
//   SNH      [Dinv(3x3 row-major), lambda_v, mu_v, alpha, cmp_lambda, cmp_mu]
//                                                      stableNeoHookeanEnergy.cpp:64-108
// and the nine further particle energies (types 6-14), with diagonal stiffness matrices:
//   STVK_TET [Dinv(3x3), lambda V, mu V, cmp(0,0), cmp(1,1)]   stvkEnergy.cpp:61-108
//   SSNH     [Dinv(3x3), lambda V, mu V, cmp(0,0), cmp(1,1)]   stableSquaredNeoHookeanEnergy.cpp:33-75
//   BW_MEMB  [Dinv(2x2), k diag(3), cmp diag(3)]               membraneBaraffWitkinEnergy.cpp:28-70
//   CHOI     [Dinv(2x2), k diag(4), cmp diag(4)]               membraneChoiEnergy.cpp:31-73
//   BW_BEND  [theta0, k, cmp]                                  baraffWitkinBendingEnergy.cpp:40-76
//   QBEND    [c0, c1, c2, c3, k, cmp]                          quadraticBendingEnergy.cpp:32-93
//   SPRING_C, SPRING_SQ_C [L0, k L0, cmp]                      springContinuumEnergy.cpp:19-34
//   LOAD     [k, dx, dy, dz]                                   staticLoadEnergy.h (addStencil)
#pragma once

#include "ad.h"

namespace oracle {

enum EnergyType {
    kSpring = 1,
    kAnchor = 2,
    kBending = 3,
    kStvk = 4,
    kSnh = 5,
    kStvkTet = 6,
    kSsnh = 7,
    kBwMembrane = 8,
    kChoi = 9,
    kBwBending = 10,
    kQuadBending = 11,
    kSpringCont = 12,
    kSpringSqCont = 13,
    kStaticLoad = 14
};

inline int stencil_size(int type)
{
    switch (type) {
    case kSpring: return 2;
    case kAnchor: return 1;
    case kBending: return 4;
    case kStvk: return 3;
    case kSnh: return 4;
    case kStvkTet: return 4;
    case kSsnh: return 4;
    case kBwMembrane: return 3;
    case kChoi: return 3;
    case kBwBending: return 4;
    case kQuadBending: return 4;
    case kSpringCont: return 2;
    case kSpringSqCont: return 2;
    case kStaticLoad: return 1;
    default: return 0;
    }
}

inline int param_count(int type)
{
    switch (type) {
    case kSpring: return 3;
    case kAnchor: return 5;
    case kBending: return 3;
    case kStvk: return 22;
    case kSnh: return 14;
    case kStvkTet: return 13;
    case kSsnh: return 13;
    case kBwMembrane: return 10;
    case kChoi: return 12;
    case kBwBending: return 3;
    case kQuadBending: return 6;
    case kSpringCont: return 3;
    case kSpringSqCont: return 3;
    case kStaticLoad: return 4;
    default: return 0;
    }
}

// ---------------------------------------------------------------------------------------
// StVK membrane: constraint lambda membraneStvkEnergy.cpp:9-28; energy = 1/2 C^T K C via the
// default StencilBlockEnergy::dEnergy (energy.h:336-347).
template <typename T>
inline void stvk_constraints(const V3<T> *x, const double *p, T *C)
{
    const V3<T> u = x[1] - x[0];
    const V3<T> v = x[2] - x[0];
    // F = [u v] * Dinv (3x2); Dinv row-major p[0..3]
    V3<T> f0, f1;
    for (int a = 0; a < 3; ++a) {
        f0[a] = u[a] * p[0] + v[a] * p[2];
        f1[a] = u[a] * p[1] + v[a] * p[3];
    }
    // E = 1/2 (F^T F - I)
    const T e00 = 0.5 * (dot(f0, f0) - 1.0);
    const T e11 = 0.5 * (dot(f1, f1) - 1.0);
    const T e01 = 0.5 * dot(f0, f1);
    C[0] = e00;
    C[1] = e11;
    C[2] = 2.0 * e01;
}

template <typename T>
inline T stvk_energy(const V3<T> *x, const double *p)
{
    T C[3];
    stvk_constraints(x, p, C);
    const double *K = p + 4;
    T e = T(0.0);
    for (int i = 0; i < 3; ++i) {
        T kc = K[i * 3 + 0] * C[0] + K[i * 3 + 1] * C[1] + K[i * 3 + 2] * C[2];
        e = e + C[i] * kc;
    }
    return 0.5 * e;
}

// ---------------------------------------------------------------------------------------
// Stable Neo-Hookean: energy lambda stableNeoHookeanEnergy.cpp:33-61 (used for VBD), and the
// constraint lambda :9-31 (used by the XPBD projection).
template <typename T>
inline void snh_deformation(const V3<T> *x, const double *D, T F[3][3])
{
    const V3<T> u = x[1] - x[0];
    const V3<T> v = x[2] - x[0];
    const V3<T> w = x[3] - x[0];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) F[a][b] = u[a] * D[0 * 3 + b] + v[a] * D[1 * 3 + b] + w[a] * D[2 * 3 + b];
}

template <typename T>
inline T det3(const T F[3][3])
{
    return F[0][0] * (F[1][1] * F[2][2] - F[1][2] * F[2][1]) - F[0][1] * (F[1][0] * F[2][2] - F[1][2] * F[2][0]) +
           F[0][2] * (F[1][0] * F[2][1] - F[1][1] * F[2][0]);
}

template <typename T>
inline T snh_energy(const V3<T> *x, const double *p)
{
    T F[3][3];
    snh_deformation(x, p, F);
    const double lambda = p[9], mu = p[10], alpha = p[11];
    const T hydro = det3(F) - alpha;
    T tr = T(0.0);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) tr = tr + F[a][b] * F[a][b];
    const T dev = tr - 3.0;
    return 0.5 * lambda * hydro * hydro + 0.5 * mu * dev;
}

template <typename T>
inline void snh_constraints(const V3<T> *x, const double *p, T *C)
{
    T F[3][3];
    snh_deformation(x, p, F);
    T tr = T(0.0);
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) tr = tr + F[a][b] * F[a][b];
    using oracle::sqrt;
    C[0] = det3(F) - p[11];
    C[1] = sqrt(tr);
}

// ---------------------------------------------------------------------------------------
// Discrete bending (Tamstorf 2013): constraint lambda discreteBendingEnergy.cpp:9-30; energy
// 1/2 k_eff C^2 via energy.h:336-347.
template <typename T>
inline T bending_constraint(const V3<T> *x, const double *p)
{
    const V3<T> e0 = x[1] - x[0];
    const V3<T> e3 = x[2] - x[1];
    const V3<T> e4 = x[3] - x[1];
    const V3<T> n1 = normalized(cross(e0, e3));
    const V3<T> n2 = -normalized(cross(e0, e4));
    using oracle::atan2;
    const T theta = atan2(dot(cross(n1, n2), normalized(e0)), dot(n1, n2));
    return theta - p[0];
}

template <typename T>
inline T bending_energy(const V3<T> *x, const double *p)
{
    const T c = bending_constraint(x, p);
    return 0.5 * (c * (p[1] * c));
}

// ---------------------------------------------------------------------------------------
// Spring anchor: energy lambda springAnchorEnergy.cpp:21-26 (uses the model stiffness);
// constraint lambda :8-19 with its zero-norm guard.
template <typename T>
inline T anchor_energy(const V3<T> *x, const double *p)
{
    const V3<T> a{T(p[0]), T(p[1]), T(p[2])};
    return 0.5 * p[3] * squaredNorm(x[0] - a);
}

template <typename T>
inline T anchor_constraint(const V3<T> *x, const double *p)
{
    const V3<T> a{T(p[0]), T(p[1]), T(p[2])};
    T c = norm(x[0] - a);
    if (value_of(c) == 0.0) c = T(0.0);
    return c;
}

// ---------------------------------------------------------------------------------------
// Spring: energy lambda springEnergy.cpp:20-30 (only used here for AD cross-checks; the
// reference overrides gradient/Hessian analytically, :101-133, restated in oracle.cpp).
template <typename T>
inline T spring_energy(const V3<T> *x, const double *p)
{
    const T d = norm(x[0] - x[1]) - p[0];
    return 0.5 * p[1] * d * d;
}

template <typename T>
inline T spring_constraint(const V3<T> *x, const double *p)
{
    return norm(x[0] - x[1]) - p[0];
}

// ---------------------------------------------------------------------------------------
// Types 6-14. Constraint energies use E = 1/2 C^T K C with the diagonal K of the params
// (StencilBlockEnergy::dEnergy, energy.h:336-347).

template <typename T>
inline void tet_columns(const V3<T> *x, const double *D, V3<T> f[3])
{
    const V3<T> u = x[1] - x[0], v = x[2] - x[0], w = x[3] - x[0];
    for (int c = 0; c < 3; ++c) f[c] = scale(u, D[c]) + scale(v, D[3 + c]) + scale(w, D[6 + c]);
}

template <typename T>
inline void tri_columns(const V3<T> *x, const double *D, V3<T> f[2])
{
    const V3<T> u = x[1] - x[0], v = x[2] - x[0];
    for (int c = 0; c < 2; ++c) f[c] = scale(u, D[c]) + scale(v, D[2 + c]);
}

template <typename T>
inline T constraint_energy(const T *C, const double *k, int n)
{
    T e = T(0.0);
    for (int i = 0; i < n; ++i) e = e + 0.5 * k[i] * C[i] * C[i];
    return e;
}

// StvkEnergy (tet), stvkEnergy.cpp:37-60: E = 1/2 lambda tr(G)^2 + mu tr(G^T G),
// G = 1/2 (F^T F - I), lambda and mu volume-weighted. Constraints (:9-35):
// [tr G, sqrt(2 tr(G G))], the second set to 0 when its value is 0.
template <typename T>
inline T stvk_tet_energy(const V3<T> *x, const double *p)
{
    V3<T> f[3];
    tet_columns(x, p, f);
    T tr = T(0.0), sq = T(0.0);
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            T G = 0.5 * dot(f[a], f[c]);
            if (a == c) G = G - 0.5;
            if (a == c) tr = tr + G;
            sq = sq + G * G;
        }
    return 0.5 * p[9] * tr * tr + p[10] * sq;
}

template <typename T>
inline void stvk_tet_constraints(const V3<T> *x, const double *p, T *C)
{
    V3<T> f[3];
    tet_columns(x, p, f);
    T tr = T(0.0), sq = T(0.0);
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            T G = 0.5 * dot(f[a], f[c]);
            if (a == c) G = G - 0.5;
            if (a == c) tr = tr + G;
            sq = sq + G * G;
        }
    C[0] = tr;
    C[1] = value_of(sq) == 0.0 ? T(0.0) : sqrt(2.0 * sq);
}

// StableSquaredNeoHookeanEnergy, stableSquaredNeoHookeanEnergy.cpp:9-31:
// C = [det F - 1, tr(F^T F) - 3].
template <typename T>
inline void ssnh_constraints(const V3<T> *x, const double *p, T *C)
{
    V3<T> f[3];
    tet_columns(x, p, f);
    C[0] = dot(f[0], cross(f[1], f[2])) - 1.0;
    C[1] = dot(f[0], f[0]) + dot(f[1], f[1]) + dot(f[2], f[2]) - 3.0;
}

template <typename T>
inline T ssnh_energy(const V3<T> *x, const double *p)
{
    T C[2];
    ssnh_constraints(x, p, C);
    return constraint_energy(C, p + 9, 2);
}

// MembraneBaraffWitkinEnergy, membraneBaraffWitkinEnergy.cpp:9-26: C = [|F0| - 1, |F1| - 1, F0.F1].
template <typename T>
inline void bw_membrane_constraints(const V3<T> *x, const double *p, T *C)
{
    V3<T> f[2];
    tri_columns(x, p, f);
    C[0] = norm(f[0]) - 1.0;
    C[1] = norm(f[1]) - 1.0;
    C[2] = dot(f[0], f[1]);
}

template <typename T>
inline T bw_membrane_energy(const V3<T> *x, const double *p)
{
    T C[3];
    bw_membrane_constraints(x, p, C);
    return constraint_energy(C, p + 4, 3);
}

// MembraneChoiEnergy, membraneChoiEnergy.cpp:9-29: stretch of the warp, weft and both
// diagonal directions.
template <typename T>
inline void choi_constraints(const V3<T> *x, const double *p, T *C)
{
    V3<T> f[2];
    tri_columns(x, p, f);
    const double s = 1.0 / std::sqrt(2.0);
    C[0] = norm(f[0]) - 1.0;
    C[1] = norm(f[1]) - 1.0;
    C[2] = norm(scale(f[0] + f[1], s)) - 1.0;
    C[3] = norm(scale(f[0] - f[1], s)) - 1.0;
}

template <typename T>
inline T choi_energy(const V3<T> *x, const double *p)
{
    T C[4];
    choi_constraints(x, p, C);
    return constraint_energy(C, p + 4, 4);
}

// BaraffWitkinBendingEnergy, baraffWitkinBendingEnergy.cpp:9-38: the dihedral angle with the
// edge and normal norms taken as constants (their values only).
template <typename T>
inline T bw_bending_constraint(const V3<T> *x, const double *p)
{
    const V3<T> e0 = x[1] - x[0], e3 = x[2] - x[1], e4 = x[3] - x[1];
    const double e0i = 1.0 / value_of(norm(e0));
    const V3<T> n1 = cross(e0, e3);
    const double n1i = 1.0 / value_of(norm(n1));
    const V3<T> n2 = -cross(e0, e4);
    const double n2i = 1.0 / value_of(norm(n2));
    const V3<T> a = scale(n1, n1i), c = scale(n2, n2i);
    return atan2(dot(cross(a, c), scale(e0, e0i)), dot(a, c)) - p[0];
}

template <typename T>
inline T bw_bending_energy(const V3<T> *x, const double *p)
{
    const T c = bw_bending_constraint(x, p);
    return 0.5 * p[1] * c * c;
}

// QuadraticBendingEnergy, quadraticBendingEnergy.cpp:9-30: C = L x with the 3x12 Laplacian
// L = [c0 I, c1 I, c2 I, c3 I]; E = 1/2 k |C|^2 (K = k I).
template <typename T>
inline void quad_bending_constraints(const V3<T> *x, const double *p, T *C)
{
    const V3<T> s = scale(x[0], p[0]) + scale(x[1], p[1]) + scale(x[2], p[2]) + scale(x[3], p[3]);
    C[0] = s[0];
    C[1] = s[1];
    C[2] = s[2];
}

template <typename T>
inline T quad_bending_energy(const V3<T> *x, const double *p)
{
    T C[3];
    quad_bending_constraints(x, p, C);
    const double k[3] = {p[4], p[4], p[4]};
    return constraint_energy(C, k, 3);
}

// SpringContinuumEnergy (springContinuumEnergy.cpp:8-17) and SpringSquaredContinuumEnergy
// (springSquaredContinuumEnergy.cpp:8-17).
template <typename T>
inline T spring_cont_constraint(const V3<T> *x, const double *p)
{
    return norm(x[0] - x[1]) / p[0] - 1.0;
}

template <typename T>
inline T spring_sq_cont_constraint(const V3<T> *x, const double *p)
{
    return squaredNorm(x[0] - x[1]) / (p[0] * p[0]) - 1.0;
}

template <typename T>
inline T spring_cont_energy(const V3<T> *x, const double *p)
{
    const T c = spring_cont_constraint(x, p);
    return 0.5 * p[1] * c * c;
}

template <typename T>
inline T spring_sq_cont_energy(const V3<T> *x, const double *p)
{
    const T c = spring_sq_cont_constraint(x, p);
    return 0.5 * p[1] * c * c;
}

// StaticLoadEnergy, staticLoadEnergy.cpp:17-23: E = k * -(d . x).
template <typename T>
inline T static_load_energy(const V3<T> *x, const double *p)
{
    return p[0] * -(p[1] * x[0][0] + p[2] * x[0][1] + p[3] * x[0][2]);
}

}  // namespace oracle
