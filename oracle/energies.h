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
#pragma once

#include "ad.h"

namespace oracle {

enum EnergyType { kSpring = 1, kAnchor = 2, kBending = 3, kStvk = 4, kSnh = 5 };

inline int stencil_size(int type)
{
    switch (type) {
    case kSpring: return 2;
    case kAnchor: return 1;
    case kBending: return 4;
    case kStvk: return 3;
    case kSnh: return 4;
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

}  // namespace oracle
