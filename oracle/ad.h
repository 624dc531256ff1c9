// ORACLE — test infrastructure only. Nothing in the shipped library links this file.
//
// Forward-mode automatic differentiation scalar, a restatement of the semantics of
// TinyAD::Scalar<N, double, hess> (github.com/patr-schm/TinyAD; the submodule pin is not
// recorded in the reference checkout, so no version can be named). The reference seeds one
// scalar per degree of freedom (`RealT(x0p.x(), 0)`, e.g. spg/source/sim/energy/
// membraneStvkEnergy.cpp:15-17) and reads `.val`, `.grad` and `.Hess` back
// (spg/include/spg/sim/energy/energy.h:264-266, 348-362).
//
// Each value carries its gradient over N seeded variables and, when Hess is true, the dense
// N x N Hessian. Every operation applies the first- and second-order chain rule.
#pragma once

#include <array>
#include <cmath>
#include <type_traits>

namespace oracle {

template <int N, bool Hess>
struct Dual {
    static constexpr int kN = N;
    double val{0};
    std::array<double, N> grad{};
    std::array<double, Hess ? N * N : 1> hess{};

    Dual() = default;
    Dual(double v) : val(v) {}  // NOLINT: implicit constant promotion like TinyAD
    Dual(double v, int idx) : val(v) { grad[idx] = 1.0; }

    double &H(int i, int j) { return hess[i * N + j]; }
    double H(int i, int j) const { return hess[i * N + j]; }
};

// Unary chain rule: r = f(a) with first derivative d1 and second derivative d2 at a.val.
template <int N, bool Hs>
inline Dual<N, Hs> chain1(const Dual<N, Hs> &a, double fval, double d1, double d2)
{
    Dual<N, Hs> r;
    r.val = fval;
    for (int i = 0; i < N; ++i) r.grad[i] = d1 * a.grad[i];
    if constexpr (Hs) {
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) r.H(i, j) = d1 * a.H(i, j) + d2 * a.grad[i] * a.grad[j];
    }
    return r;
}

template <int N, bool Hs>
inline Dual<N, Hs> operator+(const Dual<N, Hs> &a, const Dual<N, Hs> &b)
{
    Dual<N, Hs> r;
    r.val = a.val + b.val;
    for (int i = 0; i < N; ++i) r.grad[i] = a.grad[i] + b.grad[i];
    if constexpr (Hs)
        for (int i = 0; i < N * N; ++i) r.hess[i] = a.hess[i] + b.hess[i];
    return r;
}

template <int N, bool Hs>
inline Dual<N, Hs> operator-(const Dual<N, Hs> &a, const Dual<N, Hs> &b)
{
    Dual<N, Hs> r;
    r.val = a.val - b.val;
    for (int i = 0; i < N; ++i) r.grad[i] = a.grad[i] - b.grad[i];
    if constexpr (Hs)
        for (int i = 0; i < N * N; ++i) r.hess[i] = a.hess[i] - b.hess[i];
    return r;
}

template <int N, bool Hs>
inline Dual<N, Hs> operator-(const Dual<N, Hs> &a)
{
    Dual<N, Hs> r;
    r.val = -a.val;
    for (int i = 0; i < N; ++i) r.grad[i] = -a.grad[i];
    if constexpr (Hs)
        for (int i = 0; i < N * N; ++i) r.hess[i] = -a.hess[i];
    return r;
}

template <int N, bool Hs>
inline Dual<N, Hs> operator*(const Dual<N, Hs> &a, const Dual<N, Hs> &b)
{
    Dual<N, Hs> r;
    r.val = a.val * b.val;
    for (int i = 0; i < N; ++i) r.grad[i] = a.val * b.grad[i] + b.val * a.grad[i];
    if constexpr (Hs) {
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                r.H(i, j) = a.val * b.H(i, j) + b.val * a.H(i, j) + a.grad[i] * b.grad[j] + b.grad[i] * a.grad[j];
    }
    return r;
}

template <int N, bool Hs>
inline Dual<N, Hs> operator*(double s, const Dual<N, Hs> &a)
{
    Dual<N, Hs> r;
    r.val = s * a.val;
    for (int i = 0; i < N; ++i) r.grad[i] = s * a.grad[i];
    if constexpr (Hs)
        for (int i = 0; i < N * N; ++i) r.hess[i] = s * a.hess[i];
    return r;
}
template <int N, bool Hs>
inline Dual<N, Hs> operator*(const Dual<N, Hs> &a, double s)
{
    return s * a;
}

template <int N, bool Hs>
inline Dual<N, Hs> operator/(const Dual<N, Hs> &a, const Dual<N, Hs> &b)
{
    const double inv = 1.0 / b.val;
    return a * chain1(b, inv, -inv * inv, 2.0 * inv * inv * inv);
}
template <int N, bool Hs>
inline Dual<N, Hs> operator/(const Dual<N, Hs> &a, double s)
{
    return (1.0 / s) * a;
}

template <int N, bool Hs>
inline Dual<N, Hs> operator+(const Dual<N, Hs> &a, double s)
{
    Dual<N, Hs> r = a;
    r.val += s;
    return r;
}
template <int N, bool Hs>
inline Dual<N, Hs> operator-(const Dual<N, Hs> &a, double s)
{
    Dual<N, Hs> r = a;
    r.val -= s;
    return r;
}

template <int N, bool Hs>
inline Dual<N, Hs> sqrt(const Dual<N, Hs> &a)
{
    const double s = std::sqrt(a.val);
    return chain1(a, s, 0.5 / s, -0.25 / (s * a.val));
}

// atan2(y, x) with the two-argument chain rule.
template <int N, bool Hs>
inline Dual<N, Hs> atan2(const Dual<N, Hs> &y, const Dual<N, Hs> &x)
{
    Dual<N, Hs> r;
    const double r2 = x.val * x.val + y.val * y.val;
    r.val = std::atan2(y.val, x.val);
    const double fy = x.val / r2;
    const double fx = -y.val / r2;
    for (int i = 0; i < N; ++i) r.grad[i] = fy * y.grad[i] + fx * x.grad[i];
    if constexpr (Hs) {
        const double r4 = r2 * r2;
        const double fyy = -2.0 * x.val * y.val / r4;
        const double fxx = 2.0 * x.val * y.val / r4;
        const double fxy = (y.val * y.val - x.val * x.val) / r4;
        for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j)
                r.H(i, j) = fy * y.H(i, j) + fx * x.H(i, j) + fyy * y.grad[i] * y.grad[j] +
                            fxx * x.grad[i] * x.grad[j] + fxy * (x.grad[i] * y.grad[j] + y.grad[i] * x.grad[j]);
    }
    return r;
}

// Plain-double overloads so templated energy code can be instantiated on double.
inline double sqrt(double a) { return std::sqrt(a); }
// The value of a scalar with its derivatives dropped (TinyAD's `.val`).
inline double value_of(double a) { return a; }
template <int N, bool Hs>
inline double value_of(const Dual<N, Hs> &a)
{
    return a.val;
}
inline double atan2(double y, double x) { return std::atan2(y, x); }

template <typename T>
inline double value_of(const T &a)
{
    if constexpr (std::is_same_v<T, double>)
        return a;
    else
        return a.val;
}

// Minimal fixed 3-vector over any scalar, with the Eigen operations the reference uses
// (cross, dot, norm, normalized, squaredNorm).
template <typename T>
struct V3 {
    T c[3];
    V3() : c{T(0.0), T(0.0), T(0.0)} {}
    V3(const T &a, const T &b, const T &d) : c{a, b, d} {}
    T &operator[](int i) { return c[i]; }
    const T &operator[](int i) const { return c[i]; }
};

template <typename T>
inline V3<T> operator+(const V3<T> &a, const V3<T> &b)
{
    return {a[0] + b[0], a[1] + b[1], a[2] + b[2]};
}
template <typename T>
inline V3<T> operator-(const V3<T> &a, const V3<T> &b)
{
    return {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
}
template <typename T>
inline V3<T> operator-(const V3<T> &a)
{
    return {-a[0], -a[1], -a[2]};
}
template <typename T, typename S>
inline V3<T> scale(const V3<T> &a, const S &s)
{
    return {a[0] * s, a[1] * s, a[2] * s};
}
template <typename T>
inline T dot(const V3<T> &a, const V3<T> &b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
template <typename T>
inline V3<T> cross(const V3<T> &a, const V3<T> &b)
{
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
template <typename T>
inline T squaredNorm(const V3<T> &a)
{
    return dot(a, a);
}
template <typename T>
inline T norm(const V3<T> &a)
{
    using oracle::sqrt;
    return sqrt(squaredNorm(a));
}
template <typename T>
inline V3<T> normalized(const V3<T> &a)
{
    const T n = norm(a);
    return {a[0] / n, a[1] / n, a[2] / n};
}

}  // namespace oracle
