// Eigen-free stand-ins for the small fixed-size types of spg/include/spg/types.h:8-39, with
// the operations the hot-path energies and scene builders use. Real is double as in the
// reference.
#pragma once

#include <array>
#include <cmath>

namespace spg {

using Real = double;
using Int2 = std::array<int, 2>;
using Int3 = std::array<int, 3>;
using Int4 = std::array<int, 4>;

struct Vector3 {
    Real v[3]{0, 0, 0};
    Vector3() = default;
    Vector3(Real a, Real b, Real c) : v{a, b, c} {}
    Real &operator[](int i) { return v[i]; }
    Real operator[](int i) const { return v[i]; }
    Real x() const { return v[0]; }
    Real y() const { return v[1]; }
    Real z() const { return v[2]; }
    Vector3 operator+(const Vector3 &o) const { return {v[0] + o.v[0], v[1] + o.v[1], v[2] + o.v[2]}; }
    Vector3 operator-(const Vector3 &o) const { return {v[0] - o.v[0], v[1] - o.v[1], v[2] - o.v[2]}; }
    Vector3 operator-() const { return {-v[0], -v[1], -v[2]}; }
    Vector3 operator*(Real s) const { return {v[0] * s, v[1] * s, v[2] * s}; }
    Vector3 operator/(Real s) const { return {v[0] / s, v[1] / s, v[2] / s}; }
    Vector3 &operator+=(const Vector3 &o)
    {
        for (int i = 0; i < 3; ++i) v[i] += o.v[i];
        return *this;
    }
    Real dot(const Vector3 &o) const { return v[0] * o.v[0] + v[1] * o.v[1] + v[2] * o.v[2]; }
    Vector3 cross(const Vector3 &o) const
    {
        return {v[1] * o.v[2] - v[2] * o.v[1], v[2] * o.v[0] - v[0] * o.v[2], v[0] * o.v[1] - v[1] * o.v[0]};
    }
    Real squaredNorm() const { return dot(*this); }
    Real norm() const { return std::sqrt(squaredNorm()); }
    Vector3 normalized() const { return *this / norm(); }
    static Vector3 Zero() { return {}; }
};

inline Vector3 operator*(Real s, const Vector3 &a) { return a * s; }

// Row-major fixed matrix with the closed-form inverse / determinant the energies need.
template <int R, int C = R>
struct Matrix {
    Real m[R * C]{};
    Real &operator()(int i, int j) { return m[i * C + j]; }
    Real operator()(int i, int j) const { return m[i * C + j]; }
};
using Matrix1 = Matrix<1>;
using Matrix2 = Matrix<2>;
using Matrix3 = Matrix<3>;

inline Real determinant(const Matrix3 &A)
{
    return A(0, 0) * (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) - A(0, 1) * (A(1, 0) * A(2, 2) - A(1, 2) * A(2, 0)) +
           A(0, 2) * (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0));
}

inline Matrix3 inverse(const Matrix3 &A)
{
    Matrix3 I;
    const Real c00 = A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1);
    const Real c01 = A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2);
    const Real c02 = A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0);
    const Real id = 1.0 / (A(0, 0) * c00 + A(0, 1) * c01 + A(0, 2) * c02);
    I(0, 0) = c00 * id;
    I(0, 1) = (A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2)) * id;
    I(0, 2) = (A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1)) * id;
    I(1, 0) = c01 * id;
    I(1, 1) = (A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0)) * id;
    I(1, 2) = (A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2)) * id;
    I(2, 0) = c02 * id;
    I(2, 1) = (A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1)) * id;
    I(2, 2) = (A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0)) * id;
    return I;
}

inline Matrix2 inverse(const Matrix2 &A)
{
    Matrix2 I;
    const Real det = A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0);
    I(0, 0) = A(1, 1) / det;
    I(0, 1) = -A(0, 1) / det;
    I(1, 0) = -A(1, 0) / det;
    I(1, 1) = A(0, 0) / det;
    return I;
}

enum class Verbosity { None, Performance, Debug };

}  // namespace spg
