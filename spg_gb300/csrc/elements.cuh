// Hand-derived per-vertex gradient segments and 3x3 Hessian blocks of the five energies on
// SPG's VBD hot path, and the constraint gradients its XPBD projection needs.
//
// The reference obtains these by forward-mode AD of the whole element and then keeps one
// block (StencilBlockEnergy::accumulateVertexForce / accumulateVertexHessian,
// spg/include/spg/sim/energy/energy.h:240-258; no PSD projection, :354-361). Here each block
// is written in closed form for the one vertex that needs it. The functions are templates on
// the scalar so the solver runs them in FP32 while a CPU check instantiates them in FP64.
//
// Block convention: f accumulates the force -dE/dx_v, h the symmetric Hessian block
// (h[0..5] = H00 H01 H02 H11 H12 H22).
#pragma once

#if defined(__CUDACC__)
#define SPGX_HD __host__ __device__ __forceinline__
#else
#define SPGX_HD inline
#endif

#include <math.h>

namespace spgx {

template <typename T>
struct Vec3 {
    T x, y, z;
};

template <typename T>
SPGX_HD Vec3<T> mk(T a, T b, T c)
{
    Vec3<T> r;
    r.x = a;
    r.y = b;
    r.z = c;
    return r;
}
template <typename T>
SPGX_HD Vec3<T> operator+(Vec3<T> a, Vec3<T> b)
{
    return mk(a.x + b.x, a.y + b.y, a.z + b.z);
}
template <typename T>
SPGX_HD Vec3<T> operator-(Vec3<T> a, Vec3<T> b)
{
    return mk(a.x - b.x, a.y - b.y, a.z - b.z);
}
template <typename T>
SPGX_HD Vec3<T> operator*(T s, Vec3<T> a)
{
    return mk(s * a.x, s * a.y, s * a.z);
}
template <typename T>
SPGX_HD T dot(Vec3<T> a, Vec3<T> b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
SPGX_HD Vec3<T> cross(Vec3<T> a, Vec3<T> b)
{
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

SPGX_HD float sq_root(float a) { return sqrtf(a); }
SPGX_HD double sq_root(double a) { return sqrt(a); }
// 1/x and 1/sqrt(x). On the device the FP32 forms use the hardware's approximate reciprocal
// (PTX rcp.approx.f32, within 1 ulp) and reciprocal square root (about 2 ulp): single
// instructions instead of rounding sequences in the element blocks' dependency chains. The CPU
// instantiations keep plain division.
SPGX_HD float recip(float a)
{
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
#else
    return 1.f / a;
#endif
}
SPGX_HD double recip(double a) { return 1.0 / a; }
SPGX_HD float rsqrt_of(float a)
{
#if defined(__CUDA_ARCH__)
    return rsqrtf(a);
#else
    return 1.f / sqrtf(a);
#endif
}
SPGX_HD double rsqrt_of(double a) { return 1.0 / sqrt(a); }
// FP32 atan2 on the device: t = min(|x|, |y|) / max(|x|, |y|) in [0, 1], atan(t) = t P(t^2)
// with P the degree-8 minimax polynomial in relative error (Remez exchange; atan_poly_fit.py
// beside this file fits it: 2 ulp in FP32 Horner form), then the octant is restored:
// pi/2 - r when |y| > |x|, pi - r when x is negative (or -0), and the sign of y. Finite
// arguments only, as the hinge angles of non-degenerate triangles are; atan2(+-0, +0) = +-0
// and atan2(+-0, -0) = +-pi as in C.
SPGX_HD float arctan2(float y, float x)
{
#if defined(__CUDA_ARCH__)
    const float ax = fabsf(x), ay = fabsf(y);
    const float hi = fmaxf(ax, ay), lo = fminf(ax, ay);
    const float t = hi > 0.f ? lo * recip(hi) : 0.f;
    const float s = t * t;
    float p = 0.002849889686331153f;
    p = fmaf(p, s, -0.016068629920482635f);
    p = fmaf(p, s, 0.04269152134656906f);
    p = fmaf(p, s, -0.07504294812679291f);
    p = fmaf(p, s, 0.10640934109687805f);
    p = fmaf(p, s, -0.14203643798828125f);
    p = fmaf(p, s, 0.1999261975288391f);
    p = fmaf(p, s, -0.3333307206630707f);
    p = fmaf(p, s, 1.0f);
    float r = t * p;
    if (ay > ax) r = 1.5707963267948966f - r;
    if (signbit(x)) r = 3.141592653589793f - r;
    return copysignf(r, y);
#else
    return atan2f(y, x);
#endif
}
SPGX_HD double arctan2(double y, double x) { return atan2(y, x); }

template <typename T>
struct Block {
    T f[3];
    T h[6];
};

template <typename T>
SPGX_HD void block_zero(Block<T> &b)
{
    for (int i = 0; i < 3; ++i) b.f[i] = T(0);
    for (int i = 0; i < 6; ++i) b.h[i] = T(0);
}

// f -= s * g
template <typename T>
SPGX_HD void sub_force(Block<T> &b, Vec3<T> g, T s)
{
    b.f[0] -= s * g.x;
    b.f[1] -= s * g.y;
    b.f[2] -= s * g.z;
}
// h += s * u u^T
template <typename T>
SPGX_HD void add_outer(Block<T> &b, Vec3<T> u, T s)
{
    const Vec3<T> su = s * u;
    b.h[0] += su.x * u.x;
    b.h[1] += su.x * u.y;
    b.h[2] += su.x * u.z;
    b.h[3] += su.y * u.y;
    b.h[4] += su.y * u.z;
    b.h[5] += su.z * u.z;
}
// h += s * (u v^T + v u^T)
template <typename T>
SPGX_HD void add_sym_outer(Block<T> &b, Vec3<T> u, Vec3<T> v, T s)
{
    b.h[0] += s * (T(2) * u.x * v.x);
    b.h[1] += s * (u.x * v.y + v.x * u.y);
    b.h[2] += s * (u.x * v.z + v.x * u.z);
    b.h[3] += s * (T(2) * u.y * v.y);
    b.h[4] += s * (u.y * v.z + v.y * u.z);
    b.h[5] += s * (T(2) * u.z * v.z);
}
// h += s * I
template <typename T>
SPGX_HD void add_diag(Block<T> &b, T s)
{
    b.h[0] += s;
    b.h[3] += s;
    b.h[5] += s;
}

// ---------------------------------------------------------------------------------------
// SpringAnchorEnergy: E = 1/2 k |x - a|^2 (springAnchorEnergy.cpp:21-26).
template <typename T>
SPGX_HD void anchor_block(Vec3<T> x, Vec3<T> a, T k, Block<T> &b)
{
    sub_force(b, x - a, k);
    add_diag(b, k);
}

SPGX_HD float fmadd(float a, float b, float c) { return fmaf(a, b, c); }
SPGX_HD double fmadd(double a, double b, double c) { return fma(a, b, c); }
// A product and a sum that the device compiler never fuses into an FMA with a neighbouring
// operation (error-free transformations need each one rounded on its own; the host build
// disables contraction altogether).
#if defined(__CUDA_ARCH__)
SPGX_HD float mul_rn(float a, float b) { return __fmul_rn(a, b); }
SPGX_HD double mul_rn(double a, double b) { return __dmul_rn(a, b); }
SPGX_HD float add_rn(float a, float b) { return __fadd_rn(a, b); }
SPGX_HD double add_rn(double a, double b) { return __dadd_rn(a, b); }
#else
SPGX_HD float mul_rn(float a, float b) { return a * b; }
SPGX_HD double mul_rn(double a, double b) { return a * b; }
SPGX_HD float add_rn(float a, float b) { return a + b; }
SPGX_HD double add_rn(double a, double b) { return a + b; }
#endif

// Knuth's error-free sum: a + b = s + e exactly, for any ordering of |a| and |b|.
template <typename T>
SPGX_HD void two_sum(T a, T b, T &s, T &e)
{
    s = add_rn(a, b);
    const T bb = add_rn(s, -a);
    e = add_rn(add_rn(a, -add_rn(s, -bb)), add_rn(b, -bb));
}

// Spring stretch l - L0 for the spring vector s = sh + sl (sl a small remainder of sh's
// rounding), with l ~ |sh| for the denominator. Near rest l - L0 is a small difference of
// two nearly equal lengths, and forming it as l - L0 from a rounded l leaves a relative error
// of about (rounding of l) / strain: 1e-7 / 1e-5 = 1e-2 at a strain of 1e-5. Here
// |s|^2 - L0^2 is formed without that cancellation: the squares are error-free products
// (p + e = a * a exactly, e from one FMA), their sum and the subtraction of L0^2 are
// error-free sums, and only the small remainders are rounded. Then
// l - L0 = (|s|^2 - L0^2) / (l + L0), where the rounding of l no longer cancels.
template <typename T>
SPGX_HD T spring_stretch(Vec3<T> sh, Vec3<T> sl, T L0, T l)
{
    const T px = mul_rn(sh.x, sh.x), py = mul_rn(sh.y, sh.y), pz = mul_rn(sh.z, sh.z), q = mul_rn(L0, L0);
    const T ex = fmadd(sh.x, sh.x, -px), ey = fmadd(sh.y, sh.y, -py);
    const T ez = fmadd(sh.z, sh.z, -pz), eq = fmadd(L0, L0, -q);
    T s1, t1, s2, t2, s3, t3;
    two_sum(px, py, s1, t1);
    two_sum(s1, pz, s2, t2);
    two_sum(s2, -q, s3, t3);
    const T tail = ((ex + ey) + (ez - eq)) + ((t1 + t2) + t3) + T(2) * dot(sh, sl);
    return (s3 + tail) * recip(l + L0);
}

// SpringEnergy gradient / Hessian (springEnergy.cpp:101-133) for the vertex xi of a spring
// whose other end is xo: g = k (l - L0) s / l with s = xi - xo, and
// H = k [(1 - L0/l)(I - s s^T / l^2) + s s^T / l^2] = k (1 - L0/l) I + k L0 / l^3 s s^T.
// sl is the remainder of the spring vector's rounding (s = (xi - xo) + sl exactly, or as
// exactly as the caller knows it); it enters only the stretch l - L0.
template <typename T>
SPGX_HD void spring_block(Vec3<T> xi, Vec3<T> xo, Vec3<T> sl, T L0, T k, Block<T> &b)
{
    const Vec3<T> s = xi - xo;
    const T l2 = dot(s, s);
    const T il = rsqrt_of(l2);
    const T l = l2 * il;
    const T c = k * spring_stretch(s, sl, L0, l) * il;  // k (l - L0) / l = k (1 - L0 / l)
    sub_force(b, s, c);
    add_diag(b, c);
    add_outer(b, s, k * L0 * il * il * il);
}

template <typename T>
SPGX_HD void spring_block(Vec3<T> xi, Vec3<T> xo, T L0, T k, Block<T> &b)
{
    spring_block(xi, xo, mk(T(0), T(0), T(0)), L0, k, b);
}

// ---------------------------------------------------------------------------------------
// Discrete bending (discreteBendingEnergy.cpp:9-30): for the stencil (p0, p1, p2, p3) with
// hinge e = p1 - p0, flaps a = p2 - p0, b = p3 - p0, Na = e x a, Nb = e x b, the reference's
// theta = atan2((n1 x n2).e_hat, n1.n2) with n1 = Na/|Na|, n2 = -Nb/|Nb| equals
// atan2(-|e| (Na . b), -(Na . Nb)). E = 1/2 k_eff (theta - theta0)^2, so
// g = k C dtheta and H = k (dtheta dtheta^T + C d2theta) with C = theta - theta0 (no PSD
// projection, like the reference).
//
// Exchanging p2 and p3, or p0 and p1, negates theta, so the slot-3 block is the slot-2
// formula on (p0, p1, p3, p2) with -theta0, and the slot-0 block the slot-1 formula on
// (p1, p0, p2, p3) with -theta0.
template <typename T>
SPGX_HD T hinge_angle(Vec3<T> e, Vec3<T> Na, Vec3<T> Nb, Vec3<T> b, T L)
{
    return arctan2(-L * dot(Na, b), -dot(Na, Nb));
}

// Flap vertex p2: dtheta/dp2 = -|e| Na / |Na|^2 and
// d2theta/dp2^2 = -(|e| / |Na|^4) (M Na^T + Na M^T) with M = e x Na.
template <typename T>
SPGX_HD void bending_flap_block(Vec3<T> p0, Vec3<T> p1, Vec3<T> p2, Vec3<T> p3, T theta0, T k, Block<T> &blk)
{
    const Vec3<T> e = p1 - p0;
    const Vec3<T> a = p2 - p0;
    const Vec3<T> b = p3 - p0;
    const Vec3<T> Na = cross(e, a);
    const Vec3<T> Nb = cross(e, b);
    const T L2 = dot(e, e);
    const T L = L2 * rsqrt_of(L2);
    const T nua = dot(Na, Na);
    const T C = hinge_angle(e, Na, Nb, b, L) - theta0;
    const T ina = recip(nua);
    const Vec3<T> g = (-L * ina) * Na;
    sub_force(blk, g, k * C);
    add_outer(blk, g, k);
    const Vec3<T> M = cross(e, Na);
    add_sym_outer(blk, M, Na, -k * C * L * ina * ina);
}

// Hinge vertex p1 (p0 fixed): with Q(c) = (c.e) (e x c) / (|e| |e x c|^2),
// dtheta/dp1 = Q(a) - Q(b), and the symmetric part of dQ(c)/de is
// sym(N u^T) / (|e| |N|^2) with N = e x c, u = c - (c.e)/|e|^2 e + 2 (c.e)/|N|^2 (N x c)
// (the antisymmetric [c]x term cancels between the two triangles).
template <typename T>
SPGX_HD void bending_hinge_block(Vec3<T> p0, Vec3<T> p1, Vec3<T> p2, Vec3<T> p3, T theta0, T k, Block<T> &blk)
{
    const Vec3<T> e = p1 - p0;
    const Vec3<T> a = p2 - p0;
    const Vec3<T> b = p3 - p0;
    const Vec3<T> Na = cross(e, a);
    const Vec3<T> Nb = cross(e, b);
    const T L2 = dot(e, e);
    const T iL = rsqrt_of(L2);
    const T L = L2 * iL;
    const T iL2 = iL * iL;
    const T ina = recip(dot(Na, Na));
    const T inb = recip(dot(Nb, Nb));
    const T C = hinge_angle(e, Na, Nb, b, L) - theta0;
    const T sa = dot(a, e);
    const T sb = dot(b, e);
    const Vec3<T> g = (sa * iL * ina) * Na - (sb * iL * inb) * Nb;
    sub_force(blk, g, k * C);
    add_outer(blk, g, k);
    const Vec3<T> ua = a - (sa * iL2) * e + (T(2) * sa * ina) * cross(Na, a);
    const Vec3<T> ub = b - (sb * iL2) * e + (T(2) * sb * inb) * cross(Nb, b);
    const T kc = k * C * T(0.5) * iL;
    add_sym_outer(blk, Na, ua, kc * ina);
    add_sym_outer(blk, Nb, ub, -kc * inb);
}

template <typename T>
SPGX_HD void bending_block(const Vec3<T> *p, int slot, T theta0, T k, Block<T> &blk)
{
    switch (slot) {
    case 0: bending_hinge_block(p[1], p[0], p[2], p[3], -theta0, k, blk); break;
    case 1: bending_hinge_block(p[0], p[1], p[2], p[3], theta0, k, blk); break;
    case 2: bending_flap_block(p[0], p[1], p[2], p[3], theta0, k, blk); break;
    default: bending_flap_block(p[0], p[1], p[3], p[2], -theta0, k, blk); break;
    }
}

// ---------------------------------------------------------------------------------------
// StVK membrane (membraneStvkEnergy.cpp:9-28, energy 1/2 C^T K C): F = [x1-x0, x2-x0] Dinv
// = sum_j x_j w_j^T with w_1 = Dinv row 0, w_2 = Dinv row 1, w_0 = -(w_1 + w_2). For the
// vertex's (p, q) = w_slot: dC0 = p f0, dC1 = q f1, dC2 = q f0 + p f1, so
// g = F S w with S = K C, and H = J K J^T + (S0 p^2 + S1 q^2 + 2 S2 p q) I.
// K is symmetric: Ks = (K00, K01, K02, K11, K12, K22).
template <typename T>
SPGX_HD void stvk_block(const Vec3<T> *x, int slot, const T *D, const T *Ks, Block<T> &blk)
{
    const Vec3<T> u = x[1] - x[0];
    const Vec3<T> v = x[2] - x[0];
    const Vec3<T> f0 = D[0] * u + D[2] * v;
    const Vec3<T> f1 = D[1] * u + D[3] * v;
    const T C0 = T(0.5) * (dot(f0, f0) - T(1));
    const T C1 = T(0.5) * (dot(f1, f1) - T(1));
    const T C2 = dot(f0, f1);
    const T S0 = Ks[0] * C0 + Ks[1] * C1 + Ks[2] * C2;
    const T S1 = Ks[1] * C0 + Ks[3] * C1 + Ks[4] * C2;
    const T S2 = Ks[2] * C0 + Ks[4] * C1 + Ks[5] * C2;
    T p, q;
    if (slot == 0) {
        p = -(D[0] + D[2]);
        q = -(D[1] + D[3]);
    } else if (slot == 1) {
        p = D[0];
        q = D[1];
    } else {
        p = D[2];
        q = D[3];
    }
    const Vec3<T> g = (S0 * p + S2 * q) * f0 + (S2 * p + S1 * q) * f1;
    sub_force(blk, g, T(1));
    const Vec3<T> J0 = p * f0;
    const Vec3<T> J1 = q * f1;
    const Vec3<T> J2 = q * f0 + p * f1;
    add_outer(blk, J0, Ks[0]);
    add_outer(blk, J1, Ks[3]);
    add_outer(blk, J2, Ks[5]);
    add_sym_outer(blk, J0, J1, Ks[1]);
    add_sym_outer(blk, J0, J2, Ks[2]);
    add_sym_outer(blk, J1, J2, Ks[4]);
    add_diag(blk, S0 * p * p + S1 * q * q + T(2) * S2 * p * q);
}

// ---------------------------------------------------------------------------------------
// Stable Neo-Hookean (stableNeoHookeanEnergy.cpp:33-61):
// E = 1/2 lambda (J - alpha)^2 + 1/2 mu (tr F^T F - 3), F = [x1-x0, x2-x0, x3-x0] Dinv
// = sum_j x_j w_j^T. J is linear in any single vertex (rank-one update), so with
// c = cof(F) w: g = lambda (J - alpha) c + mu F w and H = mu |w|^2 I + lambda c c^T.
template <typename T>
SPGX_HD void snh_deformation(const Vec3<T> *x, const T *D, Vec3<T> &f0, Vec3<T> &f1, Vec3<T> &f2)
{
    const Vec3<T> u = x[1] - x[0];
    const Vec3<T> v = x[2] - x[0];
    const Vec3<T> w = x[3] - x[0];
    f0 = D[0] * u + D[3] * v + D[6] * w;
    f1 = D[1] * u + D[4] * v + D[7] * w;
    f2 = D[2] * u + D[5] * v + D[8] * w;
}

template <typename T>
SPGX_HD Vec3<T> snh_weights(const T *D, int slot)
{
    if (slot == 0) return mk(-(D[0] + D[3] + D[6]), -(D[1] + D[4] + D[7]), -(D[2] + D[5] + D[8]));
    if (slot == 1) return mk(D[0], D[1], D[2]);
    if (slot == 2) return mk(D[3], D[4], D[5]);
    return mk(D[6], D[7], D[8]);
}

template <typename T>
SPGX_HD void snh_block(const Vec3<T> *x, int slot, const T *D, T lambda, T mu, T alpha, Block<T> &blk)
{
    Vec3<T> f0, f1, f2;
    snh_deformation(x, D, f0, f1, f2);
    const Vec3<T> c0 = cross(f1, f2);
    const Vec3<T> c1 = cross(f2, f0);
    const Vec3<T> c2 = cross(f0, f1);
    const T J = dot(f0, c0);
    const Vec3<T> w = snh_weights(D, slot);
    const Vec3<T> cw = w.x * c0 + w.y * c1 + w.z * c2;
    const Vec3<T> Fw = w.x * f0 + w.y * f1 + w.z * f2;
    const Vec3<T> g = (lambda * (J - alpha)) * cw + mu * Fw;
    sub_force(blk, g, T(1));
    add_diag(blk, mu * dot(w, w));
    add_outer(blk, cw, lambda);
}

// ---------------------------------------------------------------------------------------
// Constraint values and gradients for the XPBD projection (energy.h:117-153 uses
// dConstraintsAndGradient). grad[c * S + j] is dC_c / dx_j (stencil slot j).

// SpringAnchorEnergy constraint |x - a| with the zero-norm guard (springAnchorEnergy.cpp:8-19).
template <typename T>
SPGX_HD void anchor_constraint(Vec3<T> x, Vec3<T> a, T *C, Vec3<T> *grad)
{
    const Vec3<T> d = x - a;
    const T n = sq_root(dot(d, d));
    if (n == T(0)) {
        C[0] = T(0);
        grad[0] = mk(T(0), T(0), T(0));
    } else {
        C[0] = n;
        grad[0] = (T(1) / n) * d;
    }
}

// Bending constraint theta - theta0 and its gradient over the four stencil vertices.
template <typename T>
SPGX_HD void bending_constraint(const Vec3<T> *p, T theta0, T *C, Vec3<T> *grad)
{
    const Vec3<T> e = p[1] - p[0];
    const Vec3<T> a = p[2] - p[0];
    const Vec3<T> b = p[3] - p[0];
    const Vec3<T> Na = cross(e, a);
    const Vec3<T> Nb = cross(e, b);
    const T L = sq_root(dot(e, e));
    const T iL = T(1) / L;
    const T ina = T(1) / dot(Na, Na);
    const T inb = T(1) / dot(Nb, Nb);
    C[0] = hinge_angle(e, Na, Nb, b, L) - theta0;
    const Vec3<T> g2 = (-L * ina) * Na;
    const Vec3<T> g3 = (L * inb) * Nb;
    const Vec3<T> g1 = (dot(a, e) * iL * ina) * Na - (dot(b, e) * iL * inb) * Nb;
    grad[0] = mk(T(0), T(0), T(0)) - (g1 + g2 + g3);
    grad[1] = g1;
    grad[2] = g2;
    grad[3] = g3;
}

// StVK constraints [E00, E11, 2 E01] (membraneStvkEnergy.cpp:9-28).
template <typename T>
SPGX_HD void stvk_constraints(const Vec3<T> *x, const T *D, T *C, Vec3<T> *grad)
{
    const Vec3<T> u = x[1] - x[0];
    const Vec3<T> v = x[2] - x[0];
    const Vec3<T> f0 = D[0] * u + D[2] * v;
    const Vec3<T> f1 = D[1] * u + D[3] * v;
    C[0] = T(0.5) * (dot(f0, f0) - T(1));
    C[1] = T(0.5) * (dot(f1, f1) - T(1));
    C[2] = dot(f0, f1);
    const T ps[3] = {-(D[0] + D[2]), D[0], D[2]};
    const T qs[3] = {-(D[1] + D[3]), D[1], D[3]};
    for (int j = 0; j < 3; ++j) {
        grad[0 * 3 + j] = ps[j] * f0;
        grad[1 * 3 + j] = qs[j] * f1;
        grad[2 * 3 + j] = qs[j] * f0 + ps[j] * f1;
    }
}

// SNH constraints [det F - alpha, sqrt(tr F^T F)] (stableNeoHookeanEnergy.cpp:9-31).
template <typename T>
SPGX_HD void snh_constraints(const Vec3<T> *x, const T *D, T alpha, T *C, Vec3<T> *grad)
{
    Vec3<T> f0, f1, f2;
    snh_deformation(x, D, f0, f1, f2);
    const Vec3<T> c0 = cross(f1, f2);
    const Vec3<T> c1 = cross(f2, f0);
    const Vec3<T> c2 = cross(f0, f1);
    const T J = dot(f0, c0);
    const T nF = sq_root(dot(f0, f0) + dot(f1, f1) + dot(f2, f2));
    C[0] = J - alpha;
    C[1] = nF;
    const T inF = T(1) / nF;
    for (int j = 0; j < 4; ++j) {
        const Vec3<T> w = snh_weights(D, j);
        grad[0 * 4 + j] = w.x * c0 + w.y * c1 + w.z * c2;
        grad[1 * 4 + j] = inF * (w.x * f0 + w.y * f1 + w.z * f2);
    }
}

}  // namespace spgx
