// Test-only CPU instantiation of the solver's element derivative templates
// (spg_gb300/csrc/elements.cuh) in FP64 and FP32, so the closed-form blocks can be checked
// against the oracle's automatic differentiation without a GPU. The shipped library never
// calls this; its GPU kernels instantiate the same templates in FP32.
#include "elements.cuh"
#include "generic.cuh"

#include <cmath>
#include <cstdint>

using namespace spgx;

namespace {
int ssize(int type)
{
    static const int kSize[15] = {0, 2, 1, 4, 3, 4, 4, 4, 3, 3, 4, 4, 2, 2, 1};
    return type >= 1 && type <= 14 ? kSize[type] : 0;
}

template <typename T>
void eval_block(int type, const double *X, const double *p, int slot, double *g, double *H)
{
    Vec3<T> x[4];
    const int S = ssize(type);
    for (int j = 0; j < S; ++j) x[j] = mk(T(X[3 * j]), T(X[3 * j + 1]), T(X[3 * j + 2]));
    Block<T> b;
    block_zero(b);
    switch (type) {
    case 1: spring_block(x[slot], x[1 - slot], T(p[0]), T(p[1]), b); break;
    case 2: anchor_block(x[0], mk(T(p[0]), T(p[1]), T(p[2])), T(p[3]), b); break;
    case 3: bending_block(x, slot, T(p[0]), T(p[1]), b); break;
    case 4: {
        const T D[4] = {T(p[0]), T(p[1]), T(p[2]), T(p[3])};
        const double *K = p + 4;
        const T Ks[6] = {T(K[0]), T(0.5 * (K[1] + K[3])), T(0.5 * (K[2] + K[6])), T(K[4]), T(0.5 * (K[5] + K[7])), T(K[8])};
        stvk_block(x, slot, D, Ks, b);
        break;
    }
    case 5: {
        T D[9];
        for (int i = 0; i < 9; ++i) D[i] = T(p[i]);
        snh_block(x, slot, D, T(p[9]), T(p[10]), T(p[11]), b);
        break;
    }
    default: {  // types 6-14: the per-vertex forward-mode path, on positions relative to the vertex
        static const int kParams[15] = {0, 3, 5, 3, 22, 14, 13, 13, 10, 12, 3, 6, 3, 3, 4};
        T prm[13] = {};
        for (int i = 0; i < kParams[type]; ++i) prm[i] = T(p[i]);
        Vec3<T> r[4];
        for (int j = 0; j < 4; ++j) r[j] = j < S ? x[j] - x[slot] : mk(T(0), T(0), T(0));
        generic_block(type, r, slot, prm, b);
        break;
    }
    }
    for (int a = 0; a < 3; ++a) g[a] = -double(b.f[a]);
    const int m[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};
    for (int i = 0; i < 9; ++i) H[i] = double(b.h[m[i]]);
}

template <typename T>
void eval_constraints(int type, const double *X, const double *p, double *C, double *G)
{
    Vec3<T> x[4];
    const int S = ssize(type);
    for (int j = 0; j < S; ++j) x[j] = mk(T(X[3 * j]), T(X[3 * j + 1]), T(X[3 * j + 2]));
    T c[3];
    Vec3<T> g[12];
    int nc = 1;
    switch (type) {
    case 2: anchor_constraint(x[0], mk(T(p[0]), T(p[1]), T(p[2])), c, g); break;
    case 3: bending_constraint(x, T(p[0]), c, g); break;
    case 4: {
        const T D[4] = {T(p[0]), T(p[1]), T(p[2]), T(p[3])};
        stvk_constraints(x, D, c, g);
        nc = 3;
        break;
    }
    case 5: {
        T D[9];
        for (int i = 0; i < 9; ++i) D[i] = T(p[i]);
        snh_constraints(x, D, T(p[11]), c, g);
        nc = 2;
        break;
    }
    default: return;
    }
    for (int i = 0; i < nc; ++i) {
        C[i] = double(c[i]);
        for (int j = 0; j < S; ++j) {
            G[i * 3 * S + 3 * j + 0] = double(g[i * S + j].x);
            G[i * 3 * S + 3 * j + 1] = double(g[i * S + j].y);
            G[i * 3 * S + 3 * j + 2] = double(g[i * S + j].z);
        }
    }
}
}  // namespace

extern "C" {
void host_block_f64(int type, const double *X, const double *p, int slot, double *g, double *H)
{
    eval_block<double>(type, X, p, slot, g, H);
}
void host_block_f32(int type, const double *X, const double *p, int slot, double *g, double *H)
{
    eval_block<float>(type, X, p, slot, g, H);
}
void host_constraints_f64(int type, const double *X, const double *p, double *C, double *G)
{
    eval_constraints<double>(type, X, p, C, G);
}
}
