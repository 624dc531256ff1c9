// ORACLE — test infrastructure only. Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg load this library, and only as the checker / timed CPU restatement of
// the reference. The shipped library (spg_gb300/) never links or calls it.
//
// FP64 CPU restatement of SPG's Vertex Block Descent hot path and its XPBD counterpart
// (alexrodag/spg). The reference itself cannot be built here: its Eigen and TinyAD
// submodules are empty and neither library exists on the system. Each function below cites
// the reference lines it restates. Only the reference's graph colouring
// (spg/source/utils/graphColoring.cpp, STL only) compiles from its own sources; it is built
// into oracle/_ref/ by oracle/build_ref.sh and pins the colouring restated here.
//
// Derivative evaluation follows the reference literally in kFullAD mode (full element
// gradient and dense element Hessian per incidence, then the vertex's block:
// energy.h:240-258). kVertexAD evaluates the same block with the AD seeded on the vertex's
// three coordinates only, which is mathematically the same block at a fraction of the cost.
#include "energies.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <list>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

struct EnergyBlock {
    int type{0};
    std::vector<int> stencils;
    std::vector<double> params;
    int n() const { return static_cast<int>(stencils.size()) / stencil_size(type); }
};

// ParticleGroup state (spg/include/spg/sim/simObject/particleGroup.h:51-56), flat FP64.
struct Object {
    std::vector<double> x, x0, v, m, w;
    std::vector<EnergyBlock> energies;
    int nv() const { return static_cast<int>(m.size()); }
    // ParticleGroup::addParticle, particleGroup.cpp:74-82
    void addParticle(const double *p, const double *p0, double mass)
    {
        for (int k = 0; k < 3; ++k) {
            x.push_back(p[k]);
            x0.push_back(p0[k]);
            v.push_back(0.0);
        }
        m.push_back(mass);
        w.push_back(mass == 0 ? 0 : 1 / mass);
    }
};

static thread_local std::string g_error;

// ---------------------------------------------------------------------------------------
// Small dense helpers (Eigen's closed-form 2x2 / 3x3 inverse and determinant).
static double det3x3(const double *A)
{
    return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
           A[2] * (A[3] * A[7] - A[4] * A[6]);
}

static void inverse3x3(const double *A, double *Ai)
{
    const double c00 = A[4] * A[8] - A[5] * A[7];
    const double c01 = A[5] * A[6] - A[3] * A[8];
    const double c02 = A[3] * A[7] - A[4] * A[6];
    const double det = A[0] * c00 + A[1] * c01 + A[2] * c02;
    const double id = 1.0 / det;
    Ai[0] = c00 * id;
    Ai[1] = (A[2] * A[7] - A[1] * A[8]) * id;
    Ai[2] = (A[1] * A[5] - A[2] * A[4]) * id;
    Ai[3] = c01 * id;
    Ai[4] = (A[0] * A[8] - A[2] * A[6]) * id;
    Ai[5] = (A[2] * A[3] - A[0] * A[5]) * id;
    Ai[6] = c02 * id;
    Ai[7] = (A[1] * A[6] - A[0] * A[7]) * id;
    Ai[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

// n x n inverse by Gauss-Jordan elimination with partial pivoting (Eigen's inverse() for the
// 4x4 XPBD system of the Choi membrane).
static void inverse_gauss_jordan(const double *A, double *Ai, int n)
{
    double M[4][8];
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < 2 * n; ++c) M[r][c] = c < n ? A[r * n + c] : (c - n == r ? 1.0 : 0.0);
    for (int k = 0; k < n; ++k) {
        int piv = k;
        for (int r = k + 1; r < n; ++r)
            if (std::fabs(M[r][k]) > std::fabs(M[piv][k])) piv = r;
        for (int c = 0; c < 2 * n; ++c) std::swap(M[k][c], M[piv][c]);
        const double ip = 1.0 / M[k][k];
        for (int c = 0; c < 2 * n; ++c) M[k][c] *= ip;
        for (int r = 0; r < n; ++r)
            if (r != k) {
                const double f = M[r][k];
                for (int c = 0; c < 2 * n; ++c) M[r][c] -= f * M[k][c];
            }
    }
    for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) Ai[r * n + c] = M[r][n + c];
}

static void inverse2x2(const double *A, double *Ai)
{
    const double det = A[0] * A[3] - A[1] * A[2];
    Ai[0] = A[3] / det;
    Ai[1] = -A[1] / det;
    Ai[2] = -A[2] / det;
    Ai[3] = A[0] / det;
}

// ---------------------------------------------------------------------------------------
// Energy construction: addStencil + preparePrecomputations of each energy.

// SpringEnergy::addStencil, springEnergy.cpp:33-46
static void spring_add(EnergyBlock &E, int a, int b, double L0, double k)
{
    if (L0 <= 0) throw std::runtime_error("Zero/negative rest length invalid");
    E.stencils.push_back(a);
    E.stencils.push_back(b);
    E.params.insert(E.params.end(), {L0, k, 1.0 / k});
}

// SpringAnchorEnergy::addStencil, springAnchorEnergy.cpp:29-39
static void anchor_add(EnergyBlock &E, int a, const double *pos, double k)
{
    E.stencils.push_back(a);
    E.params.insert(E.params.end(), {pos[0], pos[1], pos[2], k, 1.0 / k});
}

// DiscreteBendingEnergy::addStencil + preparePrecomputations, discreteBendingEnergy.cpp:33-72
static void bending_add(EnergyBlock &E, const std::array<int, 4> &s, double restTheta, double k)
{
    if (restTheta < -3.12 || restTheta > 3.12) throw std::runtime_error("Invalid restTheta");
    E.stencils.insert(E.stencils.end(), s.begin(), s.end());
    E.params.insert(E.params.end(), {restTheta, k, 1.0 / k});
}

static void bending_prepare(EnergyBlock &E, const Object &obj)
{
    const int n = E.n();
    for (int i = 0; i < n; ++i) {
        const int *s = &E.stencils[4 * i];
        V3<double> p[4];
        for (int j = 0; j < 4; ++j) p[j] = V3<double>(obj.x0[3 * s[j]], obj.x0[3 * s[j] + 1], obj.x0[3 * s[j] + 2]);
        const V3<double> e0 = p[1] - p[0];
        const V3<double> e3 = p[2] - p[1];
        const V3<double> e4 = p[3] - p[1];
        const double constantFactor = 2. * 3. * squaredNorm(e0) / (0.5 * (norm(cross(e0, e3)) + norm(cross(e0, e4))));
        const double k = E.params[3 * i + 1];
        const double modelCompliance = 1.0 / k;
        const double effCompliance = modelCompliance / constantFactor;
        E.params[3 * i + 2] = effCompliance;
        E.params[3 * i + 1] = 1.0 / effCompliance;
        const V3<double> n1 = normalized(cross(e0, e3));
        const V3<double> n2 = -normalized(cross(e0, e4));
        E.params[3 * i + 0] = std::atan2(dot(cross(n1, n2), normalized(e0)), dot(n1, n2));
    }
}

// MembraneStvkEnergy::addStencil + preparePrecomputations, membraneStvkEnergy.cpp:31-71
static void stvk_add(EnergyBlock &E, const std::array<int, 3> &s, double young, double poisson)
{
    E.stencils.insert(E.stencils.end(), s.begin(), s.end());
    const double yc = young / (1 - poisson * poisson);
    const double C[9] = {yc, yc * poisson, 0, yc * poisson, yc, 0, 0, 0, yc * (1 - poisson) / 2};
    double Ci[9];
    inverse3x3(C, Ci);
    E.params.insert(E.params.end(), {0, 0, 0, 0});
    E.params.insert(E.params.end(), C, C + 9);
    E.params.insert(E.params.end(), Ci, Ci + 9);
}

static void stvk_prepare(EnergyBlock &E, const Object &obj)
{
    const int n = E.n();
    for (int i = 0; i < n; ++i) {
        const int *s = &E.stencils[3 * i];
        const double *x0 = &obj.x0[3 * s[0]];
        const double *x1 = &obj.x0[3 * s[1]];
        const double *x2 = &obj.x0[3 * s[2]];
        if (x0[2] != 0.0 || x1[2] != 0.0 || x2[2] != 0.0)
            throw std::runtime_error("Rest positions of triangles for membrane StVK energy must have coordinate z=0");
        const double u[2] = {x1[0] - x0[0], x1[1] - x0[1]};
        const double v[2] = {x2[0] - x0[0], x2[1] - x0[1]};
        const double Dm[4] = {u[0], v[0], u[1], v[1]};
        double *p = &E.params[22 * i];
        inverse2x2(Dm, p);
        const double area = (u[0] * v[1] - v[0] * u[1]) * 0.5;
        if (area <= 0) throw std::runtime_error("Rest area of membrane StVK triangle is not positive");
        for (int k = 0; k < 9; ++k) {
            p[13 + k] = p[13 + k] / area;
            p[4 + k] = p[4 + k] * area;
        }
    }
}

// StableNeoHookeanEnergy::addStencil + preparePrecomputations, stableNeoHookeanEnergy.cpp:64-108
static void snh_add(EnergyBlock &E, const std::array<int, 4> &s, double young, double poisson)
{
    E.stencils.insert(E.stencils.end(), s.begin(), s.end());
    const double mu = young / (2 * (1 + poisson));
    const double lambda = mu / (1 - 2 * poisson);
    E.params.insert(E.params.end(), {0, 0, 0, 0, 0, 0, 0, 0, 0, lambda, mu, 1 + mu / lambda, 1.0 / lambda, 1.0 / mu});
}

static void snh_prepare(EnergyBlock &E, const Object &obj)
{
    const int n = E.n();
    for (int i = 0; i < n; ++i) {
        const int *s = &E.stencils[4 * i];
        double Dm[9];
        for (int a = 0; a < 3; ++a) {
            Dm[a * 3 + 0] = obj.x0[3 * s[1] + a] - obj.x0[3 * s[0] + a];
            Dm[a * 3 + 1] = obj.x0[3 * s[2] + a] - obj.x0[3 * s[0] + a];
            Dm[a * 3 + 2] = obj.x0[3 * s[3] + a] - obj.x0[3 * s[0] + a];
        }
        const double volume = 1. / 6. * det3x3(Dm);
        if (volume <= 0) throw std::runtime_error("SNH tetrahedron rest volume is not positive");
        double *p = &E.params[14 * i];
        inverse3x3(Dm, p);
        p[12] = p[12] / volume;
        p[13] = p[13] / volume;
        p[9] = p[9] * volume;
        p[10] = p[10] * volume;
    }
}

// ---------------------------------------------------------------------------------------
// Scene builders (apps/solverCompare.cpp) and the new ones the benchmark configurations need.

struct TriMesh {
    std::vector<double> verts, verts0;  // 3V each
    std::vector<std::array<int, 3>> faces;
    std::vector<std::array<int, 2>> edges;
    std::vector<std::vector<int>> opposing;  // opposing vertex ids per edge, face order
};

// TriangleMesh constructor edge map, spg/include/spg/geom/triangleMesh.h:16-51
static void triangle_mesh_edges(TriMesh &M, int nv)
{
    for (const auto &f : M.faces) {
        for (int i = 0; i < 3; ++i)
            if (f[i] < 0 || f[i] >= nv) throw std::runtime_error("Triangle mesh face contains index to invalid vertex");
        if (f[0] == f[1] || f[1] == f[2] || f[2] == f[0])
            throw std::runtime_error("Triangle mesh face contains repeated vertex index");
    }
    std::map<std::array<int, 2>, std::vector<int>> edges;
    for (int f = 0; f < static_cast<int>(M.faces.size()); ++f) {
        const auto &face = M.faces[f];
        for (int i = 0; i < 3; ++i) {
            const int id0 = face[i];
            const int id1 = face[(i + 1) % 3];
            const int id2 = face[(i + 2) % 3];
            edges[{std::min(id0, id1), std::max(id0, id1)}].push_back(id2);
        }
    }
    for (const auto &kv : edges) {
        M.edges.push_back(kv.first);
        M.opposing.push_back(kv.second);
    }
}

// buildTriangleSquareMesh, apps/solverCompare.cpp:332-365 (float arithmetic kept).
static TriMesh build_triangle_square_mesh(float width, float height, int rows, int cols)
{
    TriMesh M;
    const float rowStep = height / (rows - 1);
    const float colStep = width / (cols - 1);
    for (int row = 0; row < rows; ++row) {
        for (int col = 0; col < cols; ++col) {
            M.verts0.insert(M.verts0.end(), {double(colStep * col), double(rowStep * row), 0.0});
            M.verts.insert(M.verts.end(), {double(colStep * col), 0.0, double(-rowStep * row)});
            if (row != 0 && col != 0) {
                if ((row + col) % 2 == 0) {
                    M.faces.push_back({row * cols + col - 1, (row - 1) * cols + col - 1, (row - 1) * cols + col});
                    M.faces.push_back({row * cols + col - 1, (row - 1) * cols + col, row * cols + col});
                } else {
                    M.faces.push_back({(row - 1) * cols + col - 1, row * cols + col, row * cols + col - 1});
                    M.faces.push_back({(row - 1) * cols + col - 1, (row - 1) * cols + col, row * cols + col});
                }
            }
        }
    }
    return M;
}

// Deterministic generator shared (by specification, not by code) with the shipped scene
// builders: splitmix64 and Box-Muller.
struct SplitMix64 {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
};

static double signed_area_xy(const std::vector<double> &P, const std::array<int, 3> &f)
{
    const double ax = P[3 * f[1]] - P[3 * f[0]], ay = P[3 * f[1] + 1] - P[3 * f[0] + 1];
    const double bx = P[3 * f[2]] - P[3 * f[0]], by = P[3 * f[2] + 1] - P[3 * f[0] + 1];
    return 0.5 * (ax * by - ay * bx);
}

// In-plane jitter of rest positions: N(0, sigma^2) per axis, resampled (up to 64 draws) when
// an incident triangle would drop below 10 % of its nominal signed area; the base position
// is kept if no draw passes. Vertices are visited in index order.
static void jitter_rest_positions(std::vector<double> &P, const std::vector<std::array<int, 3>> &faces, double sigma,
                                  uint64_t seed)
{
    const int nv = static_cast<int>(P.size() / 3);
    std::vector<std::vector<int>> vf(nv);
    for (int f = 0; f < static_cast<int>(faces.size()); ++f)
        for (int k = 0; k < 3; ++k) vf[faces[f][k]].push_back(f);
    std::vector<double> nominal(faces.size());
    for (size_t f = 0; f < faces.size(); ++f) nominal[f] = signed_area_xy(P, faces[f]);
    SplitMix64 rng{seed};
    const double twoPi = 6.283185307179586;
    for (int v = 0; v < nv; ++v) {
        const double bx = P[3 * v], by = P[3 * v + 1];
        bool accepted = false;
        for (int attempt = 0; attempt < 64 && !accepted; ++attempt) {
            const double u1 = rng.uniform(), u2 = rng.uniform();
            const double r = std::sqrt(-2.0 * std::log(u1));
            P[3 * v] = bx + sigma * (r * std::cos(twoPi * u2));
            P[3 * v + 1] = by + sigma * (r * std::sin(twoPi * u2));
            accepted = true;
            for (int f : vf[v])
                if (signed_area_xy(P, faces[f]) < 0.1 * nominal[f]) accepted = false;
        }
        if (!accepted) {
            P[3 * v] = bx;
            P[3 * v + 1] = by;
        }
    }
}

// Lumped masses from rest triangle areas, apps/solverCompare.cpp:383-400.
static void add_cloth_particles(Object &obj, const TriMesh &M, double mass, bool restInitial)
{
    const int nv = static_cast<int>(M.verts0.size() / 3);
    std::vector<double> particleAreas(nv, 0.0);
    double totalArea = 0;
    for (const auto &face : M.faces) {
        V3<double> x[3];
        for (int k = 0; k < 3; ++k) x[k] = V3<double>(M.verts0[3 * face[k]], M.verts0[3 * face[k] + 1], M.verts0[3 * face[k] + 2]);
        const V3<double> e0 = x[1] - x[0];
        const V3<double> e3 = x[2] - x[1];
        const double area = 0.5 * norm(cross(e0, e3));
        totalArea += area;
        for (int k = 0; k < 3; ++k) particleAreas[face[k]] += area / 3.0;
    }
    const double density = mass / totalArea;
    for (int i = 0; i < nv; ++i)
        obj.addParticle(restInitial ? &M.verts0[3 * i] : &M.verts[3 * i], &M.verts0[3 * i], particleAreas[i] * density);
}

// Bending stencils on interior edges, apps/solverCompare.cpp:441-452, then prepare.
static EnergyBlock cloth_bending(const TriMesh &M, const Object &obj, double k)
{
    EnergyBlock E;
    E.type = kBending;
    for (size_t i = 0; i < M.edges.size(); ++i)
        if (M.opposing[i].size() == 2)
            bending_add(E, {M.edges[i][0], M.edges[i][1], M.opposing[i][0], M.opposing[i][1]}, 0., k);
    bending_prepare(E, obj);
    return E;
}

// createCloth, apps/solverCompare.cpp:367-498, with the material constants, bending
// stiffness, anchor set and initial state as parameters (energy order: bending, membrane,
// anchor, as :460, :493, :496).
static Object create_cloth(double mass, float width, float height, int rows, int cols, double young, double poisson,
                           double bendK, double anchorK, const std::vector<int> &anchorIds, bool restInitial)
{
    TriMesh M = build_triangle_square_mesh(width, height, rows, cols);
    const int nv = rows * cols;
    triangle_mesh_edges(M, nv);
    Object obj;
    add_cloth_particles(obj, M, mass, restInitial);
    EnergyBlock anchors;
    anchors.type = kAnchor;
    for (int id : anchorIds) anchor_add(anchors, id, &obj.x[3 * id], anchorK);
    obj.energies.push_back(cloth_bending(M, obj, bendK));
    EnergyBlock membrane;
    membrane.type = kStvk;
    for (const auto &f : M.faces) stvk_add(membrane, f, young, poisson);
    stvk_prepare(membrane, obj);
    obj.energies.push_back(std::move(membrane));
    obj.energies.push_back(std::move(anchors));
    return obj;
}

// Spring cloth with jittered rest positions (large-cloth benchmark scene). New builder in the
// style of createCloth and createSpringBeam (apps/solverCompare.cpp:191-258): bending on
// interior edges, springs on every mesh edge with rest length from the rest positions, anchors
// on row 0. Energy order: bending, spring, anchor.
static Object create_spring_cloth(double mass, float width, float height, int rows, int cols, double springK,
                                  double bendK, double anchorK, double jitterFrac, uint64_t seed)
{
    TriMesh M = build_triangle_square_mesh(width, height, rows, cols);
    const int nv = rows * cols;
    if (jitterFrac > 0) {
        const double edge = double(width) / (cols - 1);
        jitter_rest_positions(M.verts0, M.faces, jitterFrac * edge, seed);
    }
    triangle_mesh_edges(M, nv);
    Object obj;
    add_cloth_particles(obj, M, mass, true);
    obj.energies.push_back(cloth_bending(M, obj, bendK));
    EnergyBlock springs;
    springs.type = kSpring;
    for (const auto &e : M.edges) {
        const V3<double> a(obj.x0[3 * e[0]], obj.x0[3 * e[0] + 1], obj.x0[3 * e[0] + 2]);
        const V3<double> b(obj.x0[3 * e[1]], obj.x0[3 * e[1] + 1], obj.x0[3 * e[1] + 2]);
        spring_add(springs, e[0], e[1], norm(a - b), springK);
    }
    obj.energies.push_back(std::move(springs));
    EnergyBlock anchors;
    anchors.type = kAnchor;
    for (int id = 0; id < cols; ++id) anchor_add(anchors, id, &obj.x[3 * id], anchorK);
    obj.energies.push_back(std::move(anchors));
    return obj;
}

// tetrahedralVolume, apps/solverCompare.cpp:104-117
static double tet_volume(const double *a, const double *b, const double *c, const double *d)
{
    double M[9];
    for (int k = 0; k < 3; ++k) {
        M[k * 3 + 0] = b[k] - a[k];
        M[k * 3 + 1] = c[k] - a[k];
        M[k * 3 + 2] = d[k] - a[k];
    }
    return det3x3(M) / 6.0;
}

struct TetMesh {
    std::vector<double> verts, verts0;
    std::vector<std::array<int, 4>> tets;
};

// buildTetrahedralBeamMesh, apps/solverCompare.cpp:118-189 (split == 5, with mirroring), and
// the 6-tet split of each cell along its (i,j,k) -> (i+1,j+1,k+1) diagonal (split == 6, new;
// conforming without mirroring). Both keep the reference's positive-volume reorder (:174-179).
static TetMesh build_tet_beam(float sx, float sy, float sz, int nx, int ny, int nz, int split)
{
    TetMesh M;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const double p[3] = {double(-sx * 0.5f + i * sx / (nx - 1)), double(-sy * 0.5f + j * sy / (ny - 1)),
                                     double(-sz * 0.5f + k * sz / (nz - 1))};
                M.verts.insert(M.verts.end(), p, p + 3);
                M.verts0.insert(M.verts0.end(), p, p + 3);
            }
    auto positive = [&M](int a, int b, int c, int d) -> std::array<int, 4> {
        if (tet_volume(&M.verts0[3 * a], &M.verts0[3 * b], &M.verts0[3 * c], &M.verts0[3 * d]) > 0) return {a, b, c, d};
        return {b, a, c, d};
    };
    auto id = [ny, nz](int i, int j, int k) { return i * ny * nz + j * nz + k; };
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < ny - 1; ++j)
            for (int k = 0; k < nz - 1; ++k) {
                if (split == 5) {
                    int id1 = id(i, j, k), id2 = id(i + 1, j, k), id3 = id(i, j, k + 1), id4 = id(i + 1, j, k + 1);
                    int id5 = id(i, j + 1, k), id6 = id(i + 1, j + 1, k), id7 = id(i, j + 1, k + 1),
                        id8 = id(i + 1, j + 1, k + 1);
                    if (i % 2 == 1) {
                        std::swap(id1, id2);
                        std::swap(id3, id4);
                        std::swap(id5, id6);
                        std::swap(id7, id8);
                    }
                    if (j % 2 == 1) {
                        std::swap(id1, id5);
                        std::swap(id2, id6);
                        std::swap(id3, id7);
                        std::swap(id4, id8);
                    }
                    if (k % 2 == 1) {
                        std::swap(id1, id3);
                        std::swap(id2, id4);
                        std::swap(id5, id7);
                        std::swap(id6, id8);
                    }
                    M.tets.push_back(positive(id1, id3, id4, id7));
                    M.tets.push_back(positive(id7, id8, id4, id6));
                    M.tets.push_back(positive(id4, id2, id1, id6));
                    M.tets.push_back(positive(id1, id5, id7, id6));
                    M.tets.push_back(positive(id7, id4, id6, id1));
                } else {
                    // Axis orders (x,y,z),(x,z,y),(y,x,z),(y,z,x),(z,x,y),(z,y,x): path from
                    // corner (0,0,0) to (1,1,1) adding one axis at a time.
                    static const int orders[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
                    for (const auto &o : orders) {
                        int c[3] = {0, 0, 0};
                        int t[4];
                        t[0] = id(i, j, k);
                        for (int s = 0; s < 3; ++s) {
                            c[o[s]] = 1;
                            t[s + 1] = id(i + c[0], j + c[1], k + c[2]);
                        }
                        M.tets.push_back(positive(t[0], t[1], t[2], t[3]));
                    }
                }
            }
    return M;
}

// createTetrahedralBeam, apps/solverCompare.cpp:260-330 with SNH, anchors on the x-min face
// (energy order: anchor, tet).
static Object create_tet_beam(double mass, float sx, float sy, float sz, int nx, int ny, int nz, double young,
                              double poisson, double anchorK, int split)
{
    TetMesh M = build_tet_beam(sx, sy, sz, nx, ny, nz, split);
    const int nv = nx * ny * nz;
    for (const auto &t : M.tets) {
        for (int k = 0; k < 4; ++k)
            if (t[k] < 0 || t[k] >= nv) throw std::runtime_error("Tetrahedral mesh cell contains index to invalid vertex");
    }
    std::vector<double> vol(nv, 0.0);
    double totalVolume = 0;
    for (const auto &t : M.tets) {
        const double tv = tet_volume(&M.verts0[3 * t[0]], &M.verts0[3 * t[1]], &M.verts0[3 * t[2]], &M.verts0[3 * t[3]]);
        totalVolume += tv;
        for (int k = 0; k < 4; ++k) vol[t[k]] += tv / 4.0;
    }
    const double density = mass / totalVolume;
    Object obj;
    for (int i = 0; i < nv; ++i) obj.addParticle(&M.verts[3 * i], &M.verts0[3 * i], vol[i] * density);
    EnergyBlock anchors;
    anchors.type = kAnchor;
    for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) {
            const int idv = j * nz + k;
            anchor_add(anchors, idv, &obj.x0[3 * idv], anchorK);
        }
    EnergyBlock snh;
    snh.type = kSnh;
    for (const auto &t : M.tets) snh_add(snh, t, young, poisson);
    obj.energies.push_back(std::move(anchors));
    obj.energies.push_back(std::move(snh));
    snh_prepare(obj.energies.back(), obj);
    return obj;
}

// ---------------------------------------------------------------------------------------
// Greedy colouring restated literally: Graph::addEdge / greedyColoring / colorVertices /
// colorStencils, spg/source/utils/graphColoring.cpp:12-84.
struct Graph {
    std::vector<std::list<int>> adj;
    void setNumNodes(int n) { adj.resize(n); }
    void addEdge(int i, int j)
    {
        if (i >= static_cast<int>(adj.size()) || j >= static_cast<int>(adj.size()))
            throw std::runtime_error("Trying to add edge to graph with invalid node indices");
        adj[i].push_back(j);
        adj[j].push_back(i);
    }
    std::vector<int> greedyColoring()
    {
        const int nbNodes = static_cast<int>(adj.size());
        std::vector<int> nodeColors(nbNodes, -1);
        if (nbNodes == 0) return nodeColors;
        nodeColors[0] = 0;
        std::vector<char> colorIsAvailable(nbNodes);
        for (int n = 1; n < nbNodes; n++) {
            std::fill(colorIsAvailable.begin(), colorIsAvailable.end(), static_cast<char>(1));
            for (int nb : adj[n])
                if (nodeColors[nb] != -1) colorIsAvailable[nodeColors[nb]] = 0;
            for (int color = 0; color < nbNodes; ++color) {
                if (colorIsAvailable[color] == 1) {
                    nodeColors[n] = color;
                    break;
                }
            }
        }
        return nodeColors;
    }
};

static std::vector<int> color_vertices(const Object &obj)
{
    Graph g;
    g.setNumNodes(obj.nv());
    for (const auto &E : obj.energies) {
        const int S = stencil_size(E.type);
        const int n = static_cast<int>(E.stencils.size());
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j % S != 0; ++j) g.addEdge(E.stencils[i], E.stencils[j]);
    }
    return g.greedyColoring();
}

static std::vector<int> color_stencils(const EnergyBlock &E)
{
    Graph g;
    std::vector<std::list<int>> stencilsPerVertex;
    const int S = stencil_size(E.type);
    for (int i = 0; i < static_cast<int>(E.stencils.size()); ++i) {
        const int vertexId = E.stencils[i];
        const int stencilId = i / S;
        stencilsPerVertex.resize(std::max(stencilsPerVertex.size(), static_cast<size_t>(vertexId + 1)));
        stencilsPerVertex[vertexId].push_back(stencilId);
    }
    g.setNumNodes(static_cast<int>(E.stencils.size()) / S);
    for (const auto &vs : stencilsPerVertex)
        for (auto it1 = vs.begin(); it1 != vs.end(); ++it1)
            for (auto it2 = std::next(it1); it2 != vs.end(); ++it2) g.addEdge(*it1, *it2);
    return g.greedyColoring();
}

// ---------------------------------------------------------------------------------------
// Per-incidence derivative evaluation.

enum DerivMode { kFullAD = 0, kVertexAD = 1 };

template <int S>
static void load_stencil(const double *X, const int *st, V3<double> *p)
{
    for (int j = 0; j < S; ++j) p[j] = V3<double>(X[3 * st[j]], X[3 * st[j] + 1], X[3 * st[j] + 2]);
}

// Evaluates the energy on AD scalars and returns the slot's gradient segment and Hessian block.
template <int S, typename Fn>
static void ad_block(Fn fn, const V3<double> *p, const double *params, int slot, int mode, double *g, double *H)
{
    if (mode == kFullAD) {
        using D = Dual<3 * S, true>;
        V3<D> q[S];
        for (int j = 0; j < S; ++j)
            for (int a = 0; a < 3; ++a) q[j][a] = D(p[j][a], 3 * j + a);
        const D e = fn(q, params);
        for (int a = 0; a < 3; ++a) {
            g[a] = e.grad[3 * slot + a];
            for (int b = 0; b < 3; ++b) H[a * 3 + b] = e.H(3 * slot + a, 3 * slot + b);
        }
    } else {
        using D = Dual<3, true>;
        V3<D> q[S];
        for (int j = 0; j < S; ++j)
            for (int a = 0; a < 3; ++a) q[j][a] = (j == slot) ? D(p[j][a], a) : D(p[j][a]);
        const D e = fn(q, params);
        for (int a = 0; a < 3; ++a) {
            g[a] = e.grad[a];
            for (int b = 0; b < 3; ++b) H[a * 3 + b] = e.H(a, b);
        }
    }
}

// SpringEnergy::energyGradient / energyHessian, springEnergy.cpp:101-133 (full 6x6 as the
// reference builds it; the slot's block is returned).
static void spring_block(const V3<double> *p, const double *params, int slot, double *g, double *H)
{
    const double k = params[1];
    const double L0 = params[0];
    const V3<double> s = p[0] - p[1];
    const double sNorm = norm(s);
    const V3<double> gradx0 = scale(s, k * (sNorm - L0) / sNorm);
    const V3<double> sn = scale(s, 1.0 / sNorm);
    const double sgn = slot == 0 ? 1.0 : -1.0;
    for (int a = 0; a < 3; ++a) {
        g[a] = sgn * gradx0[a];
        for (int b = 0; b < 3; ++b) {
            const double sst = sn[a] * sn[b];
            H[a * 3 + b] = k * ((1 - L0 / sNorm) * ((a == b ? 1.0 : 0.0) - sst) + sst);
        }
    }
}

// One incidence's energy gradient segment and Hessian block (the quantities
// accumulateVertexForce / accumulateVertexHessian add, energy.h:240-258).
static void incidence_block(int type, const double *X, const int *st, const double *params, int slot, int mode,
                            double *g, double *H)
{
    switch (type) {
    case kSpring: {
        V3<double> p[2];
        load_stencil<2>(X, st, p);
        spring_block(p, params, slot, g, H);
        break;
    }
    case kAnchor: {
        V3<double> p[1];
        load_stencil<1>(X, st, p);
        ad_block<1>([](const auto *q, const double *pp) { return anchor_energy(q, pp); }, p, params, slot, mode, g, H);
        break;
    }
    case kBending: {
        V3<double> p[4];
        load_stencil<4>(X, st, p);
        ad_block<4>([](const auto *q, const double *pp) { return bending_energy(q, pp); }, p, params, slot, mode, g, H);
        break;
    }
    case kStvk: {
        V3<double> p[3];
        load_stencil<3>(X, st, p);
        ad_block<3>([](const auto *q, const double *pp) { return stvk_energy(q, pp); }, p, params, slot, mode, g, H);
        break;
    }
    case kSnh: {
        V3<double> p[4];
        load_stencil<4>(X, st, p);
        ad_block<4>([](const auto *q, const double *pp) { return snh_energy(q, pp); }, p, params, slot, mode, g, H);
        break;
    }
#define ORACLE_GENERIC_CASE(KIND, S, FN)                                                                          \
    case KIND: {                                                                                                  \
        V3<double> p[S];                                                                                          \
        load_stencil<S>(X, st, p);                                                                                \
        ad_block<S>([](const auto *q, const double *pp) { return FN(q, pp); }, p, params, slot, mode, g, H);       \
        break;                                                                                                    \
    }
        ORACLE_GENERIC_CASE(kStvkTet, 4, stvk_tet_energy)
        ORACLE_GENERIC_CASE(kSsnh, 4, ssnh_energy)
        ORACLE_GENERIC_CASE(kBwMembrane, 3, bw_membrane_energy)
        ORACLE_GENERIC_CASE(kChoi, 3, choi_energy)
        ORACLE_GENERIC_CASE(kBwBending, 4, bw_bending_energy)
        ORACLE_GENERIC_CASE(kQuadBending, 4, quad_bending_energy)
        ORACLE_GENERIC_CASE(kSpringCont, 2, spring_cont_energy)
        ORACLE_GENERIC_CASE(kSpringSqCont, 2, spring_sq_cont_energy)
        ORACLE_GENERIC_CASE(kStaticLoad, 1, static_load_energy)
#undef ORACLE_GENERIC_CASE
    default: throw std::runtime_error("unsupported energy type");
    }
}

static double element_energy(int type, const V3<double> *p, const double *params)
{
    switch (type) {
    case kSpring: return spring_energy(p, params);
    case kAnchor: return anchor_energy(p, params);
    case kBending: return bending_energy(p, params);
    case kStvk: return stvk_energy(p, params);
    case kSnh: return snh_energy(p, params);
    case kStvkTet: return stvk_tet_energy(p, params);
    case kSsnh: return ssnh_energy(p, params);
    case kBwMembrane: return bw_membrane_energy(p, params);
    case kChoi: return choi_energy(p, params);
    case kBwBending: return bw_bending_energy(p, params);
    case kQuadBending: return quad_bending_energy(p, params);
    case kSpringCont: return spring_cont_energy(p, params);
    case kSpringSqCont: return spring_sq_cont_energy(p, params);
    case kStaticLoad: return static_load_energy(p, params);
    default: throw std::runtime_error("unsupported energy type");
    }
}

// Constraint values and gradients (dConstraintsAndGradient, energy.h:317-332) for the XPBD
// projection. gradC is column-major: gradC[c * 3S + dof].
template <int S, int NC, typename Fn>
static void constraints_and_gradient(Fn fn, const V3<double> *p, const double *params, double *C, double *gradC)
{
    using D = Dual<3 * S, false>;
    V3<D> q[S];
    for (int j = 0; j < S; ++j)
        for (int a = 0; a < 3; ++a) q[j][a] = D(p[j][a], 3 * j + a);
    D c[NC];
    fn(q, params, c);
    for (int i = 0; i < NC; ++i) {
        C[i] = c[i].val;
        for (int d = 0; d < 3 * S; ++d) gradC[i * 3 * S + d] = c[i].grad[d];
    }
}

static int n_constraints(int type)
{
    switch (type) {
    case kStvk: return 3;
    case kSnh: return 2;
    case kStvkTet: return 2;
    case kSsnh: return 2;
    case kBwMembrane: return 3;
    case kChoi: return 4;
    case kQuadBending: return 3;
    case kStaticLoad: return 0;
    default: return 1;
    }
}

static void element_constraints(int type, const V3<double> *p, const double *params, double *C, double *gradC)
{
    switch (type) {
    case kSpring:
        constraints_and_gradient<2, 1>([](const auto *q, const double *pp, auto *c) { c[0] = spring_constraint(q, pp); },
                                       p, params, C, gradC);
        break;
    case kAnchor:
        constraints_and_gradient<1, 1>([](const auto *q, const double *pp, auto *c) { c[0] = anchor_constraint(q, pp); },
                                       p, params, C, gradC);
        break;
    case kBending:
        constraints_and_gradient<4, 1>([](const auto *q, const double *pp, auto *c) { c[0] = bending_constraint(q, pp); },
                                       p, params, C, gradC);
        break;
    case kStvk:
        constraints_and_gradient<3, 3>([](const auto *q, const double *pp, auto *c) { stvk_constraints(q, pp, c); }, p,
                                       params, C, gradC);
        break;
    case kSnh:
        constraints_and_gradient<4, 2>([](const auto *q, const double *pp, auto *c) { snh_constraints(q, pp, c); }, p,
                                       params, C, gradC);
        break;
    case kStvkTet:
        constraints_and_gradient<4, 2>([](const auto *q, const double *pp, auto *c) { stvk_tet_constraints(q, pp, c); },
                                       p, params, C, gradC);
        break;
    case kSsnh:
        constraints_and_gradient<4, 2>([](const auto *q, const double *pp, auto *c) { ssnh_constraints(q, pp, c); }, p,
                                       params, C, gradC);
        break;
    case kBwMembrane:
        constraints_and_gradient<3, 3>([](const auto *q, const double *pp, auto *c) { bw_membrane_constraints(q, pp, c); },
                                       p, params, C, gradC);
        break;
    case kChoi:
        constraints_and_gradient<3, 4>([](const auto *q, const double *pp, auto *c) { choi_constraints(q, pp, c); }, p,
                                       params, C, gradC);
        break;
    case kBwBending:
        constraints_and_gradient<4, 1>(
            [](const auto *q, const double *pp, auto *c) { c[0] = bw_bending_constraint(q, pp); }, p, params, C, gradC);
        break;
    case kQuadBending:
        constraints_and_gradient<4, 3>([](const auto *q, const double *pp, auto *c) { quad_bending_constraints(q, pp, c); },
                                       p, params, C, gradC);
        break;
    case kSpringCont:
        constraints_and_gradient<2, 1>(
            [](const auto *q, const double *pp, auto *c) { c[0] = spring_cont_constraint(q, pp); }, p, params, C, gradC);
        break;
    case kSpringSqCont:
        constraints_and_gradient<2, 1>(
            [](const auto *q, const double *pp, auto *c) { c[0] = spring_sq_cont_constraint(q, pp); }, p, params, C,
            gradC);
        break;
    default: throw std::runtime_error("unsupported energy type");
    }
}

// ---------------------------------------------------------------------------------------
// VBD solver: VBD::step, VBD::computeParallelVertexGroups, VBD::computeStencilInfoPerVertex
// (spg/source/sim/solver/vbd.cpp:12-268). One object per solver instance: the reference's
// iteration loop never advances objId (vbd.cpp:91), so batches run one instance per object.
struct Vbd {
    Object obj;
    double dt{0.01};
    int substeps{1};
    int iterations{1};
    double g[3]{0, -9.8, 0};
    int mode{kVertexAD};
    bool prepared{false};
    std::vector<int> colors;
    std::vector<std::vector<int>> groups;
    // adjacency[v][e] = list of (stencilIdx, vertexIdxInStencil), vbd.cpp:231-268
    std::vector<std::vector<std::vector<std::array<int, 2>>>> adjacency;
    std::vector<double> xOld, xInertial;

    void prepare()
    {
        colors = color_vertices(obj);
        groups.clear();
        for (int i = 0; i < static_cast<int>(colors.size()); ++i) {
            groups.resize(std::max(groups.size(), static_cast<size_t>(colors[i] + 1)));
            groups[colors[i]].push_back(i);
        }
        const int nv = obj.nv();
        const int ne = static_cast<int>(obj.energies.size());
        adjacency.assign(nv, std::vector<std::vector<std::array<int, 2>>>(ne));
        for (int e = 0; e < ne; ++e) {
            const auto &E = obj.energies[e];
            const int S = stencil_size(E.type);
            for (int s = 0; s < static_cast<int>(E.stencils.size()); ++s)
                adjacency[E.stencils[s]][e].push_back({s / S, s % S});
        }
        // Before the first substep the inertial target is the current state (zero inertia).
        xInertial = obj.x;
        xOld = obj.x;
        prepared = true;
    }

    // vbd.cpp:46-83: store x_old, v += dt g, x += dt v, x_inertial = x
    void begin_substep(double h)
    {
        if (!prepared) prepare();
        xOld = obj.x;
        const int nv = obj.nv();
        for (int i = 0; i < nv; ++i)
            for (int a = 0; a < 3; ++a) {
                obj.v[3 * i + a] += h * g[a];
                obj.x[3 * i + a] += obj.v[3 * i + a] * h;
            }
        xInertial = obj.x;
    }

    // l_vertexDescent, vbd.cpp:100-147
    void vertex_descent(int vIdx, double invdtSquared)
    {
        const double mOverdtSquared = obj.m[vIdx] * invdtSquared;
        double f[3], H[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int a = 0; a < 3; ++a) f[a] = -mOverdtSquared * (obj.x[3 * vIdx + a] - xInertial[3 * vIdx + a]);
        H[0] = H[4] = H[8] = mOverdtSquared;
        for (int e = 0; e < static_cast<int>(obj.energies.size()); ++e) {
            const auto &E = obj.energies[e];
            const int S = stencil_size(E.type);
            const int P = param_count(E.type);
            for (const auto &ent : adjacency[vIdx][e]) {
                double ge[3], He[9];
                incidence_block(E.type, obj.x.data(), &E.stencils[S * ent[0]], &E.params[P * ent[0]], ent[1], mode, ge,
                                He);
                for (int a = 0; a < 3; ++a) f[a] += -ge[a];
                for (int a = 0; a < 9; ++a) H[a] += He[a];
            }
        }
        if (det3x3(H) > 1e-10) {
            double Hi[9];
            inverse3x3(H, Hi);
            for (int a = 0; a < 3; ++a)
                obj.x[3 * vIdx + a] += Hi[a * 3 + 0] * f[0] + Hi[a * 3 + 1] * f[1] + Hi[a * 3 + 2] * f[2];
        }
    }

    // vbd.cpp:90-169 (the colour loop with an OpenMP parallel-for per colour group)
    void iterate(int n, double h)
    {
        const double invdt = 1. / h;
        const double invdtSquared = invdt * invdt;
        for (int it = 0; it < n; ++it) {
            for (const auto &group : groups) {
                const int cnt = static_cast<int>(group.size());
#pragma omp parallel for schedule(static)
                for (int v = 0; v < cnt; ++v) vertex_descent(group[v], invdtSquared);
            }
        }
    }

    // vbd.cpp:174-185 -> ParticleGroup::computeIntegratedVelocities, particleGroup.cpp:65-72
    void end_substep(double h)
    {
        const double invdt = 1. / h;
        for (size_t i = 0; i < obj.x.size(); ++i) obj.v[i] = (obj.x[i] - xOld[i]) * invdt;
    }

    void step()
    {
        const double h = dt / substeps;
        for (int s = 0; s < substeps; ++s) {
            begin_substep(h);
            iterate(iterations, h);
            end_substep(h);
        }
    }

    // Gradient of the total potential (all energies) at the current positions, 3V.
    void energy_gradient(std::vector<double> &grad) const
    {
        const int nv = obj.nv();
        grad.assign(3 * nv, 0.0);
        for (int v = 0; v < nv; ++v) {
            for (int e = 0; e < static_cast<int>(obj.energies.size()); ++e) {
                const auto &E = obj.energies[e];
                const int S = stencil_size(E.type);
                const int P = param_count(E.type);
                for (const auto &ent : adjacency[v][e]) {
                    double ge[3], He[9];
                    incidence_block(E.type, obj.x.data(), &E.stencils[S * ent[0]], &E.params[P * ent[0]], ent[1],
                                    kVertexAD, ge, He);
                    for (int a = 0; a < 3; ++a) grad[3 * v + a] += ge[a];
                }
            }
        }
    }

    // Incremental-potential residual r = M/h^2 (x - y) + grad E(x) (FP64), per component.
    void residual(std::vector<double> &r, double h) const
    {
        energy_gradient(r);
        const double invdtSquared = 1.0 / (h * h);
        for (int v = 0; v < obj.nv(); ++v)
            for (int a = 0; a < 3; ++a)
                r[3 * v + a] += obj.m[v] * invdtSquared * (obj.x[3 * v + a] - xInertial[3 * v + a]);
    }
};

// ---------------------------------------------------------------------------------------
// XPBD solver: XPBD::step, computeParallelStencilGroups (spg/source/sim/solver/xpbd.cpp:16-160),
// StencilBlockEnergy::projectPosition (energy.h:117-153), SpringEnergy::projectPosition
// (springEnergy.cpp:48-68).
struct Xpbd {
    Object obj;
    double dt{0.01};
    int substeps{1};
    double g[3]{0, -9.8, 0};
    bool prepared{false};
    std::vector<std::vector<std::vector<int>>> groups;  // per energy, per colour
    std::vector<double> xOld;

    void prepare()
    {
        groups.clear();
        for (const auto &E : obj.energies) {
            const auto colors = color_stencils(E);
            std::vector<std::vector<int>> gs;
            for (int i = 0; i < static_cast<int>(colors.size()); ++i) {
                gs.resize(std::max(gs.size(), static_cast<size_t>(colors[i] + 1)));
                gs[colors[i]].push_back(i);
            }
            groups.push_back(std::move(gs));
        }
        prepared = true;
    }

    void project_spring(const EnergyBlock &E, int i, double h)
    {
        const int a = E.stencils[2 * i], b = E.stencils[2 * i + 1];
        const double w0 = obj.w[a], w1 = obj.w[b];
        const double wSum = w0 + w1;
        const double eps = 1.0e-6;
        if (wSum < eps) return;
        const double alphaTilde = E.params[3 * i + 2] / (h * h);
        double n[3];
        for (int k = 0; k < 3; ++k) n[k] = obj.x[3 * b + k] - obj.x[3 * a + k];
        const double d = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (d < eps) return;
        for (int k = 0; k < 3; ++k) n[k] = n[k] / d;
        const double s = (d - E.params[3 * i]) / (wSum + alphaTilde);
        for (int k = 0; k < 3; ++k) {
            const double corr = n[k] * s;
            obj.x[3 * a + k] += w0 * corr;
            obj.x[3 * b + k] -= w1 * corr;
        }
    }

    void project_generic(const EnergyBlock &E, int i, double h)
    {
        const int S = stencil_size(E.type);
        const int P = param_count(E.type);
        const int NC = n_constraints(E.type);
        const int *st = &E.stencils[S * i];
        const double *params = &E.params[P * i];
        V3<double> p[4];
        for (int j = 0; j < S; ++j) p[j] = V3<double>(obj.x[3 * st[j]], obj.x[3 * st[j] + 1], obj.x[3 * st[j] + 2]);
        double C[4], gradC[4 * 12];
        element_constraints(E.type, p, params, C, gradC);
        // Effective compliance matrix (NC x NC)
        double cmp[16] = {};
        if (E.type >= kStvkTet) {  // diagonal compliances of types 6-13 (parameter layouts above)
            const int off = (E.type == kStvkTet || E.type == kSsnh) ? 11
                            : E.type == kBwMembrane                 ? 7
                            : E.type == kChoi                       ? 8
                            : E.type == kQuadBending                ? 5
                                                                    : 2;
            for (int c = 0; c < NC; ++c) cmp[c * NC + c] = params[E.type == kQuadBending ? off : off + c];
        } else if (E.type == kStvk) {
            for (int k = 0; k < 9; ++k) cmp[k] = params[13 + k];
        } else if (E.type == kSnh) {
            cmp[0] = params[12];
            cmp[3] = params[13];
        } else if (E.type == kBending) {
            cmp[0] = params[2];
        } else if (E.type == kAnchor) {
            cmp[0] = params[4];
        } else {
            cmp[0] = params[2];
        }
        // WgradC and A = gradC^T W gradC + cmp / dt^2 + 1e-10 I
        double WgradC[4 * 12];
        for (int c = 0; c < NC; ++c)
            for (int j = 0; j < S; ++j)
                for (int a = 0; a < 3; ++a) WgradC[c * 3 * S + 3 * j + a] = obj.w[st[j]] * gradC[c * 3 * S + 3 * j + a];
        double A[16];
        for (int r = 0; r < NC; ++r)
            for (int c = 0; c < NC; ++c) {
                double acc = 0;
                for (int d = 0; d < 3 * S; ++d) acc += gradC[r * 3 * S + d] * WgradC[c * 3 * S + d];
                A[r * NC + c] = acc + cmp[r * NC + c] / (h * h) + (r == c ? 1e-10 : 0.0);
            }
        double Ai[16];
        if (NC == 1)
            Ai[0] = 1.0 / A[0];
        else if (NC == 2)
            inverse2x2(A, Ai);
        else if (NC == 3)
            inverse3x3(A, Ai);
        else
            inverse_gauss_jordan(A, Ai, NC);
        double dl[4];
        for (int r = 0; r < NC; ++r) {
            double acc = 0;
            for (int c = 0; c < NC; ++c) acc += Ai[r * NC + c] * C[c];
            dl[r] = -acc;
        }
        for (int j = 0; j < S; ++j)
            for (int a = 0; a < 3; ++a) {
                double acc = 0;
                for (int c = 0; c < NC; ++c) acc += WgradC[c * 3 * S + 3 * j + a] * dl[c];
                obj.x[3 * st[j] + a] += acc;
            }
    }

    void step()
    {
        if (!prepared) prepare();
        const double h = dt / substeps;
        const double invdt = 1 / h;
        const int nv = obj.nv();
        for (int s = 0; s < substeps; ++s) {
            xOld = obj.x;
            for (int i = 0; i < nv; ++i)
                for (int a = 0; a < 3; ++a) {
                    obj.v[3 * i + a] += h * g[a];
                    obj.x[3 * i + a] += obj.v[3 * i + a] * h;
                }
            for (size_t e = 0; e < obj.energies.size(); ++e) {
                const auto &E = obj.energies[e];
                for (const auto &group : groups[e]) {
                    const int cnt = static_cast<int>(group.size());
#pragma omp parallel for schedule(static)
                    for (int i = 0; i < cnt; ++i) {
                        if (E.type == kSpring)
                            project_spring(E, group[i], h);
                        else
                            project_generic(E, group[i], h);
                    }
                }
            }
            for (size_t i = 0; i < obj.x.size(); ++i) obj.v[i] = (obj.x[i] - xOld[i]) * invdt;
        }
    }
};

}  // namespace oracle

// =======================================================================================
// C API for the Python test harness (ctypes). Descriptor layout matches include/spgx.h.
using namespace oracle;

extern "C" {

struct oracle_energy_desc {
    int32_t type;
    int32_t n_stencils;
    const int32_t *stencils;
    const double *params;
};

struct oracle_object_desc {
    int32_t n_vertices;
    const double *x;
    const double *v;
    const double *mass;
    int32_t n_energies;
    const oracle_energy_desc *energies;
};

const char *oracle_last_error() { return g_error.c_str(); }

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int oracle_max_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// ---- builders -> Object handles --------------------------------------------------------
void *oracle_build_cloth(double mass, float width, float height, int rows, int cols, double young, double poisson,
                         double bendK, double anchorK, int restInitial, int nAnchors, const int *anchorIds)
{
    try {
        std::vector<int> ids;
        if (nAnchors < 0)
            ids = {0, rows - 1};
        else
            ids.assign(anchorIds, anchorIds + nAnchors);
        return new Object(create_cloth(mass, width, height, rows, cols, young, poisson, bendK, anchorK, ids, restInitial != 0));
    } catch (const std::exception &e) {
        g_error = e.what();
        return nullptr;
    }
}

void *oracle_build_spring_cloth(double mass, float width, float height, int rows, int cols, double springK,
                                double bendK, double anchorK, double jitterFrac, uint64_t seed)
{
    try {
        return new Object(create_spring_cloth(mass, width, height, rows, cols, springK, bendK, anchorK, jitterFrac, seed));
    } catch (const std::exception &e) {
        g_error = e.what();
        return nullptr;
    }
}

void *oracle_build_tet_beam(double mass, float sx, float sy, float sz, int nx, int ny, int nz, double young,
                            double poisson, double anchorK, int split)
{
    try {
        return new Object(create_tet_beam(mass, sx, sy, sz, nx, ny, nz, young, poisson, anchorK, split));
    } catch (const std::exception &e) {
        g_error = e.what();
        return nullptr;
    }
}

// Batch of independent square patches (batched-solve benchmark scene): per patch, in this
// draw order from one splitmix64 stream: side vertex count n ~ U{nMin..nMax}, mu, lambda
// ~ logU[muLo, muHi], bending k ~ logU[kbLo, kbHi], anchored corner ~ U{0..3}. Each patch is a
// 1 m cloth (createCloth layout) with total mass `mass`, flat rest state and one anchor.
int oracle_build_patch_batch(int nPatches, int nMin, int nMax, double muLo, double muHi, double kbLo, double kbHi,
                             double mass, double anchorK, uint64_t seed, void **out)
{
    try {
        SplitMix64 rng{seed};
        for (int p = 0; p < nPatches; ++p) {
            const int n = nMin + static_cast<int>(rng.next() % static_cast<uint64_t>(nMax - nMin + 1));
            const double mu = std::exp(std::log(muLo) + rng.uniform() * (std::log(muHi) - std::log(muLo)));
            const double lam = std::exp(std::log(muLo) + rng.uniform() * (std::log(muHi) - std::log(muLo)));
            const double kb = std::exp(std::log(kbLo) + rng.uniform() * (std::log(kbHi) - std::log(kbLo)));
            const int corner = static_cast<int>(rng.next() % 4);
            const int cornerIds[4] = {0, n - 1, n * (n - 1), n * n - 1};
            const double poisson = lam / (2 * mu + lam);
            const double young = (2 * mu + lam) * (1 - poisson * poisson);
            out[p] = new Object(create_cloth(mass, 1.0f, 1.0f, n, n, young, poisson, kb, anchorK, {cornerIds[corner]}, true));
        }
        return 0;
    } catch (const std::exception &e) {
        g_error = e.what();
        return 1;
    }
}

void oracle_object_free(void *h) { delete static_cast<Object *>(h); }
int oracle_object_nv(void *h) { return static_cast<Object *>(h)->nv(); }
int oracle_object_n_energies(void *h) { return static_cast<int>(static_cast<Object *>(h)->energies.size()); }
void oracle_object_arrays(void *h, const double **x, const double **x0, const double **v, const double **m)
{
    auto *o = static_cast<Object *>(h);
    *x = o->x.data();
    *x0 = o->x0.data();
    *v = o->v.data();
    *m = o->m.data();
}
void oracle_object_energy(void *h, int e, int *type, int *n, const int **stencils, const double **params)
{
    auto *o = static_cast<Object *>(h);
    const auto &E = o->energies[e];
    *type = E.type;
    *n = E.n();
    *stencils = E.stencils.data();
    *params = E.params.data();
}

// ---- solvers on a descriptor ---------------------------------------------------------
static Object object_from_desc(const oracle_object_desc *d)
{
    Object o;
    const int nv = d->n_vertices;
    o.x.assign(d->x, d->x + 3 * nv);
    o.x0 = o.x;
    if (d->v)
        o.v.assign(d->v, d->v + 3 * nv);
    else
        o.v.assign(3 * nv, 0.0);
    o.m.assign(d->mass, d->mass + nv);
    o.w.resize(nv);
    for (int i = 0; i < nv; ++i) o.w[i] = o.m[i] == 0 ? 0 : 1 / o.m[i];
    for (int e = 0; e < d->n_energies; ++e) {
        const auto &ed = d->energies[e];
        EnergyBlock E;
        E.type = ed.type;
        const int S = stencil_size(E.type), P = param_count(E.type);
        if (S == 0) throw std::runtime_error("unsupported energy type");
        E.stencils.assign(ed.stencils, ed.stencils + S * ed.n_stencils);
        E.params.assign(ed.params, ed.params + P * ed.n_stencils);
        for (int s : E.stencils)
            if (s < 0 || s >= nv) throw std::runtime_error("stencil index out of range");
        o.energies.push_back(std::move(E));
    }
    return o;
}

void *oracle_vbd_create(const oracle_object_desc *d, double dt, int substeps, int iterations, const double *g, int mode)
{
    try {
        auto *s = new Vbd();
        s->obj = object_from_desc(d);
        s->dt = dt;
        s->substeps = substeps;
        s->iterations = iterations;
        for (int a = 0; a < 3; ++a) s->g[a] = g[a];
        s->mode = mode;
        s->prepare();
        return s;
    } catch (const std::exception &e) {
        g_error = e.what();
        return nullptr;
    }
}
void oracle_vbd_free(void *h) { delete static_cast<Vbd *>(h); }
void oracle_vbd_set_mode(void *h, int mode) { static_cast<Vbd *>(h)->mode = mode; }
void oracle_vbd_step(void *h) { static_cast<Vbd *>(h)->step(); }
void oracle_vbd_begin_substep(void *h)
{
    auto *s = static_cast<Vbd *>(h);
    s->begin_substep(s->dt / s->substeps);
}
void oracle_vbd_iterate(void *h, int n)
{
    auto *s = static_cast<Vbd *>(h);
    s->iterate(n, s->dt / s->substeps);
}
// Runs the vertex descent of one colour group only (for bounded CPU-baseline samples).
void oracle_vbd_iterate_color(void *h, int color)
{
    auto *s = static_cast<Vbd *>(h);
    const double hh = s->dt / s->substeps;
    const double invdt2 = 1.0 / (hh * hh);
    const auto &group = s->groups[color];
    const int cnt = static_cast<int>(group.size());
#pragma omp parallel for schedule(static)
    for (int v = 0; v < cnt; ++v) s->vertex_descent(group[v], invdt2);
}
void oracle_vbd_end_substep(void *h)
{
    auto *s = static_cast<Vbd *>(h);
    s->end_substep(s->dt / s->substeps);
}
void oracle_vbd_get_state(void *h, double *x, double *v)
{
    auto *s = static_cast<Vbd *>(h);
    if (x) std::memcpy(x, s->obj.x.data(), sizeof(double) * s->obj.x.size());
    if (v) std::memcpy(v, s->obj.v.data(), sizeof(double) * s->obj.v.size());
}
void oracle_vbd_set_state(void *h, const double *x, const double *v)
{
    auto *s = static_cast<Vbd *>(h);
    if (x) std::memcpy(s->obj.x.data(), x, sizeof(double) * s->obj.x.size());
    if (v) std::memcpy(s->obj.v.data(), v, sizeof(double) * s->obj.v.size());
}
void oracle_vbd_get_inertial(void *h, double *y)
{
    auto *s = static_cast<Vbd *>(h);
    std::memcpy(y, s->xInertial.data(), sizeof(double) * s->xInertial.size());
}
int oracle_vbd_n_colors(void *h) { return static_cast<int>(static_cast<Vbd *>(h)->groups.size()); }
int oracle_vbd_color_size(void *h, int c) { return static_cast<int>(static_cast<Vbd *>(h)->groups[c].size()); }
void oracle_vbd_colors(void *h, int *out)
{
    auto *s = static_cast<Vbd *>(h);
    std::copy(s->colors.begin(), s->colors.end(), out);
}
// Adjacency export: counts[v * nE + e] and, in the same (v, e) order, (stencil, slot) pairs.
long long oracle_vbd_adjacency_size(void *h)
{
    auto *s = static_cast<Vbd *>(h);
    long long n = 0;
    for (const auto &pv : s->adjacency)
        for (const auto &pe : pv) n += static_cast<long long>(pe.size());
    return n;
}
void oracle_vbd_adjacency(void *h, int *counts, int *entries)
{
    auto *s = static_cast<Vbd *>(h);
    long long k = 0;
    int c = 0;
    for (const auto &pv : s->adjacency)
        for (const auto &pe : pv) {
            counts[c++] = static_cast<int>(pe.size());
            for (const auto &en : pe) {
                entries[2 * k] = en[0];
                entries[2 * k + 1] = en[1];
                ++k;
            }
        }
}
// Residual norm ||M/h^2 (x - y) + grad E(x)||_2 at the current state against the current
// inertial target y; optionally the per-component residual.
double oracle_vbd_residual(void *h, double *out)
{
    auto *s = static_cast<Vbd *>(h);
    std::vector<double> r;
    s->residual(r, s->dt / s->substeps);
    double acc = 0;
    for (double q : r) acc += q * q;
    if (out) std::memcpy(out, r.data(), sizeof(double) * r.size());
    return std::sqrt(acc);
}

void *oracle_xpbd_create(const oracle_object_desc *d, double dt, int substeps, const double *g)
{
    try {
        auto *s = new Xpbd();
        s->obj = object_from_desc(d);
        s->dt = dt;
        s->substeps = substeps;
        for (int a = 0; a < 3; ++a) s->g[a] = g[a];
        s->prepare();
        return s;
    } catch (const std::exception &e) {
        g_error = e.what();
        return nullptr;
    }
}
void oracle_xpbd_free(void *h) { delete static_cast<Xpbd *>(h); }
void oracle_xpbd_step(void *h) { static_cast<Xpbd *>(h)->step(); }
void oracle_xpbd_get_state(void *h, double *x, double *v)
{
    auto *s = static_cast<Xpbd *>(h);
    if (x) std::memcpy(x, s->obj.x.data(), sizeof(double) * s->obj.x.size());
    if (v) std::memcpy(v, s->obj.v.data(), sizeof(double) * s->obj.v.size());
}
int oracle_xpbd_n_groups(void *h, int e) { return static_cast<int>(static_cast<Xpbd *>(h)->groups[e].size()); }
void oracle_xpbd_stencil_colors(void *h, int e, int *out)
{
    auto *s = static_cast<Xpbd *>(h);
    const auto &gs = s->groups[e];
    for (int c = 0; c < static_cast<int>(gs.size()); ++c)
        for (int i : gs[c]) out[i] = c;
}

// ---- element-level evaluation -----------------------------------------------------------
// X: 3*S positions of the stencil's vertices (in stencil order), params: one stencil's
// parameters. Returns the slot's gradient segment (3) and Hessian block (9, row-major).
int oracle_element_block(int type, const double *X, const double *params, int slot, int mode, double *g, double *H)
{
    try {
        const int S = stencil_size(type);
        std::vector<int> st(S);
        for (int j = 0; j < S; ++j) st[j] = j;
        incidence_block(type, X, st.data(), params, slot, mode, g, H);
        return 0;
    } catch (const std::exception &e) {
        g_error = e.what();
        return 1;
    }
}

double oracle_element_energy(int type, const double *X, const double *params)
{
    const int S = stencil_size(type);
    V3<double> p[4];
    for (int j = 0; j < S; ++j) p[j] = V3<double>(X[3 * j], X[3 * j + 1], X[3 * j + 2]);
    return element_energy(type, p, params);
}

// Full element gradient (3S) and dense Hessian (3S x 3S) on the AD scalar (reference path).
int oracle_element_full(int type, const double *X, const double *params, double *grad, double *hess)
{
    const int S = stencil_size(type);
    if (S == 0) return 1;
    for (int slot = 0; slot < S; ++slot) {
        double g[3], H[9];
        oracle_element_block(type, X, params, slot, kFullAD, g, H);
        for (int a = 0; a < 3; ++a) grad[3 * slot + a] = g[a];
    }
    // Dense Hessian through the AD scalar seeded on all dofs.
    auto fill = [&](auto fn, auto sz) {
        constexpr int SS = decltype(sz)::value;
        using D = Dual<3 * SS, true>;
        V3<D> q[SS];
        for (int j = 0; j < SS; ++j)
            for (int a = 0; a < 3; ++a) q[j][a] = D(X[3 * j + a], 3 * j + a);
        const D e = fn(q, params);
        for (int i = 0; i < 3 * SS; ++i)
            for (int j = 0; j < 3 * SS; ++j) hess[i * 3 * SS + j] = e.H(i, j);
    };
    switch (type) {
    case kSpring: fill([](const auto *q, const double *pp) { return spring_energy(q, pp); }, std::integral_constant<int, 2>{}); break;
    case kAnchor: fill([](const auto *q, const double *pp) { return anchor_energy(q, pp); }, std::integral_constant<int, 1>{}); break;
    case kBending: fill([](const auto *q, const double *pp) { return bending_energy(q, pp); }, std::integral_constant<int, 4>{}); break;
    case kStvk: fill([](const auto *q, const double *pp) { return stvk_energy(q, pp); }, std::integral_constant<int, 3>{}); break;
    case kSnh: fill([](const auto *q, const double *pp) { return snh_energy(q, pp); }, std::integral_constant<int, 4>{}); break;
    case kStvkTet: fill([](const auto *q, const double *pp) { return stvk_tet_energy(q, pp); }, std::integral_constant<int, 4>{}); break;
    case kSsnh: fill([](const auto *q, const double *pp) { return ssnh_energy(q, pp); }, std::integral_constant<int, 4>{}); break;
    case kBwMembrane: fill([](const auto *q, const double *pp) { return bw_membrane_energy(q, pp); }, std::integral_constant<int, 3>{}); break;
    case kChoi: fill([](const auto *q, const double *pp) { return choi_energy(q, pp); }, std::integral_constant<int, 3>{}); break;
    case kBwBending: fill([](const auto *q, const double *pp) { return bw_bending_energy(q, pp); }, std::integral_constant<int, 4>{}); break;
    case kQuadBending: fill([](const auto *q, const double *pp) { return quad_bending_energy(q, pp); }, std::integral_constant<int, 4>{}); break;
    case kSpringCont: fill([](const auto *q, const double *pp) { return spring_cont_energy(q, pp); }, std::integral_constant<int, 2>{}); break;
    case kSpringSqCont: fill([](const auto *q, const double *pp) { return spring_sq_cont_energy(q, pp); }, std::integral_constant<int, 2>{}); break;
    case kStaticLoad: fill([](const auto *q, const double *pp) { return static_load_energy(q, pp); }, std::integral_constant<int, 1>{}); break;
    default: return 1;
    }
    return 0;
}

// Constraint values and their gradients (column-major, 3S per constraint).
int oracle_element_constraints(int type, const double *X, const double *params, double *C, double *gradC)
{
    const int S = stencil_size(type);
    if (S == 0) return 1;
    V3<double> p[4];
    for (int j = 0; j < S; ++j) p[j] = V3<double>(X[3 * j], X[3 * j + 1], X[3 * j + 2]);
    element_constraints(type, p, params, C, gradC);
    return 0;
}

int oracle_n_constraints(int type) { return n_constraints(type); }

// Literal greedy colouring of an arbitrary object (graphColoring.cpp:72-84).
int oracle_color_vertices(const oracle_object_desc *d, int *out)
{
    try {
        const Object o = object_from_desc(d);
        const auto c = color_vertices(o);
        std::copy(c.begin(), c.end(), out);
        return 0;
    } catch (const std::exception &e) {
        g_error = e.what();
        return 1;
    }
}

}  // extern "C"
