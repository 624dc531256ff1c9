// Headless scene builders (see spg/scenes.h).
#include "spg/scenes.h"

#include <cmath>
#include <memory>
#include <stdexcept>

namespace spg::scenes {

namespace {

struct SplitMix64 {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // Uniform in (0, 1) from the top 53 bits.
    double uniform() { return (double(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
};

double signedAreaXY(const std::vector<Vector3> &P, const Int3 &f)
{
    const double ax = P[f[1]].x() - P[f[0]].x(), ay = P[f[1]].y() - P[f[0]].y();
    const double bx = P[f[2]].x() - P[f[0]].x(), by = P[f[2]].y() - P[f[0]].y();
    return 0.5 * (ax * by - ay * bx);
}

void jitterRestPositions(std::vector<Vector3> &P, const std::vector<Int3> &faces, double sigma, uint64_t seed)
{
    const int nv = static_cast<int>(P.size());
    std::vector<std::vector<int>> vertexFaces(nv);
    for (int f = 0; f < static_cast<int>(faces.size()); ++f)
        for (int k = 0; k < 3; ++k) vertexFaces[faces[f][k]].push_back(f);
    std::vector<double> nominal(faces.size());
    for (size_t f = 0; f < faces.size(); ++f) nominal[f] = signedAreaXY(P, faces[f]);
    SplitMix64 rng{seed};
    const double twoPi = 6.283185307179586;
    for (int v = 0; v < nv; ++v) {
        const double bx = P[v].x(), by = P[v].y();
        bool accepted = false;
        for (int attempt = 0; attempt < 64 && !accepted; ++attempt) {
            const double u1 = rng.uniform(), u2 = rng.uniform();
            const double r = std::sqrt(-2.0 * std::log(u1));
            P[v][0] = bx + sigma * (r * std::cos(twoPi * u2));
            P[v][1] = by + sigma * (r * std::sin(twoPi * u2));
            accepted = true;
            for (int f : vertexFaces[v])
                if (signedAreaXY(P, faces[f]) < 0.1 * nominal[f]) accepted = false;
        }
        if (!accepted) {
            P[v][0] = bx;
            P[v][1] = by;
        }
    }
}

// Lumped masses: a third of each rest triangle's area (solverCompare.cpp:383-400).
void addClothParticles(ParticleGroup &pGroup, const TriangleMesh &mesh, Real mass, bool restInitial)
{
    const auto &V = mesh.vertices();
    const auto &V0 = mesh.vertices0();
    std::vector<Real> particleAreas(V.size(), 0);
    Real totalArea = 0;
    for (const auto &face : mesh.faces()) {
        const Vector3 e0 = V0[face[1]] - V0[face[0]];
        const Vector3 e3 = V0[face[2]] - V0[face[1]];
        const Real area = 0.5 * (e0.cross(e3).norm());
        totalArea += area;
        for (int k = 0; k < 3; ++k) particleAreas[face[k]] += area / 3.0;
    }
    const Real density = mass / totalArea;
    for (size_t i = 0; i < V.size(); ++i) pGroup.addParticle(restInitial ? V0[i] : V[i], V0[i], particleAreas[i] * density);
}

// Bending stencils on edges with two opposing vertices (solverCompare.cpp:441-452).
std::shared_ptr<DiscreteBendingEnergy> clothBending(const TriangleMesh &mesh, Real stiffness)
{
    auto bending = std::make_shared<DiscreteBendingEnergy>();
    const auto &edges = mesh.edges();
    const auto &opp = mesh.opposingVerticesPerEdge();
    for (size_t i = 0; i < edges.size(); ++i)
        if (opp[i].size() == 2)
            bending->addStencil({edges[i][0], edges[i][1], opp[i][0].vertexId, opp[i][1].vertexId}, 0., stiffness);
    return bending;
}

Real tetrahedralVolume(const Vector3 &x0, const Vector3 &x1, const Vector3 &x2, const Vector3 &x3)
{
    Matrix3 M;
    for (int a = 0; a < 3; ++a) {
        M(a, 0) = x1[a] - x0[a];
        M(a, 1) = x2[a] - x0[a];
        M(a, 2) = x3[a] - x0[a];
    }
    return determinant(M) / 6.0;
}

}  // namespace

TriangleMesh buildTriangleSquareMesh(float width, float height, int rows, int cols)
{
    std::vector<Vector3> vertices, vertices0;
    std::vector<Int3> faces;
    const float rowStep = height / (rows - 1);
    const float colStep = width / (cols - 1);
    for (int row = 0; row < rows; ++row)
        for (int col = 0; col < cols; ++col) {
            vertices0.push_back({double(colStep * col), double(rowStep * row), 0.0});
            vertices.push_back({double(colStep * col), 0.0, double(-rowStep * row)});
            if (row != 0 && col != 0) {
                if ((row + col) % 2 == 0) {
                    faces.push_back({row * cols + col - 1, (row - 1) * cols + col - 1, (row - 1) * cols + col});
                    faces.push_back({row * cols + col - 1, (row - 1) * cols + col, row * cols + col});
                } else {
                    faces.push_back({(row - 1) * cols + col - 1, row * cols + col, row * cols + col - 1});
                    faces.push_back({(row - 1) * cols + col - 1, (row - 1) * cols + col, row * cols + col});
                }
            }
        }
    return TriangleMesh(vertices, vertices0, faces);
}

ParticleGroup createCloth(Real mass, float width, float height, int rows, int cols, Real young, Real poisson,
                          Real bendingStiffness, Real anchorStiffness, const std::vector<int> &anchorIds,
                          bool restInitial)
{
    const TriangleMesh mesh = buildTriangleSquareMesh(width, height, rows, cols);
    ParticleGroup pGroup;
    addClothParticles(pGroup, mesh, mass, restInitial);
    auto anchors = std::make_shared<SpringAnchorEnergy>();
    for (int id : anchorIds) anchors->addStencil({id}, pGroup.positions()[id], anchorStiffness);
    auto bending = clothBending(mesh, bendingStiffness);
    pGroup.addEnergy(bending);
    bending->preparePrecomputations(pGroup);
    auto membrane = std::make_shared<MembraneStvkEnergy>();
    for (const auto &f : mesh.faces()) membrane->addStencil({f[0], f[1], f[2]}, young, poisson);
    pGroup.addEnergy(membrane);
    membrane->preparePrecomputations(pGroup);
    pGroup.addEnergy(anchors);
    return pGroup;
}

ParticleGroup createSpringCloth(Real mass, float width, float height, int rows, int cols, Real springStiffness,
                                Real bendingStiffness, Real anchorStiffness, Real jitter, uint64_t seed)
{
    const TriangleMesh grid = buildTriangleSquareMesh(width, height, rows, cols);
    std::vector<Vector3> rest = grid.vertices0();
    if (jitter > 0) jitterRestPositions(rest, grid.faces(), jitter * (double(width) / (cols - 1)), seed);
    const TriangleMesh mesh(rest, rest, grid.faces());
    ParticleGroup pGroup;
    addClothParticles(pGroup, mesh, mass, true);
    auto bending = clothBending(mesh, bendingStiffness);
    pGroup.addEnergy(bending);
    bending->preparePrecomputations(pGroup);
    auto springs = std::make_shared<SpringEnergy>();
    for (const auto &e : mesh.edges())
        springs->addStencil({e[0], e[1]}, (pGroup.positions0()[e[0]] - pGroup.positions0()[e[1]]).norm(),
                            springStiffness);
    pGroup.addEnergy(springs);
    auto anchors = std::make_shared<SpringAnchorEnergy>();
    for (int id = 0; id < cols; ++id) anchors->addStencil({id}, pGroup.positions()[id], anchorStiffness);
    pGroup.addEnergy(anchors);
    return pGroup;
}

ParticleGroup createTetrahedralBeam(Real mass, float sx, float sy, float sz, int nx, int ny, int nz, Real young,
                                    Real poisson, Real anchorStiffness, int split)
{
    if (split != 5 && split != 6) throw std::runtime_error("beam split must be 5 or 6 tets per cell");
    std::vector<Vector3> vertices;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k)
                vertices.push_back({double(-sx * 0.5f + i * sx / (nx - 1)), double(-sy * 0.5f + j * sy / (ny - 1)),
                                    double(-sz * 0.5f + k * sz / (nz - 1))});
    auto id = [ny, nz](int i, int j, int k) { return i * ny * nz + j * nz + k; };
    auto positive = [&vertices](int a, int b, int c, int d) -> Int4 {
        if (tetrahedralVolume(vertices[a], vertices[b], vertices[c], vertices[d]) > 0) return {a, b, c, d};
        return {b, a, c, d};
    };
    std::vector<Int4> tets;
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < ny - 1; ++j)
            for (int k = 0; k < nz - 1; ++k) {
                if (split == 5) {
                    int c[8] = {id(i, j, k),         id(i + 1, j, k),     id(i, j, k + 1),     id(i + 1, j, k + 1),
                                id(i, j + 1, k),     id(i + 1, j + 1, k), id(i, j + 1, k + 1), id(i + 1, j + 1, k + 1)};
                    if (i % 2 == 1) {
                        std::swap(c[0], c[1]);
                        std::swap(c[2], c[3]);
                        std::swap(c[4], c[5]);
                        std::swap(c[6], c[7]);
                    }
                    if (j % 2 == 1) {
                        std::swap(c[0], c[4]);
                        std::swap(c[1], c[5]);
                        std::swap(c[2], c[6]);
                        std::swap(c[3], c[7]);
                    }
                    if (k % 2 == 1) {
                        std::swap(c[0], c[2]);
                        std::swap(c[1], c[3]);
                        std::swap(c[4], c[6]);
                        std::swap(c[5], c[7]);
                    }
                    tets.push_back(positive(c[0], c[2], c[3], c[6]));
                    tets.push_back(positive(c[6], c[7], c[3], c[5]));
                    tets.push_back(positive(c[3], c[1], c[0], c[5]));
                    tets.push_back(positive(c[0], c[4], c[6], c[5]));
                    tets.push_back(positive(c[6], c[3], c[5], c[0]));
                } else {
                    static const int orders[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
                    for (const auto &o : orders) {
                        int d[3] = {0, 0, 0};
                        int t[4];
                        t[0] = id(i, j, k);
                        for (int s = 0; s < 3; ++s) {
                            d[o[s]] = 1;
                            t[s + 1] = id(i + d[0], j + d[1], k + d[2]);
                        }
                        tets.push_back(positive(t[0], t[1], t[2], t[3]));
                    }
                }
            }
    const TetrahedralMesh mesh(vertices, vertices, tets);
    std::vector<Real> volumes(vertices.size(), 0);
    Real totalVolume = 0;
    for (const auto &t : tets) {
        const Real v = tetrahedralVolume(vertices[t[0]], vertices[t[1]], vertices[t[2]], vertices[t[3]]);
        totalVolume += v;
        for (int k = 0; k < 4; ++k) volumes[t[k]] += v / 4.0;
    }
    const Real density = mass / totalVolume;
    ParticleGroup pGroup;
    for (size_t i = 0; i < vertices.size(); ++i) pGroup.addParticle(vertices[i], vertices[i], volumes[i] * density);
    auto anchors = std::make_shared<SpringAnchorEnergy>();
    for (int j = 0; j < ny; ++j)
        for (int k = 0; k < nz; ++k) anchors->addStencil({id(0, j, k)}, pGroup.positions0()[id(0, j, k)], anchorStiffness);
    auto snh = std::make_shared<StableNeoHookeanEnergy>();
    for (const auto &t : mesh.tets()) snh->addStencil(t, young, poisson);
    pGroup.addEnergy(anchors);
    pGroup.addEnergy(snh);
    snh->preparePrecomputations(pGroup);
    return pGroup;
}

ParticleGroup createTriangleMeshShell(const std::vector<Vector3> &vertices, const std::vector<Int3> &faces, Real mass,
                                      Real springStiffness, Real bendingStiffness, Real anchorStiffness,
                                      const std::vector<int> &anchorIds)
{
    const TriangleMesh mesh(vertices, vertices, faces);
    ParticleGroup pGroup;
    addClothParticles(pGroup, mesh, mass, true);
    auto bending = clothBending(mesh, bendingStiffness);
    pGroup.addEnergy(bending);
    bending->preparePrecomputations(pGroup);
    auto springs = std::make_shared<SpringEnergy>();
    for (const auto &e : mesh.edges())
        springs->addStencil({e[0], e[1]}, (pGroup.positions0()[e[0]] - pGroup.positions0()[e[1]]).norm(),
                            springStiffness);
    pGroup.addEnergy(springs);
    auto anchors = std::make_shared<SpringAnchorEnergy>();
    for (int id : anchorIds) anchors->addStencil({id}, pGroup.positions()[id], anchorStiffness);
    pGroup.addEnergy(anchors);
    return pGroup;
}

ParticleGroup createTetMeshSolid(const std::vector<Vector3> &vertices, const std::vector<Int4> &tets, Real mass,
                                 Real young, Real poisson, Real anchorStiffness, const std::vector<int> &anchorIds)
{
    const TetrahedralMesh mesh(vertices, vertices, tets);
    std::vector<Real> volumes(vertices.size(), 0);
    Real totalVolume = 0;
    for (const auto &t : tets) {
        const Real v = tetrahedralVolume(vertices[t[0]], vertices[t[1]], vertices[t[2]], vertices[t[3]]);
        totalVolume += v;
        for (int k = 0; k < 4; ++k) volumes[t[k]] += v / 4.0;
    }
    const Real density = mass / totalVolume;
    ParticleGroup pGroup;
    for (size_t i = 0; i < vertices.size(); ++i) pGroup.addParticle(vertices[i], vertices[i], volumes[i] * density);
    auto anchors = std::make_shared<SpringAnchorEnergy>();
    for (int id : anchorIds) anchors->addStencil({id}, pGroup.positions0()[id], anchorStiffness);
    auto snh = std::make_shared<StableNeoHookeanEnergy>();
    for (const auto &t : mesh.tets()) snh->addStencil(t, young, poisson);
    pGroup.addEnergy(anchors);
    pGroup.addEnergy(snh);
    snh->preparePrecomputations(pGroup);
    return pGroup;
}

std::vector<ParticleGroup> createPatchBatch(int nPatches, int nMin, int nMax, Real muLo, Real muHi, Real kbLo,
                                            Real kbHi, Real mass, Real anchorStiffness, uint64_t seed)
{
    SplitMix64 rng{seed};
    std::vector<ParticleGroup> out;
    out.reserve(nPatches);
    for (int p = 0; p < nPatches; ++p) {
        const int n = nMin + static_cast<int>(rng.next() % static_cast<uint64_t>(nMax - nMin + 1));
        const Real mu = std::exp(std::log(muLo) + rng.uniform() * (std::log(muHi) - std::log(muLo)));
        const Real lam = std::exp(std::log(muLo) + rng.uniform() * (std::log(muHi) - std::log(muLo)));
        const Real kb = std::exp(std::log(kbLo) + rng.uniform() * (std::log(kbHi) - std::log(kbLo)));
        const int corner = static_cast<int>(rng.next() % 4);
        const int cornerIds[4] = {0, n - 1, n * (n - 1), n * n - 1};
        const Real poisson = lam / (2 * mu + lam);
        const Real young = (2 * mu + lam) * (1 - poisson * poisson);
        out.push_back(createCloth(mass, 1.0f, 1.0f, n, n, young, poisson, kb, anchorStiffness, {cornerIds[corner]}, true));
    }
    return out;
}

}  // namespace spg::scenes
