// spg::TriangleMesh with the reference's interface (spg/include/spg/geom/triangleMesh.h:8-67):
// validated faces, the unique edge list in lexicographic (min, max) order and, per edge, its
// opposing vertices in face order. Built by sorting (edge, face, corner) records instead of a
// std::map; the order is the same.
#pragma once

#include <algorithm>
#include <stdexcept>
#include <vector>

#include "spg/types.h"

namespace spg {

class TriangleMesh {
public:
    struct OpposingVertex {
        int triangleId;
        int vertexId;
    };

    TriangleMesh(const std::vector<Vector3> &vertices, const std::vector<Vector3> &vertices0,
                 const std::vector<Int3> &faces)
        : m_vertices(vertices), m_vertices0(vertices0), m_faces(faces)
    {
        const int nV = static_cast<int>(m_vertices.size());
        for (const auto &f : m_faces)
            for (int i : f)
                if (i < 0 || i >= nV) throw std::runtime_error("Triangle mesh face contains index to invalid vertex");
        for (const auto &f : m_faces)
            if (f[0] == f[1] || f[1] == f[2] || f[2] == f[0])
                throw std::runtime_error("Triangle mesh face contains repeated vertex index");
        struct Rec {
            int a, b, face, opp;
        };
        std::vector<Rec> recs;
        recs.reserve(3 * m_faces.size());
        for (int f = 0; f < static_cast<int>(m_faces.size()); ++f)
            for (int i = 0; i < 3; ++i) {
                const int id0 = m_faces[f][i], id1 = m_faces[f][(i + 1) % 3], id2 = m_faces[f][(i + 2) % 3];
                recs.push_back({std::min(id0, id1), std::max(id0, id1), f, id2});
            }
        std::stable_sort(recs.begin(), recs.end(), [](const Rec &x, const Rec &y) {
            return x.a != y.a ? x.a < y.a : x.b < y.b;
        });
        for (size_t k = 0; k < recs.size(); ++k) {
            if (k == 0 || recs[k].a != recs[k - 1].a || recs[k].b != recs[k - 1].b) {
                m_edges.push_back({recs[k].a, recs[k].b});
                m_opposingVerticesPerEdge.emplace_back();
            }
            m_opposingVerticesPerEdge.back().push_back({recs[k].face, recs[k].opp});
        }
    }
    const std::vector<Vector3> &vertices() const { return m_vertices; }
    const std::vector<Vector3> &vertices0() const { return m_vertices0; }
    const std::vector<Int3> &faces() const { return m_faces; }
    const std::vector<Int2> &edges() const { return m_edges; }
    const std::vector<std::vector<OpposingVertex>> &opposingVerticesPerEdge() const { return m_opposingVerticesPerEdge; }

protected:
    std::vector<Vector3> m_vertices, m_vertices0;
    std::vector<Int3> m_faces;
    std::vector<Int2> m_edges;
    std::vector<std::vector<OpposingVertex>> m_opposingVerticesPerEdge;
};

// spg::TetrahedralMesh (spg/include/spg/geom/tetrahedralMesh.h:8-58): validated tets and the
// sorted unique edge list.
class TetrahedralMesh {
public:
    TetrahedralMesh(const std::vector<Vector3> &vertices, const std::vector<Vector3> &vertices0,
                    const std::vector<Int4> &tets)
        : m_vertices(vertices), m_vertices0(vertices0), m_tets(tets)
    {
        const int nV = static_cast<int>(m_vertices.size());
        for (const auto &t : m_tets)
            for (int i : t)
                if (i < 0 || i >= nV) throw std::runtime_error("Tetrahedral mesh cell contains index to invalid vertex");
        for (const auto &t : m_tets)
            if (t[0] == t[1] || t[0] == t[2] || t[0] == t[3] || t[1] == t[2] || t[1] == t[3] || t[2] == t[3])
                throw std::runtime_error("Tetrahedral mesh cell contains repeated vertex index");
        for (const auto &t : m_tets)
            for (int i = 0; i < 3; ++i)
                for (int j = i + 1; j < 4; ++j) m_edges.push_back({std::min(t[i], t[j]), std::max(t[i], t[j])});
        std::sort(m_edges.begin(), m_edges.end());
        m_edges.erase(std::unique(m_edges.begin(), m_edges.end()), m_edges.end());
    }
    const std::vector<Vector3> &vertices() const { return m_vertices; }
    const std::vector<Vector3> &vertices0() const { return m_vertices0; }
    const std::vector<Int4> &tets() const { return m_tets; }
    const std::vector<Int2> &edges() const { return m_edges; }

protected:
    std::vector<Vector3> m_vertices, m_vertices0;
    std::vector<Int4> m_tets;
    std::vector<Int2> m_edges;
};

}  // namespace spg
