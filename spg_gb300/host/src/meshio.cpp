// Mesh input: Wavefront OBJ and Gmsh MSH readers behind spg::io::loadObj / spg::io::loadMsh
// (spg/source/geom/io/obj.cpp, msh.cpp) and the C ABI spgx_load_obj / spgx_load_msh.
//
// The reference reads OBJ files with tinyobjloader and MSH files with MshIO. Both are git
// submodules whose commits are not recorded in the checkout, so no version is pinned. The
// readers below restate the published behaviour of those libraries that loadObj and loadMsh
// consume.
//
// OBJ (tinyobjloader's LoadObj with its defaults: triangulate on, real_t = float):
//  - "v x y z" adds a vertex. Coordinates are stored as float; loadObj widens them to double.
//  - "f" corners are v, v/vt, v//vn or v/vt/vn. Indices are 1-based; a negative index counts
//    back from the last vertex read so far; index 0 is an error.
//  - A face with fewer than three corners is dropped. A quad is split along its shorter
//    diagonal, compared in float: [0,1,2],[0,2,3] when |p0-p2|² < |p1-p3|², else
//    [0,1,3],[1,2,3]. A polygon of five or more corners is fanned from its first corner.
//    tinyobjloader clips ears there instead, so such files may triangulate differently.
//  - "o" and "g" close the current shape when it holds triangles. loadObj returns the
//    vertices of the whole file and the triangles of the first shape (shapes.front()).
//
// MSH (MshIO's MshSpec as loadMsh reads it): format 2.2 ASCII and 4.1 ASCII or binary.
//  - Nodes are returned in file order.
//  - Tetrahedra (element type 4) are returned in file order, each node tag mapped to its node's
//    position in the file. The reference subtracts 1 from the tag, which is the same mapping
//    when the tags run 1..N in file order, as Gmsh writes them.
//  - Blocks of other element types are skipped. The reference reads every block with the
//    tetrahedron's stride, which is only defined for files that hold tetrahedra alone.
//  - Nodes with parametric coordinates are refused: the reference reads three values per
//    node.
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../csrc/api_internal.h"
#include "spg/geom/io/msh.h"
#include "spg/geom/io/obj.h"
#include "spgx_scenes.h"

namespace spg::io {
namespace {

std::string readFile(const std::string &path)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("cannot open " + path);
    std::string data;
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) data.append(buf, n);
    const bool bad = std::ferror(f) != 0;
    std::fclose(f);
    if (bad) throw std::runtime_error("cannot read " + path);
    return data;
}

inline bool isBlank(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }

// Cursor over one buffer with the token scanning both formats need.
struct Cursor {
    const char *p, *end;

    void skipBlanks()
    {
        while (p < end && isBlank(*p)) ++p;
    }
    void skipSpace()
    {
        while (p < end && (isBlank(*p) || *p == '\n')) ++p;
    }
    void nextLine()
    {
        const void *nl = std::memchr(p, '\n', size_t(end - p));
        p = nl ? static_cast<const char *>(nl) + 1 : end;
    }
    bool atLineEnd() const { return p >= end || *p == '\n' || *p == '#'; }
    // A decimal real as std::from_chars reads it (correctly rounded), with an optional '+'.
    bool real(double &out)
    {
        const char *q = p;
        if (q < end && *q == '+') ++q;
        const auto r = std::from_chars(q, end, out, std::chars_format::general);
        if (r.ec != std::errc()) return false;
        p = r.ptr;
        return true;
    }
    bool integer(long long &out)
    {
        const char *q = p;
        if (q < end && *q == '+') ++q;
        const auto r = std::from_chars(q, end, out);
        if (r.ec != std::errc()) return false;
        p = r.ptr;
        return true;
    }
    // The next whitespace-separated token (MSH ASCII sections).
    std::string token()
    {
        skipSpace();
        const char *s = p;
        while (p < end && !isBlank(*p) && *p != '\n') ++p;
        return std::string(s, p);
    }
    double needReal(const char *what)
    {
        skipSpace();
        double v;
        if (!real(v)) throw std::runtime_error(std::string("MSH: expected a number for ") + what);
        return v;
    }
    long long needInt(const char *what)
    {
        skipSpace();
        long long v;
        if (!integer(v)) throw std::runtime_error(std::string("MSH: expected an integer for ") + what);
        return v;
    }
};

// ------------------------------------------------------------------------------------ OBJ

struct ObjResult {
    std::vector<float> v;  // x, y, z per vertex (tinyobjloader's real_t)
    std::vector<Int3> tris;
};

void triangulate(const std::vector<int> &c, const std::vector<float> &v, std::vector<Int3> &out)
{
    const size_t n = c.size();
    if (n < 3) return;
    if (n == 3) {
        out.push_back({c[0], c[1], c[2]});
        return;
    }
    if (n == 4) {
        auto sq = [&v](int a, int b) {
            const float dx = v[3 * size_t(b)] - v[3 * size_t(a)];
            const float dy = v[3 * size_t(b) + 1] - v[3 * size_t(a) + 1];
            const float dz = v[3 * size_t(b) + 2] - v[3 * size_t(a) + 2];
            return dx * dx + dy * dy + dz * dz;
        };
        if (sq(c[0], c[2]) < sq(c[1], c[3])) {
            out.push_back({c[0], c[1], c[2]});
            out.push_back({c[0], c[2], c[3]});
        } else {
            out.push_back({c[0], c[1], c[3]});
            out.push_back({c[1], c[2], c[3]});
        }
        return;
    }
    for (size_t k = 1; k + 1 < n; ++k) out.push_back({c[0], c[k], c[k + 1]});
}

ObjResult parseObj(const std::string &data)
{
    ObjResult r;
    Cursor cur{data.data(), data.data() + data.size()};
    bool shapeDone = false;  // the first shape holding triangles has been closed
    std::vector<int> corners;
    long long line = 0;
    auto fail = [&line](const std::string &what) {
        throw std::runtime_error("OBJ line " + std::to_string(line) + ": " + what);
    };
    while (cur.p < cur.end) {
        ++line;
        cur.skipBlanks();
        const char *s = cur.p;
        const size_t left = size_t(cur.end - s);
        if (left >= 2 && s[0] == 'v' && isBlank(s[1])) {
            cur.p += 2;
            float xyz[3] = {0.f, 0.f, 0.f};
            for (int k = 0; k < 3; ++k) {
                cur.skipBlanks();
                if (cur.atLineEnd()) break;
                double d;
                if (!cur.real(d)) fail("bad vertex coordinate");
                xyz[k] = static_cast<float>(d);
            }
            r.v.insert(r.v.end(), xyz, xyz + 3);
        } else if (left >= 2 && s[0] == 'f' && isBlank(s[1])) {
            cur.p += 2;
            corners.clear();
            const long long nv = static_cast<long long>(r.v.size() / 3);
            for (;;) {
                cur.skipBlanks();
                if (cur.atLineEnd()) break;
                long long idx;
                if (!cur.integer(idx)) fail("bad face index");
                if (idx == 0) fail("face index 0");
                const long long i = idx > 0 ? idx - 1 : nv + idx;
                if (i < 0 || i >= nv) fail("face index out of range");
                corners.push_back(static_cast<int>(i));
                while (cur.p < cur.end && !isBlank(*cur.p) && *cur.p != '\n') ++cur.p;  // /vt/vn
            }
            if (!shapeDone) triangulate(corners, r.v, r.tris);
        } else if (left >= 1 && (s[0] == 'o' || s[0] == 'g') && (left == 1 || isBlank(s[1]) || s[1] == '\n')) {
            if (!r.tris.empty()) shapeDone = true;
        }
        cur.nextLine();
    }
    return r;
}

// ------------------------------------------------------------------------------------ MSH

// Nodes per element of the Gmsh element types up to 31 (0 = unknown).
int nodesPerElement(long long type)
{
    static const int n[32] = {0, 2,  3,  4,  4,  8,  6,  5,  3,  6,  9,  10, 27, 18, 14, 1,
                              8, 20, 15, 13, 9,  10, 12, 15, 15, 21, 4,  5,  6,  20, 35, 56};
    return type >= 0 && type < 32 ? n[type] : 0;
}

struct MshResult {
    std::vector<Vector3> nodes;
    std::vector<long long> tags;  // node tag per node, file order
    std::vector<std::array<long long, 4>> tetTags;
};

// Moves the cursor past the line "$End<name>".
void skipSection(Cursor &cur, const std::string &name)
{
    const std::string endTag = "$End" + name;
    const char *hit = nullptr;
    for (const char *q = cur.p; q + endTag.size() <= cur.end; ++q) {
        q = static_cast<const char *>(std::memchr(q, '$', size_t(cur.end - q)));
        if (!q || q + endTag.size() > cur.end) break;
        if (std::memcmp(q, endTag.data(), endTag.size()) == 0) {
            hit = q;
            break;
        }
    }
    if (!hit) throw std::runtime_error("MSH: missing " + endTag);
    cur.p = hit + endTag.size();
    cur.nextLine();
}

template <class T>
T readBinary(Cursor &cur)
{
    if (size_t(cur.end - cur.p) < sizeof(T)) throw std::runtime_error("MSH: truncated binary section");
    T v;
    std::memcpy(&v, cur.p, sizeof(T));
    cur.p += sizeof(T);
    return v;
}

void expectSectionEnd(Cursor &cur, const char *name)
{
    const std::string t = cur.token();
    if (t != std::string("$End") + name) throw std::runtime_error(std::string("MSH: expected $End") + name);
    cur.nextLine();
}

void nodes41(Cursor &cur, bool binary, MshResult &r)
{
    uint64_t nBlocks, nNodes;
    if (binary) {
        cur.nextLine();
        nBlocks = readBinary<uint64_t>(cur);
        nNodes = readBinary<uint64_t>(cur);
        readBinary<uint64_t>(cur);
        readBinary<uint64_t>(cur);
    } else {
        nBlocks = uint64_t(cur.needInt("numEntityBlocks"));
        nNodes = uint64_t(cur.needInt("numNodes"));
        cur.needInt("minNodeTag");
        cur.needInt("maxNodeTag");
    }
    r.nodes.reserve(r.nodes.size() + nNodes);
    r.tags.reserve(r.tags.size() + nNodes);
    for (uint64_t b = 0; b < nBlocks; ++b) {
        long long parametric, n;
        if (binary) {
            readBinary<int32_t>(cur);
            readBinary<int32_t>(cur);
            parametric = readBinary<int32_t>(cur);
            n = static_cast<long long>(readBinary<uint64_t>(cur));
        } else {
            cur.needInt("entityDim");
            cur.needInt("entityTag");
            parametric = cur.needInt("parametric");
            n = cur.needInt("numNodesInBlock");
        }
        if (parametric != 0) throw std::runtime_error("MSH: parametric node coordinates are not supported");
        if (n < 0) throw std::runtime_error("MSH: negative node count");
        for (long long j = 0; j < n; ++j)
            r.tags.push_back(binary ? static_cast<long long>(readBinary<uint64_t>(cur)) : cur.needInt("nodeTag"));
        for (long long j = 0; j < n; ++j) {
            Vector3 x;
            for (int k = 0; k < 3; ++k) x[k] = binary ? readBinary<double>(cur) : cur.needReal("node coordinate");
            r.nodes.push_back(x);
        }
    }
    expectSectionEnd(cur, "Nodes");
}

void elements41(Cursor &cur, bool binary, MshResult &r)
{
    uint64_t nBlocks;
    if (binary) {
        cur.nextLine();
        nBlocks = readBinary<uint64_t>(cur);
        readBinary<uint64_t>(cur);
        readBinary<uint64_t>(cur);
        readBinary<uint64_t>(cur);
    } else {
        nBlocks = uint64_t(cur.needInt("numEntityBlocks"));
        cur.needInt("numElements");
        cur.needInt("minElementTag");
        cur.needInt("maxElementTag");
    }
    for (uint64_t b = 0; b < nBlocks; ++b) {
        long long type, n;
        if (binary) {
            readBinary<int32_t>(cur);
            readBinary<int32_t>(cur);
            type = readBinary<int32_t>(cur);
            n = static_cast<long long>(readBinary<uint64_t>(cur));
        } else {
            cur.needInt("entityDim");
            cur.needInt("entityTag");
            type = cur.needInt("elementType");
            n = cur.needInt("numElementsInBlock");
        }
        const int k = nodesPerElement(type);
        if (k == 0) throw std::runtime_error("MSH: unsupported element type " + std::to_string(type));
        if (n < 0) throw std::runtime_error("MSH: negative element count");
        for (long long j = 0; j < n; ++j) {
            std::array<long long, 4> t{};
            for (int c = 0; c <= k; ++c) {
                const long long v =
                    binary ? static_cast<long long>(readBinary<uint64_t>(cur)) : cur.needInt("element data");
                if (type == 4 && c > 0) t[c - 1] = v;
            }
            if (type == 4) r.tetTags.push_back(t);
        }
    }
    expectSectionEnd(cur, "Elements");
}

void nodes22(Cursor &cur, MshResult &r)
{
    const long long n = cur.needInt("number of nodes");
    if (n < 0) throw std::runtime_error("MSH: negative node count");
    r.nodes.reserve(size_t(n));
    r.tags.reserve(size_t(n));
    for (long long j = 0; j < n; ++j) {
        r.tags.push_back(cur.needInt("node id"));
        Vector3 x;
        for (int k = 0; k < 3; ++k) x[k] = cur.needReal("node coordinate");
        r.nodes.push_back(x);
    }
    expectSectionEnd(cur, "Nodes");
}

void elements22(Cursor &cur, MshResult &r)
{
    const long long n = cur.needInt("number of elements");
    for (long long j = 0; j < n; ++j) {
        cur.needInt("element id");
        const long long type = cur.needInt("element type");
        const long long ntags = cur.needInt("number of tags");
        const int k = nodesPerElement(type);
        if (k == 0) throw std::runtime_error("MSH: unsupported element type " + std::to_string(type));
        if (ntags < 0) throw std::runtime_error("MSH: negative tag count");
        for (long long t = 0; t < ntags; ++t) cur.needInt("element tag");
        std::array<long long, 4> t{};
        for (int c = 0; c < k; ++c) {
            const long long v = cur.needInt("element node");
            if (type == 4) t[c] = v;
        }
        if (type == 4) r.tetTags.push_back(t);
    }
    expectSectionEnd(cur, "Elements");
}

MshResult parseMsh(const std::string &data)
{
    MshResult r;
    Cursor cur{data.data(), data.data() + data.size()};
    bool haveFormat = false, binary = false, v41 = false;
    for (;;) {
        cur.skipSpace();
        if (cur.p >= cur.end) break;
        const std::string tag = cur.token();
        if (tag.empty() || tag[0] != '$') throw std::runtime_error("MSH: expected a section, got '" + tag + "'");
        const std::string name = tag.substr(1);
        if (name == "MeshFormat") {
            const std::string version = cur.token();
            const long long fileType = cur.needInt("file type");
            const long long dataSize = cur.needInt("data size");
            if (version == "4.1")
                v41 = true;
            else if (version == "2.2")
                v41 = false;
            else
                throw std::runtime_error("MSH: format " + version + " is not supported (2.2 and 4.1 are)");
            binary = fileType == 1;
            if (binary && !v41) throw std::runtime_error("MSH: binary format 2.2 is not supported");
            if (dataSize != 8) throw std::runtime_error("MSH: data size must be 8");
            cur.nextLine();
            if (binary) {
                if (readBinary<int32_t>(cur) != 1) throw std::runtime_error("MSH: big-endian binary files are not supported");
                cur.nextLine();
            }
            expectSectionEnd(cur, "MeshFormat");
            haveFormat = true;
        } else if (name == "Nodes") {
            if (!haveFormat) throw std::runtime_error("MSH: $Nodes before $MeshFormat");
            if (v41)
                nodes41(cur, binary, r);
            else
                nodes22(cur, r);
        } else if (name == "Elements") {
            if (!haveFormat) throw std::runtime_error("MSH: $Elements before $MeshFormat");
            if (v41)
                elements41(cur, binary, r);
            else
                elements22(cur, r);
        } else {
            skipSection(cur, name);
        }
    }
    if (!haveFormat) throw std::runtime_error("MSH: no $MeshFormat section");
    return r;
}

}  // namespace

std::tuple<std::vector<Vector3>, std::vector<Int3>> loadObj(const std::string &filePath)
{
    ObjResult r = parseObj(readFile(filePath));
    if (r.tris.empty()) throw std::runtime_error("OBJ file " + filePath + " holds no faces");
    std::vector<Vector3> vertices(r.v.size() / 3);
    for (size_t i = 0; i < vertices.size(); ++i) vertices[i] = {r.v[3 * i], r.v[3 * i + 1], r.v[3 * i + 2]};
    return {std::move(vertices), std::move(r.tris)};
}

std::tuple<std::vector<Vector3>, std::vector<Int4>> loadMsh(const std::string &filePath)
{
    MshResult r = parseMsh(readFile(filePath));
    // Node tag -> file position. Tags 1..N in file order (Gmsh's own numbering) map to tag - 1.
    bool sequential = true;
    for (size_t i = 0; i < r.tags.size() && sequential; ++i) sequential = r.tags[i] == static_cast<long long>(i) + 1;
    std::unordered_map<long long, int> index;
    if (!sequential) {
        index.reserve(r.tags.size());
        for (size_t i = 0; i < r.tags.size(); ++i)
            if (!index.emplace(r.tags[i], static_cast<int>(i)).second)
                throw std::runtime_error("MSH: repeated node tag " + std::to_string(r.tags[i]));
    }
    const long long nv = static_cast<long long>(r.nodes.size());
    std::vector<Int4> tets;
    tets.reserve(r.tetTags.size());
    for (const auto &t : r.tetTags) {
        Int4 q;
        for (int c = 0; c < 4; ++c) {
            if (sequential) {
                if (t[c] < 1 || t[c] > nv) throw std::runtime_error("MSH: element refers to unknown node " + std::to_string(t[c]));
                q[c] = static_cast<int>(t[c] - 1);
            } else {
                const auto it = index.find(t[c]);
                if (it == index.end()) throw std::runtime_error("MSH: element refers to unknown node " + std::to_string(t[c]));
                q[c] = it->second;
            }
        }
        tets.push_back(q);
    }
    return {std::move(r.nodes), std::move(tets)};
}

}  // namespace spg::io

struct spgx_mesh {
    std::vector<spg::Vector3> vertices;
    std::vector<int32_t> cells;
    int32_t cell_size = 0;
};

extern "C" {

spgx_status spgx_load_obj(const char *path, spgx_mesh **out)
{
    SPGX_GUARD_BEGIN
    if (!path || !out) {
        spgx::set_error("NULL path or output");
        return SPGX_ERR_INVALID_ARG;
    }
    auto m = std::make_unique<spgx_mesh>();
    auto [v, f] = spg::io::loadObj(path);
    m->vertices = std::move(v);
    m->cell_size = 3;
    m->cells.reserve(3 * f.size());
    for (const auto &t : f) m->cells.insert(m->cells.end(), t.begin(), t.end());
    *out = m.release();
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_load_msh(const char *path, spgx_mesh **out)
{
    SPGX_GUARD_BEGIN
    if (!path || !out) {
        spgx::set_error("NULL path or output");
        return SPGX_ERR_INVALID_ARG;
    }
    auto m = std::make_unique<spgx_mesh>();
    auto [v, t] = spg::io::loadMsh(path);
    m->vertices = std::move(v);
    m->cell_size = 4;
    m->cells.reserve(4 * t.size());
    for (const auto &q : t) m->cells.insert(m->cells.end(), q.begin(), q.end());
    *out = m.release();
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_mesh_info(const spgx_mesh *m, int64_t *n_vertices, int64_t *n_cells, int32_t *cell_size)
{
    if (!m) {
        spgx::set_error("NULL mesh handle");
        return SPGX_ERR_INVALID_ARG;
    }
    if (n_vertices) *n_vertices = static_cast<int64_t>(m->vertices.size());
    if (n_cells) *n_cells = m->cell_size ? static_cast<int64_t>(m->cells.size() / size_t(m->cell_size)) : 0;
    if (cell_size) *cell_size = m->cell_size;
    return SPGX_OK;
}

spgx_status spgx_mesh_copy(const spgx_mesh *m, double *vertices, int32_t *cells)
{
    if (!m) {
        spgx::set_error("NULL mesh handle");
        return SPGX_ERR_INVALID_ARG;
    }
    if (vertices)
        for (size_t i = 0; i < m->vertices.size(); ++i)
            for (int k = 0; k < 3; ++k) vertices[3 * i + size_t(k)] = m->vertices[i][k];
    if (cells && !m->cells.empty()) std::memcpy(cells, m->cells.data(), m->cells.size() * sizeof(int32_t));
    return SPGX_OK;
}

spgx_status spgx_mesh_destroy(spgx_mesh *m)
{
    delete m;
    return SPGX_OK;
}

}  // extern "C"
