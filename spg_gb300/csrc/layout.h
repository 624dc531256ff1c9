// Host-side scene packing for the GB300 VBD / XPBD solvers: validation, greedy colouring,
// incidence lists and the colour-major device layout.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "spgx.h"

namespace spgx {

// Plain host mirrors of CUDA's int4 / float4 / float2 (same size and alignment).
struct alignas(16) I4 {
    int32_t x, y, z, w;
};
struct alignas(16) F4 {
    float x, y, z, w;
};
struct alignas(8) I2 {
    int32_t x, y;
};
struct alignas(8) F2 {
    float x, y;
};

// Incidence classes, in the order the VBD kernel walks them for every vertex.
enum IncidenceClass { kClsAnchor = 0, kClsSpring, kClsFlap, kClsHinge, kClsStvk, kClsSnh, kNumClasses };

constexpr int kMaxClassCount = 0xffff;  // per vertex and class (16-bit counts in the header)

struct ObjectLayout {
    int nv{0};
    int vertex_base{0};  // offset of this object's vertices in the concatenated external order
    std::vector<int32_t> energy_types;
    std::vector<int32_t> energy_sizes;  // n_stencils per energy
    std::vector<int32_t> colors;        // greedy colour per vertex (reference order)
    int n_colors{0};
    // Incidence lists in reference order (vbd.cpp:231-268): counts[v * ne + e], pairs.
    std::vector<int32_t> adj_counts;
    std::vector<int32_t> adj_entries;
    std::vector<double> x_init;  // 3 * nv, positions given at create (BaseSolver::reset)
    // XPBD: per energy, stencil colours (graphColoring.cpp:51-70)
    std::vector<std::vector<int32_t>> stencil_colors;
};

// One device element table per energy type; stencils hold internal vertex indices.
struct ElementTables {
    std::vector<F4> anchors;       // ax, ay, az, k
    std::vector<int32_t> anchor_v; // vertex of each anchor
    std::vector<F2> anchor_cmp;    // compliance, unused
    std::vector<I4> springs;       // v0, v1, bits(L0), bits(k)
    std::vector<float> spring_cmp; // XPBD compliance
    std::vector<I4> bend_idx;      // v0..v3
    std::vector<F4> bend_prm;      // theta0, k_eff, compliance, unused
    std::vector<I4> stvk_idx;      // v0, v1, v2, unused
    std::vector<F4> stvk_D;        // Dinv row-major
    std::vector<F4> stvk_Ka;       // K00 K01 K02 K11 (symmetric part)
    std::vector<F4> stvk_Kb;       // K12 K22 unused unused
    std::vector<F4> stvk_Ca;       // compliance C00 C01 C02 C10
    std::vector<F4> stvk_Cb;       // C11 C12 C20 C21
    std::vector<float> stvk_Cc;    // C22
    std::vector<I4> snh_idx;       // v0..v3
    std::vector<F4> snh_p0;        // D00 D01 D02 D10
    std::vector<F4> snh_p1;        // D11 D12 D20 D21
    std::vector<F4> snh_p2;        // D22 lambda mu alpha
    std::vector<F2> snh_cmp;       // compliance (0,0), (1,1)
    // Types 6-14 (generic per-vertex derivatives): vertices (-1 padded), {type, param offset,
    // stencil size, 0}, parameters (the spgx.h layout, FP32).
    std::vector<I4> gen_idx;
    std::vector<I4> gen_info;
    std::vector<float> gen_prm;
};

struct SceneLayout {
    int nv{0};
    int n_colors{0};
    std::vector<int32_t> color_start;  // n_colors + 1, internal index ranges
    std::vector<int32_t> ext2int;      // concatenated external index -> internal index
    std::vector<int32_t> int2ext;
    std::vector<float> mass;           // internal order
    std::vector<double> x_ext;         // 3 * nv external order (positions at create)
    std::vector<double> v_ext;         // 3 * nv external order
    std::vector<I4> hdr;               // per internal vertex: offset, counts (16-bit pairs)
    std::vector<int32_t> adj;          // (element << 2) | slot, class-sorted per vertex
    std::vector<int32_t> gen_off;      // types 6-14: per internal vertex, range in gen_adj (empty if none)
    std::vector<int32_t> gen_adj;      // (generic element << 2) | slot, reference order per vertex
    ElementTables el;
    // Per-type element offset of each (object, energy) in the device tables.
    std::vector<std::vector<int32_t>> elem_base;
    std::vector<ObjectLayout> objects;
    int max_degree{0};
    double mean_degree{0};
    bool gen_idx_empty() const { return el.gen_idx.empty(); }
};

// Tiles of one colour for the shared-memory VBD kernel. A tile is a run of consecutive
// same-colour vertices (internal order) plus the halo of other vertices its incidences read.
// Its incidences are stored as one contiguous block of self-contained records (tile-local
// vertex indices, inline parameters): vertex by vertex in tile order, per vertex class by
// class as in the per-vertex header counts, reference order inside a class. Record sizes in
// 16-byte units: anchor 1, spring 1, flap 1, hinge 1, StVK 3, SNH 4.
constexpr int kTileMaxLocal = 1024;  // tile vertices + halo vertices
constexpr int kTileMaxVerts = 128;
constexpr int kTileMaxRecords = 4096;  // 16-byte record units per tile

struct TileLayout {
    int tile_vertices{0};
    int max_local{0};
    int max_records{0};
    std::vector<int32_t> color_tiles;  // n_colors + 1: tile index range of each colour
    // Per tile: {vstart, nvt, halo_off, n_halo}, {rec_off, n_rec, 0, 0} (16-byte units).
    std::vector<I4> hdr;
    std::vector<int32_t> halo;
    std::vector<I4> records;
    std::vector<int32_t> vrec;  // per internal vertex: record offset inside its tile's block
};

spgx_status build_tiles(const SceneLayout &L, int tile_vertices, TileLayout &out, std::string &err);

int stencil_size(int type);
// Types 6-14 run through the generic per-vertex derivative path (lanes kernel only).
inline bool is_generic_type(int type) { return type >= SPGX_ENERGY_STVK && type <= SPGX_ENERGY_STATIC_LOAD; }
int param_count(int type);

// Greedy first-fit vertex colouring in index order (graphColoring.cpp:21-49, 72-84),
// bit-exact with the reference, in O(incidences) instead of O(V^2).
std::vector<int32_t> greedy_color_vertices(int nv, const spgx_object_desc &obj);
// Greedy colouring of one energy's stencils (graphColoring.cpp:51-70), bit-exact.
std::vector<int32_t> greedy_color_stencils(int type, int n_stencils, const int32_t *stencils);

// Validates the scene and builds the device layout. with_xpbd also computes stencil colours.
spgx_status build_scene_layout(const spgx_scene_desc *scene, bool with_xpbd, SceneLayout &out, std::string &err);

}  // namespace spgx
