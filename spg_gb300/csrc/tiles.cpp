// Tile records for the shared-memory VBD kernel (see TileLayout in layout.h).
#include <algorithm>
#include <cstring>

#include "layout.h"

namespace spgx {

namespace {

int32_t fb(float f)
{
    int32_t b;
    std::memcpy(&b, &f, sizeof(b));
    return b;
}

struct Incidence {
    int cls;
    int elem;
    int slot;
};

// Energies of types 6-14 follow the six classes in a vertex's record block, one unit each:
// {local v0 | v1 << 16, local v2 | v3 << 16, type | slot << 8 | stencil size << 16,
// parameter offset in the generic parameter table}.
constexpr int kClsGeneric = kNumClasses;
constexpr int kRecordUnits[kNumClasses + 1] = {1, 1, 1, 1, 3, 4, 1};

// Vertices read by one incidence other than its own vertex.
int others(const ElementTables &T, const Incidence &inc, int self, int *out)
{
    int n = 0;
    auto push = [&](int v) {
        if (v != self) out[n++] = v;
    };
    switch (inc.cls) {
    case kClsAnchor: break;
    case kClsSpring: push(T.springs[inc.elem].x), push(T.springs[inc.elem].y); break;
    case kClsFlap:
    case kClsHinge: {
        const I4 &s = T.bend_idx[inc.elem];
        push(s.x), push(s.y), push(s.z), push(s.w);
        break;
    }
    case kClsStvk: {
        const I4 &s = T.stvk_idx[inc.elem];
        push(s.x), push(s.y), push(s.z);
        break;
    }
    case kClsGeneric: {
        const I4 &s = T.gen_idx[inc.elem];
        const int S = T.gen_info[inc.elem].z;
        const int all[4] = {s.x, s.y, s.z, s.w};
        for (int j = 0; j < S; ++j) push(all[j]);
        break;
    }
    default: {
        const I4 &s = T.snh_idx[inc.elem];
        push(s.x), push(s.y), push(s.z), push(s.w);
        break;
    }
    }
    return n;
}

void incidences(const SceneLayout &L, int v, std::vector<Incidence> &list)
{
    list.clear();
    const I4 &h = L.hdr[v];
    const int cnt[kNumClasses] = {h.y & 0xffff, (h.y >> 16) & 0xffff, h.z & 0xffff,
                                  (h.z >> 16) & 0xffff, h.w & 0xffff, (h.w >> 16) & 0xffff};
    int off = h.x;
    for (int c = 0; c < kNumClasses; ++c)
        for (int k = 0; k < cnt[c]; ++k, ++off) list.push_back({c, L.adj[off] >> 2, L.adj[off] & 3});
    if (!L.gen_off.empty())
        for (int k = L.gen_off[v]; k < L.gen_off[v + 1]; ++k) list.push_back({kClsGeneric, L.gen_adj[k] >> 2, L.gen_adj[k] & 3});
}

int record_units(const std::vector<Incidence> &list)
{
    int n = 0;
    for (const auto &i : list) n += kRecordUnits[i.cls];
    return n;
}

void emit(const ElementTables &T, const Incidence &i, const std::vector<int32_t> &local,
          std::vector<I4> &out)
{
    switch (i.cls) {
    case kClsAnchor: {
        const F4 &a = T.anchors[i.elem];
        out.push_back({fb(a.x), fb(a.y), fb(a.z), fb(a.w)});
        break;
    }
    case kClsSpring: {
        const I4 &s = T.springs[i.elem];
        const int other = i.slot == 0 ? s.y : s.x;
        out.push_back({local[other], s.z, s.w, 0});
        break;
    }
    case kClsFlap: {
        const I4 &s = T.bend_idx[i.elem];
        const F4 &p = T.bend_prm[i.elem];
        const int oth = i.slot == 2 ? s.w : s.z;
        out.push_back({local[s.x] | (local[s.y] << 16), local[oth], fb(i.slot == 2 ? p.x : -p.x), fb(p.y)});
        break;
    }
    case kClsHinge: {
        const I4 &s = T.bend_idx[i.elem];
        const F4 &p = T.bend_prm[i.elem];
        const int origin = i.slot == 1 ? s.x : s.y;
        out.push_back({local[origin], local[s.z] | (local[s.w] << 16), fb(i.slot == 1 ? p.x : -p.x), fb(p.y)});
        break;
    }
    case kClsStvk: {
        const I4 &s = T.stvk_idx[i.elem];
        const F4 &D = T.stvk_D[i.elem];
        const F4 &Ka = T.stvk_Ka[i.elem];
        const F4 &Kb = T.stvk_Kb[i.elem];
        out.push_back({local[s.x] | (local[s.y] << 16), local[s.z] | (i.slot << 16), fb(D.x), fb(D.y)});
        out.push_back({fb(D.z), fb(D.w), fb(Ka.x), fb(Ka.y)});
        out.push_back({fb(Ka.z), fb(Ka.w), fb(Kb.x), fb(Kb.y)});
        break;
    }
    case kClsGeneric: {
        const I4 &s = T.gen_idx[i.elem];
        const I4 &info = T.gen_info[i.elem];
        const int S = info.z;
        auto loc = [&](int j, int v) { return j < S ? local[v] : 0; };
        out.push_back({loc(0, s.x) | (loc(1, s.y) << 16), loc(2, s.z) | (loc(3, s.w) << 16),
                       info.x | (i.slot << 8) | (S << 16), info.y});
        break;
    }
    default: {
        const I4 &s = T.snh_idx[i.elem];
        const F4 &a = T.snh_p0[i.elem];
        const F4 &b = T.snh_p1[i.elem];
        const F4 &c = T.snh_p2[i.elem];
        out.push_back({local[s.x] | (local[s.y] << 16), local[s.z] | (local[s.w] << 16), i.slot, fb(a.x)});
        out.push_back({fb(a.y), fb(a.z), fb(a.w), fb(b.x)});
        out.push_back({fb(b.y), fb(b.z), fb(b.w), fb(c.x)});
        out.push_back({fb(c.y), fb(c.z), fb(c.w), 0});
        break;
    }
    }
}

}  // namespace

spgx_status build_tiles(const SceneLayout &L, int tile_vertices, TileLayout &out, std::string &err)
{
    out = TileLayout();
    if (tile_vertices < 1 || tile_vertices > kTileMaxVerts) {
        err = "tile_vertices must be in [1, 128]";
        return SPGX_ERR_INVALID_ARG;
    }
    out.tile_vertices = tile_vertices;
    out.vrec.assign(L.nv, 0);
    const auto &T = L.el;
    std::vector<int32_t> mark(L.nv, -1), local(L.nv, -1);
    std::vector<Incidence> inc;
    std::vector<int32_t> add;
    int o[4];
    int tile_id = 0;
    out.color_tiles.assign(L.n_colors + 1, 0);
    for (int c = 0; c < L.n_colors; ++c) {
        out.color_tiles[c] = tile_id;
        int v = L.color_start[c];
        const int ce = L.color_start[c + 1];
        while (v < ce) {
            // Grow the tile while its vertices, halo and records fit the shared-memory budget.
            const int vstart = v;
            std::vector<int32_t> halo;
            int units = 0;
            while (v < ce && v - vstart < tile_vertices) {
                incidences(L, v, inc);
                add.clear();
                for (const auto &i : inc) {
                    const int n = others(T, i, v, o);
                    for (int k = 0; k < n; ++k)
                        if (mark[o[k]] != tile_id) {
                            mark[o[k]] = tile_id;
                            add.push_back(o[k]);
                        }
                }
                const int u = record_units(inc);
                const bool fits = (v - vstart + 1) + static_cast<int>(halo.size() + add.size()) <= kTileMaxLocal &&
                                  units + u <= kTileMaxRecords;
                if (!fits) {
                    for (int a : add) mark[a] = -1;
                    if (v == vstart) {
                        err = "a vertex neighbourhood exceeds the tile capacity";
                        return SPGX_ERR_INVALID_ARG;
                    }
                    break;
                }
                halo.insert(halo.end(), add.begin(), add.end());
                units += u;
                ++v;
            }
            const int nvt = v - vstart;
            std::sort(halo.begin(), halo.end());
            for (int k = 0; k < nvt; ++k) local[vstart + k] = k;
            for (size_t k = 0; k < halo.size(); ++k) local[halo[k]] = nvt + static_cast<int>(k);
            out.max_local = std::max(out.max_local, nvt + static_cast<int>(halo.size()));
            out.max_records = std::max(out.max_records, units);
            const int rec_off = static_cast<int>(out.records.size());
            out.hdr.push_back({vstart, nvt, static_cast<int32_t>(out.halo.size()), static_cast<int32_t>(halo.size())});
            out.hdr.push_back({rec_off, units, 0, 0});
            out.halo.insert(out.halo.end(), halo.begin(), halo.end());
            for (int k = 0; k < nvt; ++k) {
                out.vrec[vstart + k] = static_cast<int32_t>(out.records.size()) - rec_off;
                incidences(L, vstart + k, inc);
                for (const auto &i : inc) emit(T, i, local, out.records);
            }
            for (int k = 0; k < nvt; ++k) local[vstart + k] = -1;
            for (int a : halo) local[a] = -1;
            ++tile_id;
        }
    }
    out.color_tiles[L.n_colors] = tile_id;
    return SPGX_OK;
}

}  // namespace spgx
