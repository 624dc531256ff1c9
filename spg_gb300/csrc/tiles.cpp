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
    default: {
        const I4 &s = T.snh_idx[inc.elem];
        push(s.x), push(s.y), push(s.z), push(s.w);
        break;
    }
    }
    return n;
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
    const auto &T = L.el;
    std::vector<int32_t> mark(L.nv, -1), local(L.nv, -1);
    auto incidences = [&L](int v, std::vector<Incidence> &list) {
        list.clear();
        const I4 &h = L.hdr[v];
        const int cnt[kNumClasses] = {h.y & 0xffff, (h.y >> 16) & 0xffff, h.z & 0xffff,
                                      (h.z >> 16) & 0xffff, h.w & 0xffff, (h.w >> 16) & 0xffff};
        int off = h.x;
        for (int c = 0; c < kNumClasses; ++c)
            for (int k = 0; k < cnt[c]; ++k, ++off) list.push_back({c, L.adj[off] >> 2, L.adj[off] & 3});
    };
    std::vector<Incidence> inc;
    int tile_id = 0;
    out.color_tiles.assign(L.n_colors + 1, 0);
    for (int c = 0; c < L.n_colors; ++c) {
        out.color_tiles[c] = tile_id;
        int v = L.color_start[c];
        const int ce = L.color_start[c + 1];
        while (v < ce) {
            // Grow the tile while the local set fits.
            const int vstart = v;
            std::vector<int32_t> halo;
            int o[4];
            while (v < ce && v - vstart < tile_vertices) {
                incidences(v, inc);
                std::vector<int32_t> add;
                for (const auto &i : inc) {
                    const int n = others(T, i, v, o);
                    for (int k = 0; k < n; ++k)
                        if (mark[o[k]] != tile_id) {
                            mark[o[k]] = tile_id;
                            add.push_back(o[k]);
                        }
                }
                if (v > vstart && (v - vstart + 1) + static_cast<int>(halo.size() + add.size()) > kTileMaxLocal) {
                    for (int a : add) mark[a] = -1;
                    break;
                }
                if (1 + static_cast<int>(halo.size() + add.size()) > kTileMaxLocal) {
                    err = "a vertex neighbourhood exceeds the tile capacity";
                    return SPGX_ERR_INVALID_ARG;
                }
                halo.insert(halo.end(), add.begin(), add.end());
                ++v;
            }
            const int nvt = v - vstart;
            std::sort(halo.begin(), halo.end());
            for (int k = 0; k < nvt; ++k) local[vstart + k] = k;
            for (size_t k = 0; k < halo.size(); ++k) local[halo[k]] = nvt + static_cast<int>(k);
            out.max_local = std::max(out.max_local, nvt + static_cast<int>(halo.size()));
            const I4 h0 = {vstart, nvt, static_cast<int32_t>(out.halo.size()), static_cast<int32_t>(halo.size())};
            out.halo.insert(out.halo.end(), halo.begin(), halo.end());
            // Records, class by class, vertex-interleaved.
            std::vector<std::vector<Incidence>> per_vertex(nvt);
            for (int k = 0; k < nvt; ++k) incidences(vstart + k, per_vertex[k]);
            int cls_off[kNumClasses], cls_n[kNumClasses];
            cls_off[kClsAnchor] = static_cast<int>(out.rec_anchor.size() / 2);
            cls_off[kClsSpring] = static_cast<int>(out.rec_spring.size());
            cls_off[kClsFlap] = static_cast<int>(out.rec_flap.size());
            cls_off[kClsHinge] = static_cast<int>(out.rec_hinge.size());
            cls_off[kClsStvk] = static_cast<int>(out.rec_stvk.size() / 3);
            cls_off[kClsSnh] = static_cast<int>(out.rec_snh.size() / 4);
            for (int cls = 0; cls < kNumClasses; ++cls) {
                std::vector<std::vector<const Incidence *>> lists(nvt);
                size_t rounds = 0;
                for (int k = 0; k < nvt; ++k) {
                    for (const auto &i : per_vertex[k])
                        if (i.cls == cls) lists[k].push_back(&i);
                    rounds = std::max(rounds, lists[k].size());
                }
                int count = 0;
                for (size_t r = 0; r < rounds; ++r)
                    for (int k = 0; k < nvt; ++k) {
                        if (r >= lists[k].size()) continue;
                        const Incidence &i = *lists[k][r];
                        const int self = k;
                        ++count;
                        switch (cls) {
                        case kClsAnchor: {
                            const F4 &a = T.anchors[i.elem];
                            out.rec_anchor.push_back({self, fb(a.w), 0, 0});
                            out.rec_anchor.push_back({fb(a.x), fb(a.y), fb(a.z), 0});
                            break;
                        }
                        case kClsSpring: {
                            const I4 &s = T.springs[i.elem];
                            const int other = i.slot == 0 ? s.y : s.x;
                            out.rec_spring.push_back({self | (local[other] << 16), s.z, s.w, 0});
                            break;
                        }
                        case kClsFlap: {
                            const I4 &s = T.bend_idx[i.elem];
                            const F4 &p = T.bend_prm[i.elem];
                            const int oth = i.slot == 2 ? s.w : s.z;
                            out.rec_flap.push_back({self | (local[s.x] << 16), local[s.y] | (local[oth] << 16),
                                                    fb(i.slot == 2 ? p.x : -p.x), fb(p.y)});
                            break;
                        }
                        case kClsHinge: {
                            const I4 &s = T.bend_idx[i.elem];
                            const F4 &p = T.bend_prm[i.elem];
                            const int origin = i.slot == 1 ? s.x : s.y;
                            out.rec_hinge.push_back({self | (local[origin] << 16), local[s.z] | (local[s.w] << 16),
                                                     fb(i.slot == 1 ? p.x : -p.x), fb(p.y)});
                            break;
                        }
                        case kClsStvk: {
                            const I4 &s = T.stvk_idx[i.elem];
                            const F4 &D = T.stvk_D[i.elem];
                            const F4 &Ka = T.stvk_Ka[i.elem];
                            const F4 &Kb = T.stvk_Kb[i.elem];
                            out.rec_stvk.push_back({local[s.x] | (local[s.y] << 16), local[s.z] | (i.slot << 16), fb(D.x),
                                                    fb(D.y)});
                            out.rec_stvk.push_back({fb(D.z), fb(D.w), fb(Ka.x), fb(Ka.y)});
                            out.rec_stvk.push_back({fb(Ka.z), fb(Ka.w), fb(Kb.x), fb(Kb.y)});
                            break;
                        }
                        default: {
                            const I4 &s = T.snh_idx[i.elem];
                            const F4 &a = T.snh_p0[i.elem];
                            const F4 &b = T.snh_p1[i.elem];
                            const F4 &cc = T.snh_p2[i.elem];
                            out.rec_snh.push_back({local[s.x] | (local[s.y] << 16), local[s.z] | (local[s.w] << 16), i.slot,
                                                   fb(a.x)});
                            out.rec_snh.push_back({fb(a.y), fb(a.z), fb(a.w), fb(b.x)});
                            out.rec_snh.push_back({fb(b.y), fb(b.z), fb(b.w), fb(cc.x)});
                            out.rec_snh.push_back({fb(cc.y), fb(cc.z), fb(cc.w), 0});
                            break;
                        }
                        }
                    }
                cls_n[cls] = count;
            }
            out.hdr.push_back(h0);
            out.hdr.push_back({cls_off[0], cls_off[1], cls_off[2], cls_off[3]});
            out.hdr.push_back({cls_off[4], cls_off[5], cls_n[0], cls_n[1]});
            out.hdr.push_back({cls_n[2], cls_n[3], cls_n[4], cls_n[5]});
            for (int k = 0; k < nvt; ++k) local[vstart + k] = -1;
            for (int a : halo) local[a] = -1;
            ++tile_id;
        }
    }
    out.color_tiles[L.n_colors] = tile_id;
    return SPGX_OK;
}

}  // namespace spgx
