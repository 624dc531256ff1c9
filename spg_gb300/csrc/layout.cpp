// Host-side scene packing: validation, bit-exact greedy colouring, reference-order incidence
// lists and the colour-major, class-sorted device layout the GB300 kernels read.
#include "layout.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace spgx {

int stencil_size(int type)
{
    switch (type) {
    case SPGX_ENERGY_SPRING: return 2;
    case SPGX_ENERGY_SPRING_ANCHOR: return 1;
    case SPGX_ENERGY_DISCRETE_BENDING: return 4;
    case SPGX_ENERGY_MEMBRANE_STVK: return 3;
    case SPGX_ENERGY_STABLE_NEO_HOOKEAN: return 4;
    case SPGX_ENERGY_STVK: return 4;
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: return 4;
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN: return 3;
    case SPGX_ENERGY_MEMBRANE_CHOI: return 3;
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING: return 4;
    case SPGX_ENERGY_QUADRATIC_BENDING: return 4;
    case SPGX_ENERGY_SPRING_CONTINUUM: return 2;
    case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM: return 2;
    case SPGX_ENERGY_STATIC_LOAD: return 1;
    default: return 0;
    }
}

int param_count(int type)
{
    switch (type) {
    case SPGX_ENERGY_SPRING: return 3;
    case SPGX_ENERGY_SPRING_ANCHOR: return 5;
    case SPGX_ENERGY_DISCRETE_BENDING: return 3;
    case SPGX_ENERGY_MEMBRANE_STVK: return 22;
    case SPGX_ENERGY_STABLE_NEO_HOOKEAN: return 14;
    case SPGX_ENERGY_STVK: return 13;
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: return 13;
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN: return 10;
    case SPGX_ENERGY_MEMBRANE_CHOI: return 12;
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING: return 3;
    case SPGX_ENERGY_QUADRATIC_BENDING: return 6;
    case SPGX_ENERGY_SPRING_CONTINUUM: return 3;
    case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM: return 3;
    case SPGX_ENERGY_STATIC_LOAD: return 4;
    default: return 0;
    }
}

static int32_t fbits(double v)
{
    const float f = static_cast<float>(v);
    int32_t b;
    std::memcpy(&b, &f, sizeof(b));
    return b;
}

// The reference joins every pair of vertices inside every stencil (graphColoring.cpp:72-84)
// and colours nodes first-fit in index order with node 0 forced to colour 0 (:21-49). Only
// already-coloured neighbours (lower index, plus node 0) constrain a node, so stamping the
// neighbours' colours per node gives the identical assignment without the O(V) refill.
std::vector<int32_t> greedy_color_vertices(int nv, const spgx_object_desc &obj)
{
    std::vector<int32_t> colors(nv, -1);
    if (nv == 0) return colors;
    std::vector<int64_t> start(static_cast<size_t>(nv) + 1, 0);
    for (int e = 0; e < obj.n_energies; ++e) {
        const auto &E = obj.energies[e];
        const int S = stencil_size(E.type);
        for (int64_t s = 0; s < E.n_stencils; ++s) {
            const int32_t *st = E.stencils + s * S;
            for (int i = 0; i < S; ++i)
                for (int j = i + 1; j < S; ++j) {
                    ++start[st[i] + 1];
                    ++start[st[j] + 1];
                }
        }
    }
    for (int v = 0; v < nv; ++v) start[v + 1] += start[v];
    std::vector<int32_t> nbr(static_cast<size_t>(start[nv]));
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    int64_t maxdeg = 0;
    for (int e = 0; e < obj.n_energies; ++e) {
        const auto &E = obj.energies[e];
        const int S = stencil_size(E.type);
        for (int64_t s = 0; s < E.n_stencils; ++s) {
            const int32_t *st = E.stencils + s * S;
            for (int i = 0; i < S; ++i)
                for (int j = i + 1; j < S; ++j) {
                    nbr[fill[st[i]]++] = st[j];
                    nbr[fill[st[j]]++] = st[i];
                }
        }
    }
    for (int v = 0; v < nv; ++v) maxdeg = std::max<int64_t>(maxdeg, start[v + 1] - start[v]);
    std::vector<int32_t> stamp(static_cast<size_t>(maxdeg) + 2, -1);
    colors[0] = 0;
    for (int n = 1; n < nv; ++n) {
        for (int64_t k = start[n]; k < start[n + 1]; ++k) {
            const int c = colors[nbr[k]];
            if (c >= 0) stamp[c] = n;
        }
        int c = 0;
        while (stamp[c] == n) ++c;
        colors[n] = c;
    }
    return colors;
}

// colorStencils (graphColoring.cpp:51-70): stencils are joined when they share a vertex.
std::vector<int32_t> greedy_color_stencils(int type, int n_stencils, const int32_t *stencils)
{
    const int S = stencil_size(type);
    std::vector<int32_t> colors(n_stencils, -1);
    if (n_stencils == 0) return colors;
    int32_t maxv = -1;
    for (int64_t i = 0; i < int64_t(n_stencils) * S; ++i) maxv = std::max(maxv, stencils[i]);
    const int nv = maxv + 1;
    std::vector<int64_t> start(static_cast<size_t>(nv) + 1, 0);
    for (int64_t i = 0; i < int64_t(n_stencils) * S; ++i) ++start[stencils[i] + 1];
    for (int v = 0; v < nv; ++v) start[v + 1] += start[v];
    std::vector<int32_t> list(static_cast<size_t>(start[nv]));
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int64_t i = 0; i < int64_t(n_stencils) * S; ++i) list[fill[stencils[i]]++] = static_cast<int32_t>(i / S);
    std::vector<int32_t> stamp(static_cast<size_t>(n_stencils) + 1, -1);
    colors[0] = 0;
    for (int n = 1; n < n_stencils; ++n) {
        for (int j = 0; j < S; ++j) {
            const int v = stencils[int64_t(n) * S + j];
            for (int64_t k = start[v]; k < start[v + 1]; ++k) {
                const int m = list[k];
                if (m == n) continue;
                const int c = colors[m];
                if (c >= 0) stamp[c] = n;
            }
        }
        int c = 0;
        while (stamp[c] == n) ++c;
        colors[n] = c;
    }
    return colors;
}

static int incidence_class(int type, int slot)
{
    switch (type) {
    case SPGX_ENERGY_SPRING_ANCHOR: return kClsAnchor;
    case SPGX_ENERGY_SPRING: return kClsSpring;
    case SPGX_ENERGY_DISCRETE_BENDING: return slot >= 2 ? kClsFlap : kClsHinge;
    case SPGX_ENERGY_MEMBRANE_STVK: return kClsStvk;
    default: return kClsSnh;
    }
}

spgx_status build_scene_layout(const spgx_scene_desc *scene, bool with_xpbd, SceneLayout &L, std::string &err)
{
    if (!scene || scene->n_objects < 0 || (scene->n_objects > 0 && !scene->objects)) {
        err = "invalid scene descriptor";
        return SPGX_ERR_INVALID_ARG;
    }
    L = SceneLayout();
    const int nobj = scene->n_objects;
    int64_t total_v = 0;
    for (int o = 0; o < nobj; ++o) {
        const auto &ob = scene->objects[o];
        if (ob.n_vertices < 0 || (ob.n_vertices > 0 && (!ob.x || !ob.mass)) || ob.n_energies < 0 ||
            (ob.n_energies > 0 && !ob.energies)) {
            err = "invalid object descriptor " + std::to_string(o);
            return SPGX_ERR_INVALID_ARG;
        }
        for (int e = 0; e < ob.n_energies; ++e) {
            const auto &E = ob.energies[e];
            if (stencil_size(E.type) == 0) {
                err = "unsupported energy type " + std::to_string(E.type) + " (object " + std::to_string(o) + ", energy " +
                      std::to_string(e) + ")";
                return SPGX_ERR_UNSUPPORTED_ENERGY;
            }
            if (E.n_stencils < 0 || (E.n_stencils > 0 && (!E.stencils || !E.params))) {
                err = "invalid energy descriptor";
                return SPGX_ERR_INVALID_ARG;
            }
            const int S = stencil_size(E.type);
            for (int64_t i = 0; i < int64_t(E.n_stencils) * S; ++i)
                if (E.stencils[i] < 0 || E.stencils[i] >= ob.n_vertices) {
                    err = "stencil contains index to invalid vertex (object " + std::to_string(o) + ", energy " +
                          std::to_string(e) + ")";
                    return SPGX_ERR_INVALID_ARG;
                }
        }
        total_v += ob.n_vertices;
    }
    if (total_v >= (int64_t(1) << 29)) {
        err = "scene too large";
        return SPGX_ERR_INVALID_ARG;
    }
    const int nv = static_cast<int>(total_v);
    L.nv = nv;
    L.objects.resize(nobj);
    L.x_ext.resize(3 * size_t(nv));
    L.v_ext.assign(3 * size_t(nv), 0.0);
    std::vector<int32_t> color_ext(nv);
    std::vector<float> mass_ext(nv);
    int base = 0;
    for (int o = 0; o < nobj; ++o) {
        const auto &ob = scene->objects[o];
        auto &OL = L.objects[o];
        OL.nv = ob.n_vertices;
        OL.vertex_base = base;
        std::memcpy(&L.x_ext[3 * size_t(base)], ob.x, sizeof(double) * 3 * ob.n_vertices);
        if (ob.v) std::memcpy(&L.v_ext[3 * size_t(base)], ob.v, sizeof(double) * 3 * ob.n_vertices);
        OL.x_init.assign(ob.x, ob.x + 3 * size_t(ob.n_vertices));
        for (int v = 0; v < ob.n_vertices; ++v) mass_ext[base + v] = static_cast<float>(ob.mass[v]);
        OL.colors = greedy_color_vertices(ob.n_vertices, ob);
        for (int v = 0; v < ob.n_vertices; ++v) {
            color_ext[base + v] = OL.colors[v];
            OL.n_colors = std::max(OL.n_colors, OL.colors[v] + 1);
        }
        L.n_colors = std::max(L.n_colors, OL.n_colors);
        const int ne = ob.n_energies;
        for (int e = 0; e < ne; ++e) {
            OL.energy_types.push_back(ob.energies[e].type);
            OL.energy_sizes.push_back(ob.energies[e].n_stencils);
        }
        // Reference-order incidence lists (vbd.cpp:231-268).
        OL.adj_counts.assign(size_t(ob.n_vertices) * ne, 0);
        for (int e = 0; e < ne; ++e) {
            const auto &E = ob.energies[e];
            const int S = stencil_size(E.type);
            for (int64_t i = 0; i < int64_t(E.n_stencils) * S; ++i) ++OL.adj_counts[size_t(E.stencils[i]) * ne + e];
        }
        std::vector<int64_t> off(size_t(ob.n_vertices) * ne + 1, 0);
        for (size_t k = 0; k < OL.adj_counts.size(); ++k) off[k + 1] = off[k] + OL.adj_counts[k];
        OL.adj_entries.assign(2 * size_t(off.back()), 0);
        for (int e = 0; e < ne; ++e) {
            const auto &E = ob.energies[e];
            const int S = stencil_size(E.type);
            for (int64_t i = 0; i < int64_t(E.n_stencils) * S; ++i) {
                const int64_t k = off[size_t(E.stencils[i]) * ne + e]++;
                OL.adj_entries[2 * k] = static_cast<int32_t>(i / S);
                OL.adj_entries[2 * k + 1] = static_cast<int32_t>(i % S);
            }
        }
        if (with_xpbd) {
            for (int e = 0; e < ne; ++e)
                OL.stencil_colors.push_back(
                    greedy_color_stencils(ob.energies[e].type, ob.energies[e].n_stencils, ob.energies[e].stencils));
        }
        base += ob.n_vertices;
    }

    // Colour-major internal order. Inside a colour, vertices are grouped by object and ordered
    // along a Morton curve of their initial positions, so a tile of consecutive same-colour
    // vertices is spatially compact and its neighbourhoods overlap. The order inside a colour
    // does not change the result (the colour's vertices are updated independently).
    L.color_start.assign(L.n_colors + 1, 0);
    for (int v = 0; v < nv; ++v) ++L.color_start[color_ext[v] + 1];
    for (int c = 0; c < L.n_colors; ++c) L.color_start[c + 1] += L.color_start[c];
    L.ext2int.resize(nv);
    L.int2ext.resize(nv);
    {
        std::vector<uint64_t> key(nv);
        for (int o = 0; o < nobj; ++o) {
            const auto &OL = L.objects[o];
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            for (int k = 0; k < OL.nv; ++k)
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::min(lo[a], OL.x_init[3 * k + a]);
                    hi[a] = std::max(hi[a], OL.x_init[3 * k + a]);
                }
            for (int k = 0; k < OL.nv; ++k) {
                uint64_t m = 0;
                uint32_t q[3];
                for (int a = 0; a < 3; ++a) {
                    const double ext = hi[a] - lo[a];
                    const double t = ext > 0 ? (OL.x_init[3 * k + a] - lo[a]) / ext : 0.0;
                    const double qt = std::min(1023.0, std::max(0.0, std::floor(t * 1023.0 + 0.5)));
                    q[a] = std::isfinite(qt) ? static_cast<uint32_t>(qt) : 0u;
                }
                for (int b = 9; b >= 0; --b)
                    for (int a = 0; a < 3; ++a) m = (m << 1) | ((q[a] >> b) & 1u);
                key[OL.vertex_base + k] = (uint64_t(o) << 32) | m;
            }
        }
        std::vector<int32_t> order(nv);
        {
            std::vector<int32_t> fill(L.color_start.begin(), L.color_start.end() - (L.n_colors > 0 ? 1 : 0));
            for (int v = 0; v < nv; ++v) order[fill[color_ext[v]]++] = v;
        }
        for (int c = 0; c < L.n_colors; ++c)
            std::stable_sort(order.begin() + L.color_start[c], order.begin() + L.color_start[c + 1],
                             [&key](int32_t a, int32_t b) { return key[a] < key[b]; });
        for (int i = 0; i < nv; ++i) {
            L.int2ext[i] = order[i];
            L.ext2int[order[i]] = i;
        }
    }
    L.mass.resize(nv);
    for (int v = 0; v < nv; ++v) L.mass[L.ext2int[v]] = mass_ext[v];

    // Element tables (internal vertex indices) and per-vertex class-sorted incidences.
    auto &T = L.el;
    L.elem_base.resize(nobj);
    std::vector<int64_t> cls_count(size_t(nv) * kNumClasses, 0);
    std::vector<int64_t> gen_count(size_t(nv), 0);
    for (int o = 0; o < nobj; ++o) {
        const auto &ob = scene->objects[o];
        const int vb = L.objects[o].vertex_base;
        for (int e = 0; e < ob.n_energies; ++e) {
            const auto &E = ob.energies[e];
            const int S = stencil_size(E.type);
            const int P = param_count(E.type);
            int32_t eb = 0;
            for (int s = 0; s < E.n_stencils; ++s) {
                const int32_t *st = E.stencils + int64_t(s) * S;
                const double *p = E.params + int64_t(s) * P;
                int iv[4] = {0, 0, 0, 0};
                for (int k = 0; k < S; ++k) iv[k] = L.ext2int[vb + st[k]];
                if (is_generic_type(E.type)) {
                    if (s == 0) eb = static_cast<int32_t>(T.gen_idx.size());
                    T.gen_idx.push_back({iv[0], S > 1 ? iv[1] : -1, S > 2 ? iv[2] : -1, S > 3 ? iv[3] : -1});
                    T.gen_info.push_back({E.type, static_cast<int32_t>(T.gen_prm.size()), S, 0});
                    for (int k = 0; k < P; ++k) T.gen_prm.push_back(static_cast<float>(p[k]));
                    for (int k = 0; k < S; ++k) ++gen_count[iv[k]];
                    continue;
                }
                switch (E.type) {
                case SPGX_ENERGY_SPRING_ANCHOR:
                    if (s == 0) eb = static_cast<int32_t>(T.anchors.size());
                    T.anchors.push_back({float(p[0]), float(p[1]), float(p[2]), float(p[3])});
                    T.anchor_v.push_back(iv[0]);
                    T.anchor_cmp.push_back({float(p[4]), 0.f});
                    break;
                case SPGX_ENERGY_SPRING:
                    if (s == 0) eb = static_cast<int32_t>(T.springs.size());
                    T.springs.push_back({iv[0], iv[1], fbits(p[0]), fbits(p[1])});
                    T.spring_cmp.push_back(float(p[2]));
                    break;
                case SPGX_ENERGY_DISCRETE_BENDING:
                    if (s == 0) eb = static_cast<int32_t>(T.bend_idx.size());
                    T.bend_idx.push_back({iv[0], iv[1], iv[2], iv[3]});
                    T.bend_prm.push_back({float(p[0]), float(p[1]), float(p[2]), 0.f});
                    break;
                case SPGX_ENERGY_MEMBRANE_STVK: {
                    if (s == 0) eb = static_cast<int32_t>(T.stvk_idx.size());
                    T.stvk_idx.push_back({iv[0], iv[1], iv[2], 0});
                    T.stvk_D.push_back({float(p[0]), float(p[1]), float(p[2]), float(p[3])});
                    const double *K = p + 4;
                    T.stvk_Ka.push_back({float(K[0]), float(0.5 * (K[1] + K[3])), float(0.5 * (K[2] + K[6])), float(K[4])});
                    T.stvk_Kb.push_back({float(0.5 * (K[5] + K[7])), float(K[8]), 0.f, 0.f});
                    const double *Cm = p + 13;
                    T.stvk_Ca.push_back({float(Cm[0]), float(Cm[1]), float(Cm[2]), float(Cm[3])});
                    T.stvk_Cb.push_back({float(Cm[4]), float(Cm[5]), float(Cm[6]), float(Cm[7])});
                    T.stvk_Cc.push_back(float(Cm[8]));
                    break;
                }
                default:
                    if (s == 0) eb = static_cast<int32_t>(T.snh_idx.size());
                    T.snh_idx.push_back({iv[0], iv[1], iv[2], iv[3]});
                    T.snh_p0.push_back({float(p[0]), float(p[1]), float(p[2]), float(p[3])});
                    T.snh_p1.push_back({float(p[4]), float(p[5]), float(p[6]), float(p[7])});
                    T.snh_p2.push_back({float(p[8]), float(p[9]), float(p[10]), float(p[11])});
                    T.snh_cmp.push_back({float(p[12]), float(p[13])});
                    break;
                }
                for (int k = 0; k < S; ++k) ++cls_count[size_t(iv[k]) * kNumClasses + incidence_class(E.type, k)];
            }
            L.elem_base[o].push_back(eb);
        }
    }
    const size_t n_elems = T.anchors.size() + T.springs.size() + T.bend_idx.size() + T.stvk_idx.size() +
                           T.snh_idx.size() + T.gen_idx.size();
    if (n_elems >= (size_t(1) << 29)) {
        err = "too many elements";
        return SPGX_ERR_INVALID_ARG;
    }
    // Offsets: per internal vertex, classes in order.
    std::vector<int64_t> voff(size_t(nv) + 1, 0);
    for (int v = 0; v < nv; ++v) {
        int64_t tot = 0;
        for (int c = 0; c < kNumClasses; ++c) {
            const int64_t n = cls_count[size_t(v) * kNumClasses + c];
            if (n > kMaxClassCount) {
                err = "vertex has more than 65535 incidences of one energy class";
                return SPGX_ERR_INVALID_ARG;
            }
            tot += n;
        }
        voff[v + 1] = voff[v] + tot;
        L.max_degree = std::max<int>(L.max_degree, static_cast<int>(tot + gen_count[v]));
    }
    if (voff[nv] >= (int64_t(1) << 31)) {
        err = "too many incidences";
        return SPGX_ERR_INVALID_ARG;
    }
    int64_t n_gen = 0;
    for (int v = 0; v < nv; ++v) n_gen += gen_count[v];
    if (n_gen >= (int64_t(1) << 31)) {
        err = "too many incidences";
        return SPGX_ERR_INVALID_ARG;
    }
    L.mean_degree = nv ? double(voff[nv] + n_gen) / nv : 0.0;
    std::vector<int64_t> gen_fill;
    if (n_gen > 0) {
        L.gen_off.assign(size_t(nv) + 1, 0);
        for (int v = 0; v < nv; ++v) L.gen_off[v + 1] = L.gen_off[v] + static_cast<int32_t>(gen_count[v]);
        L.gen_adj.assign(size_t(n_gen), 0);
        gen_fill.assign(L.gen_off.begin(), L.gen_off.end() - 1);
    }
    L.hdr.resize(nv);
    std::vector<int64_t> cls_fill(size_t(nv) * kNumClasses);
    for (int v = 0; v < nv; ++v) {
        const int64_t *cc = &cls_count[size_t(v) * kNumClasses];
        int64_t o = voff[v];
        for (int c = 0; c < kNumClasses; ++c) {
            cls_fill[size_t(v) * kNumClasses + c] = o;
            o += cc[c];
        }
        L.hdr[v] = {static_cast<int32_t>(voff[v]), static_cast<int32_t>(cc[0] | (cc[1] << 16)),
                    static_cast<int32_t>(cc[2] | (cc[3] << 16)), static_cast<int32_t>(cc[4] | (cc[5] << 16))};
    }
    L.adj.assign(size_t(voff[nv]), 0);
    // Fill in reference order (objects, energies, flat stencil entries) so each class keeps it.
    for (int o = 0; o < nobj; ++o) {
        const auto &ob = scene->objects[o];
        const int vb = L.objects[o].vertex_base;
        for (int e = 0; e < ob.n_energies; ++e) {
            const auto &E = ob.energies[e];
            const int S = stencil_size(E.type);
            const int32_t eb = L.elem_base[o][e];
            for (int64_t i = 0; i < int64_t(E.n_stencils) * S; ++i) {
                const int slot = static_cast<int>(i % S);
                const int iv = L.ext2int[vb + E.stencils[i]];
                if (is_generic_type(E.type)) {
                    L.gen_adj[gen_fill[iv]++] = static_cast<int32_t>(((eb + i / S) << 2) | slot);
                    continue;
                }
                const int64_t k = cls_fill[size_t(iv) * kNumClasses + incidence_class(E.type, slot)]++;
                L.adj[k] = static_cast<int32_t>(((eb + i / S) << 2) | slot);
            }
        }
    }
    return SPGX_OK;
}

}  // namespace spgx
