// Host-only C ABI: colouring and incidence lists of one object, without a device.
#include <algorithm>

#include "api_internal.h"
#include "layout.h"

extern "C" {

spgx_status spgx_color_vertices(const spgx_object_desc *obj, int32_t *colors)
{
    SPGX_GUARD_BEGIN
    if (!obj || (obj->n_vertices > 0 && !colors)) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    spgx_scene_desc scene{1, obj};
    spgx::SceneLayout L;
    std::string err;
    const spgx_status st = spgx::build_scene_layout(&scene, false, L, err);
    if (st != SPGX_OK) {
        spgx::set_error(err);
        return st;
    }
    std::copy(L.objects[0].colors.begin(), L.objects[0].colors.end(), colors);
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_color_stencils(const spgx_energy_desc *energy, int32_t *colors)
{
    SPGX_GUARD_BEGIN
    if (!energy || energy->n_stencils < 0 || (energy->n_stencils > 0 && (!colors || !energy->stencils))) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    const int S = spgx::stencil_size(energy->type);
    if (S == 0) {
        spgx::set_error("unsupported energy type");
        return SPGX_ERR_UNSUPPORTED_ENERGY;
    }
    for (int64_t i = 0; i < int64_t(energy->n_stencils) * S; ++i)
        if (energy->stencils[i] < 0) {
            spgx::set_error("negative vertex index");
            return SPGX_ERR_INVALID_ARG;
        }
    const auto c = spgx::greedy_color_stencils(energy->type, energy->n_stencils, energy->stencils);
    std::copy(c.begin(), c.end(), colors);
    return SPGX_OK;
    SPGX_GUARD_END
}

spgx_status spgx_incidences(const spgx_object_desc *obj, int32_t *counts, int32_t *entries, int64_t *total)
{
    SPGX_GUARD_BEGIN
    if (!obj || !total) {
        spgx::set_error("invalid argument");
        return SPGX_ERR_INVALID_ARG;
    }
    spgx_scene_desc scene{1, obj};
    spgx::SceneLayout L;
    std::string err;
    const spgx_status st = spgx::build_scene_layout(&scene, false, L, err);
    if (st != SPGX_OK) {
        spgx::set_error(err);
        return st;
    }
    const auto &O = L.objects[0];
    *total = static_cast<int64_t>(O.adj_entries.size() / 2);
    if (counts) std::copy(O.adj_counts.begin(), O.adj_counts.end(), counts);
    if (entries) std::copy(O.adj_entries.begin(), O.adj_entries.end(), entries);
    return SPGX_OK;
    SPGX_GUARD_END
}

}  // extern "C"
