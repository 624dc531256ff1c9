// C ABI entry points that need no device: version, descriptor sizes, defaults, errors.
#include <string>

#include "api_internal.h"
#include "layout.h"

namespace spgx {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
void clear_error() { g_last_error.clear(); }

}  // namespace spgx

extern "C" {

int32_t spgx_api_version(void) { return SPGX_API_VERSION; }

int32_t spgx_stencil_size(int32_t type) { return spgx::stencil_size(type); }

int32_t spgx_param_count(int32_t type) { return spgx::param_count(type); }

int32_t spgx_num_constraints(int32_t type)
{
    switch (type) {
    case SPGX_ENERGY_MEMBRANE_STVK: return 3;
    case SPGX_ENERGY_STABLE_NEO_HOOKEAN: return 2;
    case SPGX_ENERGY_SPRING:
    case SPGX_ENERGY_SPRING_ANCHOR:
    case SPGX_ENERGY_DISCRETE_BENDING: return 1;
    case SPGX_ENERGY_STVK:
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: return 2;
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN: return 3;
    case SPGX_ENERGY_MEMBRANE_CHOI: return 4;
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING: return 1;
    case SPGX_ENERGY_QUADRATIC_BENDING: return 3;
    case SPGX_ENERGY_SPRING_CONTINUUM:
    case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM: return 1;
    default: return 0;  // including the static load, which has no constraint form
    }
}

const char *spgx_last_error_string(void) { return spgx::g_last_error.c_str(); }

void spgx_vbd_params_default(spgx_vbd_params *p)
{
    if (!p) return;
    p->dt = 0.01;
    p->substeps = 1;
    p->iterations = 1;
    p->gravity[0] = 0.0;
    p->gravity[1] = -9.8;
    p->gravity[2] = 0.0;
    p->tolerance = 0.0;
    p->max_iterations = 1000;
    p->check_interval = 10;
    p->fallback_condition = 1e6;
    p->lanes_per_vertex = 0;
    p->block_size = 0;
    p->use_graph = 1;
    p->device = 0;
    p->kernel = 0;
    p->tile_vertices = 0;
}

void spgx_xpbd_params_default(spgx_xpbd_params *p)
{
    if (!p) return;
    p->dt = 0.01;
    p->substeps = 1;
    p->gravity[0] = 0.0;
    p->gravity[1] = -9.8;
    p->gravity[2] = 0.0;
    p->block_size = 0;
    p->use_graph = 1;
    p->device = 0;
    p->kernel = 0;
}

}  // extern "C"
