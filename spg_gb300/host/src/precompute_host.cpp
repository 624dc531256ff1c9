// Host counterpart of spgx_precompute_params: the same per-stencil material values through the
// host energy classes' addStencil + preparePrecomputations (the reference's own setup path,
// e.g. apps/solverCompare.cpp:328, 461) and the C ABI packing.
#include <array>
#include <cstring>
#include <memory>
#include <string>

#include "../../csrc/api_internal.h"
#include "spg/sim/solver/gpuPacking.h"

namespace {

using namespace spg;

template <int S>
std::array<int, S> stencil_at(const int32_t *st, int i)
{
    std::array<int, S> s;
    for (int k = 0; k < S; ++k) s[k] = st[size_t(i) * S + k];
    return s;
}

Real rest_length(const ParticleGroup &g, const std::array<int, 2> &s, Real given)
{
    return given > 0 ? given : (g.positions0()[s[0]] - g.positions0()[s[1]]).norm();
}

std::shared_ptr<Energy<ParticleGroup>> make_energy(int type, int n, const int32_t *st, const ParticleGroup &g,
                                                   const double *material, int stride)
{
    auto row = [&](int i) { return material + size_t(stride) * size_t(i); };
    switch (type) {
    case SPGX_ENERGY_SPRING: {
        auto e = std::make_shared<SpringEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<2>(st, i), rest_length(g, stencil_at<2>(st, i), row(i)[0]), row(i)[1]);
        return e;
    }
    case SPGX_ENERGY_SPRING_ANCHOR: {
        auto e = std::make_shared<SpringAnchorEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<1>(st, i), Vector3(row(i)[0], row(i)[1], row(i)[2]), row(i)[3]);
        return e;
    }
    case SPGX_ENERGY_DISCRETE_BENDING: {
        auto e = std::make_shared<DiscreteBendingEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<4>(st, i), row(i)[0], row(i)[1]);
        return e;
    }
    case SPGX_ENERGY_MEMBRANE_STVK: {
        auto e = std::make_shared<MembraneStvkEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<3>(st, i), row(i)[0], row(i)[1]);
        return e;
    }
    case SPGX_ENERGY_STABLE_NEO_HOOKEAN: {
        auto e = std::make_shared<StableNeoHookeanEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<4>(st, i), row(i)[0], row(i)[1]);
        return e;
    }
    case SPGX_ENERGY_STVK: {
        auto e = std::make_shared<StvkEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<4>(st, i), row(i)[0], row(i)[1]);
        return e;
    }
    case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: {
        auto e = std::make_shared<StableSquaredNeoHookeanEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<4>(st, i), row(i)[0], row(i)[1]);
        return e;
    }
    case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN: {
        auto e = std::make_shared<MembraneBaraffWitkinEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<3>(st, i), row(i)[0], row(i)[1], row(i)[2]);
        return e;
    }
    case SPGX_ENERGY_MEMBRANE_CHOI: {
        auto e = std::make_shared<MembraneChoiEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<3>(st, i), row(i)[0], row(i)[1], row(i)[2]);
        return e;
    }
    case SPGX_ENERGY_BARAFF_WITKIN_BENDING: {
        auto e = std::make_shared<BaraffWitkinBendingEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<4>(st, i), row(i)[0], row(i)[1]);
        return e;
    }
    case SPGX_ENERGY_QUADRATIC_BENDING: {
        auto e = std::make_shared<QuadraticBendingEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<4>(st, i), row(i)[0], row(i)[1]);
        return e;
    }
    case SPGX_ENERGY_SPRING_CONTINUUM:
    case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM: {
        auto e = type == SPGX_ENERGY_SPRING_CONTINUUM ? std::make_shared<SpringContinuumEnergy>()
                                                      : std::make_shared<SpringSquaredContinuumEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<2>(st, i), rest_length(g, stencil_at<2>(st, i), row(i)[0]), row(i)[1]);
        return e;
    }
    case SPGX_ENERGY_STATIC_LOAD: {
        auto e = std::make_shared<StaticLoadEnergy>();
        for (int i = 0; i < n; ++i) e->addStencil(stencil_at<1>(st, i), Vector3(row(i)[1], row(i)[2], row(i)[3]), row(i)[0]);
        return e;
    }
    default: return nullptr;
    }
}

}  // namespace

extern "C" spgx_status spgx_precompute_params_host(int32_t type, int32_t n_stencils, const int32_t *stencils,
                                                   int32_t n_vertices, const double *x0, const double *material,
                                                   int32_t material_stride, double *params)
{
    SPGX_GUARD_BEGIN
    const int S = spgx_stencil_size(type), M = spgx_material_count(type), P = spgx_param_count(type);
    if (S == 0 || M == 0) {
        spgx::set_error("unsupported energy type " + std::to_string(type));
        return SPGX_ERR_UNSUPPORTED_ENERGY;
    }
    if (n_stencils < 0 || n_vertices < 0 || (n_stencils > 0 && (!stencils || !material || !params)) ||
        (n_vertices > 0 && !x0) || (material_stride != 0 && material_stride < M)) {
        spgx::set_error("invalid precompute arguments");
        return SPGX_ERR_INVALID_ARG;
    }
    for (int64_t i = 0; i < int64_t(n_stencils) * S; ++i)
        if (stencils[i] < 0 || stencils[i] >= n_vertices) {
            spgx::set_error("stencil contains index to invalid vertex");
            return SPGX_ERR_INVALID_ARG;
        }
    ParticleGroup g;
    for (int i = 0; i < n_vertices; ++i) {
        const Vector3 p(x0[3 * i], x0[3 * i + 1], x0[3 * i + 2]);
        g.addParticle(p, p, 1.0);
    }
    auto e = make_energy(type, n_stencils, stencils, g, material, material_stride);
    e->preparePrecomputations(g);
    g.addEnergy(e);
    gpu::PackedObject out;
    gpu::pack(g, out);
    if (n_stencils) std::memcpy(params, out.params[0].data(), sizeof(double) * size_t(n_stencils) * size_t(P));
    return SPGX_OK;
    SPGX_GUARD_END
}
