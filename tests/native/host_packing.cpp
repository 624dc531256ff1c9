// Test-only: builds ParticleGroups with the library's C++ host layer (spg_gb300/host), runs the
// energies' addStencil + preparePrecomputations and the C ABI packing, and returns the packed
// parameters, so the tests can compare them with the numpy restatement of the reference.
#include <cstring>
#include <memory>
#include <vector>

#include "spg/sim/energy/energy.h"
#include "spg/sim/solver/gpuPacking.h"

using namespace spg;

extern "C" int host_pack(int type, int nv, const double *x0, int n_stencils, const int *stencils, const double *a,
                         double *params_out)
{
    try {
        ParticleGroup g;
        for (int i = 0; i < nv; ++i) {
            const Vector3 p(x0[3 * i], x0[3 * i + 1], x0[3 * i + 2]);
            g.addParticle(p, p, 1.0);
        }
        std::shared_ptr<Energy<ParticleGroup>> e;
        switch (type) {
        case SPGX_ENERGY_SPRING: {
            auto en = std::make_shared<SpringEnergy>();
            for (int s = 0; s < n_stencils; ++s) {
                const Vector3 d = g.positions0()[stencils[2 * s]] - g.positions0()[stencils[2 * s + 1]];
                en->addStencil({stencils[2 * s], stencils[2 * s + 1]}, d.norm(), a[0]);
            }
            e = en;
            break;
        }
        case SPGX_ENERGY_SPRING_ANCHOR: {
            auto en = std::make_shared<SpringAnchorEnergy>();
            for (int s = 0; s < n_stencils; ++s) en->addStencil({stencils[s]}, g.positions0()[stencils[s]], a[0]);
            e = en;
            break;
        }
        case SPGX_ENERGY_DISCRETE_BENDING: {
            auto en = std::make_shared<DiscreteBendingEnergy>();
            for (int s = 0; s < n_stencils; ++s)
                en->addStencil({stencils[4 * s], stencils[4 * s + 1], stencils[4 * s + 2], stencils[4 * s + 3]}, 0.0, a[0]);
            e = en;
            break;
        }
        case SPGX_ENERGY_MEMBRANE_STVK: {
            auto en = std::make_shared<MembraneStvkEnergy>();
            for (int s = 0; s < n_stencils; ++s)
                en->addStencil({stencils[3 * s], stencils[3 * s + 1], stencils[3 * s + 2]}, a[0], a[1]);
            e = en;
            break;
        }
        case SPGX_ENERGY_STABLE_NEO_HOOKEAN: {
            auto en = std::make_shared<StableNeoHookeanEnergy>();
            for (int s = 0; s < n_stencils; ++s)
                en->addStencil({stencils[4 * s], stencils[4 * s + 1], stencils[4 * s + 2], stencils[4 * s + 3]}, a[0], a[1]);
            e = en;
            break;
        }
        case SPGX_ENERGY_STVK: {
            auto en = std::make_shared<StvkEnergy>();
            for (int s = 0; s < n_stencils; ++s)
                en->addStencil({stencils[4 * s], stencils[4 * s + 1], stencils[4 * s + 2], stencils[4 * s + 3]}, a[0], a[1]);
            e = en;
            break;
        }
        case SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN: {
            auto en = std::make_shared<StableSquaredNeoHookeanEnergy>();
            for (int s = 0; s < n_stencils; ++s)
                en->addStencil({stencils[4 * s], stencils[4 * s + 1], stencils[4 * s + 2], stencils[4 * s + 3]}, a[0], a[1]);
            e = en;
            break;
        }
        case SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN: {
            auto en = std::make_shared<MembraneBaraffWitkinEnergy>();
            for (int s = 0; s < n_stencils; ++s)
                en->addStencil({stencils[3 * s], stencils[3 * s + 1], stencils[3 * s + 2]}, a[0], a[1], a[2]);
            e = en;
            break;
        }
        case SPGX_ENERGY_MEMBRANE_CHOI: {
            auto en = std::make_shared<MembraneChoiEnergy>();
            for (int s = 0; s < n_stencils; ++s)
                en->addStencil({stencils[3 * s], stencils[3 * s + 1], stencils[3 * s + 2]}, a[0], a[1], a[2]);
            e = en;
            break;
        }
        case SPGX_ENERGY_BARAFF_WITKIN_BENDING: {
            auto en = std::make_shared<BaraffWitkinBendingEnergy>();
            for (int s = 0; s < n_stencils; ++s)
                en->addStencil({stencils[4 * s], stencils[4 * s + 1], stencils[4 * s + 2], stencils[4 * s + 3]}, 0.0, a[0]);
            e = en;
            break;
        }
        case SPGX_ENERGY_QUADRATIC_BENDING: {
            auto en = std::make_shared<QuadraticBendingEnergy>();
            for (int s = 0; s < n_stencils; ++s)
                en->addStencil({stencils[4 * s], stencils[4 * s + 1], stencils[4 * s + 2], stencils[4 * s + 3]}, 0.0, a[0]);
            e = en;
            break;
        }
        case SPGX_ENERGY_SPRING_CONTINUUM:
        case SPGX_ENERGY_SPRING_SQUARED_CONTINUUM: {
            auto en = type == SPGX_ENERGY_SPRING_CONTINUUM ? std::make_shared<SpringContinuumEnergy>()
                                                           : std::make_shared<SpringSquaredContinuumEnergy>();
            for (int s = 0; s < n_stencils; ++s) {
                const Vector3 d = g.positions0()[stencils[2 * s]] - g.positions0()[stencils[2 * s + 1]];
                en->addStencil({stencils[2 * s], stencils[2 * s + 1]}, d.norm(), a[0]);
            }
            e = en;
            break;
        }
        case SPGX_ENERGY_STATIC_LOAD: {
            auto en = std::make_shared<StaticLoadEnergy>();
            for (int s = 0; s < n_stencils; ++s) en->addStencil({stencils[s]}, Vector3(a[1], a[2], a[3]), a[0]);
            e = en;
            break;
        }
        default: return 1;
        }
        e->preparePrecomputations(g);
        g.addEnergy(e);
        gpu::PackedObject out;
        gpu::pack(g, out);
        if (out.energies.size() != 1 || out.energies[0].type != type) return 2;
        std::memcpy(params_out, out.params[0].data(), sizeof(double) * out.params[0].size());
        return 0;
    } catch (...) {
        return 3;
    }
}
