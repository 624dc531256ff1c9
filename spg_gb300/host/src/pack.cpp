// Packing of ParticleGroups into the C ABI descriptor (spgx_object_desc): the reference's
// accessors for each energy's precomputed per-stencil data, in the order spgx.h documents.
#include <algorithm>
#include <stdexcept>
#include <string>
#include <typeinfo>

#include "spg/sim/solver/gpuPacking.h"

namespace spg::gpu {

// [Dinv (3x3 row-major), effectiveStiffness(0,0), (1,1), effectiveCompliance(0,0), (1,1)]
template <class E>
static void pack_tet(const E &en, std::vector<double> &p, const char *name)
{
    if (!en.prepared()) throw std::runtime_error(std::string(name) + " used before preparePrecomputations");
    for (int i = 0; i < en.nStencils(); ++i) {
        const auto &D = en.inverseReferenceMats()[i];
        p.insert(p.end(), D.m, D.m + 9);
        p.insert(p.end(), {en.effectiveStiffness()[i](0, 0), en.effectiveStiffness()[i](1, 1),
                           en.effectiveCompliance()[i](0, 0), en.effectiveCompliance()[i](1, 1)});
    }
}

// [Dinv (2x2 row-major), effectiveStiffness diagonal, effectiveCompliance diagonal]
template <class E>
static void pack_membrane(const E &en, std::vector<double> &p, const char *name)
{
    if (!en.prepared()) throw std::runtime_error(std::string(name) + " used before preparePrecomputations");
    for (int i = 0; i < en.nStencils(); ++i) {
        const auto &D = en.inverseReferenceMats()[i];
        p.insert(p.end(), D.m, D.m + 4);
        const auto &K = en.effectiveStiffness()[i];
        const auto &Cm = en.effectiveCompliance()[i];
        const int n = static_cast<int>(sizeof(K.m) / sizeof(K.m[0]) == 9 ? 3 : 4);
        for (int a = 0; a < n; ++a) p.push_back(K(a, a));
        for (int a = 0; a < n; ++a) p.push_back(Cm(a, a));
    }
}

void pack(const ParticleGroup &g, PackedObject &out, int nEnergies)
{
    const int nv = g.size();
    out = PackedObject();
    out.x.resize(3 * nv);
    out.v.resize(3 * nv);
    out.mass.assign(g.masses().begin(), g.masses().end());
    for (int i = 0; i < nv; ++i)
        for (int a = 0; a < 3; ++a) {
            out.x[3 * i + a] = g.positions()[i][a];
            out.v[3 * i + a] = g.velocities()[i][a];
        }
    const int ne = nEnergies < 0 ? static_cast<int>(g.energies().size())
                                  : std::min(nEnergies, static_cast<int>(g.energies().size()));
    for (int ei = 0; ei < ne; ++ei) {
        const auto *e = g.energies()[ei].get();
        std::vector<int32_t> st;
        for (int s : e->flatStencils()) st.push_back(s);
        std::vector<double> p;
        int type = 0;
        if (auto *sp = dynamic_cast<const SpringEnergy *>(e)) {
            type = SPGX_ENERGY_SPRING;
            for (int i = 0; i < sp->nStencils(); ++i)
                p.insert(p.end(), {sp->restLengths()[i], sp->effectiveStiffness()[i](0, 0),
                                   sp->effectiveCompliance()[i](0, 0)});
        } else if (auto *an = dynamic_cast<const SpringAnchorEnergy *>(e)) {
            type = SPGX_ENERGY_SPRING_ANCHOR;
            for (int i = 0; i < an->nStencils(); ++i)
                p.insert(p.end(), {an->anchors()[i][0], an->anchors()[i][1], an->anchors()[i][2],
                                   an->modelStiffness()[i](0, 0), an->effectiveCompliance()[i](0, 0)});
        } else if (auto *bd = dynamic_cast<const DiscreteBendingEnergy *>(e)) {
            type = SPGX_ENERGY_DISCRETE_BENDING;
            for (int i = 0; i < bd->nStencils(); ++i)
                p.insert(p.end(), {bd->restThetas()[i], bd->effectiveStiffness()[i](0, 0),
                                   bd->effectiveCompliance()[i](0, 0)});
        } else if (auto *mb = dynamic_cast<const MembraneStvkEnergy *>(e)) {
            type = SPGX_ENERGY_MEMBRANE_STVK;
            if (!mb->prepared()) throw std::runtime_error("MembraneStvkEnergy used before preparePrecomputations");
            for (int i = 0; i < mb->nStencils(); ++i) {
                const auto &D = mb->inverseReferenceMats()[i];
                p.insert(p.end(), D.m, D.m + 4);
                const auto &K = mb->effectiveStiffness()[i];
                p.insert(p.end(), K.m, K.m + 9);
                const auto &Cm = mb->effectiveCompliance()[i];
                p.insert(p.end(), Cm.m, Cm.m + 9);
            }
        } else if (auto *sn = dynamic_cast<const StableNeoHookeanEnergy *>(e)) {
            type = SPGX_ENERGY_STABLE_NEO_HOOKEAN;
            if (!sn->prepared()) throw std::runtime_error("StableNeoHookeanEnergy used before preparePrecomputations");
            for (int i = 0; i < sn->nStencils(); ++i) {
                const auto &D = sn->inverseReferenceMats()[i];
                p.insert(p.end(), D.m, D.m + 9);
                p.insert(p.end(), {sn->effectiveStiffness()[i](0, 0), sn->effectiveStiffness()[i](1, 1),
                                   sn->hydrostaticCorrectionTerms()[i], sn->effectiveCompliance()[i](0, 0),
                                   sn->effectiveCompliance()[i](1, 1)});
            }
        } else if (auto *st4 = dynamic_cast<const StvkEnergy *>(e)) {
            type = SPGX_ENERGY_STVK;
            pack_tet(*st4, p, "StvkEnergy");
        } else if (auto *ss = dynamic_cast<const StableSquaredNeoHookeanEnergy *>(e)) {
            type = SPGX_ENERGY_STABLE_SQUARED_NEO_HOOKEAN;
            pack_tet(*ss, p, "StableSquaredNeoHookeanEnergy");
        } else if (auto *bw = dynamic_cast<const MembraneBaraffWitkinEnergy *>(e)) {
            type = SPGX_ENERGY_MEMBRANE_BARAFF_WITKIN;
            pack_membrane(*bw, p, "MembraneBaraffWitkinEnergy");
        } else if (auto *ch = dynamic_cast<const MembraneChoiEnergy *>(e)) {
            type = SPGX_ENERGY_MEMBRANE_CHOI;
            pack_membrane(*ch, p, "MembraneChoiEnergy");
        } else if (auto *bb = dynamic_cast<const BaraffWitkinBendingEnergy *>(e)) {
            type = SPGX_ENERGY_BARAFF_WITKIN_BENDING;
            for (int i = 0; i < bb->nStencils(); ++i)
                p.insert(p.end(), {bb->restThetas()[i], bb->effectiveStiffness()[i](0, 0),
                                   bb->effectiveCompliance()[i](0, 0)});
        } else if (auto *qb = dynamic_cast<const QuadraticBendingEnergy *>(e)) {
            type = SPGX_ENERGY_QUADRATIC_BENDING;
            if (!qb->prepared()) throw std::runtime_error("QuadraticBendingEnergy used before preparePrecomputations");
            for (int i = 0; i < qb->nStencils(); ++i) {
                const auto &c = qb->laplacianWeights()[i];
                p.insert(p.end(), {c[0], c[1], c[2], c[3], qb->effectiveStiffness()[i](0, 0),
                                   qb->effectiveCompliance()[i](0, 0)});
            }
        } else if (auto *sq = dynamic_cast<const SpringSquaredContinuumEnergy *>(e)) {
            type = SPGX_ENERGY_SPRING_SQUARED_CONTINUUM;
            for (int i = 0; i < sq->nStencils(); ++i)
                p.insert(p.end(), {sq->restLengths()[i], sq->effectiveStiffness()[i](0, 0),
                                   sq->effectiveCompliance()[i](0, 0)});
        } else if (auto *sc = dynamic_cast<const SpringContinuumEnergy *>(e)) {
            type = SPGX_ENERGY_SPRING_CONTINUUM;
            for (int i = 0; i < sc->nStencils(); ++i)
                p.insert(p.end(), {sc->restLengths()[i], sc->effectiveStiffness()[i](0, 0),
                                   sc->effectiveCompliance()[i](0, 0)});
        } else if (auto *ld = dynamic_cast<const StaticLoadEnergy *>(e)) {
            type = SPGX_ENERGY_STATIC_LOAD;
            for (int i = 0; i < ld->nStencils(); ++i)
                p.insert(p.end(), {ld->modelStiffness()[i](0, 0), ld->loadDirections()[i][0],
                                   ld->loadDirections()[i][1], ld->loadDirections()[i][2]});
        } else {
            throw std::runtime_error(std::string("energy type not supported by the GPU solver: ") + typeid(*e).name());
        }
        out.stencils.push_back(std::move(st));
        out.params.push_back(std::move(p));
        out.energies.push_back({type, e->nStencils(), nullptr, nullptr});
    }
    for (size_t k = 0; k < out.energies.size(); ++k) {
        out.energies[k].stencils = out.stencils[k].data();
        out.energies[k].params = out.params[k].data();
    }
    out.desc = {nv, out.x.data(), out.v.data(), out.mass.data(), static_cast<int32_t>(out.energies.size()),
                out.energies.data()};
}

void pack(const std::vector<ParticleGroup> &groups, PackedScene &out, const std::vector<int> &nEnergies)
{
    out.objects.clear();
    out.objects.resize(groups.size());
    out.descs.clear();
    for (size_t i = 0; i < groups.size(); ++i) {
        pack(groups[i], out.objects[i], i < nEnergies.size() ? nEnergies[i] : -1);
        out.descs.push_back(out.objects[i].desc);
    }
    out.desc = {static_cast<int32_t>(out.descs.size()), out.descs.data()};
}

}  // namespace spg::gpu
