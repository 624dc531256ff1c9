// Packing of ParticleGroups into the C ABI descriptor and the GpuVBD / GpuXPBD drop-in solvers.
#include <stdexcept>
#include <typeinfo>

#include "spg/sim/solver/gpuPacking.h"
#include "spg/sim/solver/gpuSolvers.h"

namespace spg::gpu {

void pack(const ParticleGroup &g, PackedObject &out)
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
    for (const auto &ep : g.energies()) {
        const auto *e = ep.get();
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

void pack(const std::vector<ParticleGroup> &groups, PackedScene &out)
{
    out.objects.clear();
    out.objects.resize(groups.size());
    out.descs.clear();
    for (size_t i = 0; i < groups.size(); ++i) {
        pack(groups[i], out.objects[i]);
        out.descs.push_back(out.objects[i].desc);
    }
    out.desc = {static_cast<int32_t>(out.descs.size()), out.descs.data()};
}

}  // namespace spg::gpu

namespace spg::solver {

static void check(spgx_status s)
{
    if (s != SPGX_OK) throw std::runtime_error(spgx_last_error_string());
}

GpuVBD::GpuVBD() { spgx_vbd_params_default(&m_params); }

GpuVBD::~GpuVBD() { spgx_vbd_destroy(m_handle); }

void GpuVBD::setIterations(int iterations)
{
    m_params.iterations = iterations;
    m_params.tolerance = 0;
    if (m_handle) check(spgx_vbd_set_params(m_handle, &m_params));
}

void GpuVBD::setTolerance(Real relativeResidual, int maxIterations, int checkInterval)
{
    m_params.tolerance = relativeResidual;
    m_params.max_iterations = maxIterations;
    m_params.check_interval = checkInterval;
    if (m_handle) check(spgx_vbd_set_params(m_handle, &m_params));
}

void GpuVBD::setLaunch(int lanesPerVertex, int blockSize)
{
    m_params.lanes_per_vertex = lanesPerVertex;
    m_params.block_size = blockSize;
    if (m_handle) check(spgx_vbd_set_params(m_handle, &m_params));
}

// First step (or after requirePrecomputationUpdate): colouring and incidence lists are
// built from the current ParticleGroups, like VBD::step's precomputation (vbd.cpp:14-18).
void GpuVBD::prepare()
{
    spgx_vbd_destroy(m_handle);
    m_handle = nullptr;
    gpu::PackedScene scene;
    gpu::pack(m_objects, scene);
    check(spgx_vbd_create(&scene.desc, &m_params, &m_handle));
    m_dirty = false;
    m_hostDirty = false;
}

void GpuVBD::pushState()
{
    for (int o = 0; o < numSimObjects(); ++o) {
        const auto &g = m_objects[o];
        std::vector<double> x(3 * g.size()), v(3 * g.size());
        for (int i = 0; i < g.size(); ++i)
            for (int a = 0; a < 3; ++a) {
                x[3 * i + a] = g.positions()[i][a];
                v[3 * i + a] = g.velocities()[i][a];
            }
        check(spgx_vbd_set_state(m_handle, o, x.data(), v.data()));
    }
    m_hostDirty = false;
}

void GpuVBD::pullState()
{
    for (int o = 0; o < numSimObjects(); ++o) {
        auto &g = m_objects[o];
        std::vector<double> x(3 * g.size()), v(3 * g.size());
        check(spgx_vbd_get_state(m_handle, o, x.data(), v.data()));
        for (int i = 0; i < g.size(); ++i) {
            g.positions()[i] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
            g.velocities()[i] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
        }
    }
}

void GpuVBD::step()
{
    m_params.dt = m_dtStep;
    m_params.substeps = m_nsubsteps;
    for (int a = 0; a < 3; ++a) m_params.gravity[a] = m_gravity[a];
    if (m_dirty || !m_handle) {
        prepare();
    } else {
        check(spgx_vbd_set_params(m_handle, &m_params));
        if (m_hostDirty) pushState();
    }
    check(spgx_vbd_step(m_handle, &m_stats));
    pullState();
}

void GpuVBD::reset()
{
    BaseSolver::reset();
    m_dirty = true;
}

GpuXPBD::GpuXPBD() { spgx_xpbd_params_default(&m_params); }

GpuXPBD::~GpuXPBD() { spgx_xpbd_destroy(m_handle); }

void GpuXPBD::prepare()
{
    spgx_xpbd_destroy(m_handle);
    m_handle = nullptr;
    gpu::PackedScene scene;
    gpu::pack(m_objects, scene);
    check(spgx_xpbd_create(&scene.desc, &m_params, &m_handle));
    m_dirty = false;
    m_hostDirty = false;
}

void GpuXPBD::step()
{
    m_params.dt = m_dtStep;
    m_params.substeps = m_nsubsteps;
    for (int a = 0; a < 3; ++a) m_params.gravity[a] = m_gravity[a];
    if (m_dirty || !m_handle) {
        prepare();
    } else {
        check(spgx_xpbd_set_params(m_handle, &m_params));
        if (m_hostDirty) {
            for (int o = 0; o < numSimObjects(); ++o) {
                const auto &g = m_objects[o];
                std::vector<double> x(3 * g.size()), v(3 * g.size());
                for (int i = 0; i < g.size(); ++i)
                    for (int a = 0; a < 3; ++a) {
                        x[3 * i + a] = g.positions()[i][a];
                        v[3 * i + a] = g.velocities()[i][a];
                    }
                check(spgx_xpbd_set_state(m_handle, o, x.data(), v.data()));
            }
            m_hostDirty = false;
        }
    }
    check(spgx_xpbd_step(m_handle, nullptr));
    for (int o = 0; o < numSimObjects(); ++o) {
        auto &g = m_objects[o];
        std::vector<double> x(3 * g.size()), v(3 * g.size());
        check(spgx_xpbd_get_state(m_handle, o, x.data(), v.data()));
        for (int i = 0; i < g.size(); ++i) {
            g.positions()[i] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
            g.velocities()[i] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
        }
    }
}

void GpuXPBD::reset()
{
    BaseSolver::reset();
    m_dirty = true;
}

}  // namespace spg::solver
