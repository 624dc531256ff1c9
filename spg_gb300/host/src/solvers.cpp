// The GpuVBD / GpuXPBD drop-in solvers (packing: pack.cpp).
#include <stdexcept>
#include <typeinfo>

#include "spg/sim/solver/gpuPacking.h"
#include "spg/sim/solver/gpuSolvers.h"

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

void GpuVBD::setKernel(int kernel, int tileVertices)
{
    m_params.kernel = kernel;
    if (tileVertices != m_params.tile_vertices) {  // fixed at creation: rebuild on the next step
        m_params.tile_vertices = tileVertices;
        spgx_vbd_destroy(m_handle);
        m_handle = nullptr;
        m_packedEnergies.clear();
        m_dirty = true;
    } else if (m_handle) {
        check(spgx_vbd_set_params(m_handle, &m_params));
    }
}

void GpuVBD::classify(std::vector<int> &packed, std::vector<Pick> &picks) const
{
    packed.assign(m_objects.size(), 0);
    picks.clear();
    for (int o = 0; o < numSimObjects(); ++o) {
        const auto &E = m_objects[o].energies();
        int n = static_cast<int>(E.size());
        std::vector<Pick> mine;
        while (n > 0) {
            const auto *a = dynamic_cast<const SpringAnchorEnergy *>(E[n - 1].get());
            if (!a || a->nStencils() != 1 || picks.size() + mine.size() >= SPGX_MAX_PICKS) break;
            mine.push_back({o, a});
            --n;
        }
        packed[o] = n;
        picks.insert(picks.end(), mine.rbegin(), mine.rend());
    }
}

// First step, or after requirePrecomputationUpdate: colouring and incidence lists are built
// from the current ParticleGroups, like VBD::step's precomputation (vbd.cpp:14-18). When the
// only change since the last build is in the trailing one-stencil anchors (picking adds,
// moves and removes such an energy, solverCompare.cpp:717-726, 1496-1524), the solver is
// kept: an anchor adds no edge to the colouring graph, so the reference's recolouring
// yields the same colours, and the anchors run as the solver's dynamic anchors.
void GpuVBD::prepare()
{
    std::vector<int> packed;
    std::vector<Pick> picks;
    classify(packed, picks);
    std::vector<std::vector<const void *>> ids(m_objects.size());
    for (int o = 0; o < numSimObjects(); ++o)
        for (int e = 0; e < packed[o]; ++e) ids[o].push_back(m_objects[o].energies()[e].get());
    if (!m_handle || ids != m_packedEnergies) {
        spgx_vbd_destroy(m_handle);
        m_handle = nullptr;
        gpu::PackedScene scene;
        gpu::pack(m_objects, scene, packed);
        check(spgx_vbd_create(&scene.desc, &m_params, &m_handle));
        m_packedEnergies = std::move(ids);
        m_hostDirty = false;
    } else {
        check(spgx_vbd_set_params(m_handle, &m_params));
        if (m_hostDirty) pushState();
    }
    m_picks = std::move(picks);
    m_pickData.clear();
    m_dirty = false;
}

// Uploads the picks' targets and stiffnesses when they changed (updateAnchor between steps).
void GpuVBD::uploadPicks()
{
    std::vector<double> data;
    for (const auto &p : m_picks) {
        const Vector3 &a = p.energy->anchors()[0];
        data.insert(data.end(), {a[0], a[1], a[2], p.energy->modelStiffness()[0](0, 0)});
    }
    if (data == m_pickData) return;
    const int n = static_cast<int>(m_picks.size());
    std::vector<int32_t> obj(n), vert(n);
    std::vector<double> tgt(3 * size_t(n)), k(n);
    for (int q = 0; q < n; ++q) {
        obj[q] = m_picks[q].object;
        vert[q] = m_picks[q].energy->stencils()[0][0];
        for (int a = 0; a < 3; ++a) tgt[3 * q + a] = data[4 * q + a];
        k[q] = data[4 * q + 3];
    }
    check(spgx_vbd_set_picks(m_handle, n, obj.data(), vert.data(), tgt.data(), k.data()));
    m_pickData = std::move(data);
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
        check(spgx_vbd_set_picks(m_handle, 0, nullptr, nullptr, nullptr, nullptr));
    } else {
        check(spgx_vbd_set_params(m_handle, &m_params));
        if (m_hostDirty) pushState();
    }
    uploadPicks();
    check(spgx_vbd_step(m_handle, &m_stats));
    pullState();
}

void GpuVBD::reset()
{
    BaseSolver::reset();
    spgx_vbd_destroy(m_handle);  // a reset rebuilds everything from the host state
    m_handle = nullptr;
    m_packedEnergies.clear();
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

GpuImplicit::GpuImplicit(spgx_implicit_method method)
{
    spgx_implicit_params_default(&m_params);
    m_params.method = method;
}

GpuImplicit::~GpuImplicit() { spgx_implicit_destroy(m_handle); }

// First step or after a topology change: the system pattern is built from the current groups.
void GpuImplicit::prepare()
{
    spgx_implicit_destroy(m_handle);
    m_handle = nullptr;
    gpu::PackedScene scene;
    gpu::pack(m_objects, scene);
    check(spgx_implicit_create(&scene.desc, &m_params, &m_handle));
    m_dirty = false;
    m_hostDirty = false;
}

void GpuImplicit::step()
{
    m_params.dt = m_dtStep;
    m_params.substeps = m_nsubsteps;
    for (int a = 0; a < 3; ++a) m_params.gravity[a] = m_gravity[a];
    if (m_dirty || !m_handle) {
        prepare();
    } else {
        // setDt / setNumSubsteps / setGravity between steps: the handle keeps its step control
        // and BDF2 history, as the reference's solver object does.
        check(spgx_implicit_set_params(m_handle, &m_params));
    }
    if (m_hostDirty) {
        for (int o = 0; o < numSimObjects(); ++o) {
            const auto &g = m_objects[o];
            std::vector<double> x(3 * g.size()), v(3 * g.size());
            for (int i = 0; i < g.size(); ++i)
                for (int a = 0; a < 3; ++a) {
                    x[3 * i + a] = g.positions()[i][a];
                    v[3 * i + a] = g.velocities()[i][a];
                }
            check(spgx_implicit_set_state(m_handle, o, x.data(), v.data()));
        }
        m_hostDirty = false;
    }
    check(spgx_implicit_step(m_handle, &m_stats));
    for (int o = 0; o < numSimObjects(); ++o) {
        auto &g = m_objects[o];
        std::vector<double> x(3 * g.size()), v(3 * g.size());
        check(spgx_implicit_get_state(m_handle, o, x.data(), v.data()));
        for (int i = 0; i < g.size(); ++i) {
            g.positions()[i] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
            g.velocities()[i] = {v[3 * i], v[3 * i + 1], v[3 * i + 2]};
        }
    }
}

void GpuImplicit::reset()
{
    BaseSolver::reset();
    spgx_implicit_destroy(m_handle);  // also restarts the step control and BDF2's history
    m_handle = nullptr;
    m_dirty = true;
}

}  // namespace spg::solver
