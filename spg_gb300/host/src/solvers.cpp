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
