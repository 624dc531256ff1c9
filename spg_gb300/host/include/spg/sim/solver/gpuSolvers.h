// Drop-in GPU solvers behind SPG's solver plugin interface (BaseSolver,
// spg/include/spg/sim/solver/baseSolver.h:14-41): GpuVBD replaces spg::solver::VBD and GpuXPBD
// replaces spg::solver::XPBD. step() runs on the GB300 through the spgx C ABI; the host
// ParticleGroups are refreshed from the device after every step.
#pragma once

#include <string>
#include <vector>

#include "spg/sim/simObject/particleGroup.h"
#include "spg/sim/solver/gpuPacking.h"
#include "spgx.h"

namespace spg::solver {

class BaseSolver {
public:
    virtual ~BaseSolver() = default;
    virtual void step() = 0;
    void addObject(const ParticleGroup &object) { m_objects.push_back(object); }
    std::vector<ParticleGroup> &particleGroups() { return m_objects; }
    const std::vector<ParticleGroup> &particleGroups() const { return m_objects; }
    int numSimObjects() const { return static_cast<int>(m_objects.size()); }
    void setDt(Real dt) { m_dtStep = dt; }
    Real dt() const { return m_dtStep; }
    void setNumSubsteps(int n) { m_nsubsteps = n; }
    int numSubsteps() const { return m_nsubsteps; }
    virtual void reset()
    {
        for (auto &o : m_objects) o.reset();
    }
    void setVerbosity(Verbosity v) { m_verbosity = v; }
    void setGravity(const Vector3 &g) { m_gravity = g; }

protected:
    std::vector<ParticleGroup> m_objects;
    Vector3 m_gravity{0, -9.8, 0};
    Real m_dtStep{0.01};
    int m_nsubsteps{1};
    Verbosity m_verbosity{Verbosity::None};
};

class GpuVBD : public BaseSolver {
public:
    enum class InitialGuessType { InertialWithAcceleration };
    GpuVBD();
    ~GpuVBD() override;
    void step() override;
    void reset() override;
    void setInitialGuessType(InitialGuessType type) { m_initialGuessType = type; }
    void requirePrecomputationUpdate() { m_dirty = true; }
    // Extensions over the reference (vbd.h:33 hard-codes one iteration).
    void setIterations(int iterations);
    void setTolerance(Real relativeResidual, int maxIterations, int checkInterval = 10);
    void setLaunch(int lanesPerVertex, int blockSize);
    // 0 = autotune, 1 = lanes kernel, 2 = tile kernel, 3 = dataflow kernel; tile size 0 = autotune.
    void setKernel(int kernel, int tileVertices = 0);
    // Pushes host-side edits of positions/velocities to the device before the next step.
    void markHostStateDirty() { m_hostDirty = true; }
    const spgx_step_stats &lastStats() const { return m_stats; }
    spgx_vbd *handle() { return m_handle; }

private:
    struct Pick {
        int object;
        const SpringAnchorEnergy *energy;
    };
    // Splits every group's energies into the packed prefix and the trailing one-stencil
    // SpringAnchorEnergy objects (at most SPGX_MAX_PICKS in all), which run as dynamic anchors.
    void classify(std::vector<int> &packed, std::vector<Pick> &picks) const;
    void prepare();
    void uploadPicks();
    void pushState();
    void pullState();
    std::vector<std::vector<const void *>> m_packedEnergies;  // identity of the packed energies
    std::vector<Pick> m_picks;
    std::vector<double> m_pickData;  // targets and stiffnesses last uploaded
    InitialGuessType m_initialGuessType{InitialGuessType::InertialWithAcceleration};
    spgx_vbd_params m_params{};
    spgx_vbd *m_handle{nullptr};
    spgx_step_stats m_stats{};
    bool m_dirty{true};
    bool m_hostDirty{false};
};

class GpuXPBD : public BaseSolver {
public:
    GpuXPBD();
    ~GpuXPBD() override;
    void step() override;
    void reset() override;
    void requirePrecomputationUpdate() { m_dirty = true; }
    void markHostStateDirty() { m_hostDirty = true; }

private:
    void prepare();
    spgx_xpbd_params m_params{};
    spgx_xpbd *m_handle{nullptr};
    bool m_dirty{true};
    bool m_hostDirty{false};
};

// The global solvers (implicitEulerNewtonDx/Dv/Robust, implicitEulerBaraffWitkin, bdf2,
// staticNewton, quasiStaticNewton(Robust), simplecticEuler) behind one BaseSolver: the
// method picks which reference class it replaces (spgx_implicit_method).
class GpuImplicit : public BaseSolver {
public:
    explicit GpuImplicit(spgx_implicit_method method = SPGX_IMPLICIT_NEWTON_DX);
    ~GpuImplicit() override;
    void step() override;
    void reset() override;
    void requirePrecomputationUpdate() { m_dirty = true; }
    void markHostStateDirty() { m_hostDirty = true; }
    const spgx_step_stats &lastStats() const { return m_stats; }

private:
    void prepare();
    spgx_implicit_params m_params{};
    spgx_implicit *m_handle{nullptr};
    spgx_step_stats m_stats{};
    bool m_dirty{true};
    bool m_hostDirty{false};
};

// The reference's class names over GpuImplicit.
struct GpuImplicitEulerNewtonDx : GpuImplicit {
    GpuImplicitEulerNewtonDx() : GpuImplicit(SPGX_IMPLICIT_NEWTON_DX) {}
};
struct GpuImplicitEulerNewtonDv : GpuImplicit {
    GpuImplicitEulerNewtonDv() : GpuImplicit(SPGX_IMPLICIT_NEWTON_DV) {}
};
struct GpuImplicitEulerNewtonRobust : GpuImplicit {
    GpuImplicitEulerNewtonRobust() : GpuImplicit(SPGX_IMPLICIT_NEWTON_ROBUST) {}
};
struct GpuImplicitEulerBaraffWitkin : GpuImplicit {
    GpuImplicitEulerBaraffWitkin() : GpuImplicit(SPGX_IMPLICIT_BARAFF_WITKIN) {}
};
struct GpuBDF2 : GpuImplicit {
    GpuBDF2() : GpuImplicit(SPGX_IMPLICIT_BDF2) {}
};
struct GpuStaticNewton : GpuImplicit {
    GpuStaticNewton() : GpuImplicit(SPGX_STATIC_NEWTON) {}
};
struct GpuQuasiStaticNewton : GpuImplicit {
    GpuQuasiStaticNewton() : GpuImplicit(SPGX_QUASI_STATIC_NEWTON) {}
};
struct GpuQuasiStaticNewtonRobust : GpuImplicit {
    GpuQuasiStaticNewtonRobust() : GpuImplicit(SPGX_QUASI_STATIC_NEWTON_ROBUST) {}
};
struct GpuSimplecticEuler : GpuImplicit {
    GpuSimplecticEuler() : GpuImplicit(SPGX_SYMPLECTIC_EULER) {}
};

}  // namespace spg::solver
