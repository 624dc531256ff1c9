// spg::ParticleGroup with the reference's interface (particleGroup.h:14-60): FP64 host-side
// particle state and the energy list a solver packs for the GPU.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "spg/types.h"

namespace spg {

template <class TSimObject>
class Energy;

class ParticleGroup {
public:
    static constexpr int s_nDOFs = 3;
    using EnergyT = Energy<ParticleGroup>;

    const std::vector<Vector3> &positions() const { return m_x; }
    std::vector<Vector3> &positions() { return m_x; }
    const std::vector<Vector3> &positions0() const { return m_x0; }
    std::vector<Vector3> &velocities() { return m_v; }
    const std::vector<Vector3> &velocities() const { return m_v; }
    const std::vector<Real> &invMasses() const { return m_w; }
    const std::vector<Real> &masses() const { return m_m; }
    std::vector<std::shared_ptr<EnergyT>> &energies() { return m_energies; }
    const std::vector<std::shared_ptr<EnergyT>> &energies() const { return m_energies; }
    int nDOF() const { return static_cast<int>(m_x.size()) * 3; }
    int size() const { return static_cast<int>(m_x.size()); }

    // particleGroup.cpp:74-82
    void addParticle(const Vector3 &position, const Vector3 &position0, Real mass)
    {
        m_x.push_back(position);
        m_xInitial.push_back(position);
        m_x0.push_back(position0);
        m_v.push_back(Vector3::Zero());
        m_m.push_back(mass);
        m_w.push_back(mass == 0 ? 0 : 1 / mass);
    }
    void addEnergy(std::shared_ptr<EnergyT> energy) { m_energies.push_back(std::move(energy)); }
    void removeEnergy(const std::shared_ptr<EnergyT> &energy);
    void scaleMasses(Real scaleFactor);
    void setName(std::string name) { m_name = std::move(name); }
    // particleGroup.cpp:97-103
    void reset()
    {
        m_x = m_xInitial;
        for (auto &v : m_v) v = Vector3::Zero();
    }

protected:
    std::string m_name;
    std::vector<Vector3> m_x, m_xInitial, m_x0, m_v;
    std::vector<Real> m_m, m_w;
    std::vector<std::shared_ptr<EnergyT>> m_energies;
};

}  // namespace spg
