// Setup-time parts of the five hot-path energies: addStencil and preparePrecomputations with
// the reference's formulas and validation (the per-vertex derivatives run on the GPU).
#include <algorithm>
#include <cmath>
#include <string>
#include <utility>

#include "spg/sim/energy/energy.h"

namespace spg {

void ParticleGroup::removeEnergy(const std::shared_ptr<EnergyT> &energy)
{
    m_energies.erase(std::remove(m_energies.begin(), m_energies.end(), energy), m_energies.end());
}

// particleGroup.cpp:105-113
void ParticleGroup::scaleMasses(Real scaleFactor)
{
    for (size_t i = 0; i < m_m.size(); ++i)
        if (m_m[i] != 0) {
            m_m[i] *= scaleFactor;
            m_w[i] /= scaleFactor;
        }
}

// springEnergy.cpp:33-46
void SpringEnergy::addStencil(const std::array<int, 2> &stencil, Real restLength, Real stiffness)
{
    m_stencils.push_back(stencil);
    if (restLength <= 0) throw std::runtime_error("Zero/negative rest length invalid");
    m_restLength.push_back(restLength);
    Matrix1 K;
    K(0, 0) = stiffness;
    pushStiffness(K);
}

// springAnchorEnergy.cpp:29-39
void SpringAnchorEnergy::addStencil(std::array<int, 1> stencil, const Vector3 &anchor, Real stiffness)
{
    m_stencils.push_back(stencil);
    Matrix1 K;
    K(0, 0) = stiffness;
    pushStiffness(K);
    m_anchor.push_back(anchor);
}

// discreteBendingEnergy.cpp:33-46
void DiscreteBendingEnergy::addStencil(const std::array<int, 4> &stencil, Real restTheta, Real stiffness)
{
    m_stencils.push_back(stencil);
    if (restTheta < -3.12 || restTheta > 3.12) throw std::runtime_error("Invalid restTheta");
    m_restTheta.push_back(restTheta);
    Matrix1 K;
    K(0, 0) = stiffness;
    pushStiffness(K);
}

// discreteBendingEnergy.cpp:48-72: k_eff = k * 6 |e0|^2 / (|e0 x e3| + |e0 x e4|) (written as
// the inverse of the scaled compliance) and theta0 from the rest positions.
void DiscreteBendingEnergy::preparePrecomputations(const ParticleGroup &pGroup)
{
    const auto &X0 = pGroup.positions0();
    for (size_t i = 0; i < m_stencils.size(); ++i) {
        const auto &s = m_stencils[i];
        const Vector3 e0 = X0[s[1]] - X0[s[0]];
        const Vector3 e3 = X0[s[2]] - X0[s[1]];
        const Vector3 e4 = X0[s[3]] - X0[s[1]];
        const Real constantFactor = 2. * 3. * e0.squaredNorm() / (0.5 * (e0.cross(e3).norm() + e0.cross(e4).norm()));
        m_effectiveCompliance[i](0, 0) = m_modelCompliance[i](0, 0) / constantFactor;
        m_effectiveStiffness[i](0, 0) = 1.0 / m_effectiveCompliance[i](0, 0);
        const Vector3 n1 = e0.cross(e3).normalized();
        const Vector3 n2 = -e0.cross(e4).normalized();
        m_restTheta[i] = std::atan2(n1.cross(n2).dot(e0.normalized()), n1.dot(n2));
    }
    Energy<ParticleGroup>::preparePrecomputations(pGroup);
}

// membraneStvkEnergy.cpp:31-43: plane-stress StVK matrix.
void MembraneStvkEnergy::addStencil(const std::array<int, 3> &stencil, Real young, Real poisson)
{
    m_stencils.push_back(stencil);
    const Real yc = young / (1 - poisson * poisson);
    Matrix3 C;
    C(0, 0) = yc;
    C(0, 1) = yc * poisson;
    C(1, 0) = yc * poisson;
    C(1, 1) = yc;
    C(2, 2) = yc * (1 - poisson) / 2;
    pushStiffness(C);
}

// membraneStvkEnergy.cpp:45-71
void MembraneStvkEnergy::preparePrecomputations(const ParticleGroup &pGroup)
{
    const auto &X0 = pGroup.positions0();
    m_inverseReferenceMat.resize(m_stencils.size());
    for (size_t i = 0; i < m_stencils.size(); ++i) {
        const auto &s = m_stencils[i];
        const Vector3 &x0 = X0[s[0]], &x1 = X0[s[1]], &x2 = X0[s[2]];
        if (x0.z() != 0.0 || x1.z() != 0.0 || x2.z() != 0.0)
            throw std::runtime_error("Rest positions of triangles for membrane StVK energy must have coordinate z=0");
        const Real u[2] = {x1.x() - x0.x(), x1.y() - x0.y()};
        const Real v[2] = {x2.x() - x0.x(), x2.y() - x0.y()};
        Matrix2 Dm;
        Dm(0, 0) = u[0];
        Dm(1, 0) = u[1];
        Dm(0, 1) = v[0];
        Dm(1, 1) = v[1];
        m_inverseReferenceMat[i] = inverse(Dm);
        const Real area = (u[0] * v[1] - v[0] * u[1]) * 0.5;
        if (area <= 0) throw std::runtime_error("Rest area of membrane StVK triangle is not positive");
        for (int k = 0; k < 9; ++k) {
            m_effectiveCompliance[i].m[k] = m_modelCompliance[i].m[k] / area;
            m_effectiveStiffness[i].m[k] = m_modelStiffness[i].m[k] * area;
        }
    }
    Energy<ParticleGroup>::preparePrecomputations(pGroup);
}

// stableNeoHookeanEnergy.cpp:64-80: mu = E / (2 (1 + nu)), lambda = mu / (1 - 2 nu).
void StableNeoHookeanEnergy::addStencil(const std::array<int, 4> &stencil, Real young, Real poisson)
{
    m_stencils.push_back(stencil);
    const Real mu = young / (2 * (1 + poisson));
    const Real lambda = mu / (1 - 2 * poisson);
    Matrix2 C;
    C(0, 0) = lambda;
    C(1, 1) = mu;
    Matrix2 Ci;
    Ci(0, 0) = 1.0 / lambda;
    Ci(1, 1) = 1.0 / mu;
    m_modelStiffness.push_back(C);
    m_effectiveStiffness.push_back(C);
    m_modelCompliance.push_back(Ci);
    m_effectiveCompliance.push_back(Ci);
    m_hydrostaticCorrectionTerm.push_back(1 + mu / lambda);
}

// stableNeoHookeanEnergy.cpp:82-108
void StableNeoHookeanEnergy::preparePrecomputations(const ParticleGroup &pGroup)
{
    const auto &X0 = pGroup.positions0();
    m_inverseReferenceMat.resize(m_stencils.size());
    for (size_t i = 0; i < m_stencils.size(); ++i) {
        const auto &s = m_stencils[i];
        Matrix3 Dm;
        for (int a = 0; a < 3; ++a) {
            Dm(a, 0) = X0[s[1]][a] - X0[s[0]][a];
            Dm(a, 1) = X0[s[2]][a] - X0[s[0]][a];
            Dm(a, 2) = X0[s[3]][a] - X0[s[0]][a];
        }
        const Real volume = 1. / 6. * determinant(Dm);
        if (volume <= 0) throw std::runtime_error("SNH tetrahedron rest volume is not positive");
        m_inverseReferenceMat[i] = inverse(Dm);
        for (int k = 0; k < 4; ++k) {
            m_effectiveCompliance[i].m[k] = m_modelCompliance[i].m[k] / volume;
            m_effectiveStiffness[i].m[k] = m_modelStiffness[i].m[k] * volume;
        }
    }
    Energy<ParticleGroup>::preparePrecomputations(pGroup);
}

// ---------------------------------------------------------------------------------------
// Types 6-14

static std::pair<Real, Real> lame(Real young, Real poisson)
{
    const Real mu = young / (2 * (1 + poisson));
    // Epsilon guards a zero lambda against the compliance's division (stvkEnergy.cpp:69-71).
    const Real lambda = young * poisson / ((1 + poisson) * (1 - 2 * poisson)) + 1e-20;
    return {lambda, mu};
}

// Inverse rest matrix and volume of a tet (stvkEnergy.cpp:84-108).
static Real tet_rest(const ParticleGroup &g, const std::array<int, 4> &s, Matrix3 &inv, const char *what)
{
    const auto &X0 = g.positions0();
    Matrix3 Dm;
    for (int a = 0; a < 3; ++a) {
        Dm(a, 0) = X0[s[1]][a] - X0[s[0]][a];
        Dm(a, 1) = X0[s[2]][a] - X0[s[0]][a];
        Dm(a, 2) = X0[s[3]][a] - X0[s[0]][a];
    }
    const Real volume = 1. / 6. * determinant(Dm);
    if (volume <= 0) throw std::runtime_error(std::string(what) + " tetrahedron rest volume is not positive");
    inv = inverse(Dm);
    return volume;
}

// Inverse rest matrix and area of a z = 0 triangle (membraneBaraffWitkinEnergy.cpp:42-70).
static Real tri_rest(const ParticleGroup &g, const std::array<int, 3> &s, Matrix2 &inv, const char *what)
{
    const auto &X0 = g.positions0();
    const Vector3 &x0 = X0[s[0]], &x1 = X0[s[1]], &x2 = X0[s[2]];
    if (x0.z() != 0.0 || x1.z() != 0.0 || x2.z() != 0.0)
        throw std::runtime_error(std::string("Rest positions of triangles for ") + what +
                                 " must have coordinate z=0");
    const Real u[2] = {x1.x() - x0.x(), x1.y() - x0.y()};
    const Real v[2] = {x2.x() - x0.x(), x2.y() - x0.y()};
    Matrix2 Dm;
    Dm(0, 0) = u[0];
    Dm(1, 0) = u[1];
    Dm(0, 1) = v[0];
    Dm(1, 1) = v[1];
    inv = inverse(Dm);
    const Real area = (u[0] * v[1] - v[0] * u[1]) * 0.5;
    if (area <= 0) throw std::runtime_error(std::string("Rest area of ") + what + " triangle is not positive");
    return area;
}

void StvkEnergy::addStencil(const std::array<int, 4> &stencil, Real young, Real poisson)
{
    m_stencils.push_back(stencil);
    const auto lm = lame(young, poisson);
    pushDiagonalStiffness({lm.first, lm.second});
}

void StvkEnergy::preparePrecomputations(const ParticleGroup &pGroup)
{
    m_inverseReferenceMat.resize(m_stencils.size());
    for (size_t i = 0; i < m_stencils.size(); ++i)
        scaleEffective(i, tet_rest(pGroup, m_stencils[i], m_inverseReferenceMat[i], "SNH"));
    Energy<ParticleGroup>::preparePrecomputations(pGroup);
}

void StableSquaredNeoHookeanEnergy::addStencil(const std::array<int, 4> &stencil, Real young, Real poisson)
{
    m_stencils.push_back(stencil);
    const auto lm = lame(young, poisson);
    pushDiagonalStiffness({lm.first, lm.second});
}

void StableSquaredNeoHookeanEnergy::preparePrecomputations(const ParticleGroup &pGroup)
{
    m_inverseReferenceMat.resize(m_stencils.size());
    for (size_t i = 0; i < m_stencils.size(); ++i)
        scaleEffective(i, tet_rest(pGroup, m_stencils[i], m_inverseReferenceMat[i], "SSNH"));
    Energy<ParticleGroup>::preparePrecomputations(pGroup);
}

void MembraneBaraffWitkinEnergy::addStencil(const std::array<int, 3> &stencil, Real kWeft, Real kWarp, Real kBias)
{
    m_stencils.push_back(stencil);
    pushDiagonalStiffness({kWeft, kWarp, kBias});
}

void MembraneBaraffWitkinEnergy::preparePrecomputations(const ParticleGroup &pGroup)
{
    m_inverseReferenceMat.resize(m_stencils.size());
    for (size_t i = 0; i < m_stencils.size(); ++i)
        scaleEffective(i, tri_rest(pGroup, m_stencils[i], m_inverseReferenceMat[i], "membrane BaraffWitkin energy"));
    Energy<ParticleGroup>::preparePrecomputations(pGroup);
}

void MembraneChoiEnergy::addStencil(const std::array<int, 3> &stencil, Real kWeft, Real kWarp, Real kBias)
{
    m_stencils.push_back(stencil);
    pushDiagonalStiffness({kWeft, kWarp, kBias, kBias});
}

void MembraneChoiEnergy::preparePrecomputations(const ParticleGroup &pGroup)
{
    m_inverseReferenceMat.resize(m_stencils.size());
    for (size_t i = 0; i < m_stencils.size(); ++i)
        scaleEffective(i, tri_rest(pGroup, m_stencils[i], m_inverseReferenceMat[i], "membrane Choi energy"));
    Energy<ParticleGroup>::preparePrecomputations(pGroup);
}

void BaraffWitkinBendingEnergy::addStencil(const std::array<int, 4> &stencil, Real restTheta, Real stiffness)
{
    m_stencils.push_back(stencil);
    if (restTheta < -3.12 || restTheta > 3.12) throw std::runtime_error("Invalid restTheta");
    m_restTheta.push_back(restTheta);
    pushDiagonalStiffness({stiffness});
}

// baraffWitkinBendingEnergy.cpp:55-76: theta0 from the rest positions, no area weighting.
void BaraffWitkinBendingEnergy::preparePrecomputations(const ParticleGroup &pGroup)
{
    const auto &X0 = pGroup.positions0();
    for (size_t i = 0; i < m_stencils.size(); ++i) {
        const auto &s = m_stencils[i];
        const Vector3 e0 = X0[s[1]] - X0[s[0]];
        const Vector3 e3 = X0[s[2]] - X0[s[1]];
        const Vector3 e4 = X0[s[3]] - X0[s[1]];
        const Vector3 n1 = e0.cross(e3).normalized();
        const Vector3 n2 = -e0.cross(e4).normalized();
        m_restTheta[i] = std::atan2(n1.cross(n2).dot(e0.normalized()), n1.dot(n2));
    }
    Energy<ParticleGroup>::preparePrecomputations(pGroup);
}

void QuadraticBendingEnergy::addStencil(const std::array<int, 4> &stencil, Real restTheta, Real stiffness)
{
    if (restTheta != 0) throw std::runtime_error("Rest theta != 0 not supported for quadratic bending");
    m_stencils.push_back(stencil);
    m_weights.push_back({0, 0, 0, 0});
    m_stiffnessFactor.push_back(stiffness);
    pushDiagonalStiffness({1, 1, 1});
}

// quadraticBendingEnergy.cpp:48-93: cotangent weights and k * 3 / (area of the two triangles).
void QuadraticBendingEnergy::preparePrecomputations(const ParticleGroup &pGroup)
{
    const auto &X0 = pGroup.positions0();
    auto cot = [](const Vector3 &a, const Vector3 &b) { return a.dot(b) / a.cross(b).norm(); };
    for (size_t i = 0; i < m_stencils.size(); ++i) {
        const auto &s = m_stencils[i];
        const Vector3 e0 = X0[s[1]] - X0[s[0]];
        const Vector3 e1 = X0[s[2]] - X0[s[0]];
        const Vector3 e2 = X0[s[3]] - X0[s[0]];
        const Vector3 e3 = X0[s[2]] - X0[s[1]];
        const Vector3 e4 = X0[s[3]] - X0[s[1]];
        const Real c01 = cot(e0, e1), c02 = cot(e0, e2), c03 = cot(-e0, e3), c04 = cot(-e0, e4);
        m_weights[i] = {c03 + c04, c01 + c02, -c01 - c03, -c02 - c04};
        const Real k = m_stiffnessFactor[i] * (3 / (0.5 * (e0.cross(e1).norm() + e0.cross(e2).norm())));
        for (int a = 0; a < 3; ++a) {
            m_effectiveStiffness[i](a, a) = k;
            m_modelStiffness[i](a, a) = k;
            m_effectiveCompliance[i](a, a) = 1 / k;
            m_modelCompliance[i](a, a) = 1 / k;
        }
    }
    Energy<ParticleGroup>::preparePrecomputations(pGroup);
}

// springContinuumEnergy.cpp:19-34: the element integral makes the stiffness k L0.
void SpringContinuumEnergy::addStencil(const std::array<int, 2> &stencil, Real restLength, Real stiffness)
{
    m_stencils.push_back(stencil);
    if (restLength <= 0) throw std::runtime_error("Zero/negative rest length invalid");
    m_restLength.push_back(restLength);
    pushDiagonalStiffness({stiffness});
    scaleEffective(m_stencils.size() - 1, restLength);
}

}  // namespace spg
