// Energy plugin interface of SPG (spg/include/spg/sim/energy/energy.h:21-69) and the
// StencilBlockEnergy data layout (:75-369), restricted to what a GPU solver packs: stencils
// and the precomputed stiffness / compliance per stencil. The per-vertex derivatives run on
// the GPU (spg_gb300/csrc/elements.cuh); there is no host evaluation path.
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "spg/sim/simObject/particleGroup.h"
#include "spg/types.h"

namespace spg {

template <class TSimObject>
class Energy {
public:
    static constexpr int s_nDOFs = TSimObject::s_nDOFs;
    virtual ~Energy() = default;
    virtual int nStencils() const = 0;
    virtual int stencilSize() const = 0;
    virtual std::vector<int> flatStencils() const = 0;
    virtual int nDOFs() const = 0;

    // energy.h:54-61: a single preparation is accepted.
    virtual void preparePrecomputations(const TSimObject & /*obj*/)
    {
        if (m_prepared) throw std::runtime_error("Energy was already prepared");
        m_prepared = true;
    }
    bool prepared() const { return m_prepared; }
    void setName(const std::string &name) { m_name = name; }
    std::string name() { return m_name; }

protected:
    bool m_prepared{false};
    std::string m_name;
};

inline Matrix1 inverse(const Matrix1 &A)
{
    Matrix1 I;
    I(0, 0) = 1.0 / A(0, 0);
    return I;
}

template <int TstencilSize, int TnConstraints = 1, class TSimObject = ParticleGroup>
class StencilBlockEnergy : public Energy<TSimObject> {
protected:
    static constexpr int s_stencilSize{TstencilSize};
    using StiffnessMat = Matrix<TnConstraints>;

public:
    int nStencils() const override { return static_cast<int>(m_stencils.size()); }
    int stencilSize() const override { return TstencilSize; }
    int nDOFs() const override { return TSimObject::s_nDOFs; }
    std::vector<int> flatStencils() const override
    {
        std::vector<int> flat;
        flat.reserve(m_stencils.size() * TstencilSize);
        for (const auto &s : m_stencils) flat.insert(flat.end(), s.begin(), s.end());
        return flat;
    }
    const std::vector<std::array<int, TstencilSize>> &stencils() const { return m_stencils; }
    const std::vector<StiffnessMat> &effectiveStiffness() const { return m_effectiveStiffness; }
    const std::vector<StiffnessMat> &modelStiffness() const { return m_modelStiffness; }
    const std::vector<StiffnessMat> &effectiveCompliance() const { return m_effectiveCompliance; }
    const std::vector<StiffnessMat> &modelCompliance() const { return m_modelCompliance; }

protected:
    StencilBlockEnergy() = default;
    // Diagonal model stiffness and its inverse as the compliance (the reference's
    // StiffnessMat(...) / .inverse() for the diagonal matrices of these energies).
    void pushDiagonalStiffness(const std::array<Real, TnConstraints> &k)
    {
        StiffnessMat K, Ci;
        for (int i = 0; i < TnConstraints; ++i) {
            K(i, i) = k[i];
            Ci(i, i) = 1.0 / k[i];
        }
        m_modelStiffness.push_back(K);
        m_effectiveStiffness.push_back(K);
        m_modelCompliance.push_back(Ci);
        m_effectiveCompliance.push_back(Ci);
    }
    // effective = model * s, effective compliance = model compliance / s (area or volume).
    void scaleEffective(size_t i, Real s)
    {
        for (int a = 0; a < TnConstraints * TnConstraints; ++a) {
            m_effectiveStiffness[i].m[a] = m_modelStiffness[i].m[a] * s;
            m_effectiveCompliance[i].m[a] = m_modelCompliance[i].m[a] / s;
        }
    }
    void pushStiffness(const StiffnessMat &K)
    {
        const StiffnessMat Ci = inverse(K);
        m_modelStiffness.push_back(K);
        m_effectiveStiffness.push_back(K);
        m_modelCompliance.push_back(Ci);
        m_effectiveCompliance.push_back(Ci);
    }

    std::vector<std::array<int, TstencilSize>> m_stencils;
    std::vector<StiffnessMat> m_effectiveStiffness, m_modelStiffness, m_effectiveCompliance, m_modelCompliance;
};

// SpringEnergy (springEnergy.h:9-30): 1/2 k (|x0 - x1| - L0)^2.
class SpringEnergy : public StencilBlockEnergy<2> {
public:
    SpringEnergy() { m_name = "SpringEnergy"; }
    void addStencil(const std::array<int, 2> &stencil, Real restLength, Real stiffness);
    const std::vector<Real> &restLengths() const { return m_restLength; }

protected:
    std::vector<Real> m_restLength;
};

// SpringAnchorEnergy (springAnchorEnergy.h:7-21): 1/2 k |x - a|^2.
class SpringAnchorEnergy : public StencilBlockEnergy<1> {
public:
    SpringAnchorEnergy() { m_name = "SpringAnchorEnergy"; }
    void addStencil(std::array<int, 1> stencil, const Vector3 &anchor, Real stiffness = 0);
    const std::vector<Vector3> &anchors() const { return m_anchor; }
    void updateAnchor(int i, const Vector3 &anchor) { m_anchor[i] = anchor; }

protected:
    std::vector<Vector3> m_anchor;
};

// DiscreteBendingEnergy (discreteBendingEnergy.h:9-21), Tamstorf 2013.
class DiscreteBendingEnergy : public StencilBlockEnergy<4> {
public:
    DiscreteBendingEnergy() { m_name = "DiscreteBendingEnergy"; }
    void addStencil(const std::array<int, 4> &stencil, Real restTheta, Real stiffness);
    void preparePrecomputations(const ParticleGroup &pGroup) override;
    const std::vector<Real> &restThetas() const { return m_restTheta; }

protected:
    std::vector<Real> m_restTheta;
};

// MembraneStvkEnergy (membraneStvkEnergy.h:9-21), Volino 2009.
class MembraneStvkEnergy : public StencilBlockEnergy<3, 3> {
public:
    MembraneStvkEnergy() { m_name = "MembraneStvkEnergy"; }
    void addStencil(const std::array<int, 3> &stencil, Real young, Real poisson);
    void preparePrecomputations(const ParticleGroup &pGroup) override;
    const std::vector<Matrix2> &inverseReferenceMats() const { return m_inverseReferenceMat; }

protected:
    std::vector<Matrix2> m_inverseReferenceMat;
};

// StableNeoHookeanEnergy (stableNeoHookeanEnergy.h:10-26), Smith 2018 eq. 11.
class StableNeoHookeanEnergy : public StencilBlockEnergy<4, 2> {
public:
    StableNeoHookeanEnergy() { m_name = "StableNeoHookeanEnergy"; }
    void addStencil(const std::array<int, 4> &stencil, Real young, Real poisson);
    void preparePrecomputations(const ParticleGroup &pGroup) override;
    const std::vector<Matrix3> &inverseReferenceMats() const { return m_inverseReferenceMat; }
    const std::vector<Real> &hydrostaticCorrectionTerms() const { return m_hydrostaticCorrectionTerm; }

protected:
    std::vector<Matrix3> m_inverseReferenceMat;
    std::vector<Real> m_hydrostaticCorrectionTerm;
};

// ---------------------------------------------------------------------------------------
// The further particle energies (C ABI types 6-14). Their derivatives run on the GPU's
// per-vertex forward-mode path; here only the setup data.

// StvkEnergy (stvkEnergy.h): tet StVK, stiffness diag(lambda, mu) times the rest volume.
class StvkEnergy : public StencilBlockEnergy<4, 2> {
public:
    StvkEnergy() { m_name = "StvkEnergy"; }
    void addStencil(const std::array<int, 4> &stencil, Real young, Real poisson);
    void preparePrecomputations(const ParticleGroup &pGroup) override;
    const std::vector<Matrix3> &inverseReferenceMats() const { return m_inverseReferenceMat; }

protected:
    std::vector<Matrix3> m_inverseReferenceMat;
};

// StableSquaredNeoHookeanEnergy (stableSquaredNeoHookeanEnergy.h): C = [det F - 1, tr F^T F - 3].
class StableSquaredNeoHookeanEnergy : public StencilBlockEnergy<4, 2> {
public:
    StableSquaredNeoHookeanEnergy() { m_name = "StableSquaredNeoHookeanEnergy"; }
    void addStencil(const std::array<int, 4> &stencil, Real young, Real poisson);
    void preparePrecomputations(const ParticleGroup &pGroup) override;
    const std::vector<Matrix3> &inverseReferenceMats() const { return m_inverseReferenceMat; }

protected:
    std::vector<Matrix3> m_inverseReferenceMat;
};

// MembraneBaraffWitkinEnergy (membraneBaraffWitkinEnergy.h): stiffness diag(kWeft, kWarp, kBias) * area.
class MembraneBaraffWitkinEnergy : public StencilBlockEnergy<3, 3> {
public:
    MembraneBaraffWitkinEnergy() { m_name = "MembraneBaraffWitkinEnergy"; }
    void addStencil(const std::array<int, 3> &stencil, Real kWeft, Real kWarp, Real kBias);
    void preparePrecomputations(const ParticleGroup &pGroup) override;
    const std::vector<Matrix2> &inverseReferenceMats() const { return m_inverseReferenceMat; }

protected:
    std::vector<Matrix2> m_inverseReferenceMat;
};

// MembraneChoiEnergy (membraneChoiEnergy.h): stiffness diag(kWeft, kWarp, kBias, kBias) * area.
class MembraneChoiEnergy : public StencilBlockEnergy<3, 4> {
public:
    MembraneChoiEnergy() { m_name = "MembraneChoiEnergy"; }
    void addStencil(const std::array<int, 3> &stencil, Real kWeft, Real kWarp, Real kBias);
    void preparePrecomputations(const ParticleGroup &pGroup) override;
    const std::vector<Matrix2> &inverseReferenceMats() const { return m_inverseReferenceMat; }

protected:
    std::vector<Matrix2> m_inverseReferenceMat;
};

// BaraffWitkinBendingEnergy (baraffWitkinBendingEnergy.h): dihedral angle without area weighting.
class BaraffWitkinBendingEnergy : public StencilBlockEnergy<4> {
public:
    BaraffWitkinBendingEnergy() { m_name = "BaraffWitkinBendingEnergy"; }
    void addStencil(const std::array<int, 4> &stencil, Real restTheta, Real stiffness);
    void preparePrecomputations(const ParticleGroup &pGroup) override;
    const std::vector<Real> &restThetas() const { return m_restTheta; }

protected:
    std::vector<Real> m_restTheta;
};

// QuadraticBendingEnergy (quadraticBendingEnergy.h): cotangent Laplacian per hinge.
class QuadraticBendingEnergy : public StencilBlockEnergy<4, 3> {
public:
    QuadraticBendingEnergy() { m_name = "QuadraticBendingEnergy"; }
    void addStencil(const std::array<int, 4> &stencil, Real restTheta, Real stiffness);
    void preparePrecomputations(const ParticleGroup &pGroup) override;
    // The four weights c_s of laplacians()[i] = [c0 I, c1 I, c2 I, c3 I].
    const std::vector<std::array<Real, 4>> &laplacianWeights() const { return m_weights; }

protected:
    std::vector<std::array<Real, 4>> m_weights;
    std::vector<Real> m_stiffnessFactor;
};

// SpringContinuumEnergy (springContinuumEnergy.h): C = |x0 - x1| / L0 - 1, stiffness k L0.
class SpringContinuumEnergy : public StencilBlockEnergy<2> {
public:
    SpringContinuumEnergy() { m_name = "SpringContinuumEnergy"; }
    void addStencil(const std::array<int, 2> &stencil, Real restLength, Real stiffness);
    const std::vector<Real> &restLengths() const { return m_restLength; }

protected:
    std::vector<Real> m_restLength;
};

// SpringSquaredContinuumEnergy (springSquaredContinuumEnergy.h): C = |x0 - x1|^2 / L0^2 - 1.
class SpringSquaredContinuumEnergy : public SpringContinuumEnergy {
public:
    SpringSquaredContinuumEnergy() { m_name = "SpringSquaredContinuumEnergy"; }
};

// StaticLoadEnergy (staticLoadEnergy.h): E = -k d . x with d normalized.
class StaticLoadEnergy : public StencilBlockEnergy<1> {
public:
    StaticLoadEnergy() { m_name = "StaticLoadEnergy"; }
    void addStencil(std::array<int, 1> stencil, const Vector3 &loadDirection, Real stiffness)
    {
        m_stencils.push_back(stencil);
        pushDiagonalStiffness({stiffness});
        m_loadDirection.push_back(loadDirection.normalized());
    }
    const std::vector<Vector3> &loadDirections() const { return m_loadDirection; }

protected:
    std::vector<Vector3> m_loadDirection;
};

}  // namespace spg
