// Packs a ParticleGroup and its energies into the spgx_object_desc of the C ABI, the way the
// reference's energies expose their precomputed data (stencils(), effectiveStiffness(),
// effectiveCompliance(), restLengths(), restThetas(), anchors(), inverseReferenceMats(),
// hydrostaticCorrectionTerms()).
#pragma once

#include <string>
#include <vector>

#include "spg/sim/energy/energy.h"
#include "spg/sim/simObject/particleGroup.h"
#include "spgx.h"

namespace spg::gpu {

struct PackedObject {
    std::vector<double> x, v, mass;
    std::vector<std::vector<int32_t>> stencils;
    std::vector<std::vector<double>> params;
    std::vector<spgx_energy_desc> energies;
    spgx_object_desc desc{};
};

// Throws std::runtime_error naming the energy if its type is not supported. With nEnergies >= 0
// only the group's first nEnergies energies are packed.
void pack(const ParticleGroup &pGroup, PackedObject &out, int nEnergies = -1);

struct PackedScene {
    std::vector<PackedObject> objects;
    std::vector<spgx_object_desc> descs;
    spgx_scene_desc desc{};
};

// nEnergies: per group, as above (empty = every energy).
void pack(const std::vector<ParticleGroup> &groups, PackedScene &out, const std::vector<int> &nEnergies = {});

}  // namespace spg::gpu
