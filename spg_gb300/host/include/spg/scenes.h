// Headless scene builders: the reference's solverCompare scene code (apps/solverCompare.cpp,
// whose GUI needs Polyscope/OpenGL) restated on the Eigen-free types, plus the builders the
// benchmark configurations need (jittered spring cloth, 6-tet beam, patch batch).
#pragma once

#include <cstdint>
#include <vector>

#include "spg/geom/triangleMesh.h"
#include "spg/sim/energy/energy.h"
#include "spg/sim/simObject/particleGroup.h"

namespace spg::scenes {

// buildTriangleSquareMesh (solverCompare.cpp:332-365), float grid arithmetic kept. With
// restInitial the deformed positions equal the rest positions (flat in z = 0).
TriangleMesh buildTriangleSquareMesh(float width, float height, int rows, int cols);

// createCloth (solverCompare.cpp:367-498) with material constants, bending stiffness,
// anchor set and initial state as parameters. Energy order: bending, membrane, anchor.
ParticleGroup createCloth(Real mass, float width, float height, int rows, int cols, Real young, Real poisson,
                          Real bendingStiffness, Real anchorStiffness, const std::vector<int> &anchorIds,
                          bool restInitial);

// Large spring cloth: rest positions jittered in-plane by N(0, (jitter * edge)^2) (splitmix64
// + Box-Muller from `seed`, redrawn up to 64 times while an incident triangle would fall
// below 10 % of its nominal signed area), springs on every edge (rest length from the rest
// positions), bending on interior edges, row 0 anchored. Energy order: bending, spring,
// anchor. Initial state = rest state.
ParticleGroup createSpringCloth(Real mass, float width, float height, int rows, int cols, Real springStiffness,
                                Real bendingStiffness, Real anchorStiffness, Real jitter, uint64_t seed);

// createTetrahedralBeam (solverCompare.cpp:260-330) with Stable Neo-Hookean tets, split 5
// (the reference's mirrored 5-tet cells, :118-189) or 6 (each cell split along its
// (i,j,k)->(i+1,j+1,k+1) diagonal), x-min face anchored. Energy order: anchor, tet.
ParticleGroup createTetrahedralBeam(Real mass, float sideX, float sideY, float sideZ, int nX, int nY, int nZ,
                                    Real young, Real poisson, Real anchorStiffness, int split);

// Independent 1 m square patches: per patch, from one splitmix64 stream in this order,
// side vertex count ~ U{nMin..nMax}, mu and lambda ~ logU[muLo, muHi], bending ~ logU[kbLo,
// kbHi], anchored corner ~ U{0..3}; each a createCloth patch with a flat rest state.
std::vector<ParticleGroup> createPatchBatch(int nPatches, int nMin, int nMax, Real muLo, Real muHi, Real kbLo,
                                            Real kbHi, Real mass, Real anchorStiffness, uint64_t seed);

// A shell on a loaded triangle mesh (spg::io::loadObj), assembled as createSpringCloth
// assembles its grid: masses lumped from the rest areas, springs on every edge, discrete
// bending on interior edges, anchors on the given vertices. Rest = initial = the mesh's
// vertices, which may lie anywhere in 3D. Energy order: bending, spring, anchor.
ParticleGroup createTriangleMeshShell(const std::vector<Vector3> &vertices, const std::vector<Int3> &faces, Real mass,
                                      Real springStiffness, Real bendingStiffness, Real anchorStiffness,
                                      const std::vector<int> &anchorIds);

// A solid on a loaded tetrahedral mesh (spg::io::loadMsh), assembled as createTetrahedralBeam
// assembles its bar: masses lumped from the rest volumes, Stable Neo-Hookean tets, anchors
// on the given vertices. Tets must have positive rest volume (StableNeoHookeanEnergy throws
// otherwise). Energy order: anchor, tet.
ParticleGroup createTetMeshSolid(const std::vector<Vector3> &vertices, const std::vector<Int4> &tets, Real mass,
                                 Real young, Real poisson, Real anchorStiffness, const std::vector<int> &anchorIds);

}  // namespace spg::scenes
