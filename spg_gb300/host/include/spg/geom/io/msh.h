// spg::io::loadMsh with the reference's signature (spg/include/spg/geom/io/msh.h:6-8).
#pragma once

#include <string>
#include <tuple>
#include <vector>

#include "spg/types.h"

namespace spg::io {
// Nodes and tetrahedra of a Gmsh file (spg/source/geom/io/msh.cpp:10-40).
std::tuple<std::vector<Vector3>, std::vector<Int4>> loadMsh(const std::string &filePath);
}  // namespace spg::io
