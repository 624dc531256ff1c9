// spg::io::loadObj with the reference's signature (spg/include/spg/geom/io/obj.h:6-8).
#pragma once

#include <string>
#include <tuple>
#include <vector>

#include "spg/types.h"

namespace spg::io {
// Vertices of the whole file and the triangles of its first shape (spg/source/geom/io/obj.cpp:9-35).
std::tuple<std::vector<Vector3>, std::vector<Int3>> loadObj(const std::string &filePath);
}  // namespace spg::io
