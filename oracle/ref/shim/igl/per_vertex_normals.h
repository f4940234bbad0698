// Declaration-only stand-in for libigl's per_vertex_normals header (BVH path only).
#pragma once
#include <stdexcept>
namespace igl {
enum PerVertexNormalsWeightingType { PER_VERTEX_NORMALS_WEIGHTING_TYPE_ANGLE = 0 };
template <typename... Ts>
void per_vertex_normals(const Ts&...) { throw std::runtime_error("igl::per_vertex_normals unavailable in oracle build"); }
}  // namespace igl
