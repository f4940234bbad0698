// Declaration-only stand-in for libigl's per_edge_normals header (BVH path only).
#pragma once
#include <stdexcept>
namespace igl {
enum PerEdgeNormalsWeightingType { PER_EDGE_NORMALS_WEIGHTING_TYPE_UNIFORM = 0 };
template <typename... Ts>
void per_edge_normals(const Ts&...) { throw std::runtime_error("igl::per_edge_normals unavailable in oracle build"); }
}  // namespace igl
