// Declaration-only stand-in for libigl's per_face_normals header (BVH path only).
#pragma once
#include <stdexcept>
namespace igl {
template <typename... Ts>
void per_face_normals(const Ts&...) { throw std::runtime_error("igl::per_face_normals unavailable in oracle build"); }
}  // namespace igl
