// Declaration-only stand-in for libigl's signed_distance header (BVH path only).
#pragma once
#include <stdexcept>
namespace igl {
template <typename... Ts>
void signed_distance_pseudonormal(const Ts&...) { throw std::runtime_error("igl::signed_distance unavailable in oracle build"); }
}  // namespace igl
