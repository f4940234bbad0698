// Declaration-only stand-in for libigl's AABB header. The reference's libigl
// submodule is empty; only its BVH body type (never used by the SDF contact
// path) names these symbols, so every body here throws if it is ever reached.
#pragma once
#include <stdexcept>
namespace igl {
template <typename DerivedV, int DIM>
class AABB {
 public:
  template <typename DV, typename DF>
  void init(const DV&, const DF&) { throw std::runtime_error("igl::AABB unavailable in oracle build"); }
  template <typename DV, typename DF, typename DP, typename DS, typename DI, typename DC>
  void squared_distance(const DV&, const DF&, const DP&, DS&, DI&, DC&) const {
    throw std::runtime_error("igl::AABB unavailable in oracle build");
  }
};
}  // namespace igl
