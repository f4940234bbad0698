// Kernels of the batched point-vs-SDF contact evaluation (sm_103a).
//
// One evaluation of a batch of pair instances (contact body A's points against
// SDF body B's grid, each instance with its own poses) runs three launches:
//
//   detect_kernel    one CTA per tile of kTile points of one instance.  Every
//                    point is transformed into B's grid frame and its distance
//                    evaluated in FP32 with a rigorous error bound; points whose
//                    FP32 distance lies inside the bound ("guard band") or near
//                    the box faces are re-evaluated in FP64 exactly as the
//                    reference does.  Active ids (distance < 0) are compacted
//                    in ascending order per tile (ballot + CTA scan), which is
//                    the order the reference's detection loop produces
//                    (simulation/redmax/CollisionDetection/CollisionDetection.cpp:124-147).
//   force_kernel     one CTA per (instance, slot).  The instance's active
//                    contacts are cut into chunks of kChunk; slot s takes chunks
//                    s, s+kSlots, ...  Each thread evaluates one contact in FP64;
//                    the per-contact force (12 values) and, with derivatives, the
//                    24 Jacobian columns (288 values) are summed over the warp
//                    with shuffles and over the CTA in shared memory, in a fixed
//                    order, into one partial row per (instance, slot).
//   finalize_kernel  sums the kSlots partial rows of each instance in order and
//                    scatters them into fm / Km / Dm.
//
// No atomics touch the results: the sums are deterministic run to run.
#pragma once

#include <cuda_runtime.h>

#include "sdfc_contact.cuh"

namespace sdfc {

constexpr int kTile = 2048;          // points per detection tile
constexpr int kDetectThreads = 256;  // threads per detection CTA
constexpr int kChunk = 128;          // contacts per force chunk = threads per force CTA
constexpr int kSlots = 8;            // partial rows per instance
constexpr int kMaxTilesPerInstance = 4096;
constexpr int kOutDeriv = 300;       // fm (12) + Km (144) + Dm (144)
constexpr int kOutValue = 12;

// Fixed topology of one batch instance.
struct InstanceDesc {
    int points;  // point-set handle (contact body A)
    int grid;    // grid handle (SDF body B)
    int tile0;   // first detection tile
    int ntiles;
};

// Per-evaluation inputs, device pointers (row-major 4x4 poses, body twists).
struct BatchInputs {
    const double* EA;    // n x 16
    const double* phiA;  // n x 6
    const double* EB;    // n x 16
    const double* phiB;  // n x 6
    const double* prm;   // n x 6: kn, kt, mu, damping, scale, contact_scale
};

struct BatchOutputs {
    double* fm;      // n x 12
    double* Km;      // n x 144 (may be null for value-only evaluations)
    double* Dm;      // n x 144
    int* n_active;   // n
    int* status;     // n: bit 0 = non-finite output, bit 1 = FP64 recheck count overflow (unused)
};

struct DetectStats {
    unsigned long long rechecked;  // points re-evaluated in FP64 (diagnostic)
};

void launch_detect(const InstanceDesc* d_inst, const int* d_tile_inst, int total_tiles, BatchInputs in,
                   const GridDesc* d_grids, const PointsDesc* d_points, int* d_ids, int* d_tile_count,
                   unsigned long long* d_recheck, cudaStream_t stream);

void launch_force(const InstanceDesc* d_inst, int n_inst, BatchInputs in, const GridDesc* d_grids,
                  const PointsDesc* d_points, const int* d_ids, const int* d_tile_count, double* d_partial,
                  bool deriv, bool stencil, cudaStream_t stream);

void launch_finalize(const InstanceDesc* d_inst, int n_inst, const int* d_tile_count, const double* d_partial,
                     bool deriv, BatchOutputs out, cudaStream_t stream);

}  // namespace sdfc
