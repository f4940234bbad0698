// Kernels of the batched point-vs-SDF contact evaluation (sm_103a).
//
// One evaluation of a batch of pair instances (contact body A's points against
// SDF body B's grid, each instance with its own poses) runs these launches:
//
//   prep_kernel      one thread per instance: the FP32 point transform into B's
//                    grid frame and the error bound ("guard band") of the FP32
//                    distance, from the instance's FP64 poses.
//   detect_kernel    one CTA per tile of kTile points of one instance.  Every
//                    point's distance is evaluated in FP32; points whose FP32
//                    distance is outside the guard band are classified there,
//                    the others (and points near the box faces) are queued in
//                    the tile for an exact FP64 recheck.  Active stored indices
//                    are compacted in ascending order (ballot + CTA scan).
//   recheck_kernel   one warp per tile with queued points (detect_kernel lists
//                    those tiles): the reference's FP64 distance
//                    (BodySDFObj::distance, bit-identical), appending the active
//                    ones to the tile's list in ascending order.
//                    Detection as a whole restates
//                    simulation/redmax/CollisionDetection/CollisionDetection.cpp:124-147.
//   plan_kernel      (queue forms) one thread per instance: its items (instance, share
//                    0..S-1), appended to the item list of its force launch.  S, the
//                    instance's spread, is the number of partial sums it is cut into: its
//                    active contacts (counted by detection) over the tuned contacts per share,
//                    at most `slots` (spread_of).
//   force_kernel     one CTA per (instance, share) (the grid form), or persistent CTAs taking
//                    items from the list (force_queue_kernel).  An instance's active contacts
//                    are cut into chunks of kChunk; share s takes chunks s, s+S, ...  Each
//                    thread evaluates one contact; the
//                    per-contact force (12 values) and, with derivatives, the
//                    Jacobian columns (24 on the FP64 path; 15 on the FP32 path,
//                    which leaves body B's twist columns to finalize_kernel) are
//                    summed over the warp with shuffles and over the CTA's warps
//                    in shared memory, in a fixed order, into one partial row per
//                    (instance, share).
//                    On the FP32 path a contact whose derivative stencil could
//                    leave its cell takes the exact path (the reference's FP64
//                    stencil); the warp evaluates such contacts' 19 stencil
//                    queries together, one contact at a time across its lanes
//                    (warp_exact_jets), so that no lane runs the long FP64
//                    stencil alone while 31 wait.
//   finalize_kernel  one CTA per instance: sums its S partial rows in order,
//                    derives the FP32 path's body-B columns (Km: -Km1 Ad; Dm:
//                    -Dm1 Ad + C) and writes fm / Km / Dm, n_active and status.
//
// No atomics touch the results: which CTA takes an item does not change its sums, so they are
// deterministic run to run (the contact counts are integer atomic sums, exact in any order).
#pragma once

#include <cuda_runtime.h>

#include "sdfc_contact.cuh"

namespace sdfc {

constexpr int kTile = 2048;          // points per detection tile
constexpr int kDetectThreads = 256;  // threads per detection CTA
// contacts per force chunk = threads per force CTA, and the FP32 force CTAs resident per SM
// (their register budget is 65536 / (this x kChunk)): compile-time tuning knobs
#ifndef SDFC_FORCE_CHUNK
#define SDFC_FORCE_CHUNK 128
#endif
#ifndef SDFC_FORCE_MIN_BLOCKS
#define SDFC_FORCE_MIN_BLOCKS 4
#endif
constexpr int kChunk = SDFC_FORCE_CHUNK;
constexpr int kForceCtasPerSm = SDFC_FORCE_MIN_BLOCKS;
// the same for the force instantiation that serves every grid storage (FP16 bricks, FP32 nodes)
#ifndef SDFC_FORCE_MIN_BLOCKS_GENERAL
#define SDFC_FORCE_MIN_BLOCKS_GENERAL 5
#endif
constexpr int kForceCtasPerSmGeneral = SDFC_FORCE_MIN_BLOCKS_GENERAL;
constexpr int kMaxSlots = 128;       // partial rows per instance, at most
// Multiprocessors of the current device (cudaDevAttrMultiProcessorCount, looked up once per
// device): launch shapes follow it.
int device_sm_count();
// Default cap on an instance's partial sums for a batch of n instances: kMaxSlots, lowered so
// that the partial-row buffer (n x slots rows of kOutDeriv doubles) stays within 2^18 rows
// (630 MB).  An instance takes as many shares as its active contacts fill, up to the cap.
inline int slots_for(int n) {
    int s = kMaxSlots;
    while (s > 1 && (long long)s * n > (1LL << 18)) s /= 2;
    return s;
}
// Default chunks per share (sdfc_tuning::chunks_per_slot): an instance with c chunks of active
// contacts is cut into min(slots, ceil(c / this)) shares.
constexpr int kDefaultChunksPerSlot = 4;
constexpr int kMaxTilesPerInstance = 4096;
constexpr int kOutDeriv = 300;       // fm (12) + Km (144) + Dm (144)
constexpr int kOutValue = 12;
constexpr int kOutEnergy = 13;      // penetration energy + its 12 twist derivatives

// A convex hull on the device (the planner's disassembly check): vertices (nv x 3) and facet
// planes (nf x 4, n . x + offset <= 0 inside), with the vertices' bounds.
struct HullDesc {
    int nv, nf;
    const double* v;
    const double* planes;
    double lo[3], hi[3];
};

// The three forms of the force pass (a batch's tuning picks one; each sums each (instance,
// share) into its own partial row in a fixed order, so each is deterministic):
//   kForceCtas    force_queue_kernel: persistent CTAs of kChunk threads taking the items of
//                 plan_kernel's list from a queue, chunks of kChunk contacts, the CTA's warps
//                 merged at the end of each item;
//   kForceWorkers force_worker_kernel: persistent one-warp CTAs, chunks of 32 contacts.  No CTA
//                 barrier: a warp that finishes an item takes the next instead of waiting for
//                 its CTA.
//   kForceGrid    force_kernel: one CTA per (instance, share) for every share up to `slots`
//                 (CTAs past an instance's spread return at once), no list, no queue.
enum ForceVariant { kForceCtas = 0, kForceWorkers = 1, kForceGrid = 2 };

// Fixed topology of one batch instance.
struct InstanceDesc {
    int points;  // point-set handle (contact body A)
    int grid;    // grid handle (SDF body B)
    int tile0;   // first detection tile
    int ntiles;
};

// FP32 prefilter constants of one instance (written by prep_kernel).
struct Prefilter {
    float R[9], p[3];            // point -> grid frame: x = R xi + p
    float gmin[3], ginv[3];      // grid origin and 1/dx
    float lo_in[3], hi_in[3];    // certainly inside the box between these
    float lo_out[3], hi_out[3];  // certainly outside beyond these
    float col_th;
    float guard;                 // bound on |d32 - d64|, times a safety factor
    // a point whose cell lies in a block with least node value above this is neither active nor
    // within the guard band (GridDesc::bmin): guard - col_th plus the FP32 trilinear's error bound
    float skip_th;
};

// Per-evaluation inputs, device pointers (row-major 4x4 poses, body twists).
struct BatchInputs {
    const double* EA;    // n x 16
    const double* phiA;  // n x 6
    const double* EB;    // n x 16
    const double* phiB;  // n x 6
    const double* prm;   // n x 6: kn, kt, mu, damping, scale, contact_scale
    // optional per-instance request (null: every instance, with the launch's
    // derivative flag): 0 skip, 1 value only, 2 with derivatives
    const int* mode = nullptr;
};

struct BatchOutputs {
    double* fm;      // n x 12
    double* Km;      // n x 144 (may be null for value-only evaluations)
    double* Dm;      // n x 144
    int* n_active;   // n
    int* status;     // n: bit 0 = non-finite output, bit 1 = non-finite input
    // not null: the kernels take the five pointers from this device copy instead, which the
    // host rewrites per call (a captured graph then writes wherever the call asks, e.g. into
    // the caller's own host arrays where the device reads pageable memory)
    const BatchOutputs* dev = nullptr;
};

// One host-array evaluation as the device sees it: the caller's five input arrays
// (E_A n x 16, phi_A n x 6, E_B n x 16, phi_B n x 6, params n x 6) and its outputs.
struct HostIO {
    const double* in[5];
    BatchOutputs out;
};

// status[i] = 0 for every instance (launch_finalize does it itself with zero_status).
void launch_zero_status(BatchOutputs out, int n_inst, cudaStream_t stream);

// d (n x 50, the BatchInputs block) <- the arrays io->in point to (read by the device).
void launch_gather_inputs(const HostIO* io, double* d, int n, cudaStream_t stream);

// Scratch of a batch: device buffers sized at batch creation.
struct BatchScratch {
    Prefilter* prefilter;       // n
    int* ids;                   // total_tiles x kTile: active stored indices, queued rechecks at the tail
    int* tile_count;            // total_tiles: active count per tile
    int* tile_queue;            // total_tiles: queued recheck count per tile
    double* partial;            // n x slots x kOutDeriv
    unsigned long long* recheck;  // diagnostic counter of FP64 rechecks
    int slots;                  // partial rows per instance, at most (the spread's cap)
    PairState<float>* pair32;   // n: each instance's pair state for the FP32 kernels (written by prep_kernel)
    PairState<double>* pair64;  // n: the same for the FP64 kernels
    int* recheck_list;          // total_tiles: the tiles with queued points (appended by detect_kernel)
    // kCounters counters, reset by prep_kernel: [0] the count of recheck_list, [1..4] the queue
    // forms' queues, [5..8] the lengths of their item lists (plan_kernel).  Lists / queues by
    // launch: 0 derivative pass, 1 derivative pass on grids without the cell-corner array when the
    // FP32 fast path splits the instances by storage, 2 / 3 the same for the value pass.
    int* recheck_n;
    int* badin = nullptr;            // n: 1 where the instance's inputs are not all finite (prep_kernel)
    int force_variant = kForceCtas;  // which force kernel runs (set by the batch's tuning)
    int worker_ctas = 0;             // force workers launched (0: the device's multiprocessors x resident)
    int max_ntiles = 0;              // most detection tiles of one instance (the workers' shared prefix)
    int chunks_per_slot = kDefaultChunksPerSlot;  // chunks of active contacts per share, at least
    int* inst_total = nullptr;  // n: active contacts per instance (zeroed by prep_kernel, summed by detection)
    int* items = nullptr;       // 4 lists of n x slots items (instance x kMaxSlots + share), plan_kernel
};
constexpr int kCounters = 9;

enum Precision { kFP64 = 0, kMixed = 1 };

// plain / bricks: whether the batch has instances on grids with the FP32 cell-corner array
// (storages 0 and 1) / on grids without it (FP16 bricks, FP32 node values).
void launch_detect(const InstanceDesc* d_inst, const int* d_tile_inst, int n_inst, int total_tiles, BatchInputs in,
                   const GridDesc* d_grids, const PointsDesc* d_points, BatchScratch s, cudaStream_t stream,
                   bool plain = true, bool bricks = true);

// The force passes' item lists from detection's contact counts (after launch_detect, before
// launch_force): without a request mask every instance goes to the pass `deriv` asks for, with
// one (in.mode) each instance to the pass it requests.  One launch covers both passes.
void launch_plan(const InstanceDesc* d_inst, int n_inst, BatchInputs in, const GridDesc* d_grids, BatchScratch s,
                 bool deriv, bool stencil, int precision, cudaStream_t stream, bool plain = true, bool bricks = true);

void launch_force(const InstanceDesc* d_inst, int n_inst, BatchInputs in, const GridDesc* d_grids,
                  const PointsDesc* d_points, BatchScratch s, bool deriv, bool stencil, int precision,
                  cudaStream_t stream, bool plain = true, bool bricks = true);

// Finalizes the status words too: without a mask every instance's status is
// written outright; with one (in.mode), zero_status clears them all first, and
// only the instances whose request matches `deriv` are finalized (zero_status =
// false lets a second, value-only pass keep the first pass's status bits).
// derive_q2: the inputs of the evaluation whose force pass skipped the dq2 columns
// of Km (force_skips_q2); finalize derives them from the dq1 columns.
void launch_finalize(const InstanceDesc* d_inst, int n_inst, BatchScratch s, bool deriv, BatchOutputs out,
                     cudaStream_t stream, const int* mode = nullptr, bool zero_status = true,
                     const BatchInputs* derive_q2 = nullptr);
// Penetration energy (sum of kn d^2 / 2 over the active contacts) and its gradient wrt
// both bodies' twists, after launch_detect: energy[n], dE[n x 12] (A: w, v; B: w, v).
void launch_energy(const InstanceDesc* d_inst, int n_inst, BatchInputs in, const GridDesc* d_grids,
                   const PointsDesc* d_points, BatchScratch s, bool stencil, int precision, cudaStream_t stream);
void launch_energy_finalize(int n_inst, BatchScratch s, double* energy, double* dE, const int* mode,
                            cudaStream_t stream);
// The reference's distance (BodySDFObj::distance) of every point of every instance, FP64,
// bit-identical: min_d[n] the per-instance minimum (+inf for an empty point set) and, with d
// non-null, d[point_offset[i] + caller's index] every point's distance.
void launch_distance(const InstanceDesc* d_inst, const int* d_tile_inst, int n_inst, int total_tiles, BatchInputs in,
                     const GridDesc* d_grids, const PointsDesc* d_points, const long long* point_offset,
                     unsigned long long* key_scratch, double* min_d, double* d, cudaStream_t stream);
// SDFMesh::query_SDF at n points X (n x 3, grid frame): d[n] (may be null) and the minimum
// min_d[0] (may be null; key_scratch: one word).
void launch_grid_query(const GridDesc* d_grids, int grid, const double* X, int n, double* d,
                       unsigned long long* key_scratch, double* min_d, cudaStream_t stream);
// Whether launch_force's derivative pass leaves the dq2 columns of Km to finalize
// (the FP32-algebra path outside the stencil mode).
bool force_skips_q2(bool deriv, bool stencil, int precision);

}  // namespace sdfc
