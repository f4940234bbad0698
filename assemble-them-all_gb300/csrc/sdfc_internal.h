// Internal structures of libsdfcontact shared by its C ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <utility>
#include <vector>

#include "sdfc.h"
#include "sdfc_kernels.cuh"

struct sdfc_context {
    int device = 0;
    int sm_count = 1;  // the device's multiprocessors (cudaDevAttrMultiProcessorCount): launch shapes follow it
    cudaStream_t stream = nullptr;
    // host-array calls copy straight between the caller's pageable arrays and the device (the
    // device reads pageable memory through the host page tables, as over Grace's C2C link);
    // otherwise they stage through pinned buffers (SDFC_STAGED_COPIES forces staging)
    bool pageable_direct = false;
    std::string err;
    std::vector<sdfc::GridDesc> grids;  // host copies of the descriptors
    std::vector<sdfc::PointsDesc> points;
    std::vector<sdfc::HullDesc> hulls;  // convex hulls of the disassembly check
    std::vector<void*> allocations;  // every device allocation owned by the context
    sdfc::GridDesc* d_grids = nullptr;
    sdfc::PointsDesc* d_points = nullptr;
    int grid_cap = 0, points_cap = 0;
    int deriv_mode = SDFC_DERIV_ANALYTIC;
    int precision = SDFC_PRECISION_FP64;
    std::vector<std::vector<int>> point_order;  // per point set: stored index -> caller's index
    sdfc_batch* single = nullptr;     // cached one-instance batch of sdfc_evaluate
    int single_points = -1, single_grid = -1;
    std::vector<sdfc_batch*> batches;  // live batches, destroyed with the context
    std::vector<sdfc_sim*> sims;       // live simulations, destroyed with the context
    // tunings found by sdfc_batch_autotune, by batch shape (sdfc_impl::tune_key)
    std::vector<std::pair<std::vector<long long>, sdfc_tuning>> tunings;
};

struct sdfc_batch {
    sdfc_context* ctx = nullptr;
    int n = 0;
    int total_tiles = 0;
    int slots = sdfc::kMaxSlots;  // partial rows per instance, at most (the spread's cap)
    int partial_slots = 0;  // slots the partial-row buffer holds
    int chunks_per_slot = sdfc::kDefaultChunksPerSlot;  // chunks of active contacts per share, at least
    int force_variant = sdfc::kForceCtas;
    int worker_ctas = 0;  // one-warp force workers (0: the device's multiprocessors x resident workers)
    int max_ntiles = 0;   // most detection tiles of one instance
    float tuned_ms = 0.f;  // measured evaluation time of the configuration in use (0: not measured)
    int deriv_mode = SDFC_DERIV_ANALYTIC;
    int precision = SDFC_PRECISION_FP64;
    std::vector<sdfc::InstanceDesc> inst;
    sdfc::InstanceDesc* d_inst = nullptr;
    int* d_tile_inst = nullptr;
    int* d_ids = nullptr;
    int* d_tile_count = nullptr;
    int* d_tile_queue = nullptr;
    sdfc::Prefilter* d_prefilter = nullptr;
    sdfc::PairState<float>* d_pair32 = nullptr;
    sdfc::PairState<double>* d_pair64 = nullptr;
    int* d_recheck_list = nullptr;  // total_tiles
    int* d_recheck_n = nullptr;     // sdfc::kCounters counters (BatchScratch::recheck_n)
    int* d_badin = nullptr;         // n: non-finite inputs (BatchScratch::badin)
    int* d_inst_total = nullptr;    // n: active contacts per instance (BatchScratch::inst_total)
    int* d_items = nullptr;         // 4 x n x kMaxSlots: the force passes' item lists
    double* d_partial = nullptr;
    unsigned long long* d_recheck = nullptr;
    long long* d_point_offset = nullptr;  // n: first output row of each instance's per-point distances
    // instances on grids with the FP32 cell-corner array (storages 0, 1), on grids without it
    bool has_plain = true, has_bricks = false;
    long long total_points = 0;
    // staging of the host-array entry points
    double* d_in = nullptr;   // n x 50: EA | phiA | EB | phiB | prm
    double* d_out = nullptr;  // n x 300: fm | Km | Dm
    int* d_int = nullptr;     // n x 2: n_active | status
    double* h_in = nullptr;   // pinned
    double* h_out = nullptr;  // pinned
    int* h_int = nullptr;     // pinned
    // the direct host-array path (the device reads pageable memory): the call's array pointers,
    // written to the pinned copy and sent to the device copy before each graph launch
    sdfc::HostIO* h_io = nullptr;
    sdfc::HostIO* d_io = nullptr;
    bool timing = false;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // sdfc_batch_evaluate's device work (H2D of the staged inputs, the evaluation, D2H of the
    // results) as a graph per derivative flag, with the modes it was captured under
    cudaGraphExec_t eval_exec[2] = {nullptr, nullptr};
    int eval_key[2] = {-1, -1};
    cudaStream_t eval_stream = nullptr;
    // masked evaluations: the value pass runs on this stream beside the derivative pass
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
};

namespace sdfc_impl {

int fail(sdfc_context* ctx, int code, const std::string& msg);
int dev_alloc(sdfc_context* ctx, void** p, size_t bytes);
int use_device(sdfc_context* ctx);
int batch_create(sdfc_context* ctx, int n, const int* points, const int* grids, sdfc_batch** out);
void free_batch(sdfc_batch* b);
void free_sim(sdfc_sim* s);
// One evaluation of every instance (in.mode null) with `deriv`, or, with
// in.mode set, each instance as it requests (0 skip, 1 value, 2 derivatives).
// Penetration energy of every requested instance (in.mode: 0 skips): energy[n], dE[n x 12].
int run_energy(sdfc_batch* b, const sdfc::BatchInputs& in, double* energy, double* dE, cudaStream_t stream);
int run_batch(sdfc_batch* b, const sdfc::BatchInputs& in, bool deriv, const sdfc::BatchOutputs& out,
              cudaStream_t stream);
// The kernels' view of a batch's scratch and launch configuration.
sdfc::BatchScratch scratch_of(const sdfc_batch* b);
// Makes the batch's partial-row buffer hold `slots` rows per instance (reallocating it; not
// during a stream capture).
int ensure_partial(sdfc_batch* b, int slots);
// Times the candidate launch configurations of the force pass on these inputs (each a whole
// evaluation, CUDA events on `stream`), applies the fastest and remembers it in the context for
// batches of the same shape; `chosen` (may be null) receives it.
int autotune(sdfc_batch* b, const sdfc::BatchInputs& in, bool deriv, const sdfc::BatchOutputs& out,
             cudaStream_t stream, sdfc_tuning* chosen);
// Device-side grid preparation (sdfc_grid.cu) from the node values at d_values (FP32 or FP64,
// ni*nj*nk, i fastest, on the device): g.lip and g.vmax, and with `cells` the FP32 cell-corner
// array (owned by the context).  Fails with SDFC_ERR_INVALID_ARGUMENT on a non-finite value.
int grid_finish_device(sdfc_context* ctx, sdfc::GridDesc& g, const void* d_values, bool fp32, bool cells);
// b[0..n) = (double) a[0..n), both on the device, on the context's stream.
int widen_device(sdfc_context* ctx, const float* a, double* b, size_t n);

}  // namespace sdfc_impl

#define SDFC_CUDA_TRY(ctx, call)                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return sdfc_impl::fail((ctx), SDFC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)
