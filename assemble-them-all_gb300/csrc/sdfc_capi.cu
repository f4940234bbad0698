// C ABI of libsdfcontact (include/sdfc.h): contexts, uploads, batches.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sdfc.h"
#include "sdfc_internal.h"
#include "sdfc_kernels.cuh"

using sdfc::GridDesc;
using sdfc::InstanceDesc;
using sdfc::PointsDesc;
using sdfc_impl::dev_alloc;
using sdfc_impl::fail;
using sdfc_impl::free_batch;
using sdfc_impl::use_device;

#define CUDA_TRY(ctx, call) SDFC_CUDA_TRY(ctx, call)

namespace sdfc_impl {

int fail(sdfc_context* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int dev_alloc(sdfc_context* ctx, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(ctx, SDFC_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return SDFC_OK;
}

int use_device(sdfc_context* ctx) {
    CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    return SDFC_OK;
}

void free_batch(sdfc_batch* b) {
    if (!b) return;
    cudaFree(b->d_inst);
    cudaFree(b->d_tile_inst);
    cudaFree(b->d_ids);
    cudaFree(b->d_tile_count);
    cudaFree(b->d_tile_queue);
    cudaFree(b->d_prefilter);
    cudaFree(b->d_pair32);
    cudaFree(b->d_pair64);
    cudaFree(b->d_recheck_list);
    cudaFree(b->d_recheck_n);
    cudaFree(b->d_badin);
    cudaFree(b->d_inst_total);
    cudaFree(b->d_items);
    cudaFree(b->d_partial);
    cudaFree(b->d_recheck);
    cudaFree(b->d_point_offset);
    cudaFree(b->d_in);
    cudaFree(b->d_out);
    cudaFree(b->d_int);
    cudaFreeHost(b->h_in);
    cudaFreeHost(b->h_out);
    cudaFreeHost(b->h_int);
    cudaFreeHost(b->h_io);
    cudaFree(b->d_io);
    for (cudaEvent_t e : b->ev)
        if (e) cudaEventDestroy(e);
    for (cudaGraphExec_t g : b->eval_exec)
        if (g) cudaGraphExecDestroy(g);
    if (b->eval_stream) cudaStreamDestroy(b->eval_stream);
    if (b->aux_stream) cudaStreamDestroy(b->aux_stream);
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    if (b->join_ev) cudaEventDestroy(b->join_ev);
    delete b;
}

sdfc::BatchScratch scratch_of(const sdfc_batch* b) {
    sdfc::BatchScratch sc{b->d_prefilter, b->d_ids, b->d_tile_count, b->d_tile_queue, b->d_partial, b->d_recheck,
                         b->slots, b->d_pair32, b->d_pair64, b->d_recheck_list, b->d_recheck_n};
    sc.force_variant = b->force_variant;
    sc.worker_ctas = b->worker_ctas;
    sc.max_ntiles = b->max_ntiles;
    sc.badin = b->d_badin;
    sc.chunks_per_slot = b->chunks_per_slot;
    sc.inst_total = b->d_inst_total;
    sc.items = b->d_items;
    return sc;
}

int ensure_partial(sdfc_batch* b, int slots) {
    if (slots <= b->partial_slots) return SDFC_OK;
    void* p = nullptr;
    int rc = dev_alloc(b->ctx, &p, sizeof(double) * (size_t)b->n * slots * sdfc::kOutDeriv);
    if (rc) return rc;
    cudaFree(b->d_partial);
    b->d_partial = (double*)p;
    b->partial_slots = slots;
    return SDFC_OK;
}

int run_batch(sdfc_batch* b, const sdfc::BatchInputs& in, bool deriv, const sdfc::BatchOutputs& out,
              cudaStream_t stream) {
    sdfc_context* ctx = b->ctx;
    const sdfc::BatchScratch sc = scratch_of(b);
    const bool stencil = b->deriv_mode == SDFC_DERIV_STENCIL;
    const int prec = b->precision == SDFC_PRECISION_MIXED ? sdfc::kMixed : sdfc::kFP64;
    if (b->timing) cudaEventRecord(b->ev[0], stream);
    sdfc::launch_detect(b->d_inst, b->d_tile_inst, b->n, b->total_tiles, in, ctx->d_grids, ctx->d_points, sc, stream,
                        b->has_plain, b->has_bricks);
    if (b->timing) cudaEventRecord(b->ev[1], stream);
    sdfc::launch_plan(b->d_inst, b->n, in, ctx->d_grids, sc, deriv, stencil, prec, stream, b->has_plain,
                      b->has_bricks);
    const sdfc::BatchInputs* q2 = sdfc::force_skips_q2(true, stencil, prec) ? &in : nullptr;
    if (in.mode && !b->timing && b->aux_stream) {
        // masked evaluation: the derivative and value passes touch disjoint instances (and
        // partial rows), so the value pass runs on a forked stream beside the derivative pass
        sdfc::launch_zero_status(out, b->n, stream);
        CUDA_TRY(ctx, cudaEventRecord(b->fork_ev, stream));
        CUDA_TRY(ctx, cudaStreamWaitEvent(b->aux_stream, b->fork_ev, 0));
        sdfc::launch_force(b->d_inst, b->n, in, ctx->d_grids, ctx->d_points, sc, false, stencil, prec, b->aux_stream,
                           b->has_plain, b->has_bricks);
        sdfc::launch_finalize(b->d_inst, b->n, sc, false, out, b->aux_stream, in.mode, false);
        sdfc::launch_force(b->d_inst, b->n, in, ctx->d_grids, ctx->d_points, sc, true, stencil, prec, stream,
                           b->has_plain, b->has_bricks);
        sdfc::launch_finalize(b->d_inst, b->n, sc, true, out, stream, in.mode, false, q2);
        CUDA_TRY(ctx, cudaEventRecord(b->join_ev, b->aux_stream));
        CUDA_TRY(ctx, cudaStreamWaitEvent(stream, b->join_ev, 0));
        CUDA_TRY(ctx, cudaGetLastError());
        return SDFC_OK;
    }
    if (in.mode) {
        sdfc::launch_force(b->d_inst, b->n, in, ctx->d_grids, ctx->d_points, sc, true, stencil, prec, stream,
                           b->has_plain, b->has_bricks);
        sdfc::launch_force(b->d_inst, b->n, in, ctx->d_grids, ctx->d_points, sc, false, stencil, prec, stream,
                           b->has_plain, b->has_bricks);
    } else {
        sdfc::launch_force(b->d_inst, b->n, in, ctx->d_grids, ctx->d_points, sc, deriv, stencil, prec, stream,
                           b->has_plain, b->has_bricks);
    }
    if (b->timing) cudaEventRecord(b->ev[2], stream);
    if (in.mode) {
        sdfc::launch_finalize(b->d_inst, b->n, sc, true, out, stream, in.mode, true, q2);
        sdfc::launch_finalize(b->d_inst, b->n, sc, false, out, stream, in.mode, false);
    } else {
        sdfc::launch_finalize(b->d_inst, b->n, sc, deriv, out, stream, nullptr, true, deriv ? q2 : nullptr);
    }
    if (b->timing) cudaEventRecord(b->ev[3], stream);
    CUDA_TRY(ctx, cudaGetLastError());
    return SDFC_OK;
}

int run_energy(sdfc_batch* b, const sdfc::BatchInputs& in, double* energy, double* dE, cudaStream_t stream) {
    sdfc_context* ctx = b->ctx;
    const sdfc::BatchScratch sc = scratch_of(b);
    const bool stencil = b->deriv_mode == SDFC_DERIV_STENCIL;
    const int prec = b->precision == SDFC_PRECISION_MIXED ? sdfc::kMixed : sdfc::kFP64;
    sdfc::launch_detect(b->d_inst, b->d_tile_inst, b->n, b->total_tiles, in, ctx->d_grids, ctx->d_points, sc, stream,
                        b->has_plain, b->has_bricks);
    sdfc::launch_energy(b->d_inst, b->n, in, ctx->d_grids, ctx->d_points, sc, stencil, prec, stream);
    sdfc::launch_energy_finalize(b->n, sc, energy, dE, in.mode, stream);
    CUDA_TRY(ctx, cudaGetLastError());
    return SDFC_OK;
}

}  // namespace sdfc_impl

namespace {

template <class T>
int sync_table(sdfc_context* ctx, std::vector<T>& host, T** d_table, int* cap) {
    if ((int)host.size() > *cap) {
        int ncap = std::max(64, *cap * 2);
        while (ncap < (int)host.size()) ncap *= 2;
        void* p = nullptr;
        int rc = dev_alloc(ctx, &p, sizeof(T) * ncap);
        if (rc) return rc;
        if (*d_table) cudaFree(*d_table);
        *d_table = (T*)p;
        *cap = ncap;
    }
    CUDA_TRY(ctx, cudaMemcpy(*d_table, host.data(), sizeof(T) * host.size(), cudaMemcpyHostToDevice));
    return SDFC_OK;
}

int run_batch(sdfc_batch* b, const double* EA, const double* phiA, const double* EB, const double* phiB,
              const double* prm, bool deriv, double* fm, double* Km, double* Dm, int* n_active, int* status,
              cudaStream_t stream) {
    sdfc::BatchInputs in{EA, phiA, EB, phiB, prm};
    sdfc::BatchOutputs out{fm, Km, Dm, n_active, status};
    return sdfc_impl::run_batch(b, in, deriv, out, stream);
}

bool all_finite(const double* v, size_t n) {
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) return false;
    return true;
}

}  // namespace

int sdfc_impl::batch_create(sdfc_context* ctx, int n, const int* points, const int* grids, sdfc_batch** out) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (n <= 0 || !points || !grids || !out) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_create: bad argument");
    int rc = use_device(ctx);
    if (rc) return rc;
    auto* b = new sdfc_batch();
    b->ctx = ctx;
    b->n = n;
    b->deriv_mode = ctx->deriv_mode;
    b->slots = sdfc::slots_for(n);
    b->partial_slots = b->slots;
    b->precision = ctx->precision;
    b->inst.resize(n);
    std::vector<int> tile_inst;
    std::vector<long long> point_offset(n);
    int tiles = 0;
    for (int k = 0; k < n; ++k) {
        if (points[k] < 0 || points[k] >= (int)ctx->points.size() || grids[k] < 0 || grids[k] >= (int)ctx->grids.size()) {
            delete b;
            return fail(ctx, SDFC_ERR_NOT_FOUND, "batch_create: unknown point-set or grid handle");
        }
        int np = ctx->points[points[k]].n;
        int nt = (np + sdfc::kTile - 1) / sdfc::kTile;
        if (nt > sdfc::kMaxTilesPerInstance) {
            delete b;
            return fail(ctx, SDFC_ERR_CAPACITY, "batch_create: point set larger than kTile*kMaxTilesPerInstance");
        }
        b->inst[k] = InstanceDesc{points[k], grids[k], tiles, nt};
        b->max_ntiles = std::max(b->max_ntiles, nt);
        point_offset[k] = b->total_points;
        b->total_points += np;
        for (int t = 0; t < nt; ++t) tile_inst.push_back(k);
        tiles += nt;
    }
    b->total_tiles = tiles;
    b->has_plain = b->has_bricks = false;
    for (int k = 0; k < n; ++k) (ctx->grids[grids[k]].cells32 ? b->has_plain : b->has_bricks) = true;
    auto alloc = [&](void** p, size_t bytes) { return dev_alloc(ctx, p, bytes); };
    if ((rc = alloc((void**)&b->d_inst, sizeof(InstanceDesc) * n)) ||
        (rc = alloc((void**)&b->d_tile_inst, sizeof(int) * std::max(tiles, 1))) ||
        (rc = alloc((void**)&b->d_ids, sizeof(int) * (size_t)std::max(tiles, 1) * sdfc::kTile)) ||
        (rc = alloc((void**)&b->d_tile_count, sizeof(int) * std::max(tiles, 1))) ||
        (rc = alloc((void**)&b->d_tile_queue, sizeof(int) * std::max(tiles, 1))) ||
        (rc = alloc((void**)&b->d_prefilter, sizeof(sdfc::Prefilter) * n)) ||
        (rc = alloc((void**)&b->d_pair32, sizeof(sdfc::PairState<float>) * n)) ||
        (rc = alloc((void**)&b->d_pair64, sizeof(sdfc::PairState<double>) * n)) ||
        (rc = alloc((void**)&b->d_recheck_list, sizeof(int) * std::max(tiles, 1))) ||
        (rc = alloc((void**)&b->d_recheck_n, sdfc::kCounters * sizeof(int))) ||
        (rc = alloc((void**)&b->d_badin, sizeof(int) * (size_t)n)) ||
        (rc = alloc((void**)&b->d_inst_total, sizeof(int) * (size_t)n)) ||
        (rc = alloc((void**)&b->d_items, sizeof(int) * 4 * (size_t)n * sdfc::kMaxSlots)) ||
        (rc = alloc((void**)&b->d_partial, sizeof(double) * (size_t)n * b->slots * sdfc::kOutDeriv)) ||
        (rc = alloc((void**)&b->d_recheck, sizeof(unsigned long long))) ||
        (rc = alloc((void**)&b->d_point_offset, sizeof(long long) * n)) ||
        (rc = alloc((void**)&b->d_in, sizeof(double) * (size_t)n * 50)) ||
        (rc = alloc((void**)&b->d_out, sizeof(double) * (size_t)n * sdfc::kOutDeriv)) ||
        (rc = alloc((void**)&b->d_int, sizeof(int) * (size_t)n * 2)) ||
        (rc = alloc((void**)&b->d_io, sizeof(sdfc::HostIO)))) {
        free_batch(b);
        return rc;
    }
    if (cudaMallocHost((void**)&b->h_in, sizeof(double) * (size_t)n * 50) != cudaSuccess ||
        cudaMallocHost((void**)&b->h_out, sizeof(double) * (size_t)n * sdfc::kOutDeriv) != cudaSuccess ||
        cudaMallocHost((void**)&b->h_int, sizeof(int) * (size_t)n * 2) != cudaSuccess ||
        cudaMallocHost((void**)&b->h_io, sizeof(sdfc::HostIO)) != cudaSuccess) {
        free_batch(b);
        return fail(ctx, SDFC_ERR_CUDA, "batch_create: cudaMallocHost failed");
    }
    cudaError_t e = cudaStreamCreateWithFlags(&b->aux_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_inst, b->inst.data(), sizeof(InstanceDesc) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && tiles > 0)
        e = cudaMemcpy(b->d_tile_inst, tile_inst.data(), sizeof(int) * tiles, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_point_offset, point_offset.data(), sizeof(long long) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->d_recheck, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(b->d_tile_count, 0, sizeof(int) * std::max(tiles, 1));
    if (e == cudaSuccess) e = cudaMemset(b->d_tile_queue, 0, sizeof(int) * std::max(tiles, 1));
    if (e != cudaSuccess) {
        free_batch(b);
        return fail(ctx, SDFC_ERR_CUDA, std::string("batch_create: ") + cudaGetErrorString(e));
    }
    *out = b;
    return SDFC_OK;
}

extern "C" {

int sdfc_create(sdfc_context** out, int device) {
    if (!out) return SDFC_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) return SDFC_ERR_CUDA;
    auto* ctx = new sdfc_context();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete ctx;
        return SDFC_ERR_CUDA;
    }
    int direct = 0;
    if (cudaDeviceGetAttribute(&direct, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) != cudaSuccess)
        direct = 0;
    ctx->pageable_direct = direct != 0 && std::getenv("SDFC_STAGED_COPIES") == nullptr;
    if (cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        ctx->sm_count < 1)
        ctx->sm_count = 1;
    *out = ctx;
    return SDFC_OK;
}

void sdfc_destroy(sdfc_context* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (sdfc_sim* s : ctx->sims) sdfc_impl::free_sim(s);
    for (sdfc_batch* b : ctx->batches) free_batch(b);
    free_batch(ctx->single);
    for (void* p : ctx->allocations) cudaFree(p);
    cudaFree(ctx->d_grids);
    cudaFree(ctx->d_points);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* sdfc_last_error(const sdfc_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int sdfc_set_derivative_mode(sdfc_context* ctx, int mode) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (mode != SDFC_DERIV_ANALYTIC && mode != SDFC_DERIV_STENCIL)
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "set_derivative_mode: unknown mode");
    ctx->deriv_mode = mode;
    if (ctx->single) ctx->single->deriv_mode = mode;
    return SDFC_OK;
}

int sdfc_set_precision(sdfc_context* ctx, int precision) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (precision != SDFC_PRECISION_FP64 && precision != SDFC_PRECISION_MIXED)
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "set_precision: unknown precision");
    ctx->precision = precision;
    if (ctx->single) ctx->single->precision = precision;
    return SDFC_OK;
}

int sdfc_batch_set_precision(sdfc_batch* b, int precision) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    if (precision != SDFC_PRECISION_FP64 && precision != SDFC_PRECISION_MIXED)
        return fail(b->ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_set_precision: unknown precision");
    b->precision = precision;
    return SDFC_OK;
}

int sdfc_batch_set_derivative_mode(sdfc_batch* b, int mode) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    if (mode != SDFC_DERIV_ANALYTIC && mode != SDFC_DERIV_STENCIL)
        return fail(b->ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_set_derivative_mode: unknown mode");
    b->deriv_mode = mode;
    return SDFC_OK;
}

}  // extern "C"

// Shape, box and spacing checks shared by the grid uploads.
static int check_grid(sdfc_context* ctx, int ni, int nj, int nk, const double min_box[3], const double max_box[3],
                      const double dxyz[3], double col_th, int storage) {
    if (!min_box || !max_box || !dxyz) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid: null argument");
    if (ni < 2 || nj < 2 || nk < 2) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid: each extent must be >= 2");
    if (storage != SDFC_STORAGE_F64 && storage != SDFC_STORAGE_F32 && storage != SDFC_STORAGE_F16_BRICKS &&
        storage != SDFC_STORAGE_F32_NODES)
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid: unknown storage");
    const int nn[3] = {ni, nj, nk};
    for (int a = 0; a < 3; ++a) {
        if (!(dxyz[a] > 0.0) || !std::isfinite(dxyz[a]) || !std::isfinite(min_box[a]) || !std::isfinite(max_box[a]) ||
            !(max_box[a] > min_box[a]))
            return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid: invalid box or spacing");
        // the reference's cell index floor((x - min) / dx) must stay < n for x <= max
        if (std::floor((max_box[a] - min_box[a]) / dxyz[a]) > nn[a] - 1)
            return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid: box extends past the last grid node");
    }
    if (!std::isfinite(col_th)) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid: non-finite col_th");
    return SDFC_OK;
}

static sdfc::GridDesc grid_header(int ni, int nj, int nk, const double min_box[3], const double max_box[3],
                                  const double dxyz[3], double col_th, int storage) {
    GridDesc g{};
    g.ni = ni;
    g.nj = nj;
    g.nk = nk;
    g.storage = storage;
    for (int a = 0; a < 3; ++a) {
        g.min_box[a] = min_box[a];
        g.max_box[a] = max_box[a];
        g.dx[a] = dxyz[a];
        g.inv_dx[a] = 1.0 / dxyz[a];
        g.org[a] = min_box[a] * g.inv_dx[a];
        g.fmin[a] = (float)min_box[a];
        g.fdx[a] = (float)dxyz[a];
        g.fmax[a] = (float)max_box[a];
        g.finv_dx[a] = (float)(1.0 / dxyz[a]);
    }
    g.col_th = col_th;
    return g;
}

// Adds a prepared grid to the context's table; on failure the grid's own allocations (those
// made since `mark`) are released.
static int register_grid(sdfc_context* ctx, const GridDesc& g, size_t mark, int rc, int* grid) {
    if (rc == SDFC_OK) {
        ctx->grids.push_back(g);
        rc = sync_table(ctx, ctx->grids, &ctx->d_grids, &ctx->grid_cap);
        if (rc == SDFC_OK) {
            *grid = (int)ctx->grids.size() - 1;
            return SDFC_OK;
        }
        ctx->grids.pop_back();
    }
    for (size_t q = mark; q < ctx->allocations.size(); ++q) cudaFree(ctx->allocations[q]);
    ctx->allocations.resize(mark);
    return rc;
}

// values (FP64 grid) or, for SDFC_STORAGE_F16_BRICKS, already encoded bricks (codes_in, so_in)
static int upload_grid_impl(sdfc_context* ctx, const double* values, const unsigned short* codes_in,
                            const float* so_in, int ni, int nj, int nk, const double min_box[3],
                            const double max_box[3], const double dxyz[3], double col_th, int storage, int* grid) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if ((!values && !(codes_in && so_in)) || !grid) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid: null argument");
    int rc = check_grid(ctx, ni, nj, nk, min_box, max_box, dxyz, col_th, storage);
    if (rc) return rc;
    const size_t n = (size_t)ni * nj * nk;
    if (values && !all_finite(values, n)) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid: non-finite value");
    if ((rc = use_device(ctx))) return rc;
    GridDesc g = grid_header(ni, nj, nk, min_box, max_box, dxyz, col_th, storage);
    const size_t mark = ctx->allocations.size();
    auto upload = [&](const void* src, size_t bytes, void** dst) -> int {
        int r = dev_alloc(ctx, dst, bytes);
        if (r) return r;
        ctx->allocations.push_back(*dst);
        CUDA_TRY(ctx, cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
        return SDFC_OK;
    };

    if (storage == SDFC_STORAGE_F16_BRICKS) {
        // the values every evaluation sees are the decoded bricks; their bounds come from the host
        const int nbx = (ni + 7) / 8, nby = (nj + 7) / 8, nbz = (nk + 7) / 8;
        const size_t nb = (size_t)nbx * nby * nbz;
        std::vector<unsigned short> codes(nb * 512);
        std::vector<float> so(2 * nb);
        std::vector<double> seen(n);
        if (codes_in) {
            std::copy(codes_in, codes_in + codes.size(), codes.begin());
            std::copy(so_in, so_in + so.size(), so.begin());
        } else {
            sdfc_f16_brick_encode(values, ni, nj, nk, codes.data(), so.data());
        }
        sdfc_f16_brick_decode(codes.data(), so.data(), ni, nj, nk, seen.data());
        if (codes_in && !all_finite(seen.data(), n))
            return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid: non-finite brick value");
        double vmax = 0.0;
        for (size_t i = 0; i < n; ++i) vmax = std::max(vmax, std::fabs(seen[i]));
        // Lipschitz bound of the trilinear interpolant: per axis the largest neighbour
        // difference over the spacing
        double lip2 = 0.0;
        const size_t st[3] = {1, (size_t)ni, (size_t)ni * nj};
        const int nn[3] = {ni, nj, nk};
        for (int a = 0; a < 3; ++a) {
            double m = 0.0;
            for (int k = 0; k < nk; ++k)
                for (int j = 0; j < nj; ++j)
                    for (int i = 0; i < ni; ++i) {
                        int c[3] = {i, j, k};
                        if (c[a] + 1 >= nn[a]) continue;
                        size_t idx = i + st[1] * j + st[2] * k;
                        m = std::max(m, std::fabs(seen[idx + st[a]] - seen[idx]));
                    }
            lip2 += (m / dxyz[a]) * (m / dxyz[a]);
        }
        g.lip = (float)(std::sqrt(lip2) * 1.0001);
        g.vmax = (float)(vmax * 1.0001);
        void *pb = nullptr, *ps = nullptr;
        if ((rc = upload(codes.data(), codes.size() * sizeof(unsigned short), &pb)) ||
            (rc = upload(so.data(), so.size() * sizeof(float), &ps)))
            return register_grid(ctx, g, mark, rc, grid);
        g.b16 = (const unsigned short*)pb;
        g.bso = (const float2*)ps;
        g.nbx = nbx;
        g.nby = nby;
        return register_grid(ctx, g, mark, SDFC_OK, grid);
    }
    if (storage == SDFC_STORAGE_F32_NODES) {
        std::vector<float> v(n);
        for (size_t i = 0; i < n; ++i) v[i] = (float)values[i];
        void* p = nullptr;
        if (!(rc = upload(v.data(), n * sizeof(float), &p))) {
            g.v32 = (const float*)p;
            rc = sdfc_impl::grid_finish_device(ctx, g, p, true, false);
        }
        return register_grid(ctx, g, mark, rc, grid);
    }
    // storages 0 and 1: the FP64 values (storage 1: rounded to FP32 first) and the cell-corner array
    std::vector<double> rounded;
    if (storage == SDFC_STORAGE_F32) {
        rounded.resize(n);
        for (size_t i = 0; i < n; ++i) rounded[i] = (double)(float)values[i];
    }
    void* p64 = nullptr;
    if (!(rc = upload(rounded.empty() ? values : rounded.data(), n * sizeof(double), &p64))) {
        g.v64 = (const double*)p64;
        rc = sdfc_impl::grid_finish_device(ctx, g, p64, false, true);
    }
    return register_grid(ctx, g, mark, rc, grid);
}

extern "C" {

int sdfc_upload_grid(sdfc_context* ctx, const double* values, int ni, int nj, int nk, const double min_box[3],
                     const double max_box[3], const double dxyz[3], double col_th, int storage, int* grid) {
    return upload_grid_impl(ctx, values, nullptr, nullptr, ni, nj, nk, min_box, max_box, dxyz, col_th, storage, grid);
}

int sdfc_upload_grid_device(sdfc_context* ctx, const float* d_values, int ni, int nj, int nk,
                            const double min_box[3], const double max_box[3], const double dxyz[3], double col_th,
                            int storage, int* grid) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (!d_values || !grid) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid_device: null argument");
    if (storage != SDFC_STORAGE_F32 && storage != SDFC_STORAGE_F32_NODES)
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid_device: storage must be F32 or F32_NODES");
    int rc = check_grid(ctx, ni, nj, nk, min_box, max_box, dxyz, col_th, storage);
    if (rc) return rc;
    if ((rc = use_device(ctx))) return rc;
    const size_t n = (size_t)ni * nj * nk;
    GridDesc g = grid_header(ni, nj, nk, min_box, max_box, dxyz, col_th, storage);
    const size_t mark = ctx->allocations.size();
    void* p = nullptr;
    if (storage == SDFC_STORAGE_F32_NODES) {
        if (!(rc = dev_alloc(ctx, &p, n * sizeof(float)))) {
            ctx->allocations.push_back(p);
            cudaError_t e = cudaMemcpyAsync(p, d_values, n * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream);
            if (e != cudaSuccess) {
                rc = fail(ctx, SDFC_ERR_CUDA, std::string("upload_grid_device: ") + cudaGetErrorString(e));
            } else {
                g.v32 = (const float*)p;
                rc = sdfc_impl::grid_finish_device(ctx, g, p, true, false);
            }
        }
        return register_grid(ctx, g, mark, rc, grid);
    }
    if (!(rc = dev_alloc(ctx, &p, n * sizeof(double)))) {
        ctx->allocations.push_back(p);
        g.v64 = (const double*)p;
        if (!(rc = sdfc_impl::widen_device(ctx, d_values, (double*)p, n)))
            rc = sdfc_impl::grid_finish_device(ctx, g, d_values, true, true);
    }
    return register_grid(ctx, g, mark, rc, grid);
}

int sdfc_upload_grid_bricks(sdfc_context* ctx, const unsigned short* codes, const float* so, int ni, int nj, int nk,
                            const double min_box[3], const double max_box[3], const double dxyz[3], double col_th,
                            int* grid) {
    if (!codes || !so) return ctx ? fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid_bricks: null argument")
                                  : SDFC_ERR_INVALID_ARGUMENT;
    return upload_grid_impl(ctx, nullptr, codes, so, ni, nj, nk, min_box, max_box, dxyz, col_th,
                            SDFC_STORAGE_F16_BRICKS, grid);
}

int sdfc_grid_values(sdfc_context* ctx, int grid, double* values) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (!values) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "grid_values: null argument");
    if (grid < 0 || grid >= (int)ctx->grids.size()) return fail(ctx, SDFC_ERR_NOT_FOUND, "grid_values: unknown grid");
    int rc = use_device(ctx);
    if (rc) return rc;
    const GridDesc& g = ctx->grids[grid];
    const size_t n = (size_t)g.ni * g.nj * g.nk;
    if (g.v32) {
        std::vector<float> v(n);
        CUDA_TRY(ctx, cudaMemcpy(v.data(), g.v32, n * sizeof(float), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i) values[i] = (double)v[i];
        return SDFC_OK;
    }
    if (!g.b16) {
        CUDA_TRY(ctx, cudaMemcpy(values, g.v64, n * sizeof(double), cudaMemcpyDeviceToHost));
        return SDFC_OK;
    }
    const size_t nb = (size_t)g.nbx * g.nby * ((g.nk + 7) / 8);
    std::vector<unsigned short> codes(nb * 512);
    std::vector<float> so(2 * nb);
    CUDA_TRY(ctx, cudaMemcpy(codes.data(), g.b16, codes.size() * sizeof(unsigned short), cudaMemcpyDeviceToHost));
    CUDA_TRY(ctx, cudaMemcpy(so.data(), g.bso, so.size() * sizeof(float), cudaMemcpyDeviceToHost));
    return sdfc_f16_brick_decode(codes.data(), so.data(), g.ni, g.nj, g.nk, values);
}

static inline unsigned short half_bits(float x) {
    const __half_raw r = __half(__float2half_rn(x));
    return r.x;
}
static inline float half_value(unsigned short bits) {
    __half_raw r;
    r.x = bits;
    return __half2float(__half(r));
}

int sdfc_f16_brick_encode(const double* values, int ni, int nj, int nk, unsigned short* codes, float* so) {
    if (!values || !codes || !so || ni < 1 || nj < 1 || nk < 1) return SDFC_ERR_INVALID_ARGUMENT;
    const int nbx = (ni + 7) / 8, nby = (nj + 7) / 8, nbz = (nk + 7) / 8;
    for (int bz = 0; bz < nbz; ++bz)
        for (int by = 0; by < nby; ++by)
            for (int bx = 0; bx < nbx; ++bx) {
                const size_t b = (size_t)bx + (size_t)nbx * ((size_t)by + (size_t)nby * bz);
                auto at = [&](int ii, int jj, int kk) {  // node of the brick, the last node repeated past the end
                    const int i = std::min(8 * bx + ii, ni - 1), j = std::min(8 * by + jj, nj - 1),
                              k = std::min(8 * bz + kk, nk - 1);
                    return values[(size_t)i + (size_t)ni * ((size_t)j + (size_t)nj * k)];
                };
                double lo = INFINITY, hi = -INFINITY;
                for (int kk = 0; kk < 8; ++kk)
                    for (int jj = 0; jj < 8; ++jj)
                        for (int ii = 0; ii < 8; ++ii) {
                            const double v = at(ii, jj, kk);
                            lo = std::min(lo, v);
                            hi = std::max(hi, v);
                        }
                const float off = (lo <= 0.0 && hi >= 0.0) ? 0.0f : (float)(lo > 0.0 ? lo : hi);
                const double amax = std::max(std::fabs(hi - (double)off), std::fabs(lo - (double)off));
                const float scale = amax > 0.0 ? (float)(amax / 32768.0) : 1.0f;
                so[2 * b] = scale;
                so[2 * b + 1] = off;
                for (int kk = 0; kk < 8; ++kk)
                    for (int jj = 0; jj < 8; ++jj)
                        for (int ii = 0; ii < 8; ++ii)
                            codes[b * 512 + ii + 8 * jj + 64 * kk] =
                                half_bits((float)((at(ii, jj, kk) - (double)off) / (double)scale));
            }
    return SDFC_OK;
}

int sdfc_f16_brick_decode(const unsigned short* codes, const float* so, int ni, int nj, int nk, double* values) {
    if (!values || !codes || !so || ni < 1 || nj < 1 || nk < 1) return SDFC_ERR_INVALID_ARGUMENT;
    const int nbx = (ni + 7) / 8, nby = (nj + 7) / 8;
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                const size_t b = (size_t)(i >> 3) + (size_t)nbx * ((size_t)(j >> 3) + (size_t)nby * (k >> 3));
                const float h = half_value(codes[b * 512 + (i & 7) + 8 * (j & 7) + 64 * (k & 7)]);
                // FP32 fused multiply-add, as the device decodes (correctly rounded on both)
                values[(size_t)i + (size_t)ni * ((size_t)j + (size_t)nj * k)] =
                    (double)std::fmaf(so[2 * b], h, so[2 * b + 1]);
            }
    return SDFC_OK;
}

// Stored order of a point set: Morton (Z-order) of the points quantised to
// 2^10 cells per axis of their bounding box, ties kept in input order.  Points
// adjacent in this order are adjacent in space, so a warp's 32 points read a
// handful of grid cells and the gathers coalesce.
static std::vector<int> morton_order(const double* xyz, int n) {
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    if (n < 2) return order;
    double lo[3] = {xyz[0], xyz[1], xyz[2]}, hi[3] = {xyz[0], xyz[1], xyz[2]};
    for (int i = 1; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], xyz[3 * (size_t)i + a]);
            hi[a] = std::max(hi[a], xyz[3 * (size_t)i + a]);
        }
    auto spread = [](uint32_t v) {  // 10 bits -> every third bit
        v &= 0x3ffu;
        v = (v | (v << 16)) & 0x030000ffu;
        v = (v | (v << 8)) & 0x0300f00fu;
        v = (v | (v << 4)) & 0x030c30c3u;
        v = (v | (v << 2)) & 0x09249249u;
        return v;
    };
    std::vector<uint32_t> code(n);
    for (int i = 0; i < n; ++i) {
        uint32_t q[3];
        for (int a = 0; a < 3; ++a) {
            double ext = hi[a] - lo[a];
            double t = ext > 0 ? (xyz[3 * (size_t)i + a] - lo[a]) / ext : 0.0;
            q[a] = (uint32_t)std::min(1023.0, std::max(0.0, std::floor(t * 1024.0)));
        }
        code[i] = spread(q[0]) | (spread(q[1]) << 1) | (spread(q[2]) << 2);
    }
    // stable sort by the 30-bit code: three counting-sort passes of 10 bits each (least
    // significant first), each stable, so equal codes keep the input order
    std::vector<int> tmp(n);
    std::vector<int> count(1025);
    for (int pass = 0; pass < 3; ++pass) {
        const int shift = 10 * pass;
        std::fill(count.begin(), count.end(), 0);
        for (int k = 0; k < n; ++k) ++count[((code[order[k]] >> shift) & 1023u) + 1];
        for (int b = 0; b < 1024; ++b) count[b + 1] += count[b];
        for (int k = 0; k < n; ++k) tmp[count[(code[order[k]] >> shift) & 1023u]++] = order[k];
        order.swap(tmp);
    }
    return order;
}

// Bounding sphere (x, y, z, r) of every detection tile of a stored point set (FP32 SoA),
// r rounded up so that every FP32 point of the tile lies within it.
static std::vector<float4> tile_spheres(const std::vector<float>& s32, int n) {
    const int nt = (n + sdfc::kTile - 1) / sdfc::kTile;
    std::vector<float4> out(std::max(nt, 1), make_float4(0.f, 0.f, 0.f, 0.f));
    for (int t = 0; t < nt; ++t) {
        const int a = t * sdfc::kTile, b = std::min(n, a + sdfc::kTile);
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int k = a; k < b; ++k)
            for (int c = 0; c < 3; ++c) {
                const double v = s32[(size_t)c * n + k];
                lo[c] = std::min(lo[c], v);
                hi[c] = std::max(hi[c], v);
            }
        const float cx = (float)(0.5 * (lo[0] + hi[0])), cy = (float)(0.5 * (lo[1] + hi[1])),
                    cz = (float)(0.5 * (lo[2] + hi[2]));
        double r2 = 0.0;
        for (int k = a; k < b; ++k) {
            const double dx = s32[k] - (double)cx, dy = s32[(size_t)n + k] - (double)cy,
                         dz = s32[2 * (size_t)n + k] - (double)cz;
            r2 = std::max(r2, dx * dx + dy * dy + dz * dz);
        }
        out[t] = make_float4(cx, cy, cz, (float)(std::sqrt(r2) * (1.0 + 1e-6)) + 1e-30f);
    }
    return out;
}

int sdfc_upload_points(sdfc_context* ctx, const double* xyz, int n, int storage, int* points) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if ((!xyz && n > 0) || n < 0 || !points) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_points: bad argument");
    if (storage != SDFC_STORAGE_F64 && storage != SDFC_STORAGE_F32)
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_points: unknown storage");
    if (!all_finite(xyz, 3 * (size_t)n)) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_points: non-finite point");
    int rc = use_device(ctx);
    if (rc) return rc;
    std::vector<int> order = morton_order(xyz, n);
    std::vector<float> s32(3 * (size_t)n);
    std::vector<double> s64(3 * (size_t)n);
    double r = 0.0;
    for (int k = 0; k < n; ++k) {
        const double* q = xyz + 3 * (size_t)order[k];
        for (int a = 0; a < 3; ++a) {
            s64[(size_t)a * n + k] = q[a];
            s32[(size_t)a * n + k] = (float)q[a];
        }
        r = std::max(r, std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]));
    }
    PointsDesc P{};
    P.n = n;
    P.storage = storage;
    P.radius = (float)(r * 1.0001);
    void* p32 = nullptr;
    if ((rc = dev_alloc(ctx, &p32, s32.size() * sizeof(float)))) return rc;
    ctx->allocations.push_back(p32);
    CUDA_TRY(ctx, cudaMemcpy(p32, s32.data(), s32.size() * sizeof(float), cudaMemcpyHostToDevice));
    P.x32 = (const float*)p32;
    {
        const std::vector<float4> sph = tile_spheres(s32, n);
        void* psph = nullptr;
        if ((rc = dev_alloc(ctx, &psph, sph.size() * sizeof(float4)))) return rc;
        ctx->allocations.push_back(psph);
        CUDA_TRY(ctx, cudaMemcpy(psph, sph.data(), sph.size() * sizeof(float4), cudaMemcpyHostToDevice));
        P.tiles = (const float4*)psph;
    }
    void* pord = nullptr;
    if ((rc = dev_alloc(ctx, &pord, (size_t)n * sizeof(int)))) return rc;
    ctx->allocations.push_back(pord);
    CUDA_TRY(ctx, cudaMemcpy(pord, order.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice));
    P.orig = (const int*)pord;
    if (storage == SDFC_STORAGE_F32)  // the points as stored: FP32, widened
        for (size_t k = 0; k < s64.size(); ++k) s64[k] = (double)s32[k];
    {
        void* p64 = nullptr;
        if ((rc = dev_alloc(ctx, &p64, s64.size() * sizeof(double)))) return rc;
        ctx->allocations.push_back(p64);
        CUDA_TRY(ctx, cudaMemcpy(p64, s64.data(), s64.size() * sizeof(double), cudaMemcpyHostToDevice));
        P.x64 = (const double*)p64;
    }
    ctx->points.push_back(P);
    ctx->point_order.push_back(std::move(order));
    if ((rc = sync_table(ctx, ctx->points, &ctx->d_points, &ctx->points_cap))) {
        ctx->points.pop_back();
        ctx->point_order.pop_back();
        return rc;
    }
    *points = (int)ctx->points.size() - 1;
    return SDFC_OK;
}


int sdfc_batch_create(sdfc_context* ctx, int n, const int* points, const int* grids, sdfc_batch** out) {
    int rc = sdfc_impl::batch_create(ctx, n, points, grids, out);
    if (rc == SDFC_OK) ctx->batches.push_back(*out);
    return rc;
}

void sdfc_batch_destroy(sdfc_batch* b) {
    if (!b) return;
    sdfc_context* ctx = b->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    auto it = std::find(ctx->batches.begin(), ctx->batches.end(), b);
    if (it != ctx->batches.end()) ctx->batches.erase(it);
    free_batch(b);
}

int sdfc_batch_evaluate_device(sdfc_batch* b, const double* E_A, const double* phi_A, const double* E_B,
                               const double* phi_B, const double* params, int want_deriv, double* fm, double* Km,
                               double* Dm, int* n_active, int* status, void* stream) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    if (!E_A || !phi_A || !E_B || !phi_B || !params || !fm || !n_active || !status || (want_deriv && (!Km || !Dm)))
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_evaluate_device: null argument");
    int rc = use_device(ctx);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    return run_batch(b, E_A, phi_A, E_B, phi_B, params, want_deriv != 0, fm, Km, Dm, n_active, status, s);
}

int sdfc_batch_evaluate_masked_device(sdfc_batch* b, const double* E_A, const double* phi_A, const double* E_B,
                                      const double* phi_B, const double* params, const int* request, double* fm,
                                      double* Km, double* Dm, int* n_active, int* status, void* stream) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    if (!E_A || !phi_A || !E_B || !phi_B || !params || !request || !fm || !Km || !Dm || !n_active || !status)
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_evaluate_masked_device: null argument");
    int rc = use_device(ctx);
    if (rc) return rc;
    sdfc::BatchInputs in{E_A, phi_A, E_B, phi_B, params};
    in.mode = request;
    sdfc::BatchOutputs out{fm, Km, Dm, n_active, status};
    return sdfc_impl::run_batch(b, in, true, out, (cudaStream_t)stream);
}

int sdfc_batch_energy_device(sdfc_batch* b, const double* E_A, const double* phi_A, const double* E_B,
                             const double* phi_B, const double* params, double* energy, double* dE, void* stream) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    if (!E_A || !phi_A || !E_B || !phi_B || !params || !energy || !dE)
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_energy_device: null argument");
    int rc = use_device(ctx);
    if (rc) return rc;
    sdfc::BatchInputs in{E_A, phi_A, E_B, phi_B, params};
    return sdfc_impl::run_energy(b, in, energy, dE, (cudaStream_t)stream);
}

int sdfc_batch_energy(sdfc_batch* b, const double* E_A, const double* E_B, const sdfc_params* params, double* energy,
                      double* dE) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    if (!E_A || !E_B || !params || !energy || !dE) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_energy: null argument");
    int rc = use_device(ctx);
    if (rc) return rc;
    const size_t n = (size_t)b->n;
    double* h = b->h_in;
    std::memcpy(h, E_A, sizeof(double) * 16 * n);
    std::memset(h + 16 * n, 0, sizeof(double) * 6 * n);
    std::memcpy(h + 22 * n, E_B, sizeof(double) * 16 * n);
    std::memset(h + 38 * n, 0, sizeof(double) * 6 * n);
    for (size_t k = 0; k < n; ++k) {
        double* p = h + 44 * n + 6 * k;
        p[0] = params[k].kn;
        p[1] = params[k].kt;
        p[2] = params[k].mu;
        p[3] = params[k].damping;
        p[4] = params[k].scale;
        p[5] = params[k].contact_scale;
    }
    cudaStream_t st = ctx->stream;
    CUDA_TRY(ctx, cudaMemcpyAsync(b->d_in, h, sizeof(double) * 50 * n, cudaMemcpyHostToDevice, st));
    double* d = b->d_in;
    sdfc::BatchInputs in{d, d + 16 * n, d + 22 * n, d + 38 * n, d + 44 * n};
    double* dout = b->d_out;  // energy [n] then dE [12 n]
    if ((rc = sdfc_impl::run_energy(b, in, dout, dout + n, st))) return rc;
    CUDA_TRY(ctx, cudaMemcpyAsync(b->h_out, dout, sizeof(double) * 13 * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(ctx, cudaStreamSynchronize(st));
    std::memcpy(energy, b->h_out, sizeof(double) * n);
    std::memcpy(dE, b->h_out + n, sizeof(double) * 12 * n);
    return SDFC_OK;
}

int sdfc_batch_evaluate(sdfc_batch* b, const double* E_A, const double* phi_A, const double* E_B, const double* phi_B,
                        const sdfc_params* params, int want_deriv, double* fm, double* Km, double* Dm, int* n_active,
                        int* status) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    if (!E_A || !phi_A || !E_B || !phi_B || !params || !fm || (want_deriv && (!Km || !Dm)))
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_evaluate: null argument");
    int rc = use_device(ctx);
    if (rc) return rc;
    const size_t n = (size_t)b->n;
    cudaStream_t s = ctx->stream;
    const int dv = want_deriv ? 1 : 0;
    double* d = b->d_in;
    double* o = b->d_out;
    const size_t nout = dv ? 300 * n : 12 * n;
    static_assert(sizeof(sdfc_params) == 6 * sizeof(double), "sdfc_params rows are the kernels' 6 doubles");
    // Where the device reads pageable memory through the host page tables (Grace: the C2C
    // link), the evaluation's kernels read the caller's input arrays and write its output
    // arrays themselves (gather_inputs_kernel; finalize_kernel's indirect outputs): per call only
    // the arrays' addresses go to the device.  Elsewhere inputs and outputs are staged through
    // pinned buffers.
    const bool direct = ctx->pageable_direct;
    if (direct) {
        sdfc::HostIO* io = b->h_io;
        io->in[0] = E_A;
        io->in[1] = phi_A;
        io->in[2] = E_B;
        io->in[3] = phi_B;
        io->in[4] = reinterpret_cast<const double*>(params);
        io->out = sdfc::BatchOutputs{fm, dv ? Km : nullptr, dv ? Dm : nullptr, n_active ? n_active : b->d_int,
                                     status ? status : b->d_int + n};
        CUDA_TRY(ctx, cudaMemcpyAsync(b->d_io, io, sizeof(sdfc::HostIO), cudaMemcpyHostToDevice, s));
    } else {
        double* h = b->h_in;
        std::memcpy(h, E_A, sizeof(double) * 16 * n);
        std::memcpy(h + 16 * n, phi_A, sizeof(double) * 6 * n);
        std::memcpy(h + 22 * n, E_B, sizeof(double) * 16 * n);
        std::memcpy(h + 38 * n, phi_B, sizeof(double) * 6 * n);
        std::memcpy(h + 44 * n, params, sizeof(double) * 6 * n);
        CUDA_TRY(ctx, cudaMemcpyAsync(d, h, sizeof(double) * 50 * n, cudaMemcpyHostToDevice, s));
    }
    // the evaluation's kernels, captured once per (derivative flag, modes)
    auto enqueue = [&](cudaStream_t st) -> int {
        if (!direct)
            return run_batch(b, d, d + 16 * n, d + 22 * n, d + 38 * n, d + 44 * n, dv != 0, o, o + 12 * n,
                             o + 156 * n, b->d_int, b->d_int + n, st);
        sdfc::launch_gather_inputs(b->d_io, d, (int)n, st);
        sdfc::BatchInputs in{d, d + 16 * n, d + 22 * n, d + 38 * n, d + 44 * n};
        sdfc::BatchOutputs out{nullptr, nullptr, nullptr, nullptr, nullptr, &b->d_io->out};
        return sdfc_impl::run_batch(b, in, dv != 0, out, st);
    };
    const int key = b->precision * 2 + b->deriv_mode;
    if (b->timing) {  // the phase events need the kernels launched one by one
        if ((rc = enqueue(s))) return rc;
    } else {
        if (b->eval_exec[dv] && b->eval_key[dv] != key) {
            cudaGraphExecDestroy(b->eval_exec[dv]);
            b->eval_exec[dv] = nullptr;
        }
        if (!b->eval_exec[dv]) {
            if (!b->eval_stream) CUDA_TRY(ctx, cudaStreamCreateWithFlags(&b->eval_stream, cudaStreamNonBlocking));
            cudaGraph_t graph = nullptr;
            CUDA_TRY(ctx, cudaStreamBeginCapture(b->eval_stream, cudaStreamCaptureModeThreadLocal));
            rc = enqueue(b->eval_stream);
            cudaError_t e = cudaStreamEndCapture(b->eval_stream, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&b->eval_exec[dv], graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (e != cudaSuccess) return fail(ctx, SDFC_ERR_CUDA, std::string("batch_evaluate graph: ") + cudaGetErrorString(e));
            b->eval_key[dv] = key;
        }
        CUDA_TRY(ctx, cudaGraphLaunch(b->eval_exec[dv], s));
    }
    if (direct) {
        CUDA_TRY(ctx, cudaStreamSynchronize(s));
        return SDFC_OK;
    }
    CUDA_TRY(ctx, cudaMemcpyAsync(b->h_out, o, sizeof(double) * nout, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(ctx, cudaMemcpyAsync(b->h_int, b->d_int, sizeof(int) * 2 * n, cudaMemcpyDeviceToHost, s));
    CUDA_TRY(ctx, cudaStreamSynchronize(s));
    std::memcpy(fm, b->h_out, sizeof(double) * 12 * n);
    if (want_deriv) {
        std::memcpy(Km, b->h_out + 12 * n, sizeof(double) * 144 * n);
        std::memcpy(Dm, b->h_out + 156 * n, sizeof(double) * 144 * n);
    }
    if (n_active) std::memcpy(n_active, b->h_int, sizeof(int) * n);
    if (status) std::memcpy(status, b->h_int + n, sizeof(int) * n);
    return SDFC_OK;
}

int sdfc_batch_distance_device(sdfc_batch* b, const double* d_EA, const double* d_EB, double* d_min, double* d_d,
                               void* stream) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    if (!d_EA || !d_EB || !d_min) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_distance: null argument");
    int rc = use_device(ctx);
    if (rc) return rc;
    cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
    sdfc::BatchInputs in{d_EA, nullptr, d_EB, nullptr, nullptr};
    // d_out (n x 300 doubles) holds the minimum keys
    sdfc::launch_distance(b->d_inst, b->d_tile_inst, b->n, b->total_tiles, in, ctx->d_grids, ctx->d_points,
                          b->d_point_offset, (unsigned long long*)b->d_out, d_min, d_d, s);
    CUDA_TRY(ctx, cudaGetLastError());
    return SDFC_OK;
}

int sdfc_batch_distance(sdfc_batch* b, const double* E_A, const double* E_B, double* min_d, double* d) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    if (!E_A || !E_B || !min_d) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_distance: null argument");
    int rc = use_device(ctx);
    if (rc) return rc;
    const size_t n = (size_t)b->n;
    cudaStream_t s = ctx->stream;
    double* h = b->h_in;
    std::memcpy(h, E_A, sizeof(double) * 16 * n);
    std::memcpy(h + 16 * n, E_B, sizeof(double) * 16 * n);
    CUDA_TRY(ctx, cudaMemcpyAsync(b->d_in, h, sizeof(double) * 32 * n, cudaMemcpyHostToDevice, s));
    double* dd = nullptr;
    if (d && b->total_points > 0) CUDA_TRY(ctx, cudaMallocAsync((void**)&dd, sizeof(double) * b->total_points, s));
    double* dmin = b->d_in + 32 * n;  // n doubles after the poses
    rc = sdfc_batch_distance_device(b, b->d_in, b->d_in + 16 * n, dmin, dd, s);
    if (rc == SDFC_OK) {
        cudaError_t e = cudaMemcpyAsync(b->h_out, dmin, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && dd)
            e = cudaMemcpyAsync(d, dd, sizeof(double) * b->total_points, cudaMemcpyDeviceToHost, s);
        if (dd) cudaFreeAsync(dd, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail(ctx, SDFC_ERR_CUDA, std::string("batch_distance: ") + cudaGetErrorString(e));
        std::memcpy(min_d, b->h_out, sizeof(double) * n);
    } else if (dd) {
        cudaFreeAsync(dd, s);
        cudaStreamSynchronize(s);
    }
    return rc;
}

int sdfc_grid_distance(sdfc_context* ctx, int grid, const double* X, int n, double* d, double* min_d) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (n < 0 || (n > 0 && !X)) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "grid_distance: bad argument");
    if (grid < 0 || grid >= (int)ctx->grids.size()) return fail(ctx, SDFC_ERR_NOT_FOUND, "grid_distance: unknown grid");
    int rc = use_device(ctx);
    if (rc) return rc;
    if (!d && !min_d) return SDFC_OK;
    cudaStream_t s = ctx->stream;
    // X (n x 3), d (n), the minimum and its key, in one allocation
    const size_t words = 3 * (size_t)n + (size_t)n + 2;
    double* buf = nullptr;
    CUDA_TRY(ctx, cudaMallocAsync((void**)&buf, sizeof(double) * words, s));
    double* dX = buf;
    double* dd = buf + 3 * (size_t)n;
    double* dmin = dd + n;
    cudaError_t e = n > 0 ? cudaMemcpyAsync(dX, X, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s) : cudaSuccess;
    if (e == cudaSuccess) {
        sdfc::launch_grid_query(ctx->d_grids, grid, dX, n, d ? dd : nullptr, (unsigned long long*)(dmin + 1),
                                min_d ? dmin : nullptr, s);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && d && n > 0) e = cudaMemcpyAsync(d, dd, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && min_d) e = cudaMemcpyAsync(min_d, dmin, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(buf, s);
    const cudaError_t e2 = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return fail(ctx, SDFC_ERR_CUDA, std::string("grid_distance: ") + cudaGetErrorString(e));
    return SDFC_OK;
}

int sdfc_batch_set_timing(sdfc_batch* b, int enable) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    int rc = use_device(ctx);
    if (rc) return rc;
    if (enable && !b->ev[0])
        for (cudaEvent_t& e : b->ev) CUDA_TRY(ctx, cudaEventCreate(&e));
    b->timing = enable != 0;
    return SDFC_OK;
}

int sdfc_batch_last_timing(sdfc_batch* b, float* ms) {
    if (!b || !ms) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    if (!b->timing) return fail(ctx, SDFC_ERR_NOT_FOUND, "last_timing: timing is not enabled");
    int rc = use_device(ctx);
    if (rc) return rc;
    CUDA_TRY(ctx, cudaEventSynchronize(b->ev[3]));
    for (int k = 0; k < 3; ++k) CUDA_TRY(ctx, cudaEventElapsedTime(ms + k, b->ev[k], b->ev[k + 1]));
    return SDFC_OK;
}

int sdfc_batch_recheck_count(sdfc_batch* b, unsigned long long* count, int reset) {
    if (!b || !count) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    int rc = use_device(ctx);
    if (rc) return rc;
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    CUDA_TRY(ctx, cudaMemcpy(count, b->d_recheck, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
    if (reset) CUDA_TRY(ctx, cudaMemset(b->d_recheck, 0, sizeof(unsigned long long)));
    return SDFC_OK;
}

int sdfc_evaluate(sdfc_context* ctx, int points, int grid, const double* E_A, const double* phi_A, const double* E_B,
                  const double* phi_B, const sdfc_params* params, int want_deriv, double* fm, double* Km, double* Dm,
                  int* n_active) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (!ctx->single || ctx->single_points != points || ctx->single_grid != grid) {
        int rc = use_device(ctx);
        if (rc) return rc;
        cudaStreamSynchronize(ctx->stream);
        free_batch(ctx->single);
        ctx->single = nullptr;
        ctx->single_points = ctx->single_grid = -1;
        sdfc_batch* b = nullptr;
        rc = sdfc_impl::batch_create(ctx, 1, &points, &grid, &b);
        if (rc) return rc;
        ctx->single = b;
        ctx->single_points = points;
        ctx->single_grid = grid;
    }
    int status = 0, nact = 0;
    int rc = sdfc_batch_evaluate(ctx->single, E_A, phi_A, E_B, phi_B, params, want_deriv, fm, Km, Dm, &nact, &status);
    if (rc) return rc;
    if (n_active) *n_active = nact;
    return SDFC_OK;
}

int sdfc_active_ids(sdfc_context* ctx, int* ids, int cap, int* n) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (!n || (cap > 0 && !ids)) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "active_ids: bad argument");
    sdfc_batch* b = ctx->single;
    if (!b) return fail(ctx, SDFC_ERR_NOT_FOUND, "active_ids: no evaluation yet");
    int rc = use_device(ctx);
    if (rc) return rc;
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    const int tiles = b->total_tiles;
    std::vector<int> counts(std::max(tiles, 1));
    if (tiles > 0)
        CUDA_TRY(ctx, cudaMemcpy(counts.data(), b->d_tile_count, sizeof(int) * tiles, cudaMemcpyDeviceToHost));
    std::vector<int> all;
    for (int t = 0; t < tiles; ++t) {
        if (counts[t] <= 0) continue;
        size_t at = all.size();
        all.resize(at + counts[t]);
        CUDA_TRY(ctx, cudaMemcpy(all.data() + at, b->d_ids + (size_t)t * sdfc::kTile, sizeof(int) * counts[t],
                                 cudaMemcpyDeviceToHost));
    }
    // stored indices -> the caller's indices, ascending as the reference lists them
    const std::vector<int>& order = ctx->point_order[ctx->single_points];
    for (int& v : all) v = order[v];
    std::sort(all.begin(), all.end());
    const int total = (int)all.size();
    for (int k = 0; k < total && k < cap; ++k) ids[k] = all[k];
    *n = total;
    return SDFC_OK;
}

}  // extern "C"
