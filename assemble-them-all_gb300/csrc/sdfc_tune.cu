// Launch tuning of a batch's force pass (sdfc_batch_autotune): times each candidate
// configuration on one evaluation of the caller's inputs and keeps the fastest, per batch
// shape and context.  The candidates are the force-pass forms over the queue of (instance, share)
// items (persistent 128-thread CTAs or one-warp workers) times the chunks per share, and the
// grid of one CTA per (instance, share) times the shares per instance; the batch shape decides
// which wins (even instances favour the grid, uneven ones the queue).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "sdfc_internal.h"

namespace {

const char* const kVariantName[] = {"ctas", "workers", "grid"};

// The shape a tuning is valid for.
std::vector<long long> tune_key(const sdfc_batch* b, bool deriv, bool masked) {
    long long tiles = 0;
    for (const auto& d : b->inst) tiles += d.ntiles;
    return {b->n, tiles, b->total_points, b->max_ntiles, b->has_plain ? 1 : 0, b->has_bricks ? 1 : 0,
            b->precision, b->deriv_mode, deriv ? 1 : 0, masked ? 1 : 0};
}

bool valid_tuning(const sdfc_tuning& t) {
    const bool pow2 = t.slots >= 1 && t.slots <= sdfc::kMaxSlots && (t.slots & (t.slots - 1)) == 0;
    return pow2 && t.force_variant >= SDFC_FORCE_CTAS && t.force_variant <= SDFC_FORCE_GRID && t.worker_ctas >= 0 &&
           t.chunks_per_slot >= 1;
}

int apply(sdfc_batch* b, const sdfc_tuning& t) {
    int rc = sdfc_impl::ensure_partial(b, t.slots);
    if (rc) return rc;
    b->slots = t.slots;
    b->force_variant = t.force_variant;  // SDFC_FORCE_* = sdfc::ForceVariant
    b->worker_ctas = t.worker_ctas;
    b->chunks_per_slot = t.chunks_per_slot;
    b->tuned_ms = t.ms;
    // the captured evaluations hold the old configuration (and maybe the old partial rows)
    for (int k = 0; k < 2; ++k)
        if (b->eval_exec[k]) {
            cudaGraphExecDestroy(b->eval_exec[k]);
            b->eval_exec[k] = nullptr;
        }
    return SDFC_OK;
}

}  // namespace

namespace sdfc_impl {

int autotune(sdfc_batch* b, const sdfc::BatchInputs& in, bool deriv, const sdfc::BatchOutputs& out,
             cudaStream_t st, sdfc_tuning* chosen) {
    sdfc_context* ctx = b->ctx;
    const std::vector<long long> key = tune_key(b, deriv, in.mode != nullptr);
    for (const auto& kv : ctx->tunings)
        if (kv.first == key) {
            int rc = apply(b, kv.second);
            if (rc == SDFC_OK && chosen) *chosen = kv.second;
            return rc;
        }
    const int cap = std::max(b->slots, sdfc::slots_for(b->n));
    int rc = ensure_partial(b, cap);
    if (rc) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SDFC_CUDA_TRY(ctx, cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return fail(ctx, SDFC_ERR_CUDA, "autotune: cudaEventCreate failed");
    }
    const bool timing = b->timing;
    b->timing = false;
    sdfc_tuning best{b->slots, b->force_variant, 0, b->chunks_per_slot, 1e30f};
    constexpr int kReps = 3;
    const bool log = std::getenv("SDFC_TUNE_LOG") != nullptr;  // every candidate's time on stderr
    // the queue forms at the cap with 1-32 chunks per share; the grid form at 1-16 shares
    std::vector<sdfc_tuning> cands;
    for (int variant : {SDFC_FORCE_CTAS, SDFC_FORCE_WORKERS})
        for (int per = 1; per <= 32; per *= 2) cands.push_back(sdfc_tuning{cap, variant, 0, per, 0.f});
    for (int slots = 1; slots <= std::min(16, cap); slots *= 2)
        cands.push_back(sdfc_tuning{slots, SDFC_FORCE_GRID, 0, 1, 0.f});
    for (sdfc_tuning& cand : cands) {
        if ((rc = apply(b, cand))) break;
        if ((rc = run_batch(b, in, deriv, out, st))) break;  // warm-up
        float t_min = 1e30f;
        for (int r = 0; r < kReps && rc == SDFC_OK; ++r) {
            cudaEventRecord(e0, st);
            rc = run_batch(b, in, deriv, out, st);
            cudaEventRecord(e1, st);
            if (rc == SDFC_OK && cudaEventSynchronize(e1) != cudaSuccess)
                rc = fail(ctx, SDFC_ERR_CUDA, "autotune: evaluation failed");
            float ms = 0.f;
            if (rc == SDFC_OK && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) t_min = std::min(t_min, ms);
        }
        if (rc) break;
        if (log)
            std::fprintf(stderr, "sdfc autotune: n=%d %s slots=%d chunks_per_slot=%d %.4f ms\n", b->n,
                         kVariantName[cand.force_variant], cand.slots, cand.chunks_per_slot, t_min);
        cand.ms = t_min;
        best.ms = std::min(best.ms, t_min);
    }
    // Among the candidates within kTie of the fastest, the one that spreads an instance over the
    // most shares (its cap over its chunks per share): a batch tuned where its contacts are few
    // (a sim's opening state) times every form about equally, and the instances whose contacts
    // grow in later rounds are then spread the widest.
    if (rc == SDFC_OK) {
        constexpr float kTie = 1.01f;
        const float fastest = best.ms;
        auto spread = [](const sdfc_tuning& t) {
            const int form = t.force_variant == SDFC_FORCE_CTAS ? 2 : t.force_variant == SDFC_FORCE_GRID ? 1 : 0;
            return 64LL * t.slots / t.chunks_per_slot * 4 + form;
        };
        bool have = false;
        for (const sdfc_tuning& c : cands)
            if (c.ms <= kTie * fastest && (!have || spread(c) > spread(best) || (spread(c) == spread(best) && c.ms < best.ms))) {
                best = c;
                have = true;
            }
    }
    b->timing = timing;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if ((rc = apply(b, best))) return rc;
    ctx->tunings.emplace_back(key, best);
    if (chosen) *chosen = best;
    return SDFC_OK;
}

}  // namespace sdfc_impl

extern "C" {

int sdfc_batch_autotune(sdfc_batch* b, const double* E_A, const double* phi_A, const double* E_B,
                        const double* phi_B, const double* params, int want_deriv, double* fm, double* Km,
                        double* Dm, int* n_active, int* status, void* stream, sdfc_tuning* chosen) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = b->ctx;
    if (!E_A || !phi_A || !E_B || !phi_B || !params || !fm || !n_active || !status || (want_deriv && (!Km || !Dm)))
        return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_autotune: null argument");
    int rc = sdfc_impl::use_device(ctx);
    if (rc) return rc;
    sdfc::BatchInputs in{E_A, phi_A, E_B, phi_B, params};
    sdfc::BatchOutputs out{fm, Km, Dm, n_active, status};
    rc = sdfc_impl::autotune(b, in, want_deriv != 0, out, (cudaStream_t)stream, chosen);
    if (rc) return rc;
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize((cudaStream_t)stream));
    return SDFC_OK;
}

int sdfc_batch_get_tuning(sdfc_batch* b, sdfc_tuning* t) {
    if (!b || !t) return SDFC_ERR_INVALID_ARGUMENT;
    t->slots = b->slots;
    t->force_variant = b->force_variant;
    t->worker_ctas = b->worker_ctas;
    t->chunks_per_slot = b->chunks_per_slot;
    t->ms = b->tuned_ms;
    return SDFC_OK;
}

int sdfc_batch_set_tuning(sdfc_batch* b, const sdfc_tuning* t) {
    if (!b) return SDFC_ERR_INVALID_ARGUMENT;
    if (!t || !valid_tuning(*t))
        return sdfc_impl::fail(b->ctx, SDFC_ERR_INVALID_ARGUMENT, "batch_set_tuning: invalid configuration");
    int rc = sdfc_impl::use_device(b->ctx);
    if (rc) return rc;
    return apply(b, *t);
}

}  // extern "C"
