// Device-side preparation of uploaded SDF grids (storages 0, 1 and 3): the bounds the
// detection prefilter needs (largest |value| and, per axis, the largest difference of
// neighbouring values), detection's block table of least node values, the FP32 cell-corner
// array and the FP64 copy, built from node values already on the device, so that large grids (256^3 nodes and more) and grids generated on the
// device never pass through a host loop.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include <math_constants.h>

#include "sdfc_internal.h"

namespace {

constexpr unsigned kFullMask = 0xffffffffu;

// Non-negative doubles order like their bit patterns, so an unsigned 64-bit atomic maximum on
// the bits is the maximum of the values.
__device__ __forceinline__ void max_bits(unsigned long long* dst, double v) {
    atomicMax(dst, (unsigned long long)__double_as_longlong(v));
}

// out[0] = max |v|, out[1 + a] = max |v(node + e_a) - v(node)| along axis a, out[4] = 1 if a
// value is not finite.  Differences are taken in FP64 (exact for FP32 inputs).
template <typename T>
__global__ void grid_stats_kernel(const T* __restrict__ v, int ni, int nj, int nk, unsigned long long* __restrict__ out) {
    const size_t n = (size_t)ni * nj * nk, sj = (size_t)ni, sk = (size_t)ni * nj;
    double m[4] = {0.0, 0.0, 0.0, 0.0};
    bool bad = false;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx % sj), j = (int)((idx / sj) % nj), k = (int)(idx / sk);
        const double a = (double)v[idx];
        bad |= !isfinite(a);
        m[0] = fmax(m[0], fabs(a));
        if (i + 1 < ni) m[1] = fmax(m[1], fabs((double)v[idx + 1] - a));
        if (j + 1 < nj) m[2] = fmax(m[2], fabs((double)v[idx + sj] - a));
        if (k + 1 < nk) m[3] = fmax(m[3], fabs((double)v[idx + sk] - a));
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int o = 16; o; o >>= 1) m[q] = fmax(m[q], __shfl_xor_sync(kFullMask, m[q], o));
    const unsigned anybad = __ballot_sync(kFullMask, bad);
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (m[q] > 0.0) max_bits(out + q, m[q]);
        if (anybad) out[4] = 1ull;
    }
}

// Per cell (i fastest over the (ni-1)(nj-1)(nk-1) cells) its 8 corners in FP32:
// (c000, c100, c010, c110), (c001, c101, c011, c111).
template <typename T>
__global__ void cell_corners_kernel(const T* __restrict__ v, int ni, int nj, int nk, float4* __restrict__ cells) {
    const size_t ci = (size_t)ni - 1, cj = (size_t)nj - 1, nc = ci * cj * ((size_t)nk - 1);
    const size_t sj = (size_t)ni, sk = (size_t)ni * nj;
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < nc; c += (size_t)gridDim.x * blockDim.x) {
        const size_t i = c % ci, j = (c / ci) % cj, k = c / (ci * cj);
        const size_t b = i + sj * j + sk * k;
        cells[2 * c] = make_float4((float)v[b], (float)v[b + 1], (float)v[b + sj], (float)v[b + sj + 1]);
        cells[2 * c + 1] =
            make_float4((float)v[b + sk], (float)v[b + sk + 1], (float)v[b + sk + sj], (float)v[b + sk + sj + 1]);
    }
}

// Per block of 2^bs cells per axis, the least FP32 node value over the nodes of its cells
// (nodes bB .. min(bB + B, n - 1) per axis), block (bi, bj, bk) at bi + bnx (bj + bny bk).
template <typename T>
__global__ void block_min_kernel(const T* __restrict__ v, int ni, int nj, int nk, int bs, int bnx, int bny, int bnz,
                                 float* __restrict__ out) {
    const size_t nb = (size_t)bnx * bny * bnz, sj = (size_t)ni, sk = (size_t)ni * nj;
    const int B = 1 << bs;
    for (size_t b = blockIdx.x * (size_t)blockDim.x + threadIdx.x; b < nb; b += (size_t)gridDim.x * blockDim.x) {
        const int bi = (int)(b % bnx), bj = (int)((b / bnx) % bny), bk = (int)(b / ((size_t)bnx * bny));
        const int i0 = bi * B, j0 = bj * B, k0 = bk * B;
        const int i1 = min(i0 + B, ni - 1), j1 = min(j0 + B, nj - 1), k1 = min(k0 + B, nk - 1);
        float m = CUDART_INF_F;
        for (int k = k0; k <= k1; ++k)
            for (int j = j0; j <= j1; ++j)
                for (int i = i0; i <= i1; ++i) m = fminf(m, (float)v[(size_t)i + sj * j + sk * k]);
        out[b] = m;
    }
}

__global__ void widen_kernel(const float* __restrict__ a, double* __restrict__ b, size_t n) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
        b[q] = (double)a[q];
}

int grid_blocks(sdfc_context* ctx, size_t work) {
    return (int)std::max<size_t>(1, std::min<size_t>((work + 255) / 256, (size_t)ctx->sm_count * 8));
}

}  // namespace

namespace sdfc_impl {

int grid_finish_device(sdfc_context* ctx, sdfc::GridDesc& g, const void* d_values, bool fp32, bool cells) {
    const int ni = g.ni, nj = g.nj, nk = g.nk;
    const size_t n = (size_t)ni * nj * nk;
    cudaStream_t s = ctx->stream;
    unsigned long long* d_st = nullptr;
    int rc = dev_alloc(ctx, (void**)&d_st, 5 * sizeof(unsigned long long));
    if (rc) return rc;
    unsigned long long st[5] = {0, 0, 0, 0, 0};
    cudaError_t e = cudaMemsetAsync(d_st, 0, sizeof(st), s);
    if (e == cudaSuccess) {
        if (fp32)
            grid_stats_kernel<float><<<grid_blocks(ctx, n), 256, 0, s>>>((const float*)d_values, ni, nj, nk, d_st);
        else
            grid_stats_kernel<double><<<grid_blocks(ctx, n), 256, 0, s>>>((const double*)d_values, ni, nj, nk, d_st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(st, d_st, sizeof(st), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_st);
    if (e != cudaSuccess) return fail(ctx, SDFC_ERR_CUDA, std::string("upload_grid: ") + cudaGetErrorString(e));
    if (st[4]) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_grid: non-finite value");
    auto val = [&](int q) {
        double d;
        std::memcpy(&d, &st[q], sizeof d);
        return d;
    };
    double lip2 = 0.0;
    for (int a = 0; a < 3; ++a) lip2 += (val(1 + a) / g.dx[a]) * (val(1 + a) / g.dx[a]);
    g.lip = (float)(std::sqrt(lip2) * 1.0001);
    g.vmax = (float)(val(0) * 1.0001);
    if (cells) {
        const size_t nc = (size_t)(ni - 1) * (nj - 1) * (nk - 1);
        void* pc = nullptr;
        if ((rc = dev_alloc(ctx, &pc, nc * 2 * sizeof(float4)))) return rc;
        ctx->allocations.push_back(pc);
        if (fp32)
            cell_corners_kernel<float><<<grid_blocks(ctx, nc), 256, 0, s>>>((const float*)d_values, ni, nj, nk,
                                                                           (float4*)pc);
        else
            cell_corners_kernel<double><<<grid_blocks(ctx, nc), 256, 0, s>>>((const double*)d_values, ni, nj, nk,
                                                                            (float4*)pc);
        g.cells32 = (const float4*)pc;
        SDFC_CUDA_TRY(ctx, cudaGetLastError());
    }
    {
        // detection's block table: 2-cell blocks beside the 40-byte cell-corner layout (an eighth
        // of a node's 4 bytes more per node), 4-cell blocks beside 4-byte node values
        const int bs = cells ? 1 : 2, B = 1 << bs;
        const int bnx = (ni - 1 + B - 1) / B, bny = (nj - 1 + B - 1) / B, bnz = (nk - 1 + B - 1) / B;
        const size_t nb = (size_t)bnx * bny * bnz;
        void* pb = nullptr;
        if ((rc = dev_alloc(ctx, &pb, nb * sizeof(float)))) return rc;
        ctx->allocations.push_back(pb);
        if (fp32)
            block_min_kernel<float><<<grid_blocks(ctx, nb), 256, 0, s>>>((const float*)d_values, ni, nj, nk, bs, bnx, bny,
                                                                        bnz, (float*)pb);
        else
            block_min_kernel<double><<<grid_blocks(ctx, nb), 256, 0, s>>>((const double*)d_values, ni, nj, nk, bs, bnx,
                                                                         bny, bnz, (float*)pb);
        SDFC_CUDA_TRY(ctx, cudaGetLastError());
        g.bmin = (const float*)pb;
        g.bshift = bs;
        g.bnx = bnx;
        g.bny = bny;
    }
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return SDFC_OK;
}

int widen_device(sdfc_context* ctx, const float* a, double* b, size_t n) {
    widen_kernel<<<grid_blocks(ctx, n), 256, 0, ctx->stream>>>(a, b, n);
    SDFC_CUDA_TRY(ctx, cudaGetLastError());
    return SDFC_OK;
}

}  // namespace sdfc_impl
