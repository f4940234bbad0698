// sdfc_evaluate_noalloc: one contact evaluation that allocates no memory.
//
// Some callers cannot call cudaMalloc at the point where they need the contact
// force: a physics step driven from inside a real-time loop (cudaMalloc can
// synchronise the device and its latency is unbounded), a host application
// whose memory is owned by its own pool allocator and which forbids other
// allocations, or code running while the caller records work into a CUDA
// stream capture.  For them this entry point takes every input and output as
// caller-owned device memory and keeps its working memory in one file-scope
// device array, reserved when the library is loaded.
//
// The array holds, per call, one flag per contact point and one partial-sum
// row per block of kNaChunk points, for at most kNaMaxPoints points; every GPU
// that loads the library keeps it until the process exits.  All calls share it:
// two calls whose work overlaps on the GPU (different streams, or different
// host threads without ordering) race on it.  Each call writes every element
// it later reads before reading it, so no state carries over between calls and
// nothing needs clearing.
//
// The arithmetic is the FP64 path of the batched kernels (the same device
// functions): exact FP64 detection in the reference's operation order, FP64
// contact algebra with analytic cell derivatives, FP64 sums in a fixed order.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "sdfc.h"
#include "sdfc_contact.cuh"

namespace {

using namespace sdfc;

constexpr int kNaMaxPoints = SDFC_NOALLOC_MAX_POINTS;
constexpr int kNaChunk = 128;                                   // points per force block
constexpr int kNaRows = kNaMaxPoints / kNaChunk;                // partial rows
constexpr int kNaRowWidth = 304;                                // 300 outputs + active count, padded
constexpr unsigned kNaFull = 0xffffffffu;

// flags[kNaMaxPoints] (one byte per point) followed by partial[kNaRows][kNaRowWidth]
constexpr size_t kNaFlagBytes = ((size_t)kNaMaxPoints + 255) / 256 * 256;
constexpr size_t kNaScratchBytes = kNaFlagBytes + sizeof(double) * (size_t)kNaRows * kNaRowWidth;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

// Per-device address of g_noalloc_scratch, found once per device.
constexpr int kNaMaxDevices = 64;
std::once_flag g_once[kNaMaxDevices];
void* g_addr[kNaMaxDevices];
cudaError_t g_addr_err[kNaMaxDevices];

__device__ __forceinline__ V3 na_point(const double* p, int i) { return v3(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

// Detection: one thread per point, the reference's FP64 distance
// (CollisionDetection.cpp:136-139, BodySDFObj.cpp:207-213).
__global__ void na_detect_kernel(GridDesc g, const double* __restrict__ pts, int n, const double* __restrict__ EA,
                                 const double* __restrict__ EB, unsigned char* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Pose A = load_pose(EA), B = load_pose(EB);
    const V3 x = grid_point(B.R, B.p, world_point(A.R, A.p, na_point(pts, i)));
    flags[i] = (query_sdf(g, x, false) + g.col_th) < 0.0 ? 1 : 0;
}

// Sums 32 lanes' values into lane 0.
__device__ __forceinline__ double na_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kNaFull, v, o);
    return v;
}

template <int NV>
struct NaSink {
    double* acc;  // this warp's NV accumulators (shared memory)
    int lane;
    bool valid;
    V3 xi1, xi2;
    __device__ __forceinline__ void add(int idx, double v) {
        v = na_warp_sum(valid ? v : 0.0);
        if (lane == 0) acc[idx] += v;
    }
    __device__ __forceinline__ void add3(int idx, int stride, V3 v) {
        add(idx, v.x);
        add(idx + stride, v.y);
        add(idx + 2 * stride, v.z);
    }
    __device__ __forceinline__ void force(V3 a1, V3 f1, V3 a2, V3 f2) {
        xi1 = a1;
        xi2 = a2;
        add3(0, 1, cross(a1, f1));
        add3(3, 1, f1);
        add3(6, 1, cross(a2, f2));
        add3(9, 1, f2);
    }
    __device__ __forceinline__ void column(int c, V3 N1, V3 N2, V3 T2) {
        if constexpr (NV == 300) {
            const int base = c < 12 ? 12 + c : 156 + (c - 12);
            add3(base, 12, cross(xi1, N1));
            add3(base + 36, 12, N1);
            add3(base + 72, 12, cross(xi2, N2) + T2);
            add3(base + 108, 12, N2);
        }
    }
};

// Forces: one block per kNaChunk points; active points contribute, the block's
// sums and active count go to its own partial row.
template <bool DERIV>
__global__ void __launch_bounds__(kNaChunk) na_force_kernel(GridDesc g, const double* __restrict__ pts, int n,
                                                            const double* __restrict__ EA, const double* __restrict__ phiA,
                                                            const double* __restrict__ EB, const double* __restrict__ phiB,
                                                            const double* __restrict__ prm,
                                                            const unsigned char* __restrict__ flags,
                                                            double* __restrict__ partial) {
    constexpr int NV = DERIV ? 300 : 12;
    constexpr int NW = kNaChunk / 32;
    __shared__ double acc[NW * NV];
    __shared__ int wcount[NW];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int k = tid; k < NW * NV; k += kNaChunk) acc[k] = 0.0;
    __syncthreads();
    const int i = blockIdx.x * kNaChunk + tid;
    const bool valid = i < n && flags[i] != 0;
    const unsigned m = __ballot_sync(kNaFull, valid);
    if (lane == 0) wcount[warp] = __popc(m);
    if (m != 0) {
        PairState<double> S;
        make_pair_state(EA, phiA, EB, phiB, prm, S);
        const V3 xi = valid ? na_point(pts, i) : v3(0, 0, 0);
        NaSink<NV> sink{acc + warp * NV, lane, valid, v3(0, 0, 0), v3(0, 0, 0)};
        if constexpr (DERIV) {
            contact_force_jacobian<double>(g, xi, S, nullptr, sink, valid, false);
        } else {
            ContactForce<double> F = contact_force<double>(g, xi, S, nullptr, valid, false);
            sink.force(F.xi1, F.f1, F.xi2, F.f2);
        }
    }
    __syncthreads();
    double* row = partial + (size_t)blockIdx.x * kNaRowWidth;
    for (int k = tid; k < NV; k += kNaChunk) {
        double v = 0.0;
        for (int w = 0; w < NW; ++w) v += acc[w * NV + k];
        row[k] = v;
    }
    if (tid == 0) {
        int c = 0;
        for (int w = 0; w < NW; ++w) c += wcount[w];
        row[NV] = (double)c;
    }
}

// Sums the rows in order into the caller's outputs.
template <bool DERIV>
__global__ void na_finalize_kernel(const double* __restrict__ partial, int rows, double* __restrict__ fm,
                                   double* __restrict__ Km, double* __restrict__ Dm, int* __restrict__ n_active) {
    constexpr int NV = DERIV ? 300 : 12;
    for (int k = threadIdx.x; k <= NV; k += blockDim.x) {
        double v = 0.0;
        for (int r = 0; r < rows; ++r) v += partial[(size_t)r * kNaRowWidth + k];
        if (k == NV)
            *n_active = (int)v;
        else if (k < 12)
            fm[k] = v;
        else if (k < 156)
            Km[k - 12] = v;
        else
            Dm[k - 156] = v;
    }
}

}  // namespace

extern "C" int sdfc_evaluate_noalloc(const double* grid_values, int ni, int nj, int nk, const double* min_box,
                                     const double* max_box, const double* dxyz, double col_th, const double* points,
                                     int n, const double* E_A, const double* phi_A, const double* E_B,
                                     const double* phi_B, const double* params, int want_deriv, double* fm, double* Km,
                                     double* Dm, int* n_active, void* stream) {
    if (n < 0) return SDFC_ERR_INVALID_ARGUMENT;
    if (n > kNaMaxPoints) {
        std::fprintf(stderr, "sdfc_evaluate_noalloc: %d points exceed the maximum of %d\n", n, kNaMaxPoints);
        return SDFC_ERR_CAPACITY;
    }
    if (!grid_values || !min_box || !max_box || !dxyz || (n > 0 && !points) || !E_A || !phi_A || !E_B || !phi_B ||
        !params || !fm || !n_active || (want_deriv && (!Km || !Dm)) || ni < 2 || nj < 2 || nk < 2)
        return SDFC_ERR_INVALID_ARGUMENT;
    const int nn[3] = {ni, nj, nk};
    for (int a = 0; a < 3; ++a)
        if (!(dxyz[a] > 0.0) || !(max_box[a] > min_box[a]) ||
            std::floor((max_box[a] - min_box[a]) / dxyz[a]) > nn[a] - 1)
            return SDFC_ERR_INVALID_ARGUMENT;

    // An error left pending by an earlier, unrelated runtime call stays with the caller: this
    // call refuses to run rather than report that error as its own and clear it.
    if (cudaPeekAtLastError() != cudaSuccess) return SDFC_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return SDFC_ERR_CUDA;
    // Set-up, once per device, on the current device: the host-side name of
    // g_noalloc_scratch is not a device address; ask the runtime for it.
    std::call_once(g_once[dev], [dev] {
        g_addr_err[dev] = cudaGetSymbolAddress(&g_addr[dev], g_noalloc_scratch);
    });
    if (g_addr_err[dev] != cudaSuccess || !g_addr[dev]) return SDFC_ERR_CUDA;
    unsigned char* flags = static_cast<unsigned char*>(g_addr[dev]);
    double* partial = reinterpret_cast<double*>(flags + kNaFlagBytes);

    GridDesc g{};
    g.ni = ni;
    g.nj = nj;
    g.nk = nk;
    g.storage = SDFC_STORAGE_F64;
    for (int a = 0; a < 3; ++a) {
        g.min_box[a] = min_box[a];
        g.max_box[a] = max_box[a];
        g.dx[a] = dxyz[a];
        g.inv_dx[a] = 1.0 / dxyz[a];
        g.org[a] = min_box[a] * g.inv_dx[a];
        g.fmin[a] = (float)min_box[a];
        g.fmax[a] = (float)max_box[a];
        g.finv_dx[a] = (float)g.inv_dx[a];
        g.fdx[a] = (float)dxyz[a];
    }
    g.col_th = col_th;
    g.v64 = grid_values;
    g.cells32 = nullptr;

    cudaStream_t s = (cudaStream_t)stream;
    const int rows = (n + kNaChunk - 1) / kNaChunk;
    if (n > 0) na_detect_kernel<<<(n + 255) / 256, 256, 0, s>>>(g, points, n, E_A, E_B, flags);
    if (rows > 0) {
        if (want_deriv)
            na_force_kernel<true><<<rows, kNaChunk, 0, s>>>(g, points, n, E_A, phi_A, E_B, phi_B, params, flags,
                                                            partial);
        else
            na_force_kernel<false><<<rows, kNaChunk, 0, s>>>(g, points, n, E_A, phi_A, E_B, phi_B, params, flags,
                                                             partial);
    }
    if (want_deriv)
        na_finalize_kernel<true><<<1, 320, 0, s>>>(partial, rows, fm, Km, Dm, n_active);
    else
        na_finalize_kernel<false><<<1, 32, 0, s>>>(partial, rows, fm, Km, Dm, n_active);
    // nothing was pending on entry, so an error now comes from these launches
    return cudaGetLastError() == cudaSuccess ? SDFC_OK : SDFC_ERR_CUDA;
}
