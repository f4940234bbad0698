// Kernels of the batched point-vs-SDF contact evaluation; see sdfc_kernels.cuh.
#include <cstdint>

#include "sdfc_kernels.cuh"

namespace sdfc {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr double kU = 5.9604644775390625e-08;  // 2^-24, unit round-off of FP32

// FP32 prefilter constants of one instance, shared by a detection CTA.
struct Prefilter {
    float R[9], p[3];            // point -> grid frame: x = R xi + p
    float gmin[3], ginv[3];      // grid origin and 1/dx
    float lo_in[3], hi_in[3];    // certainly inside the box between these
    float lo_out[3], hi_out[3];  // certainly outside beyond these
    float col_th;
    float guard;                 // bound on |d32 - d64|, times a safety factor
};

// Builds the FP32 transform and the error bound of the FP32 distance.
//   Position: y32 = fl(R) fl(xi) + fl(p) in FP32 differs from the FP64 grid-frame
//   point by at most eps_pos = u (10 (sqrt3 r + |p|) + 4 (|min| + sqrt3 r + |p|))
//   (rounding of R, p, xi, the 9 multiply-adds, and the cell-coordinate
//   arithmetic (y - min) / dx expressed in length).
//   Value: the FP32 trilinear of FP32-rounded values adds <= 12 u vmax and the
//   threshold u |col_th|; a distance error is at most lip * eps_pos + those.
//   The guard band is 4x that bound.
__device__ void make_prefilter(const GridDesc& g, const PointsDesc& P, const Pose& A, const Pose& B,
                               Prefilter& f) {
    M3 R = mul(transpose(B.R), A.R);
    V3 p = mulT(B.R, A.p - B.p);
    for (int k = 0; k < 9; ++k) f.R[k] = (float)R.m[k];
    f.p[0] = (float)p.x;
    f.p[1] = (float)p.y;
    f.p[2] = (float)p.z;
    const double r = 1.7320508075688772 * (double)P.radius;
    const double pn = norm(p);
    double mn = 0.0;
    for (int a = 0; a < 3; ++a) mn = fmax(mn, fmax(fabs(g.min_box[a]), fabs(g.max_box[a])));
    const double eps_pos = kU * (10.0 * (r + pn) + 4.0 * (mn + r + pn)) + 1e-30;
    for (int a = 0; a < 3; ++a) {
        f.gmin[a] = g.fmin[a];
        f.ginv[a] = g.finv_dx[a];
        double slack = 2.0 * eps_pos + 2.0 * kU * fmax(fabs(g.min_box[a]), fabs(g.max_box[a]));
        f.lo_in[a] = (float)(g.min_box[a] + slack);
        f.hi_in[a] = (float)(g.max_box[a] - slack);
        f.lo_out[a] = (float)(g.min_box[a] - slack);
        f.hi_out[a] = (float)(g.max_box[a] + slack);
    }
    f.col_th = (float)g.col_th;
    double bound = (double)g.lip * eps_pos + 12.0 * kU * (double)g.vmax + 2.0 * kU * fabs(g.col_th);
    f.guard = (float)(4.0 * bound) + 1e-30f;
}

// FP32 trilinear interpolation for a point certainly inside the box.
__device__ __forceinline__ float trilinear32(const GridDesc& g, const Prefilter& f, float x, float y, float z) {
    float cx = (x - f.gmin[0]) * f.ginv[0];
    float cy = (y - f.gmin[1]) * f.ginv[1];
    float cz = (z - f.gmin[2]) * f.ginv[2];
    int i = min(max((int)floorf(cx), 0), g.ni - 2);
    int j = min(max((int)floorf(cy), 0), g.nj - 2);
    int k = min(max((int)floorf(cz), 0), g.nk - 2);
    float u = cx - (float)i, v = cy - (float)j, w = cz - (float)k;
    const size_t sj = (size_t)g.ni, sk = (size_t)g.ni * (size_t)g.nj;
    const float* b = g.v32 + (size_t)i + sj * (size_t)j + sk * (size_t)k;
    float c000 = __ldg(b), c100 = __ldg(b + 1);
    float c010 = __ldg(b + sj), c110 = __ldg(b + sj + 1);
    float c001 = __ldg(b + sk), c101 = __ldg(b + sk + 1);
    float c011 = __ldg(b + sk + sj), c111 = __ldg(b + sk + sj + 1);
    float a0 = fmaf(u, c100 - c000, c000), a1 = fmaf(u, c110 - c010, c010);
    float a2 = fmaf(u, c101 - c001, c001), a3 = fmaf(u, c111 - c011, c011);
    float b0 = fmaf(v, a1 - a0, a0), b1 = fmaf(v, a3 - a2, a2);
    return fmaf(w, b1 - b0, b0);
}

__device__ __forceinline__ V3 load_point(const PointsDesc& P, int id) {
    if (P.storage == 0) return v3(P.x64[id], P.x64[P.n + id], P.x64[2 * (size_t)P.n + id]);
    return v3((double)__ldg(P.x32 + id), (double)__ldg(P.x32 + P.n + id), (double)__ldg(P.x32 + 2 * (size_t)P.n + id));
}

// distance() of the reference on the FP64 path (BodySDFObj.cpp:207-213 after
// CollisionDetection.cpp:136): xw = R_A xi + p_A, x = R_B^T (xw - p_B).
__device__ __forceinline__ double exact_distance(const GridDesc& g, const Pose& A, const Pose& B, V3 xi) {
    V3 x = grid_point(B.R, B.p, world_point(A.R, A.p, xi));
    return query_sdf(g, x, false) + g.col_th;
}

// ------------------------------------------------------------------ detection
__global__ void __launch_bounds__(kDetectThreads) detect_kernel(const InstanceDesc* __restrict__ inst,
                                                                const int* __restrict__ tile_inst, BatchInputs in,
                                                                const GridDesc* __restrict__ grids,
                                                                const PointsDesc* __restrict__ points,
                                                                int* __restrict__ ids, int* __restrict__ tile_count,
                                                                unsigned long long* __restrict__ recheck) {
    __shared__ GridDesc g;
    __shared__ PointsDesc P;
    __shared__ Prefilter f;
    __shared__ Pose A, B;
    __shared__ int warp_cnt[kDetectThreads / 32];
    __shared__ int base;
    const int t = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int i = tile_inst[t];
    const InstanceDesc I = inst[i];
    if (tid == 0) {
        g = grids[I.grid];
        P = points[I.points];
        A = load_pose(in.EA + 16 * (size_t)i);
        B = load_pose(in.EB + 16 * (size_t)i);
        make_prefilter(g, P, A, B, f);
        base = 0;
    }
    __syncthreads();
    const int first = (t - I.tile0) * kTile;
    const int count = min(kTile, P.n - first);
    int* out = ids + (size_t)t * kTile;
    int n_recheck = 0;
    for (int r0 = 0; r0 < count; r0 += kDetectThreads) {
        const int local = r0 + tid;
        const int pid = first + local;
        bool active = false;
        if (local < count) {
            float xi, yi, zi;
            if (P.storage == 0) {
                xi = (float)P.x64[pid];
                yi = (float)P.x64[P.n + pid];
                zi = (float)P.x64[2 * (size_t)P.n + pid];
            } else {
                xi = __ldg(P.x32 + pid);
                yi = __ldg(P.x32 + P.n + pid);
                zi = __ldg(P.x32 + 2 * (size_t)P.n + pid);
            }
            float x = fmaf(f.R[0], xi, fmaf(f.R[1], yi, fmaf(f.R[2], zi, f.p[0])));
            float y = fmaf(f.R[3], xi, fmaf(f.R[4], yi, fmaf(f.R[5], zi, f.p[1])));
            float z = fmaf(f.R[6], xi, fmaf(f.R[7], yi, fmaf(f.R[8], zi, f.p[2])));
            bool maybe_in = x >= f.lo_out[0] && x <= f.hi_out[0] && y >= f.lo_out[1] && y <= f.hi_out[1] &&
                            z >= f.lo_out[2] && z <= f.hi_out[2];
            if (maybe_in) {
                bool surely_in = x >= f.lo_in[0] && x <= f.hi_in[0] && y >= f.lo_in[1] && y <= f.hi_in[1] &&
                                 z >= f.lo_in[2] && z <= f.hi_in[2];
                bool exact = !surely_in;
                if (surely_in) {
                    float d32 = trilinear32(g, f, x, y, z) + f.col_th;
                    if (fabsf(d32) <= f.guard)
                        exact = true;
                    else
                        active = d32 < 0.0f;
                }
                if (exact) {
                    ++n_recheck;
                    active = exact_distance(g, A, B, load_point(P, pid)) < 0.0;
                }
            }
        }
        // ordered compaction: ascending point ids within the tile
        const unsigned m = __ballot_sync(kFull, active);
        if (lane == 0) warp_cnt[warp] = __popc(m);
        __syncthreads();
        int off = base;
        for (int w = 0; w < warp; ++w) off += warp_cnt[w];
        off += __popc(m & ((1u << lane) - 1u));
        if (active) out[off] = pid;
        __syncthreads();
        if (tid == 0) {
            int s = 0;
            for (int w = 0; w < kDetectThreads / 32; ++w) s += warp_cnt[w];
            base += s;
        }
        __syncthreads();
    }
    if (tid == 0) tile_count[t] = base;
    if (recheck) {
        for (int o = 16; o > 0; o >>= 1) n_recheck += __shfl_xor_sync(kFull, n_recheck, o);
        if (lane == 0 && n_recheck) atomicAdd(recheck, (unsigned long long)n_recheck);
    }
}

// ------------------------------------------------------------------ forces
// Warp-level sink: sums each produced value over the warp's 32 contacts with a
// shuffle butterfly and adds it to the warp's shared-memory row.
template <int NV>
struct WarpSink {
    double* acc;  // this warp's NV accumulators
    int lane;
    bool valid;
    V3 xi1, xi2;

    __device__ __forceinline__ void add(int idx, double v) {
        v = valid ? v : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
        if (lane == 0) acc[idx] += v;
    }
    __device__ __forceinline__ void add3(int idx, int stride, V3 v) {
        add(idx, v.x);
        add(idx + stride, v.y);
        add(idx + 2 * stride, v.z);
    }
    // fm = [xi1 x f1; f1; xi2 x f2; f2]  (Gamma^T f, simulation/redmax/Utils.h:196)
    __device__ __forceinline__ void force(V3 a1, V3 f1, V3 a2, V3 f2) {
        xi1 = a1;
        xi2 = a2;
        add3(0, 1, cross(a1, f1));
        add3(3, 1, f1);
        add3(6, 1, cross(a2, f2));
        add3(9, 1, f2);
    }
    // column c of [Km | Dm]: rows [xi1 x N1; N1; xi2 x N2 + T2; N2]
    __device__ __forceinline__ void column(int c, V3 N1, V3 N2, V3 T2) {
        if constexpr (NV == kOutDeriv) {
            const int base = c < 12 ? 12 + c : 156 + (c - 12);
            add3(base, 12, cross(xi1, N1));
            add3(base + 36, 12, N1);
            add3(base + 72, 12, cross(xi2, N2) + T2);
            add3(base + 108, 12, N2);
        }
    }
};

template <bool DERIV, bool STENCIL>
__global__ void __launch_bounds__(kChunk) force_kernel(const InstanceDesc* __restrict__ inst, BatchInputs in,
                                                       const GridDesc* __restrict__ grids,
                                                       const PointsDesc* __restrict__ points,
                                                       const int* __restrict__ ids,
                                                       const int* __restrict__ tile_count,
                                                       double* __restrict__ partial) {
    constexpr int NV = DERIV ? kOutDeriv : kOutValue;
    constexpr int NW = kChunk / 32;
    __shared__ double acc[NW * NV];
    __shared__ int prefix[kMaxTilesPerInstance + 1];
    __shared__ GridDesc g;
    __shared__ PointsDesc P;
    const int i = blockIdx.y, s = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const InstanceDesc I = inst[i];
    if (tid == 0) {
        int run = 0;
        prefix[0] = 0;
        for (int k = 0; k < I.ntiles; ++k) {
            run += tile_count[I.tile0 + k];
            prefix[k + 1] = run;
        }
        g = grids[I.grid];
        P = points[I.points];
    }
    for (int k = tid; k < NW * NV; k += kChunk) acc[k] = 0.0;
    __syncthreads();
    const int total = prefix[I.ntiles];
    const int nchunks = (total + kChunk - 1) / kChunk;
    if (s < nchunks) {
        BodyState A, B;
        A.P = load_pose(in.EA + 16 * (size_t)i);
        B.P = load_pose(in.EB + 16 * (size_t)i);
        const double* pa = in.phiA + 6 * (size_t)i;
        const double* pb = in.phiB + 6 * (size_t)i;
        A.w = v3(pa[0], pa[1], pa[2]);
        A.v = v3(pa[3], pa[4], pa[5]);
        B.w = v3(pb[0], pb[1], pb[2]);
        B.v = v3(pb[3], pb[4], pb[5]);
        const double* pr = in.prm + 6 * (size_t)i;
        ContactParams cp;
        cp.kn = pr[0] * pr[4] * pr[5];
        cp.kt = pr[1] * pr[4] * pr[5];
        cp.mu = pr[2];
        cp.kd = pr[3];
        for (int chunk = s; chunk < nchunks; chunk += kSlots) {
            const int c = chunk * kChunk + tid;
            const bool valid = c < total;
            V3 xi = v3(0, 0, 0);
            if (valid) {
                int lo = 0, hi = I.ntiles;  // largest k with prefix[k] <= c
                while (hi - lo > 1) {
                    int mid = (lo + hi) >> 1;
                    if (prefix[mid] <= c)
                        lo = mid;
                    else
                        hi = mid;
                }
                const int pid = ids[(size_t)(I.tile0 + lo) * kTile + (c - prefix[lo])];
                xi = load_point(P, pid);
            }
            WarpSink<NV> sink{acc + warp * NV, lane, valid, v3(0, 0, 0), v3(0, 0, 0)};
            if constexpr (DERIV) {
                contact_force_jacobian(g, xi, A, B, cp, sink, valid, STENCIL);
            } else {
                ContactForce F = contact_force(g, xi, A, B, cp, valid, STENCIL);
                sink.force(F.xi1, F.f1, F.xi2, F.f2);
            }
        }
    }
    __syncthreads();
    double* row = partial + ((size_t)i * kSlots + s) * NV;
    for (int k = tid; k < NV; k += kChunk) {
        double v = 0.0;
        for (int w = 0; w < NW; ++w) v += acc[w * NV + k];
        row[k] = v;
    }
}

template <bool DERIV>
__global__ void finalize_kernel(const InstanceDesc* __restrict__ inst, int n_inst, const int* __restrict__ tile_count,
                                const double* __restrict__ partial, BatchOutputs out) {
    constexpr int NV = DERIV ? kOutDeriv : kOutValue;
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n_inst * NV) return;
    const int i = (int)(idx / NV), k = (int)(idx % NV);
    const double* p = partial + (size_t)i * kSlots * NV + k;
    double v = 0.0;
    for (int s = 0; s < kSlots; ++s) v += p[(size_t)s * NV];
    if (k < 12)
        out.fm[12 * (size_t)i + k] = v;
    else if (k < 156)
        out.Km[144 * (size_t)i + (k - 12)] = v;
    else
        out.Dm[144 * (size_t)i + (k - 156)] = v;
    if (!isfinite(v)) atomicOr(out.status + i, 1);
    if (k == 0) {
        const InstanceDesc I = inst[i];
        int n = 0;
        for (int t = 0; t < I.ntiles; ++t) n += tile_count[I.tile0 + t];
        out.n_active[i] = n;
    }
}

__global__ void zero_status_kernel(int* status, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) status[i] = 0;
}

}  // namespace

void launch_detect(const InstanceDesc* d_inst, const int* d_tile_inst, int total_tiles, BatchInputs in,
                   const GridDesc* d_grids, const PointsDesc* d_points, int* d_ids, int* d_tile_count,
                   unsigned long long* d_recheck, cudaStream_t stream) {
    if (total_tiles <= 0) return;
    detect_kernel<<<total_tiles, kDetectThreads, 0, stream>>>(d_inst, d_tile_inst, in, d_grids, d_points, d_ids,
                                                              d_tile_count, d_recheck);
}

void launch_force(const InstanceDesc* d_inst, int n_inst, BatchInputs in, const GridDesc* d_grids,
                  const PointsDesc* d_points, const int* d_ids, const int* d_tile_count, double* d_partial,
                  bool deriv, bool stencil, cudaStream_t stream) {
    if (n_inst <= 0) return;
    dim3 grid(kSlots, n_inst);
    auto* k = deriv ? (stencil ? force_kernel<true, true> : force_kernel<true, false>)
                    : (stencil ? force_kernel<false, true> : force_kernel<false, false>);
    k<<<grid, kChunk, 0, stream>>>(d_inst, in, d_grids, d_points, d_ids, d_tile_count, d_partial);
}

void launch_finalize(const InstanceDesc* d_inst, int n_inst, const int* d_tile_count, const double* d_partial,
                     bool deriv, BatchOutputs out, cudaStream_t stream) {
    if (n_inst <= 0) return;
    zero_status_kernel<<<(n_inst + 255) / 256, 256, 0, stream>>>(out.status, n_inst);
    const int NV = deriv ? kOutDeriv : kOutValue;
    const size_t total = (size_t)n_inst * NV;
    const int threads = 256;
    const unsigned blocks = (unsigned)((total + threads - 1) / threads);
    if (deriv)
        finalize_kernel<true><<<blocks, threads, 0, stream>>>(d_inst, n_inst, d_tile_count, d_partial, out);
    else
        finalize_kernel<false><<<blocks, threads, 0, stream>>>(d_inst, n_inst, d_tile_count, d_partial, out);
}

}  // namespace sdfc
