// Kernels of the batched point-vs-SDF contact evaluation; see sdfc_kernels.cuh.
#include <algorithm>
#include <atomic>
#include <math_constants.h>
#include <cstdint>

#include "sdfc_kernels.cuh"

namespace sdfc {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr double kU = 5.9604644775390625e-08;  // 2^-24, unit round-off of FP32

// ------------------------------------------------------------------ prefilter
// Builds the FP32 transform and the error bound of the FP32 distance.
//   Position: y32 = fl(R) fl(xi) + fl(p) in FP32 differs from the FP64 grid-frame
//   point by at most eps_pos = u (10 (sqrt3 r + |p|) + 4 (|min| + sqrt3 r + |p|))
//   (rounding of R, p, xi, the 9 multiply-adds, and the cell-coordinate
//   arithmetic (y - min) / dx expressed in length).
//   Value: the FP32 trilinear of FP32-rounded values adds <= 12 u vmax and the
//   threshold 2 u |col_th|; a distance error is at most lip * eps_pos + those.
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
    // The FP32 trilinear of a cell's FP32 corners is within 16 u vmax of their convex
    // combination (7 lerps, each difference and fma rounded), and the FP32 fraction of a cell
    // coordinate up to n may leave [0, 1] by n u, extrapolating by at most that times the largest
    // corner difference (lip dx); so the computed value is at least the block's least node value
    // less that margin, and its sum with col_th at least that less one more rounding.
    int nmax = max(g.ni, max(g.nj, g.nk));
    double dmax = fmax(g.dx[0], fmax(g.dx[1], g.dx[2]));
    const double margin = 16.0 * kU * (double)g.vmax + 2.0 * nmax * kU * (double)g.lip * dmax +
                          4.0 * kU * (fabs(g.col_th) + (double)f.guard + (double)g.vmax);
    const double th = (double)f.guard - (double)f.col_th + margin;
    float t = (float)th;
    if ((double)t < th) t = nextafterf(t, CUDART_INF_F);
    f.skip_th = t;
}

__global__ void prep_kernel(const InstanceDesc* __restrict__ inst, int n, BatchInputs in,
                            const GridDesc* __restrict__ grids, const PointsDesc* __restrict__ points,
                            Prefilter* __restrict__ pref, PairState<float>* __restrict__ pair32,
                            PairState<double>* __restrict__ pair64, int* __restrict__ recheck_n,
                            int* __restrict__ badin, int* __restrict__ inst_total) {
    // blockIdx.y: 0 the prefilter, 1 / 2 the FP32 / FP64 pair state every force or energy CTA of
    // the instance starts from (once per instance here, spread over three warps per 32 instances:
    // all three are FP64 arithmetic)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && blockIdx.y == 0)  // detection's list of tiles to recheck starts empty, and so do the
        for (int q = 0; q < kCounters; ++q) recheck_n[q] = 0;  // force launches' queues and item lists
    if (i < n && blockIdx.y == 0) inst_total[i] = 0;  // detection adds each tile's active count

    if (i >= n || (in.mode && in.mode[i] == 0)) return;
    const size_t o = (size_t)i;
    if (blockIdx.y == 0) {
        // an instance whose poses, twists or coefficients are not all finite is flagged (its
        // points then classify as outside the grid, as the reference's distance query has them)
        bool finite = true;
        const double* rows[5] = {in.EA + 16 * o, in.phiA + 6 * o, in.EB + 16 * o, in.phiB + 6 * o, in.prm + 6 * o};
        const int widths[5] = {16, 6, 16, 6, 6};
        for (int r = 0; r < 5; ++r)
            for (int c = 0; c < widths[r]; ++c) finite = finite && isfinite(rows[r][c]);
        badin[i] = finite ? 0 : 1;
        const InstanceDesc I = inst[i];
        Prefilter f;
        make_prefilter(grids[I.grid], points[I.points], load_pose(in.EA + 16 * o), load_pose(in.EB + 16 * o), f);
        pref[i] = f;
    } else if (blockIdx.y == 1) {
        make_pair_state(in.EA + 16 * o, in.phiA + 6 * o, in.EB + 16 * o, in.phiB + 6 * o, in.prm + 6 * o, pair32[i]);
        make_cell_map(grids[inst[i].grid], pair32[i]);
    } else {
        make_pair_state(in.EA + 16 * o, in.phiA + 6 * o, in.EB + 16 * o, in.phiB + 6 * o, in.prm + 6 * o, pair64[i]);
        make_cell_map(grids[inst[i].grid], pair64[i]);
    }
}

// dst = src by the 32 lanes of a warp, 8 bytes per lane and step
template <typename S>
__device__ __forceinline__ void warp_copy(S& dst, const S& src, int lane) {
    static_assert(sizeof(S) % 8 == 0 && alignof(S) >= 8, "8-byte words");
    const long long* a = reinterpret_cast<const long long*>(&src);
    long long* b = reinterpret_cast<long long*>(&dst);
    for (int k = lane; k < (int)(sizeof(S) / 8); k += 32) b[k] = a[k];
}

// FP32 trilinear interpolation for a point certainly inside the box, from the
// cell-corner array (GridDesc::cells32) or, with `g` non-null, from FP16 bricks.
// With the block table `bm` (GridDesc::bmin), a point whose cell's block has its least node
// value above f.skip_th returns +inf without reading the cell: its distance is then neither in
// the guard band nor active, as the trilinear would have found.
__device__ __forceinline__ float trilinear32(const float4* __restrict__ cells, const GridDesc* g, int ni, int nj,
                                             int nk, const Prefilter& f, float x, float y, float z,
                                             const float* __restrict__ bm, int bsh, int bnx, int bny) {
    float cx = (x - f.gmin[0]) * f.ginv[0];
    float cy = (y - f.gmin[1]) * f.ginv[1];
    float cz = (z - f.gmin[2]) * f.ginv[2];
    int i = min(max((int)floorf(cx), 0), ni - 2);
    int j = min(max((int)floorf(cy), 0), nj - 2);
    int k = min(max((int)floorf(cz), 0), nk - 2);
    if (bm && __ldg(bm + (i >> bsh) + bnx * ((j >> bsh) + bny * (k >> bsh))) > f.skip_th) return CUDART_INF_F;
    float u = cx - (float)i, w1 = cy - (float)j, w2 = cz - (float)k;
    float c000, c100, c010, c110, c001, c101, c011, c111;
    if (g) {
        float c[8];
        cell_corners32(*g, i, j, k, c);
        c000 = c[0]; c100 = c[1]; c010 = c[2]; c110 = c[3];
        c001 = c[4]; c101 = c[5]; c011 = c[6]; c111 = c[7];
    } else {
        const float4* q = cells + 2 * ((size_t)i + (size_t)(ni - 1) * ((size_t)j + (size_t)(nj - 1) * k));
        const float4 lo = __ldg(q), hi = __ldg(q + 1);
        c000 = lo.x; c100 = lo.y; c010 = lo.z; c110 = lo.w;
        c001 = hi.x; c101 = hi.y; c011 = hi.z; c111 = hi.w;
    }
    float a0 = fmaf(u, c100 - c000, c000), a1 = fmaf(u, c110 - c010, c010);
    float a2 = fmaf(u, c101 - c001, c001), a3 = fmaf(u, c111 - c011, c011);
    float b0 = fmaf(w1, a1 - a0, a0), b1 = fmaf(w1, a3 - a2, a2);
    return fmaf(w2, b1 - b0, b0);
}

__device__ __forceinline__ V3 load_point(const PointsDesc& P, int id) {
    return v3(__ldg(P.x64 + id), __ldg(P.x64 + P.n + id), __ldg(P.x64 + 2 * (size_t)P.n + id));
}
// The same point rounded to FP32 (exactly the stored point for FP32 storage).
__device__ __forceinline__ Vec3<float> load_point32(const PointsDesc& P, int id) {
    return vec3<float>(__ldg(P.x32 + id), __ldg(P.x32 + P.n + id), __ldg(P.x32 + 2 * (size_t)P.n + id));
}

// distance() of the reference on the FP64 path (BodySDFObj.cpp:207-213 after
// CollisionDetection.cpp:136): xw = R_A xi + p_A, x = R_B^T (xw - p_B).
__device__ __forceinline__ double exact_distance(const GridDesc& g, const Pose& A, const Pose& B, V3 xi) {
    V3 x = grid_point(B.R, B.p, world_point(A.R, A.p, xi));
    return query_sdf(g, x, false) + g.col_th;
}

// ------------------------------------------------------------------ detection
// rounds of a detection tile classified with their loads in flight together
#ifndef SDFC_DETECT_UNROLL
#define SDFC_DETECT_UNROLL 8
#endif
constexpr int kDetectUnroll = SDFC_DETECT_UNROLL;
// One instantiation per kind of grid storage: BRICKS = false reads the FP32 cell-corner array
// (storages 0 and 1), BRICKS = true every grid without one, the FP16 bricks and the FP32 node
// values (with the grid descriptor in shared memory).  A batch launches the ones its grids need;
// each leaves the other kind's tiles alone, so the cell-corner kernel keeps the registers and
// shared memory of a build without the other storages.
template <bool BRICKS>
struct DetectGrid;
template <>
struct DetectGrid<false> {
    __device__ __forceinline__ void set(const GridDesc&) {}
    __device__ __forceinline__ const GridDesc* get() { return nullptr; }
};
template <>
struct DetectGrid<true> {
    GridDesc gd;
    __device__ __forceinline__ void set(const GridDesc& g) { gd = g; }
    __device__ __forceinline__ const GridDesc* get() { return &gd; }
};

template <bool BRICKS>
__global__ void __launch_bounds__(kDetectThreads) detect_kernel(const InstanceDesc* __restrict__ inst,
                                                                const int* __restrict__ tile_inst,
                                                                const Prefilter* __restrict__ pref,
                                                                const GridDesc* __restrict__ grids,
                                                                const PointsDesc* __restrict__ points,
                                                                int* __restrict__ ids, int* __restrict__ tile_count,
                                                                int* __restrict__ tile_queue,
                                                                const int* __restrict__ mode,
                                                                int* __restrict__ recheck_list,
                                                                int* __restrict__ recheck_n,
                                                                int* __restrict__ inst_total) {
    __shared__ Prefilter f;
    __shared__ DetectGrid<BRICKS> dg;
    __shared__ const float4* gv;
    __shared__ const float* px;
    __shared__ const float* bmin;
    __shared__ int gn[3], pn, bsh, bnx, bny;
    __shared__ int cnt_a[kTile / 32], cnt_q[kTile / 32];  // per (round, warp): counts, then offsets
    const int t = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int i = tile_inst[t];
    if (mode && mode[i] == 0) {  // instance not requested this time: its tiles are empty
        if (tid == 0) {
            tile_count[t] = 0;
            tile_queue[t] = 0;
        }
        return;
    }
    const InstanceDesc I = inst[i];
    if ((grids[I.grid].cells32 == nullptr) != BRICKS) return;  // the other storage's kernel handles this tile
    if (tid < (int)(sizeof(Prefilter) / sizeof(float)))
        reinterpret_cast<float*>(&f)[tid] = reinterpret_cast<const float*>(pref + i)[tid];
    if (tid == 0) {
        const GridDesc& g = grids[I.grid];
        dg.set(g);
        gv = g.cells32;
        gn[0] = g.ni;
        gn[1] = g.nj;
        gn[2] = g.nk;
        px = points[I.points].x32;
        pn = points[I.points].n;
        bmin = g.bmin;
        bsh = g.bshift;
        bnx = g.bnx;
        bny = g.bny;
    }
    __syncthreads();
    {
        // Broad phase: the tile's points lie in a sphere (body frame); where its image in the
        // grid frame, grown by a margin well above the FP32 transform's error (a few ulps of
        // |xi| + |p|), lies wholly outside the box test below on some axis, every point of the
        // tile fails that test, so the tile is empty without reading its points.
        const PointsDesc& P = points[I.points];
        const float4 sp = __ldg(P.tiles + (t - I.tile0));
        const float cx = fmaf(f.R[0], sp.x, fmaf(f.R[1], sp.y, fmaf(f.R[2], sp.z, f.p[0])));
        const float cy = fmaf(f.R[3], sp.x, fmaf(f.R[4], sp.y, fmaf(f.R[5], sp.z, f.p[1])));
        const float cz = fmaf(f.R[6], sp.x, fmaf(f.R[7], sp.y, fmaf(f.R[8], sp.z, f.p[2])));
        const float r = sp.w * 1.00001f +
                        1e-5f * (P.radius + fabsf(f.p[0]) + fabsf(f.p[1]) + fabsf(f.p[2]) + fabsf(cx) + fabsf(cy) +
                                 fabsf(cz));
        const bool away = cx + r < f.lo_out[0] || cx - r > f.hi_out[0] || cy + r < f.lo_out[1] ||
                          cy - r > f.hi_out[1] || cz + r < f.lo_out[2] || cz - r > f.hi_out[2];
        if (away) {  // uniform over the CTA
            if (tid == 0) {
                tile_count[t] = 0;
                tile_queue[t] = 0;
            }
            return;
        }
    }
    const int n = pn;
    const int first = (t - I.tile0) * kTile;
    const int count = min(kTile, n - first);
    int* out = ids + (size_t)t * kTile;
    const float* __restrict__ xs = px;
    // classification of the tile's kRounds rounds of kDetectThreads points (several rounds' loads
    // in flight), kept as per-thread bit masks; then the ordered compaction of all rounds
    constexpr int kRounds = kTile / kDetectThreads;
    constexpr int kWarps = kDetectThreads / 32;
    static_assert(kRounds * kWarps == 64, "the compaction scan takes two (round, warp) counts per lane");
    unsigned am = 0, qm = 0;
#pragma unroll kDetectUnroll
    for (int r = 0; r < kRounds; ++r) {
        const int local = r * kDetectThreads + tid;
        const int sid = first + local;
        bool active = false, queue = false;
        if (local < count) {
            const float xi = __ldg(xs + sid), yi = __ldg(xs + n + sid), zi = __ldg(xs + 2 * (size_t)n + sid);
            const float x = fmaf(f.R[0], xi, fmaf(f.R[1], yi, fmaf(f.R[2], zi, f.p[0])));
            const float y = fmaf(f.R[3], xi, fmaf(f.R[4], yi, fmaf(f.R[5], zi, f.p[1])));
            const float z = fmaf(f.R[6], xi, fmaf(f.R[7], yi, fmaf(f.R[8], zi, f.p[2])));
            const bool maybe_in = x >= f.lo_out[0] && x <= f.hi_out[0] && y >= f.lo_out[1] && y <= f.hi_out[1] &&
                                  z >= f.lo_out[2] && z <= f.hi_out[2];
            if (maybe_in) {
                const bool surely_in = x >= f.lo_in[0] && x <= f.hi_in[0] && y >= f.lo_in[1] && y <= f.hi_in[1] &&
                                       z >= f.lo_in[2] && z <= f.hi_in[2];
                if (surely_in) {
                    const float d32 =
                        trilinear32(gv, dg.get(), gn[0], gn[1], gn[2], f, x, y, z, bmin, bsh, bnx, bny) + f.col_th;
                    if (fabsf(d32) <= f.guard)
                        queue = true;
                    else
                        active = d32 < 0.0f;
                } else {
                    queue = true;
                }
            }
        }
        am |= (unsigned)active << r;
        qm |= (unsigned)queue << r;
    }
    // ordered compaction: ascending active stored indices from the start of the tile's slots,
    // queued ones from the end (descending positions); order = round, warp, lane
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const unsigned ma = __ballot_sync(kFull, (am >> r) & 1u), mq = __ballot_sync(kFull, (qm >> r) & 1u);
        if (lane == 0) {
            cnt_a[r * kWarps + warp] = __popc(ma);
            cnt_q[r * kWarps + warp] = __popc(mq);
        }
    }
    __syncthreads();
    if (warp == 0) {  // exclusive prefix over the 64 (round, warp) counts, two per lane
        const int a0 = cnt_a[2 * lane], a1 = cnt_a[2 * lane + 1];
        const int q0 = cnt_q[2 * lane], q1 = cnt_q[2 * lane + 1];
        int ia = a0 + a1, iq = q0 + q1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int ua = __shfl_up_sync(kFull, ia, o), uq = __shfl_up_sync(kFull, iq, o);
            if (lane >= o) {
                ia += ua;
                iq += uq;
            }
        }
        const int ea = ia - (a0 + a1), eq = iq - (q0 + q1);
        cnt_a[2 * lane] = ea;
        cnt_a[2 * lane + 1] = ea + a0;
        cnt_q[2 * lane] = eq;
        cnt_q[2 * lane + 1] = eq + q0;
        if (lane == 31) {
            tile_count[t] = ia;
            tile_queue[t] = iq;
            if (iq > 0) recheck_list[atomicAdd(recheck_n, 1)] = t;  // any order: tiles are independent
            if (ia > 0) atomicAdd(inst_total + i, ia);                // integer sums: exact in any order
        }
    }
    __syncthreads();
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < kRounds; ++r) {
        const unsigned ma = __ballot_sync(kFull, (am >> r) & 1u), mq = __ballot_sync(kFull, (qm >> r) & 1u);
        const int sid = first + r * kDetectThreads + tid;
        if ((am >> r) & 1u) out[cnt_a[r * kWarps + warp] + __popc(ma & below)] = sid;
        if ((qm >> r) & 1u) out[kTile - 1 - (cnt_q[r * kWarps + warp] + __popc(mq & below))] = sid;
    }
}

// One tile with queued points, by one warp: the reference's FP64 distance for the
// queued points, appended (ascending) after the tile's FP32-classified actives.
__device__ void recheck_tile(const InstanceDesc* __restrict__ inst, const int* __restrict__ tile_inst,
                             const BatchInputs& in, const GridDesc* __restrict__ grids,
                             const PointsDesc* __restrict__ points, int* __restrict__ ids,
                             int* __restrict__ tile_count, const int* __restrict__ tile_queue,
                             unsigned long long* __restrict__ recheck, int* __restrict__ inst_total, int t, int* qs) {
    const int q = tile_queue[t];
    const int lane = threadIdx.x;
    const int i = tile_inst[t];
    const InstanceDesc I = inst[i];
    const GridDesc g = grids[I.grid];
    const PointsDesc P = points[I.points];
    const Pose A = load_pose(in.EA + 16 * (size_t)i), B = load_pose(in.EB + 16 * (size_t)i);
    int* out = ids + (size_t)t * kTile;
    // queued stored indices sit at descending positions from the end: read them
    // back in ascending order before any write can reach those slots
    __syncwarp();
    for (int k = lane; k < q; k += 32) qs[k] = out[kTile - 1 - k];
    __syncwarp();
    const int base0 = tile_count[t];
    int base = base0;
    for (int r0 = 0; r0 < q; r0 += 32) {
        const int k = r0 + lane;
        bool active = false;
        int sid = 0;
        if (k < q) {
            sid = qs[k];
            active = exact_distance(g, A, B, load_point(P, sid)) < 0.0;
        }
        const unsigned m = __ballot_sync(kFull, active);
        if (active) out[base + __popc(m & ((1u << lane) - 1u))] = sid;
        base += __popc(m);
    }
    if (lane == 0) {
        tile_count[t] = base;
        if (base > base0) atomicAdd(inst_total + i, base - base0);
        if (recheck) atomicAdd(recheck, (unsigned long long)q);
    }
}

// The warps walk the list of tiles with queued points (appended by detect_kernel in any
// order: each tile's recheck touches only that tile).
__global__ void __launch_bounds__(32) recheck_kernel(const InstanceDesc* __restrict__ inst,
                                                     const int* __restrict__ tile_inst, BatchInputs in,
                                                     const GridDesc* __restrict__ grids,
                                                     const PointsDesc* __restrict__ points, int* __restrict__ ids,
                                                     int* __restrict__ tile_count, const int* __restrict__ tile_queue,
                                                     unsigned long long* __restrict__ recheck,
                                                     const int* __restrict__ recheck_list,
                                                     const int* __restrict__ recheck_n,
                                                     int* __restrict__ inst_total) {
    __shared__ int qs[kTile];
    const int nl = *recheck_n;
    for (int w = blockIdx.x; w < nl; w += gridDim.x)
        recheck_tile(inst, tile_inst, in, grids, points, ids, tile_count, tile_queue, recheck, inst_total,
                     recheck_list[w], qs);
}

// ------------------------------------------------------------------ distances
// Order-preserving key of a double for an unsigned atomic minimum (NaN aside).
__device__ __forceinline__ unsigned long long dist_key(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dist_unkey(unsigned long long k) {
    return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

__global__ void distance_init_kernel(unsigned long long* __restrict__ key, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) key[i] = dist_key(CUDART_INF);
}

// A body-frame mesh vertex in world as Simulation::get_body_vertices computes it
// (rm/Simulation.cpp:252-264, (R2 * v + p2).eval() with a Matrix3 R2): in the reference's
// x86-64 build Eigen sums rows 0 and 1 as one SSE2 packet, (r0 v0 + r1 v1) + r2 v2, and row 2
// by its unrolled scalar reduction, r0 v0 + (r1 v1 + r2 v2).
__device__ __forceinline__ V3 vertex_world(const M3& R, V3 p, V3 v) {
    const double x = add_rn(add_rn(mul_rn(R.m[0], v.x), mul_rn(R.m[1], v.y)), mul_rn(R.m[2], v.z));
    const double y = add_rn(add_rn(mul_rn(R.m[3], v.x), mul_rn(R.m[4], v.y)), mul_rn(R.m[5], v.z));
    const double z = add_rn(mul_rn(R.m[6], v.x), add_rn(mul_rn(R.m[7], v.y), mul_rn(R.m[8], v.z)));
    return v3(add_rn(x, p.x), add_rn(y, p.y), add_rn(z, p.z));
}

// One CTA per detection tile: every vertex's FP64 distance as Simulation::get_body_distance
// computes it (rm/Simulation.cpp:276-296: get_body_vertices, then BodySDFObj::distance), the
// tile's minimum (exact: a selection) folded into the instance's by an atomic minimum.
__global__ void __launch_bounds__(kDetectThreads) distance_kernel(const InstanceDesc* __restrict__ inst,
                                                                  const int* __restrict__ tile_inst, BatchInputs in,
                                                                  const GridDesc* __restrict__ grids,
                                                                  const PointsDesc* __restrict__ points,
                                                                  const long long* __restrict__ point_offset,
                                                                  unsigned long long* __restrict__ key,
                                                                  double* __restrict__ d) {
    const int t = blockIdx.x;
    const int i = tile_inst[t];
    const InstanceDesc I = inst[i];
    const GridDesc& g = grids[I.grid];
    const PointsDesc& P = points[I.points];
    const Pose A = load_pose(in.EA + 16 * (size_t)i), B = load_pose(in.EB + 16 * (size_t)i);
    const int base = (t - I.tile0) * kTile;
    const int n = P.n;
    double m = CUDART_INF;
    for (int k = threadIdx.x; k < kTile; k += kDetectThreads) {
        const int sid = base + k;
        if (sid >= n) break;
        const double v = query_sdf(g, grid_point(B.R, B.p, vertex_world(A.R, A.p, load_point(P, sid))), false) +
                         g.col_th;
        if (d) d[point_offset[i] + __ldg(P.orig + sid)] = v;
        m = fmin(m, v);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmin(m, __shfl_xor_sync(kFull, m, o));
    if ((threadIdx.x & 31) == 0) atomicMin(key + i, dist_key(m));
}

// SDFMesh::query_SDF at caller points already in the grid frame (n x 3, AoS), no col_th.
__global__ void grid_query_kernel(const GridDesc* __restrict__ grids, int grid, const double* __restrict__ X, int n,
                                  double* __restrict__ d, unsigned long long* __restrict__ key) {
    const GridDesc& g = grids[grid];
    double m = CUDART_INF;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const double v = query_sdf(g, v3(X[3 * (size_t)q], X[3 * (size_t)q + 1], X[3 * (size_t)q + 2]), false);
        if (d) d[q] = v;
        m = fmin(m, v);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) m = fmin(m, __shfl_xor_sync(kFull, m, o));
    if (key && (threadIdx.x & 31) == 0) atomicMin(key, dist_key(m));
}

__global__ void distance_finalize_kernel(const unsigned long long* __restrict__ key, double* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = dist_unkey(key[i]);
}

// ------------------------------------------------------------------ forces
// Per-warp accumulator of one output value.  FP64 for the FP64 path; for the
// FP32 path an FP32 pair (hi, lo) updated by Knuth's TwoSum, which keeps the
// rounding error of every addition, so the running sum carries about twice
// FP32's precision without touching GB300's slow FP64 pipe.
template <typename T>
struct Accum;
template <>
struct Accum<double> {
    double v;
    __device__ __forceinline__ void zero() { v = 0.0; }
    __device__ __forceinline__ void add(double x) { v += x; }
    __device__ __forceinline__ double value() const { return v; }
};
template <>
struct Accum<float> {
    float hi, lo;
    __device__ __forceinline__ void zero() { hi = lo = 0.f; }
    __device__ __forceinline__ void add(float x) {
        const float s = hi + x;
        const float bb = s - hi;
        const float err = (hi - (s - bb)) + (x - bb);
        hi = s;
        lo += err;
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
    // this + o as an FP32 pair (TwoSum of the leading parts, trailing parts added)
    __device__ __forceinline__ void merge(const Accum<float>& o) {
        const float lo0 = lo + o.lo;
        lo = lo0;
        add(o.hi);
    }
};

// Sum over the 32 lanes of 12 values per lane by recursive halving: at each
// of the first four levels a lane keeps half of its remaining values and
// trades the other half with its partner (8 + 4 + 2 + 1 shuffles), the fifth
// level adds the two lane halves.  Lane L ends with the warp total of value
// (L >> 1) & 15 (values 12-15 are zero padding), so 12 even lanes then add
// their totals to 12 different accumulators at once.
template <typename T>
__device__ __forceinline__ T warp_reduce12(const T (&v)[12], int lane) {
    T a[8];
    const bool h16 = lane & 16;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const T lo = v[k], hi = k + 8 < 12 ? v[k + 8] : T(0);
        const T send = h16 ? lo : hi;
        a[k] = (h16 ? hi : lo) + __shfl_xor_sync(kFull, send, 16);
    }
    const bool h8 = lane & 8;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const T send = h8 ? a[k] : a[k + 4];
        a[k] = (h8 ? a[k + 4] : a[k]) + __shfl_xor_sync(kFull, send, 8);
    }
    const bool h4 = lane & 4;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const T send = h4 ? a[k] : a[k + 2];
        a[k] = (h4 ? a[k + 2] : a[k]) + __shfl_xor_sync(kFull, send, 4);
    }
    const bool h2 = lane & 2;
    {
        const T send = h2 ? a[0] : a[1];
        a[0] = (h2 ? a[1] : a[0]) + __shfl_xor_sync(kFull, send, 2);
    }
    return a[0] + __shfl_xor_sync(kFull, a[0], 1);
}

// Warp-level sink: sums each group of 12 produced values over the warp's 32
// contacts and adds the warp totals to the warp's shared-memory accumulators.
template <int NV, typename T>
struct WarpSink {
    Accum<T>* acc;  // this warp's NV accumulators
    int lane;
    bool valid;
    Vec3<T> xi1, xi2;

    // values v[r] go to accumulator base + stride * r
    __device__ __forceinline__ void add12(T (&v)[12], int base, int stride) {
        if (!valid)
#pragma unroll
            for (int r = 0; r < 12; ++r) v[r] = T(0);
        const T sum = warp_reduce12(v, lane);
        const int slot = (lane >> 1) & 15;
        if (!(lane & 1) && slot < 12) acc[base + stride * slot].add(sum);
    }
    // fm = [xi1 x f1; f1; xi2 x f2; f2]  (Gamma^T f, simulation/redmax/Utils.h:196)
    __device__ __forceinline__ void force(Vec3<T> a1, Vec3<T> f1, Vec3<T> a2, Vec3<T> f2) {
        xi1 = a1;
        xi2 = a2;
        const Vec3<T> t1 = cross(a1, f1), t2 = cross(a2, f2);
        T v[12] = {t1.x, t1.y, t1.z, f1.x, f1.y, f1.z, t2.x, t2.y, t2.z, f2.x, f2.y, f2.z};
        add12(v, 0, 1);
    }
    // column c of [Km | Dm]: rows [xi1 x N1; N1; xi2 x N2 + T2; N2].  The accumulators of Km and
    // Dm are column-major (acc_index), so a column's 12 rows are 12 adjacent accumulators (no
    // shared-memory bank conflicts); the kernel's epilogue writes the partial row in row-major order.
    __device__ __forceinline__ void column(int c, Vec3<T> N1, Vec3<T> N2, Vec3<T> T2) {
        if constexpr (NV == kOutDeriv) {
            const Vec3<T> r0 = cross(xi1, N1), r2 = cross(xi2, N2) + T2;
            T v[12] = {r0.x, r0.y, r0.z, N1.x, N1.y, N1.z, r2.x, r2.y, r2.z, N2.x, N2.y, N2.z};
            add12(v, c < 12 ? 12 + 12 * c : 156 + 12 * (c - 12), 1);
        }
    }
};

// Accumulator of output k (fm, then Km and Dm row-major) in WarpSink's layout (Km, Dm column-major).
__device__ __forceinline__ int acc_index(int k) {
    if (k < 12) return k;
    const int b = k < 156 ? 12 : 156, e = k - b;
    return b + 12 * (e % 12) + e / 12;
}

// CTAs of the FP32 path resident per SM (kForceCtasPerSm; kForceCtasPerSmGeneral for the
// instantiation that serves every storage, BR = true); the FP64 path is left its full register
// budget.
template <typename T, bool BR = false>
constexpr int force_min_blocks() {
    return std::is_same<T, float>::value ? (BR ? kForceCtasPerSmGeneral : kForceCtasPerSm) : 1;
}

// Shares of an instance with `total` active contacts in chunks of `chunk` contacts, at least
// `per` chunks a share, at most `cap` shares (none without contacts).  The force kernels, the
// plan and finalize_kernel each compute it from detection's count, so they agree.
__host__ __device__ __forceinline__ int spread_of(int total, int chunk, int per, int cap) {
    const int chunks = (total + chunk - 1) / chunk;
    const int sh = (chunks + per - 1) / per;
    return sh < cap ? sh : cap;
}

// One thread per instance: its items (instance x kMaxSlots + share, one per share), appended to
// the list of the force launch that evaluates it (list l of n x cap entries at items + l n cap;
// lengths in counters[5 + l]), one atomic per (warp, list).  Which instances land where in a list
// depends on the atomics' order; no sum does.
__global__ void plan_kernel(const InstanceDesc* __restrict__ inst, int n, const int* __restrict__ mode, int deriv,
                            const GridDesc* __restrict__ grids, int split, int chunk, int per, int cap,
                            const int* __restrict__ inst_total, int* __restrict__ items,
                            int* __restrict__ counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, lane = threadIdx.x & 31;
    int S = 0, L = 0;
    if (i < n) {
        const int m = mode ? mode[i] : (deriv ? 2 : 1);
        if (m != 0) {
            S = spread_of(inst_total[i], chunk, per, cap);
            L = (m == 2 ? 0 : 2) + (split && grids[inst[i].grid].cells32 == nullptr ? 1 : 0);
        }
    }
    for (int l = 0; l < 4; ++l) {
        const int v = L == l ? S : 0;
        int incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += u;
        }
        const int tot = __shfl_sync(kFull, incl, 31);
        if (tot == 0) continue;  // uniform over the warp
        int base = 0;
        if (lane == 31) base = atomicAdd(counters + 5 + l, tot);
        base = __shfl_sync(kFull, base, 31);
        int* out = items + (size_t)l * n * cap + base + (incl - v);
        for (int k = 0; k < v; ++k) out[k] = i * kMaxSlots + k;
    }
}

// Shared state of a force CTA of kChunk threads: the warps' accumulators, the prefix of the
// instance's tile counts and its grid, point-set and pair descriptors.
template <bool DERIV, typename T>
struct ForceSmem {
    static constexpr int NV = DERIV ? kOutDeriv : kOutValue;
    static constexpr int NW = kChunk / 32;
    Accum<T> acc[NW * NV];
    int prefix[kMaxTilesPerInstance + 1];
    GridDesc g;
    PointsDesc P;
    PairState<T> S;
};

// An item's set-up: warp 0 the inclusive prefix of the instance's tile counts (32 tiles at a
// time), warp 1 the descriptors.  The caller's barrier follows.
template <bool DERIV, typename T>
__device__ __forceinline__ void force_item_setup(ForceSmem<DERIV, T>& sm, const InstanceDesc& I, int i,
                                                 const GridDesc* __restrict__ grids,
                                                 const PointsDesc* __restrict__ points,
                                                 const int* __restrict__ tile_count,
                                                 const PairState<T>* __restrict__ pairs, int warp, int lane) {
    if (warp == 0) {
        int run = 0;
        if (lane == 0) sm.prefix[0] = 0;
        for (int k0 = 0; k0 < I.ntiles; k0 += 32) {
            const int k = k0 + lane;
            int v = k < I.ntiles ? tile_count[I.tile0 + k] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(kFull, v, o);
                if (lane >= o) v += u;
            }
            if (k < I.ntiles) sm.prefix[k + 1] = run + v;
            run += __shfl_sync(kFull, v, 31);
        }
    } else if (warp == 1) {
        warp_copy(sm.g, grids[I.grid], lane);
        warp_copy(sm.P, points[I.points], lane);
        warp_copy(sm.S, pairs[i], lane);
    }
}

// An item's contacts: chunks s, s + shares, ... of kChunk contacts, one per thread, each warp's
// sums into its accumulators.
template <bool DERIV, bool STENCIL, typename T, bool BR>
__device__ __forceinline__ void force_item_chunks(ForceSmem<DERIV, T>& sm, const InstanceDesc& I, int s, int shares,
                                                  const int* __restrict__ ids, int tid, int lane, int warp) {
    constexpr int NV = ForceSmem<DERIV, T>::NV;
    // FP32 algebra: contacts whose derivative stencil leaves the cell take the
    // exact path with the warp's help (warp_exact_jets)
    constexpr bool kWarpExact = std::is_same<T, float>::value && !STENCIL;
    const int total = sm.prefix[I.ntiles];
    const int nchunks = (total + kChunk - 1) / kChunk;
    for (int chunk = s; chunk < nchunks; chunk += shares) {
        if (chunk * kChunk + warp * 32 >= total) continue;  // a warp with no contact in this chunk
        const int c = chunk * kChunk + tid;
        const bool valid = c < total;
        V3 xi = v3(0, 0, 0);
        Vec3<float> xf = vec3<float>(0.f, 0.f, 0.f);
        int sid = 0;
        if (valid) {
            int lo = 0, hi = I.ntiles;  // largest k with prefix[k] <= c
            while (hi - lo > 1) {
                int mid = (lo + hi) >> 1;
                if (sm.prefix[mid] <= c)
                    lo = mid;
                else
                    hi = mid;
            }
            sid = ids[(size_t)(I.tile0 + lo) * kTile + (c - sm.prefix[lo])];
            xi = load_point(sm.P, sid);
            if constexpr (kWarpExact) xf = load_point32(sm.P, sid);
        }
        FastCell fc;
        const FastCell* fcp = nullptr;
        ExactJet<T> ej;
        const ExactJet<T>* ejp = nullptr;
        if constexpr (kWarpExact) {
            fc = fast_cell<T>(sm.g, sm.S.cm, xi, xf);
            fcp = &fc;
            warp_exact_jets<T>(sm.g, sm.S, xi, valid && !fc.ok && !fc.near, DERIV, ej);
            ejp = &ej;
        }
        WarpSink<NV, T> sink{sm.acc + warp * NV, lane, valid, vec3<T>(0, 0, 0), vec3<T>(0, 0, 0)};
        if constexpr (DERIV) {
            contact_force_jacobian<T, WarpSink<NV, T>, BR>(sm.g, xi, sm.S, fcp, sink, valid, STENCIL, ejp,
                                                           kWarpExact);
        } else {
            ContactForce<T> F = contact_force<T, BR>(sm.g, xi, sm.S, fcp, valid, STENCIL, ejp);
            sink.force(F.xi1, F.f1, F.xi2, F.f2);
        }
    }
}

// An item's partial row (one row stride for both passes) from the warps' accumulators, merged in
// a fixed order.  CLEAR: each accumulator is read by one thread, which clears it for the next
// item.
template <bool DERIV, typename T, bool CLEAR>
__device__ __forceinline__ void force_item_row(ForceSmem<DERIV, T>& sm, double* __restrict__ row, int tid) {
    constexpr int NV = ForceSmem<DERIV, T>::NV, NW = ForceSmem<DERIV, T>::NW;
    for (int k = tid; k < NV; k += kChunk) {
        const int a = acc_index(k);
        double v;
        if constexpr (std::is_same<T, float>::value) {
            // the warps' pairs merged in FP32 (one conversion per value on the FP64 pipe)
            Accum<float> m = sm.acc[a];
            if (CLEAR) sm.acc[a].zero();
            for (int w = 1; w < NW; ++w) {
                m.merge(sm.acc[w * NV + a]);
                if (CLEAR) sm.acc[w * NV + a].zero();
            }
            v = m.value();
        } else {
            v = 0.0;
            for (int w = 0; w < NW; ++w) {
                v += sm.acc[w * NV + a].value();
                if (CLEAR) sm.acc[w * NV + a].zero();
            }
        }
        row[k] = v;
    }
}

// The grid form (kForceGrid): CTA (s, i) = (blockIdx.x, blockIdx.y) sums share s of instance i
// (chunks s, s + S, ..., S its spread) into the share's partial row; CTAs past the spread return
// at once.  BR = false: the FP32 fast path specialised for grids with the FP32 cell-corner array
// (storages 0 and 1); BR = true serves every storage.  skip: 0 none, 1 instances on grids
// without the cell-corner array, 2 instances on grids with it (when a batch has both kinds,
// the two instantiations split its instances).
template <bool DERIV, bool STENCIL, typename T, bool BR = true>
__global__ void __launch_bounds__(kChunk, force_min_blocks<T, BR>()) force_kernel(
    const InstanceDesc* __restrict__ inst, const int* __restrict__ mode, const GridDesc* __restrict__ grids,
    const PointsDesc* __restrict__ points, const int* __restrict__ ids, const int* __restrict__ tile_count,
    const int* __restrict__ inst_total, const PairState<T>* __restrict__ pairs, double* __restrict__ partial, int skip,
    int slots, int per) {
    constexpr int NV = ForceSmem<DERIV, T>::NV, NW = ForceSmem<DERIV, T>::NW;
    __shared__ ForceSmem<DERIV, T> sm;
    const int i = blockIdx.y, s = blockIdx.x;
    if (mode && mode[i] != (DERIV ? 2 : 1)) return;  // not requested in this pass
    const int shares = spread_of(inst_total[i], kChunk, per, slots);
    if (s >= shares) return;  // uniform over the CTA
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const InstanceDesc I = inst[i];
    if (skip && (grids[I.grid].cells32 == nullptr) == (skip == 1)) return;  // the other instantiation's instance
    force_item_setup<DERIV, T>(sm, I, i, grids, points, tile_count, pairs, warp, lane);
    for (int k = tid; k < NW * NV; k += kChunk) sm.acc[k].zero();
    __syncthreads();
    force_item_chunks<DERIV, STENCIL, T, BR>(sm, I, s, shares, ids, tid, lane, warp);
    __syncthreads();
    force_item_row<DERIV, T, false>(sm, partial + ((size_t)i * slots + s) * kOutDeriv, tid);
}

// The queue form (kForceCtas): persistent CTAs, each taking the next item of its launch's list
// (queue: the launch's counter, list_n: the list's length) until the list is exhausted.  The
// next item is fetched while the current one runs (two item slots), and the row epilogue clears
// the accumulators, so an item costs two CTA barriers.
template <bool DERIV, bool STENCIL, typename T, bool BR = true>
__global__ void __launch_bounds__(kChunk, force_min_blocks<T, BR>()) force_queue_kernel(
    const InstanceDesc* __restrict__ inst, const GridDesc* __restrict__ grids, const PointsDesc* __restrict__ points,
    const int* __restrict__ ids, const int* __restrict__ tile_count, const int* __restrict__ inst_total,
    const PairState<T>* __restrict__ pairs, double* __restrict__ partial, int slots, int per,
    const int* __restrict__ items, const int* __restrict__ list_n, int* __restrict__ queue) {
    constexpr int NV = ForceSmem<DERIV, T>::NV, NW = ForceSmem<DERIV, T>::NW;
    static_assert(kChunk >= 64 && kChunk % 32 == 0, "warps 0 and 1 set an item up");
    constexpr int kFetcher = kChunk > 64 ? 64 : 0;  // the thread that fetches items (warp 2's first)
    __shared__ ForceSmem<DERIV, T> sm;
    __shared__ int item[2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int n_items = *list_n;
    auto fetch = [&]() {
        const int q = atomicAdd(queue, 1);
        return q < n_items ? items[q] : -1;
    };
    if (tid == 0) item[0] = fetch();
    for (int k = tid; k < NW * NV; k += kChunk) sm.acc[k].zero();
    __syncthreads();
    for (int it = 0;; it ^= 1) {
        // item[it] was written before the previous item's second barrier (or the one above)
        const int e = item[it];
        if (e < 0) break;  // uniform over the CTA
        const int i = e / kMaxSlots, s = e % kMaxSlots;
        const int shares = spread_of(inst_total[i], kChunk, per, slots);
        const InstanceDesc I = inst[i];
        // the next item, fetched now and stored before this item's second barrier (item[it ^ 1]
        // was last read before the previous item's first barrier)
        int pending = -1;
        if (tid == kFetcher) pending = fetch();
        // the prefix and the descriptors were last read before the previous item's second barrier
        force_item_setup<DERIV, T>(sm, I, i, grids, points, tile_count, pairs, warp, lane);
        __syncthreads();
        force_item_chunks<DERIV, STENCIL, T, BR>(sm, I, s, shares, ids, tid, lane, warp);
        if (tid == kFetcher) item[it ^ 1] = pending;
        __syncthreads();
        force_item_row<DERIV, T, true>(sm, partial + ((size_t)i * slots + s) * kOutDeriv, tid);
    }
}

// Resident one-warp force workers per SM: the FP32 path within 65536 / (32 x this) registers
// (a compile-time tuning knob, 16: 128 registers), the FP64 path within 255.
#ifndef SDFC_WORKER_MIN_BLOCKS
#define SDFC_WORKER_MIN_BLOCKS 16
#endif
template <typename T>
constexpr int worker_min_blocks() {
    return std::is_same<T, float>::value ? SDFC_WORKER_MIN_BLOCKS : 8;
}

// Force pass by persistent one-warp workers (kForceWorkers), over the same item lists as
// force_queue_kernel: item (i, s) takes instance i's 32-contact chunks s, s + S, ... in order and
// writes its own partial row, so the sums do not depend on which worker took the item.
// Dynamic shared memory: the prefix of the instance's tile counts, max_ntiles + 1 ints.
template <bool DERIV, bool STENCIL, typename T, bool BR = true>
__global__ void __launch_bounds__(32, worker_min_blocks<T>()) force_worker_kernel(
    const InstanceDesc* __restrict__ inst, const GridDesc* __restrict__ grids,
    const PointsDesc* __restrict__ points, const int* __restrict__ ids, const int* __restrict__ tile_count,
    const int* __restrict__ inst_total, const PairState<T>* __restrict__ pairs, double* __restrict__ partial,
    int slots, int per, const int* __restrict__ items, const int* __restrict__ list_n, int* __restrict__ queue) {
    constexpr int NV = DERIV ? kOutDeriv : kOutValue;
    constexpr bool kWarpExact = std::is_same<T, float>::value && !STENCIL;
    __shared__ Accum<T> acc[NV];
    __shared__ GridDesc g;
    __shared__ PointsDesc P;
    __shared__ PairState<T> S;
    extern __shared__ int prefix[];
    const int lane = threadIdx.x;
    const int n_items = *list_n;
    // lane 0 fetches the next item while the warp runs the current one; the warp reads it at
    // the top of the next round
    auto fetch = [&]() {
        int e = -1;
        if (lane == 0) {
            const int q = atomicAdd(queue, 1);
            if (q < n_items) e = items[q];
        }
        return e;
    };
    int pending = fetch();
    for (;;) {
        const int e = __shfl_sync(kFull, pending, 0);
        if (e < 0) break;
        pending = fetch();
        const int i = e / kMaxSlots, s = e % kMaxSlots;
        const int shares = spread_of(inst_total[i], 32, per, slots);
        const InstanceDesc I = inst[i];
        __syncwarp();  // the previous item's reads of the shared state are done
        {
            int run = 0;
            if (lane == 0) prefix[0] = 0;
            for (int k0 = 0; k0 < I.ntiles; k0 += 32) {
                const int k = k0 + lane;
                int v = k < I.ntiles ? tile_count[I.tile0 + k] : 0;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int u = __shfl_up_sync(kFull, v, o);
                    if (lane >= o) v += u;
                }
                if (k < I.ntiles) prefix[k + 1] = run + v;
                run += __shfl_sync(kFull, v, 31);
            }
        }
        warp_copy(g, grids[I.grid], lane);
        warp_copy(P, points[I.points], lane);
        warp_copy(S, pairs[i], lane);
        for (int k = lane; k < NV; k += 32) acc[k].zero();
        __syncwarp();
        const int total = prefix[I.ntiles];
        const int nchunks = (total + 31) >> 5;
        for (int chunk = s; chunk < nchunks; chunk += shares) {
            const int c = chunk * 32 + lane;
            const bool valid = c < total;
            V3 xi = v3(0, 0, 0);
            Vec3<float> xf = vec3<float>(0.f, 0.f, 0.f);
            if (valid) {
                int lo = 0, hi = I.ntiles;  // largest k with prefix[k] <= c
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (prefix[mid] <= c)
                        lo = mid;
                    else
                        hi = mid;
                }
                const int sid = ids[(size_t)(I.tile0 + lo) * kTile + (c - prefix[lo])];
                xi = load_point(P, sid);
                if constexpr (kWarpExact) xf = load_point32(P, sid);
            }
            FastCell fc;
            const FastCell* fcp = nullptr;
            ExactJet<T> ej;
            const ExactJet<T>* ejp = nullptr;
            if constexpr (kWarpExact) {
                fc = fast_cell<T>(g, S.cm, xi, xf);
                fcp = &fc;
                warp_exact_jets<T>(g, S, xi, valid && !fc.ok && !fc.near, DERIV, ej);
                ejp = &ej;
            }
            WarpSink<NV, T> sink{acc, lane, valid, vec3<T>(0, 0, 0), vec3<T>(0, 0, 0)};
            if constexpr (DERIV) {
                contact_force_jacobian<T, WarpSink<NV, T>, BR>(g, xi, S, fcp, sink, valid, STENCIL, ejp, kWarpExact);
            } else {
                ContactForce<T> F = contact_force<T, BR>(g, xi, S, fcp, valid, STENCIL, ejp);
                sink.force(F.xi1, F.f1, F.xi2, F.f2);
            }
        }
        __syncwarp();
        double* row = partial + ((size_t)i * slots + s) * kOutDeriv;
        for (int k = lane; k < NV; k += 32) row[k] = acc[acc_index(k)].value();
    }
}

// Penetration energy of every instance (sum over its active contacts of kn d^2 / 2) and its
// gradient wrt both bodies' twist coordinates; one CTA per (instance, share) for every share up
// to the cap (the CTAs past the instance's spread, from spread_of with chunks of kChunk, return
// at once), partial row = [e, dE/dq_A (w, v), dE/dq_B (w, v)] (kOutEnergy values).
template <bool STENCIL, typename T>
__global__ void __launch_bounds__(kChunk, force_min_blocks<T>()) energy_kernel(const InstanceDesc* __restrict__ inst,
                                                        BatchInputs in, const GridDesc* __restrict__ grids,
                                                        const PointsDesc* __restrict__ points,
                                                        const int* __restrict__ ids,
                                                        const int* __restrict__ tile_count,
                                                        const PairState<T>* __restrict__ pairs,
                                                        double* __restrict__ partial, int slots, int per,
                                                        const int* __restrict__ inst_total) {
    constexpr int NW = kChunk / 32;
    constexpr bool kWarpExact = std::is_same<T, float>::value && !STENCIL;
    __shared__ Accum<T> acc[NW * 12];
    __shared__ double eacc[NW];
    __shared__ int prefix[kMaxTilesPerInstance + 1];
    __shared__ GridDesc g;
    __shared__ PointsDesc P;
    __shared__ PairState<T> S;
    const int i = blockIdx.y;
    if (in.mode && in.mode[i] == 0) return;
    const int shares = spread_of(inst_total[i], kChunk, per, slots);
    if ((int)blockIdx.x >= shares) return;  // uniform over the CTA
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const InstanceDesc I = inst[i];
    if (warp == 0) {
        int run = 0;
        if (lane == 0) prefix[0] = 0;
        for (int k0 = 0; k0 < I.ntiles; k0 += 32) {
            const int k = k0 + lane;
            int v = k < I.ntiles ? tile_count[I.tile0 + k] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(kFull, v, o);
                if (lane >= o) v += u;
            }
            if (k < I.ntiles) prefix[k + 1] = run + v;
            run += __shfl_sync(kFull, v, 31);
        }
    } else if (warp == 1) {
        warp_copy(g, grids[I.grid], lane);
        warp_copy(P, points[I.points], lane);
        warp_copy(S, pairs[i], lane);
    }
    __syncthreads();  // the set-up above
    const int total = prefix[I.ntiles];
    const int nchunks = (total + kChunk - 1) / kChunk;
    // the CTA's shares in turn (the grid holds at most a few CTAs per instance): share s sums
    // chunks s, s + S, ... from zeroed accumulators into its own partial row
    for (int s = blockIdx.x; s < shares; s += gridDim.x) {
        for (int k = tid; k < NW * 12; k += kChunk) acc[k].zero();
        if (tid < NW) eacc[tid] = 0.0;
        __syncthreads();
        for (int chunk = s; chunk < nchunks; chunk += shares) {
            if (chunk * kChunk + warp * 32 >= total) continue;  // a warp with no contact in this chunk
            const int c = chunk * kChunk + tid;
            const bool valid = c < total;
            V3 xi = v3(0, 0, 0);
            Vec3<float> xf = vec3<float>(0.f, 0.f, 0.f);
            if (valid) {
                int lo = 0, hi = I.ntiles;
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (prefix[mid] <= c)
                        lo = mid;
                    else
                        hi = mid;
                }
                const int sid = ids[(size_t)(I.tile0 + lo) * kTile + (c - prefix[lo])];
                xi = load_point(P, sid);
                if constexpr (kWarpExact) xf = load_point32(P, sid);
            }
            FastCell fc;
            const FastCell* fcp = nullptr;
            ExactJet<T> ej;
            const ExactJet<T>* ejp = nullptr;
            if constexpr (kWarpExact) {
                fc = fast_cell<T>(g, S.cm, xi, xf);
                fcp = &fc;
                warp_exact_jets<T>(g, S, xi, valid && !fc.ok && !fc.near, false, ej);
                ejp = &ej;
            }
            const ContactEnergy<T> E = contact_energy<T>(g, xi, S, fcp, valid, STENCIL, ejp);
            WarpSink<12, T> sink{acc + warp * 12, lane, valid, vec3<T>(0, 0, 0), vec3<T>(0, 0, 0)};
            T v[12] = {E.aw.x, E.aw.y, E.aw.z, E.av.x, E.av.y, E.av.z, E.bw.x, E.bw.y, E.bw.z, E.bv.x, E.bv.y, E.bv.z};
            sink.add12(v, 0, 1);
            double e = E.e;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(kFull, e, o);
            if (lane == 0) eacc[warp] += e;
        }
        __syncthreads();
        double* row = partial + ((size_t)i * slots + s) * kOutDeriv;
        for (int k = tid; k < kOutEnergy; k += kChunk) {
            double v = 0.0;
            if (k == 0)
                for (int w = 0; w < NW; ++w) v += eacc[w];
            else
                for (int w = 0; w < NW; ++w) v += acc[w * 12 + k - 1].value();
            row[k] = v;
        }
        __syncthreads();  // the row is read before the next share zeroes the accumulators
    }
}

__global__ void energy_finalize_kernel(int n_inst, const double* __restrict__ partial, double* __restrict__ energy,
                                       double* __restrict__ dE, const int* __restrict__ mode, int slots, int per,
                                       const int* __restrict__ inst_total) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (size_t)n_inst * kOutEnergy) return;
    const int i = (int)(idx / kOutEnergy), k = (int)(idx % kOutEnergy);
    if (mode && mode[i] == 0) return;
    const double* p = partial + (size_t)i * slots * kOutDeriv + k;
    const int shares = spread_of(inst_total[i], kChunk, per, slots);
    double v = 0.0;
    for (int s = 0; s < shares; ++s) v += p[(size_t)s * kOutDeriv];
    if (k == 0)
        energy[i] = v;
    else
        dE[12 * (size_t)i + k - 1] = v;
}

// Every contact's force in the bodies' frames is unchanged when both bodies move
// together, so for a world twist eps, Km1 Ad(E_A^{-1}) eps + Km2 Ad(E_B^{-1}) eps = 0,
// i.e. Km2 = -Km1 Ad(E_A^{-1} E_B).  Dm's friction damping sees, under a common
// rotation w, the relative velocity w x (d n) of the two contact points, so
// Dm2 = -Dm1 Ad(E_A^{-1} E_B) + [C | 0] with C accumulated by force_kernel
// (contact_force_jacobian's skip_q2).
// Entry (r, c) of Ad(E_A^{-1} E_B) (6 x 6, twists ordered (w, v)):
//   [Q, 0; [t] Q, Q] with Q = R_A^T R_B and t = R_A^T (p_B - p_A).
__device__ inline double adjoint_entry(const double* EA, const double* EB, int r, int c) {
    auto q = [&](int a, int b) {
        double v = 0.0;
        for (int k = 0; k < 3; ++k) v += EA[4 * k + a] * EB[4 * k + b];  // (R_A^T R_B)_ab
        return v;
    };
    if (r < 3) return c < 3 ? q(r, c) : 0.0;
    if (c >= 3) return q(r - 3, c - 3);
    double t[3];
    for (int a = 0; a < 3; ++a) {
        t[a] = 0.0;
        for (int k = 0; k < 3; ++k) t[a] += EA[4 * k + a] * (EB[4 * k + 3] - EA[4 * k + 3]);  // R_A^T (p_B - p_A)
    }
    const int a1 = (r - 3 + 1) % 3, a2 = (r - 3 + 2) % 3;  // (t x Q e_c) component r - 3
    return t[a1] * q(a2, c) - t[a2] * q(a1, c);
}

// One CTA per instance: the instance's partial rows (one per share: spread_of with the force
// pass's chunk, chunks per share and cap) summed in order into shared memory, then written out.  EA / EB not null: the dq2 columns of Km and the dphi2 columns
// of Dm were not accumulated (force_kernel's skip_q2) and are derived here from the summed
// dq1 / dphi1 columns; the partial rows' dq2 slots of Km then hold C (Dm's correction).
template <bool DERIV>
__global__ void finalize_kernel(int n_inst, const int* __restrict__ inst_total, int chunk, int per,
                                const double* __restrict__ partial, BatchOutputs out, const int* __restrict__ mode,
                                const double* __restrict__ EA, const double* __restrict__ EB, int slots,
                                bool set_status, const int* __restrict__ badin) {
    constexpr int NV = DERIV ? kOutDeriv : kOutValue;
    __shared__ double tot[NV];
    __shared__ double ad[36];  // Ad(E_A^{-1} E_B), ad[6 c + r] = entry (r, c)
    const int i = blockIdx.x, k = threadIdx.x;
    if (i >= n_inst || (mode && mode[i] != (DERIV ? 2 : 1))) return;  // uniform over the CTA
    if (out.dev) out = *out.dev;
    const double* p = partial + (size_t)i * slots * kOutDeriv;
    const int shares = spread_of(inst_total[i], chunk, per, slots);
    if (k < NV) {
        double v = 0.0;
        for (int s = 0; s < shares; ++s) v += p[(size_t)s * kOutDeriv + k];
        tot[k] = v;
    }
    const bool derive = DERIV && EA != nullptr;
    if (derive && k < 36) ad[k] = adjoint_entry(EA + 16 * (size_t)i, EB + 16 * (size_t)i, k % 6, k / 6);
    __syncthreads();
    double v = k < NV ? tot[k] : 0.0;
    if (derive && k >= 12 && k < NV) {
        const int b = k < 156 ? 12 : 156, r = (k - b) / 12, j = (k - b) % 12;
        if (j >= 6) {  // column j of Km / Dm = -(columns 0-5) Ad e_{j-6} (+ C)
            const double* m1 = tot + b + 12 * r;
            const double* a = ad + 6 * (j - 6);
            v = 0.0;
            for (int c = 0; c < 3; ++c) v -= m1[c] * a[c] + m1[3 + c] * a[3 + c];
            if (b == 156 && j < 9) v += tot[12 + 12 * r + j];  // C column j - 6, in Km's slot (r, j)
        }
    }
    if (k < NV) {
        if (k < 12)
            out.fm[12 * (size_t)i + k] = v;
        else if (k < 156)
            out.Km[144 * (size_t)i + (k - 12)] = v;
        else
            out.Dm[144 * (size_t)i + (k - 156)] = v;
    }
    // plain stores only (the outputs may be the caller's host memory)
    const int bad = __syncthreads_or(k < NV && !isfinite(v));
    if (k == 0) {
        // bit 0: a non-finite output; bit 1: a non-finite input (prep_kernel)
        const int st = (bad ? 1 : 0) | (badin[i] ? 2 : 0);
        if (set_status)  // every instance passes through this launch: status written outright
            out.status[i] = st;
        else if (st)
            out.status[i] = st;
        out.n_active[i] = inst_total[i];
    }
}

__global__ void zero_status_kernel(BatchOutputs out, int n) {
    if (out.dev) out = *out.dev;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out.status[i] = 0;
}

__global__ void gather_inputs_kernel(const HostIO* __restrict__ io, double* __restrict__ d, int n) {
    const size_t nn = (size_t)n, total = 50 * nn;
    const size_t end[5] = {16 * nn, 22 * nn, 38 * nn, 44 * nn, 50 * nn};
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
        int seg = 0;
        while (k >= end[seg]) ++seg;
        const size_t start = seg ? end[seg - 1] : 0;
        d[k] = io->in[seg][k - start];
    }
}

// CTAs of `kernel` (block `threads`, dynamic shared memory `smem`) resident on the current
// device at once: the persistent force passes launch this many (the per-SM count looked up once
// per kernel, times the device's SMs).
template <typename K>
int resident_ctas(K kernel, int threads, size_t smem, std::atomic<int>& per_sm_cache) {
    int per_sm = per_sm_cache.load(std::memory_order_relaxed);
    if (per_sm <= 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        per_sm_cache.store(per_sm, std::memory_order_relaxed);
    }
    return per_sm * device_sm_count();
}

// Contacts per chunk of the batch's force-pass form.
int chunk_of(const BatchScratch& s) { return s.force_variant == kForceWorkers ? 32 : kChunk; }

// One force launch: for the queue forms over list `l` (BatchScratch::recheck_n),
// force_queue_kernel on persistent CTAs (as many as the SMs hold) or force_worker_kernel on
// s.worker_ctas one-warp CTAs (0: as many as the SMs hold); for the grid form force_kernel on
// (slots, n) CTAs with `skip` (force_kernel).
template <bool DERIV, bool STENCIL, typename T, bool BR>
void launch_list(int n_inst, int l, int skip, cudaStream_t stream, const InstanceDesc* d_inst, const int* mode,
                 const GridDesc* d_grids, const PointsDesc* d_points, const BatchScratch& s,
                 const PairState<T>* pairs) {
    const int per = std::max(s.chunks_per_slot, 1);
    if (s.force_variant == kForceGrid) {
        force_kernel<DERIV, STENCIL, T, BR><<<dim3(s.slots, n_inst), kChunk, 0, stream>>>(
            d_inst, mode, d_grids, d_points, s.ids, s.tile_count, s.inst_total, pairs, s.partial, skip, s.slots, per);
        return;
    }
    int* queue = s.recheck_n + 1 + l;
    const int* list_n = s.recheck_n + 5 + l;
    const int* items = s.items + (size_t)l * n_inst * s.slots;
    const long long most = (long long)n_inst * s.slots;  // items in the list, at most
    if (s.force_variant == kForceWorkers) {
        const size_t smem = sizeof(int) * ((size_t)s.max_ntiles + 1);
        int ctas = s.worker_ctas > 0 ? s.worker_ctas : device_sm_count() * worker_min_blocks<T>();
        ctas = (int)std::min<long long>(ctas, most);
        force_worker_kernel<DERIV, STENCIL, T, BR><<<ctas, 32, smem, stream>>>(
            d_inst, d_grids, d_points, s.ids, s.tile_count, s.inst_total, pairs, s.partial, s.slots, per, items,
            list_n, queue);
    } else {
        static std::atomic<int> cache{0};
        const int ctas = (int)std::min<long long>(
            resident_ctas(force_queue_kernel<DERIV, STENCIL, T, BR>, kChunk, 0, cache), most);
        force_queue_kernel<DERIV, STENCIL, T, BR><<<ctas, kChunk, 0, stream>>>(
            d_inst, d_grids, d_points, s.ids, s.tile_count, s.inst_total, pairs, s.partial, s.slots, per, items,
            list_n, queue);
    }
}

// Whether the FP32 fast path splits a batch's instances between the cell-corner specialisation
// and the general kernel (both storages present).
bool splits(bool stencil, int precision, bool plain, bool bricks) {
    return precision == kMixed && !stencil && plain && bricks;
}

template <bool DERIV, bool STENCIL>
void launch_force_t(int n_inst, int precision, cudaStream_t stream, const InstanceDesc* d_inst, const int* mode,
                    const GridDesc* d_grids, const PointsDesc* d_points, const BatchScratch& s, bool plain,
                    bool bricks) {
    const int l = DERIV ? 0 : 2;
    if (precision == kMixed && !STENCIL) {  // the FP32 fast path: specialised for brick-free grids
        if (plain)
            launch_list<DERIV, STENCIL, float, false>(n_inst, l, bricks ? 1 : 0, stream, d_inst, mode, d_grids,
                                                      d_points, s, s.pair32);
        if (bricks)
            launch_list<DERIV, STENCIL, float, true>(n_inst, plain ? l + 1 : l, plain ? 2 : 0, stream, d_inst, mode,
                                                     d_grids, d_points, s, s.pair32);
    } else if (precision == kMixed) {
        launch_list<DERIV, STENCIL, float, true>(n_inst, l, 0, stream, d_inst, mode, d_grids, d_points, s, s.pair32);
    } else {
        launch_list<DERIV, STENCIL, double, true>(n_inst, l, 0, stream, d_inst, mode, d_grids, d_points, s, s.pair64);
    }
}

}  // namespace

int device_sm_count() {
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
    if (dev < 64 && cache[dev] > 0) return cache[dev];
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 1;
    if (dev < 64) cache[dev] = n;
    return n;
}

void launch_detect(const InstanceDesc* d_inst, const int* d_tile_inst, int n_inst, int total_tiles, BatchInputs in,
                   const GridDesc* d_grids, const PointsDesc* d_points, BatchScratch s, cudaStream_t stream,
                   bool plain, bool bricks) {
    if (n_inst <= 0) return;
    prep_kernel<<<dim3((n_inst + 31) / 32, 3), 32, 0, stream>>>(d_inst, n_inst, in, d_grids, d_points, s.prefilter,
                                                                s.pair32, s.pair64, s.recheck_n, s.badin,
                                                                s.inst_total);
    if (total_tiles <= 0) return;
    if (plain)
        detect_kernel<false><<<total_tiles, kDetectThreads, 0, stream>>>(d_inst, d_tile_inst, s.prefilter, d_grids,
                                                                         d_points, s.ids, s.tile_count, s.tile_queue,
                                                                         in.mode, s.recheck_list, s.recheck_n,
                                                                         s.inst_total);
    if (bricks)
        detect_kernel<true><<<total_tiles, kDetectThreads, 0, stream>>>(d_inst, d_tile_inst, s.prefilter, d_grids,
                                                                        d_points, s.ids, s.tile_count, s.tile_queue,
                                                                        in.mode, s.recheck_list, s.recheck_n,
                                                                        s.inst_total);
    // one warp per listed tile, up to 16 warps per SM (the list is only known on the device)
    recheck_kernel<<<std::min(total_tiles, device_sm_count() * 16), 32, 0, stream>>>(d_inst, d_tile_inst, in, d_grids, d_points,
                                                                       s.ids, s.tile_count, s.tile_queue, s.recheck,
                                                                       s.recheck_list, s.recheck_n, s.inst_total);
}

void launch_distance(const InstanceDesc* d_inst, const int* d_tile_inst, int n_inst, int total_tiles, BatchInputs in,
                     const GridDesc* d_grids, const PointsDesc* d_points, const long long* point_offset,
                     unsigned long long* key_scratch, double* min_d, double* d, cudaStream_t stream) {
    if (n_inst <= 0) return;
    distance_init_kernel<<<(n_inst + 255) / 256, 256, 0, stream>>>(key_scratch, n_inst);
    if (total_tiles > 0)
        distance_kernel<<<total_tiles, kDetectThreads, 0, stream>>>(d_inst, d_tile_inst, in, d_grids, d_points,
                                                                     point_offset, key_scratch, d);
    distance_finalize_kernel<<<(n_inst + 255) / 256, 256, 0, stream>>>(key_scratch, min_d, n_inst);
}

void launch_grid_query(const GridDesc* d_grids, int grid, const double* X, int n, double* d,
                       unsigned long long* key_scratch, double* min_d, cudaStream_t stream) {
    if (min_d) distance_init_kernel<<<1, 32, 0, stream>>>(key_scratch, 1);
    if (n > 0) {
        const int blocks = std::min((n + 255) / 256, device_sm_count() * 8);
        grid_query_kernel<<<blocks, 256, 0, stream>>>(d_grids, grid, X, n, d, min_d ? key_scratch : nullptr);
    }
    if (min_d) distance_finalize_kernel<<<1, 32, 0, stream>>>(key_scratch, min_d, 1);
}

void launch_plan(const InstanceDesc* d_inst, int n_inst, BatchInputs in, const GridDesc* d_grids, BatchScratch s,
                 bool deriv, bool stencil, int precision, cudaStream_t stream, bool plain, bool bricks) {
    if (n_inst <= 0 || s.force_variant == kForceGrid) return;  // the grid form takes no list
    plan_kernel<<<(n_inst + 255) / 256, 256, 0, stream>>>(d_inst, n_inst, in.mode, deriv ? 1 : 0, d_grids,
                                                          splits(stencil, precision, plain, bricks) ? 1 : 0,
                                                          chunk_of(s), std::max(s.chunks_per_slot, 1), s.slots,
                                                          s.inst_total, s.items, s.recheck_n);
}

void launch_force(const InstanceDesc* d_inst, int n_inst, BatchInputs in, const GridDesc* d_grids,
                  const PointsDesc* d_points, BatchScratch s, bool deriv, bool stencil, int precision,
                  cudaStream_t stream, bool plain, bool bricks) {
    if (n_inst <= 0) return;
    const int* m = in.mode;
    if (deriv) {
        if (stencil)
            launch_force_t<true, true>(n_inst, precision, stream, d_inst, m, d_grids, d_points, s, plain, bricks);
        else
            launch_force_t<true, false>(n_inst, precision, stream, d_inst, m, d_grids, d_points, s, plain, bricks);
    } else {
        if (stencil)
            launch_force_t<false, true>(n_inst, precision, stream, d_inst, m, d_grids, d_points, s, plain, bricks);
        else
            launch_force_t<false, false>(n_inst, precision, stream, d_inst, m, d_grids, d_points, s, plain, bricks);
    }
}

void launch_finalize(const InstanceDesc* d_inst, int n_inst, BatchScratch s, bool deriv, BatchOutputs out,
                     cudaStream_t stream, const int* mode, bool zero_status, const BatchInputs* derive_q2) {
    (void)d_inst;
    if (n_inst <= 0) return;
    // without a request mask every instance is finalized here, which then sets each status
    // outright; with one, the statuses are cleared first and each pass sets its instances' flags
    const bool set_status = zero_status && !mode;
    if (zero_status && mode) zero_status_kernel<<<(n_inst + 255) / 256, 256, 0, stream>>>(out, n_inst);
    const double* EA = derive_q2 ? derive_q2->EA : nullptr;
    const double* EB = derive_q2 ? derive_q2->EB : nullptr;
    const int per = std::max(s.chunks_per_slot, 1);
    if (deriv)
        finalize_kernel<true><<<n_inst, 320, 0, stream>>>(n_inst, s.inst_total, chunk_of(s), per, s.partial, out, mode,
                                                          EA, EB, s.slots, set_status, s.badin);
    else
        finalize_kernel<false><<<n_inst, 64, 0, stream>>>(n_inst, s.inst_total, chunk_of(s), per, s.partial, out,
                                                          mode, nullptr, nullptr, s.slots, set_status, s.badin);
}

void launch_zero_status(BatchOutputs out, int n_inst, cudaStream_t stream) {
    if (n_inst > 0) zero_status_kernel<<<(n_inst + 255) / 256, 256, 0, stream>>>(out, n_inst);
}

void launch_gather_inputs(const HostIO* io, double* d, int n, cudaStream_t stream) {
    if (n <= 0) return;
    const int blocks = (int)std::min<size_t>((50 * (size_t)n + 255) / 256, (size_t)device_sm_count() * 4);
    gather_inputs_kernel<<<blocks, 256, 0, stream>>>(io, d, n);
}

bool force_skips_q2(bool deriv, bool stencil, int precision) { return deriv && !stencil && precision == kMixed; }

void launch_energy(const InstanceDesc* d_inst, int n_inst, BatchInputs in, const GridDesc* d_grids,
                   const PointsDesc* d_points, BatchScratch s, bool stencil, int precision, cudaStream_t stream) {
    if (n_inst <= 0) return;
    // at most kEnergyCtas CTAs per instance, each taking its shares in turn: an energy pass
    // serves batches of many small instances (rollouts), where slots x instances CTAs would
    // mostly start only to find no share
    constexpr int kEnergyCtas = 16;
    dim3 grid(std::min(s.slots, kEnergyCtas), n_inst);
    const int per = std::max(s.chunks_per_slot, 1);
    if (precision == kMixed) {
        if (stencil)
            energy_kernel<true, float><<<grid, kChunk, 0, stream>>>(d_inst, in, d_grids, d_points, s.ids, s.tile_count,
                                                                     s.pair32, s.partial, s.slots, per, s.inst_total);
        else
            energy_kernel<false, float><<<grid, kChunk, 0, stream>>>(d_inst, in, d_grids, d_points, s.ids,
                                                                      s.tile_count, s.pair32, s.partial, s.slots, per,
                                                                      s.inst_total);
    } else {
        if (stencil)
            energy_kernel<true, double><<<grid, kChunk, 0, stream>>>(d_inst, in, d_grids, d_points, s.ids,
                                                                      s.tile_count, s.pair64, s.partial, s.slots, per,
                                                                      s.inst_total);
        else
            energy_kernel<false, double><<<grid, kChunk, 0, stream>>>(d_inst, in, d_grids, d_points, s.ids,
                                                                       s.tile_count, s.pair64, s.partial, s.slots, per,
                                                                       s.inst_total);
    }
}

void launch_energy_finalize(int n_inst, BatchScratch s, double* energy, double* dE, const int* mode,
                            cudaStream_t stream) {
    if (n_inst <= 0) return;
    const size_t total = (size_t)n_inst * kOutEnergy;
    energy_finalize_kernel<<<(unsigned)((total + 255) / 256), 256, 0, stream>>>(
        n_inst, s.partial, energy, dE, mode, s.slots, std::max(s.chunks_per_slot, 1), s.inst_total);
}

}  // namespace sdfc
