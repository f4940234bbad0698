// The planner's disassembly check on the GPU, for many poses of the moving part at once.
//
// PhysicsPlanner.is_disassembled (examples/run_joint_plan.py:291-302) tests the convex hull of
// the moving part's vertices, posed by its E_0i, against the convex hull of all still parts'
// vertices with an FCL mesh-mesh collision (trimesh 3.10.8's CollisionManager over
// python-fcl 0.6.1: the hulls' triangle surfaces intersect or touch), and when the surfaces do
// not meet, calls the part disassembled unless one hull's axis-aligned box contains the
// other's.  For two convex polytopes the surfaces meet exactly when the solids intersect and
// neither solid lies inside the other, which is what one warp per pose evaluates here:
//
//   solids intersect   GJK (Gilbert, Johnson and Keerthi, IEEE J. Robotics and Automation
//                      4(2), 1988) on the Minkowski difference, boolean form: support points
//                      by warp-wide arg-max over the hull vertices, simplex reduction by the
//                      Voronoi-region tests of the line, triangle and tetrahedron; FP64;
//   containment        every vertex of one hull inside every facet plane of the other
//                      (planes n . x + offset <= 0, as qhull reports them);
//   boxes              the posed moving hull's vertex bounds against the still hull's.
//
// FP64 throughout; the decision can differ from FCL's only for poses whose hulls touch to
// within round-off.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "sdfc.h"
#include "sdfc_internal.h"

namespace {

constexpr int kHullWarps = 4;        // poses per CTA
constexpr int kGjkMaxIter = 64;      // GJK iterations before the conservative answer
constexpr double kContainTol = 1e-12;

struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 d3(double x, double y, double z) { return {x, y, z}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D3 neg(D3 a) { return d3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 cross(D3 a, D3 b) {
    return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// (a x b) x a: the component of b orthogonal to a, scaled
__device__ __forceinline__ D3 triple(D3 a, D3 b) { return cross(cross(a, b), a); }

struct Pose3 {
    double R[9];
    D3 p;
};
__device__ __forceinline__ D3 pose_apply(const Pose3& P, D3 v) {
    return d3(P.R[0] * v.x + P.R[1] * v.y + P.R[2] * v.z + P.p.x, P.R[3] * v.x + P.R[4] * v.y + P.R[5] * v.z + P.p.y,
              P.R[6] * v.x + P.R[7] * v.y + P.R[8] * v.z + P.p.z);
}
__device__ __forceinline__ D3 rot_t(const Pose3& P, D3 d) {  // R^T d
    return d3(P.R[0] * d.x + P.R[3] * d.y + P.R[6] * d.z, P.R[1] * d.x + P.R[4] * d.y + P.R[7] * d.z,
              P.R[2] * d.x + P.R[5] * d.y + P.R[8] * d.z);
}

__device__ __forceinline__ D3 ld3(const double* v, int i) { return d3(v[3 * i], v[3 * i + 1], v[3 * i + 2]); }

// Warp-wide arg-max of v . d over a hull's vertices (lowest index on ties).
__device__ int warp_support(const double* __restrict__ v, int nv, D3 d) {
    const int lane = threadIdx.x & 31;
    double best = -INFINITY;
    int arg = 0x7fffffff;
    for (int i = lane; i < nv; i += 32) {
        const double s = dot(ld3(v, i), d);
        if (s > best) {
            best = s;
            arg = i;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        const double b2 = __shfl_xor_sync(0xffffffffu, best, o);
        const int a2 = __shfl_xor_sync(0xffffffffu, arg, o);
        if (b2 > best || (b2 == best && a2 < arg)) {
            best = b2;
            arg = a2;
        }
    }
    return arg;
}

// Support point of (moving hull posed by P) minus (still hull) in direction d.
__device__ D3 mink_support(const sdfc::HullDesc& A, const Pose3& P, const sdfc::HullDesc& B, D3 d) {
    const D3 a = pose_apply(P, ld3(A.v, warp_support(A.v, A.nv, rot_t(P, d))));
    const D3 b = ld3(B.v, warp_support(B.v, B.nv, neg(d)));
    return a - b;
}

// Simplex reduction for a triangle a (newest), b, c: keeps the feature whose Voronoi region
// holds the origin and sets the search direction toward it; true when the origin lies in the
// triangle's plane inside it (touching).
__device__ __forceinline__ bool gjk_triangle(D3* s, int& n, D3& d) {
    const D3 a = s[0], b = s[1], c = s[2];
    const D3 ao = neg(a), ab = b - a, ac = c - a, abc = cross(ab, ac);
    if (dot(cross(abc, ac), ao) > 0.0) {
        if (dot(ac, ao) > 0.0) {
            s[1] = c;
            n = 2;
            d = triple(ac, ao);
        } else if (dot(ab, ao) > 0.0) {
            n = 2;
            d = triple(ab, ao);
        } else {
            n = 1;
            d = ao;
        }
    } else if (dot(cross(ab, abc), ao) > 0.0) {
        if (dot(ab, ao) > 0.0) {
            n = 2;
            d = triple(ab, ao);
        } else {
            n = 1;
            d = ao;
        }
    } else {
        const double side = dot(abc, ao);
        n = 3;
        if (side > 0.0) {
            d = abc;
        } else if (side < 0.0) {
            s[1] = c;
            s[2] = b;
            d = neg(abc);
        } else {
            return true;
        }
    }
    return dot(d, d) == 0.0;
}

// Boolean GJK: whether the posed moving hull and the still hull share a point.  Every lane
// runs the same scalar code on the same (warp-reduced) values.  Both answers are exact for the
// simplex at hand: "apart" needs a direction along which no point of the Minkowski difference
// reaches the origin, "meeting" a simplex of difference points that holds the origin.
__device__ bool gjk_intersect(const sdfc::HullDesc& A, const Pose3& P, const sdfc::HullDesc& B, D3 d, int* iters) {
    if (dot(d, d) == 0.0) d = d3(1.0, 0.0, 0.0);
    D3 s[4];
    int n = 1;
    s[0] = mink_support(A, P, B, d);
    d = neg(s[0]);
    for (int it = 0; it < kGjkMaxIter; ++it) {
        *iters = it + 1;
        if (dot(d, d) == 0.0) return true;  // the origin lies on the simplex
        const D3 a = mink_support(A, P, B, d);
        if (dot(a, d) < 0.0) return false;  // no point of the difference beyond the origin: apart
        for (int k = n; k > 0; --k) s[k] = s[k - 1];  // newest point first
        s[0] = a;
        ++n;
        const D3 ao = neg(a);
        if (n == 2) {
            const D3 ab = s[1] - a;
            if (dot(ab, ao) > 0.0) {
                d = triple(ab, ao);
                if (dot(d, d) == 0.0) return true;  // origin on the segment
            } else {
                n = 1;
                d = ao;
            }
        } else if (n == 3) {
            if (gjk_triangle(s, n, d)) return true;
        } else {  // tetrahedron a (newest), b, c, e: the origin beyond a face containing a?
            const D3 b = s[1], c = s[2], e = s[3];
            const D3 ab = b - a, ac = c - a, ae = e - a;
            D3 nabc = cross(ab, ac), nace = cross(ac, ae), naeb = cross(ae, ab);
            if (dot(nabc, ae) > 0.0) nabc = neg(nabc);  // outward: away from the opposite vertex
            if (dot(nace, ab) > 0.0) nace = neg(nace);
            if (dot(naeb, ac) > 0.0) naeb = neg(naeb);
            if (dot(nabc, ao) > 0.0) {
                n = 3;  // a, b, c
            } else if (dot(nace, ao) > 0.0) {
                s[1] = c;
                s[2] = e;
                n = 3;
            } else if (dot(naeb, ao) > 0.0) {
                s[1] = e;
                s[2] = b;
                n = 3;
            } else {
                return true;  // the origin is inside the tetrahedron
            }
            if (gjk_triangle(s, n, d)) return true;
        }
    }
    return true;  // not settled within the iteration bound: count as meeting (the safe answer)
}

// One warp per pose of the moving part: out[q] = 1 if disassembled; flags (optional) bit 0 solids
// intersect, bit 1 moving hull inside the still hull, bit 2 still hull inside the moving hull,
// bit 3 box containment, bits 8.. GJK iterations.
__global__ void __launch_bounds__(32 * kHullWarps) disassembled_kernel(sdfc::HullDesc A, sdfc::HullDesc B,
                                                                       const double* __restrict__ E, int n,
                                                                       int* __restrict__ out,
                                                                       int* __restrict__ flags) {
    const int q = blockIdx.x * kHullWarps + (threadIdx.x >> 5);
    if (q >= n) return;  // warp-uniform
    const int lane = threadIdx.x & 31;
    Pose3 P;
    const double* e = E + 16 * (size_t)q;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int c = 0; c < 3; ++c) P.R[3 * r + c] = e[4 * r + c];
    }
    P.p = d3(e[3], e[7], e[11]);
    // posed moving hull: bounds, and whether every vertex is inside the still hull
    D3 lo = d3(INFINITY, INFINITY, INFINITY), hi = d3(-INFINITY, -INFINITY, -INFINITY);
    bool a_in_b = true;
    for (int i = lane; i < A.nv; i += 32) {
        const D3 v = pose_apply(P, ld3(A.v, i));
        lo = d3(fmin(lo.x, v.x), fmin(lo.y, v.y), fmin(lo.z, v.z));
        hi = d3(fmax(hi.x, v.x), fmax(hi.y, v.y), fmax(hi.z, v.z));
        for (int f = 0; f < B.nf && a_in_b; ++f) {
            const double* pl = B.planes + 4 * f;
            a_in_b = pl[0] * v.x + pl[1] * v.y + pl[2] * v.z + pl[3] <= kContainTol;
        }
    }
    // still hull inside the posed moving hull: its vertices in the moving part's frame
    bool b_in_a = true;
    for (int i = lane; i < B.nv; i += 32) {
        const D3 w = rot_t(P, ld3(B.v, i) - P.p);
        for (int f = 0; f < A.nf && b_in_a; ++f) {
            const double* pl = A.planes + 4 * f;
            b_in_a = pl[0] * w.x + pl[1] * w.y + pl[2] * w.z + pl[3] <= kContainTol;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        lo.x = fmin(lo.x, __shfl_xor_sync(0xffffffffu, lo.x, o));
        lo.y = fmin(lo.y, __shfl_xor_sync(0xffffffffu, lo.y, o));
        lo.z = fmin(lo.z, __shfl_xor_sync(0xffffffffu, lo.z, o));
        hi.x = fmax(hi.x, __shfl_xor_sync(0xffffffffu, hi.x, o));
        hi.y = fmax(hi.y, __shfl_xor_sync(0xffffffffu, hi.y, o));
        hi.z = fmax(hi.z, __shfl_xor_sync(0xffffffffu, hi.z, o));
    }
    a_in_b = __all_sync(0xffffffffu, a_in_b);
    b_in_a = __all_sync(0xffffffffu, b_in_a);
    // initial direction: between the boxes' centres
    const D3 d0 = d3(0.5 * (lo.x + hi.x) - 0.5 * (B.lo[0] + B.hi[0]), 0.5 * (lo.y + hi.y) - 0.5 * (B.lo[1] + B.hi[1]),
                     0.5 * (lo.z + hi.z) - 0.5 * (B.lo[2] + B.hi[2]));
    int iters = 0;
    const bool meet = gjk_intersect(A, P, B, d0, &iters);
    const bool surfaces = meet && !a_in_b && !b_in_a;
    const bool move_contains = lo.x <= B.lo[0] && lo.y <= B.lo[1] && lo.z <= B.lo[2] && hi.x >= B.hi[0] &&
                               hi.y >= B.hi[1] && hi.z >= B.hi[2];
    const bool still_contains = B.lo[0] <= lo.x && B.lo[1] <= lo.y && B.lo[2] <= lo.z && B.hi[0] >= hi.x &&
                                B.hi[1] >= hi.y && B.hi[2] >= hi.z;
    if (lane == 0) {
        out[q] = (!surfaces && !(move_contains || still_contains)) ? 1 : 0;
        if (flags)
            flags[q] = (meet ? 1 : 0) | (a_in_b ? 2 : 0) | (b_in_a ? 4 : 0) |
                       ((move_contains || still_contains) ? 8 : 0) | (iters << 8);
    }
}

}  // namespace

extern "C" {

int sdfc_upload_hull(sdfc_context* ctx, const double* verts, int nv, const double* planes, int nf, int* hull) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (!verts || !planes || nv < 1 || nf < 4 || !hull)
        return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_hull: bad argument");
    for (size_t i = 0; i < 3 * (size_t)nv; ++i)
        if (!std::isfinite(verts[i])) return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_hull: non-finite vertex");
    for (size_t i = 0; i < 4 * (size_t)nf; ++i)
        if (!std::isfinite(planes[i])) return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "upload_hull: non-finite plane");
    int rc = sdfc_impl::use_device(ctx);
    if (rc) return rc;
    sdfc::HullDesc h{};
    h.nv = nv;
    h.nf = nf;
    for (int a = 0; a < 3; ++a) {
        h.lo[a] = INFINITY;
        h.hi[a] = -INFINITY;
    }
    for (int i = 0; i < nv; ++i)
        for (int a = 0; a < 3; ++a) {
            h.lo[a] = std::min(h.lo[a], verts[3 * i + a]);
            h.hi[a] = std::max(h.hi[a], verts[3 * i + a]);
        }
    void *pv = nullptr, *pp = nullptr;
    if ((rc = sdfc_impl::dev_alloc(ctx, &pv, sizeof(double) * 3 * nv))) return rc;
    ctx->allocations.push_back(pv);
    if ((rc = sdfc_impl::dev_alloc(ctx, &pp, sizeof(double) * 4 * nf))) return rc;
    ctx->allocations.push_back(pp);
    SDFC_CUDA_TRY(ctx, cudaMemcpy(pv, verts, sizeof(double) * 3 * nv, cudaMemcpyHostToDevice));
    SDFC_CUDA_TRY(ctx, cudaMemcpy(pp, planes, sizeof(double) * 4 * nf, cudaMemcpyHostToDevice));
    h.v = (const double*)pv;
    h.planes = (const double*)pp;
    ctx->hulls.push_back(h);
    *hull = (int)ctx->hulls.size() - 1;
    return SDFC_OK;
}

int sdfc_disassembled_device(sdfc_context* ctx, int hull_move, int hull_still, const double* d_E, int n, int* d_out,
                             int* d_flags, void* stream) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (n < 0 || (n > 0 && (!d_E || !d_out)))
        return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "disassembled: bad argument");
    if (hull_move < 0 || hull_move >= (int)ctx->hulls.size() || hull_still < 0 || hull_still >= (int)ctx->hulls.size())
        return sdfc_impl::fail(ctx, SDFC_ERR_NOT_FOUND, "disassembled: unknown hull");
    int rc = sdfc_impl::use_device(ctx);
    if (rc) return rc;
    if (n == 0) return SDFC_OK;
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    disassembled_kernel<<<(n + kHullWarps - 1) / kHullWarps, 32 * kHullWarps, 0, st>>>(
        ctx->hulls[hull_move], ctx->hulls[hull_still], d_E, n, d_out, d_flags);
    SDFC_CUDA_TRY(ctx, cudaGetLastError());
    return SDFC_OK;
}

int sdfc_disassembled(sdfc_context* ctx, int hull_move, int hull_still, const double* E, int n, int* out, int* flags) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (n < 0 || (n > 0 && (!E || !out))) return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "disassembled: bad argument");
    int rc = sdfc_impl::use_device(ctx);
    if (rc) return rc;
    if (n == 0) return SDFC_OK;
    cudaStream_t st = ctx->stream;
    double* dE = nullptr;
    SDFC_CUDA_TRY(ctx, cudaMallocAsync((void**)&dE, sizeof(double) * 16 * n + sizeof(int) * 2 * n, st));
    int* dout = (int*)(dE + 16 * (size_t)n);
    int* dflags = dout + n;
    cudaError_t e = cudaMemcpyAsync(dE, E, sizeof(double) * 16 * n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        rc = sdfc_disassembled_device(ctx, hull_move, hull_still, dE, n, dout, dflags, st);
        if (rc == SDFC_OK) {
            e = cudaMemcpyAsync(out, dout, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess && flags) e = cudaMemcpyAsync(flags, dflags, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
        }
    }
    cudaFreeAsync(dE, st);
    const cudaError_t e2 = cudaStreamSynchronize(st);
    if (rc) return rc;
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return sdfc_impl::fail(ctx, SDFC_ERR_CUDA, std::string("disassembled: ") + cudaGetErrorString(e));
    return SDFC_OK;
}

}  // extern "C"
