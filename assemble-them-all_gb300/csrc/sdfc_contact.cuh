// Device-side point-vs-SDF contact math for sm_103a.
//
// Restates, for one active contact, the reference redmax computation
//   BodySDFObj::collision              simulation/redmax/Body/BodySDFObj.cpp:239-377
//   ForceGeneralSDFContact::computeForce[WithDerivative](contacts, ...)
//                                      simulation/redmax/Force/ForceGeneralSDFContact.cpp:147-447
// organised for a GPU thread:
//   * the grid-frame point and the penetration depth d are FP64, computed in the
//     reference's operation order without FMA contraction, so d is bit-identical
//     to the reference's BodySDFObj::distance;
//   * the rest of the contact algebra is templated on its arithmetic type T:
//     T = double is the parity path, T = float the throughput path (GB300 runs
//     FP32 at 64x its FP64 rate); sums over contacts are always FP64;
//   * the SDF gradient / Hessian are the analytic derivatives of the trilinear
//     interpolant of the point's cell.  Inside a cell these equal the
//     reference's central differences (step 1e-5, BodySDFObj.cpp:176-205) up to
//     FP64 round-off; when any stencil point of those differences leaves the
//     cell or the box, the exact 26-query stencil is evaluated instead (and a
//     stencil-only mode evaluates it for every contact);
//   * every 6x6 block of Km/Dm is written as Gamma^T N (Gamma = [skew(xi)^T, I],
//     simulation/redmax/Utils.h:196): the body-A rows of the contact's Jacobian
//     column j are [xi1 x N1_j; N1_j] and the body-B rows
//     [xi2 x N2_j + T2_j; N2_j], with N1_j, N2_j, T2_j 3-vectors.  The 24
//     columns (q1, q2, phi1, phi2) are produced one at a time and handed to a
//     sink, so a thread never holds a 12x12 block.
#pragma once

#include <cuda_fp16.h>

#include <cfloat>
#include <cstdint>
#include <type_traits>

namespace sdfc {

// ---------------------------------------------------------------- small vectors
template <typename T>
struct Vec3 {
    T x, y, z;
};
template <typename T>
struct Mat3 {  // row-major
    T m[9];
};
using V3 = Vec3<double>;
using M3 = Mat3<double>;

template <typename T>
__device__ __forceinline__ Vec3<T> vec3(T a, T b, T c) {
    return {a, b, c};
}
__device__ __forceinline__ V3 v3(double a, double b, double c) { return {a, b, c}; }
template <typename T>
__device__ __forceinline__ Vec3<T> operator+(Vec3<T> a, Vec3<T> b) {
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename T>
__device__ __forceinline__ Vec3<T> operator-(Vec3<T> a, Vec3<T> b) {
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
__device__ __forceinline__ Vec3<T> operator-(Vec3<T> a) {
    return {-a.x, -a.y, -a.z};
}
template <typename T>
__device__ __forceinline__ Vec3<T> operator*(T s, Vec3<T> a) {
    return {s * a.x, s * a.y, s * a.z};
}
template <typename T>
__device__ __forceinline__ T dot(Vec3<T> a, Vec3<T> b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
__device__ __forceinline__ Vec3<T> cross(Vec3<T> a, Vec3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T>
__device__ __forceinline__ T norm(Vec3<T> a) {
    return sqrt(dot(a, a));
}
template <typename T>
__device__ __forceinline__ T comp(Vec3<T> a, int k) {
    return k == 0 ? a.x : (k == 1 ? a.y : a.z);
}
template <typename T>
__device__ __forceinline__ Vec3<T> unit(int k) {
    return {k == 0 ? T(1) : T(0), k == 1 ? T(1) : T(0), k == 2 ? T(1) : T(0)};
}
template <typename T, typename U>
__device__ __forceinline__ Vec3<T> cast(Vec3<U> a) {
    return {(T)a.x, (T)a.y, (T)a.z};
}
template <typename T, typename U>
__device__ __forceinline__ Mat3<T> cast(const Mat3<U>& A) {
    Mat3<T> B;
#pragma unroll
    for (int k = 0; k < 9; ++k) B.m[k] = (T)A.m[k];
    return B;
}
template <typename T>
__device__ __forceinline__ Vec3<T> mul(const Mat3<T>& A, Vec3<T> v) {
    return {A.m[0] * v.x + A.m[1] * v.y + A.m[2] * v.z, A.m[3] * v.x + A.m[4] * v.y + A.m[5] * v.z,
            A.m[6] * v.x + A.m[7] * v.y + A.m[8] * v.z};
}
template <typename T>
__device__ __forceinline__ Vec3<T> mulT(const Mat3<T>& A, Vec3<T> v) {  // A^T v
    return {A.m[0] * v.x + A.m[3] * v.y + A.m[6] * v.z, A.m[1] * v.x + A.m[4] * v.y + A.m[7] * v.z,
            A.m[2] * v.x + A.m[5] * v.y + A.m[8] * v.z};
}
template <typename T>
__device__ __forceinline__ Vec3<T> col(const Mat3<T>& A, int c) {
    return {A.m[c], A.m[3 + c], A.m[6 + c]};
}
template <typename T>
__device__ __forceinline__ Mat3<T> mul(const Mat3<T>& A, const Mat3<T>& B) {
    Mat3<T> C;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            C.m[3 * r + c] = A.m[3 * r] * B.m[c] + A.m[3 * r + 1] * B.m[3 + c] + A.m[3 * r + 2] * B.m[6 + c];
    return C;
}
template <typename T>
__device__ __forceinline__ Mat3<T> transpose(const Mat3<T>& A) {
    return {{A.m[0], A.m[3], A.m[6], A.m[1], A.m[4], A.m[7], A.m[2], A.m[5], A.m[8]}};
}

// ---------------------------------------------------------------- grids and poses
// An SDF grid as the reference's BodySDFObj holds it (BodySDFObj.h:13-16), values
// indexed [i + ni*(j + nj*k)] (simulation/externals/sdfgen/array3.h:70-79).
struct GridDesc {
    int ni, nj, nk;
    int storage;  // 0 = FP64 values, 1 = FP32 values, 2 = FP16 bricks, 3 = FP32 node values only
    double min_box[3], max_box[3], dx[3], inv_dx[3];
    double org[3];  // min_box / dx (cell coordinate of the origin), for the fast depth path
    double col_th;
    const double* v64;   // FP64 values (storage 1: the FP32 values widened), read for active contacts
    // storage 3: the FP32 node values alone (4 B per node, no FP64 copy, no cell-corner array);
    // every read widens them, so the exact paths see the same doubles as storage 1
    const float* v32;
    // storage 2: FP16 codes in 8^3-node bricks (brick b = bx + nbx (by + nby bz), node
    // (i&7) + 8 (j&7) + 64 (k&7) within it) and per brick (scale, offset); value =
    // fma(scale, code, offset), in FP64 for the exact paths and FP32 for the others
    const unsigned short* b16;
    const float2* bso;
    int nbx, nby;
    // per cell (ni-1)(nj-1)(nk-1), i fastest: its 8 FP32 corner values in two float4,
    // (c000, c100, c010, c110) and (c001, c101, c011, c111); read by detection and the
    // FP32 derivatives with two 16-byte loads instead of eight scattered gathers
    const float4* cells32;
    float fmin[3], fmax[3], finv_dx[3], fdx[3];  // FP32 constants
    float lip;        // bound on |grad| of the interpolant over the grid
    float vmax;       // max |value|
    // per block of 2^bshift cells per axis (block (bi, bj, bk) at bi + bnx (bj + bny bk)): the
    // least FP32 node value over the nodes of its cells, so detection can tell that a point is
    // far outside the surface without reading its cell (null: no table, as for FP16 bricks)
    const float* bmin;
    int bshift, bnx, bny, bpad;
};

// A contact body's points, stored on the device in a spatially sorted order
// (Morton order in the body frame) so that a warp's points share grid cells;
// `orig` maps a stored index back to the caller's point index.
struct PointsDesc {
    int n;
    int storage;       // 0 = FP64 SoA, 1 = FP32 SoA
    const float* x32;  // FP32 SoA (x[n], y[n], z[n]); exact when storage == 1
    const double* x64; // FP64 SoA (storage 1: the FP32 points widened)
    const int* orig;   // stored index -> caller's index
    float radius;      // max |xi|
    // per detection tile (kTile consecutive stored points): a sphere (x, y, z, r) in the body frame
    // holding the tile's FP32 points, so that detection can pass over tiles far from a grid box
    const float4* tiles;
};

struct Pose {
    M3 R;
    V3 p;
};

__device__ __forceinline__ Pose load_pose(const double* E) {
    Pose P;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int c = 0; c < 3; ++c) P.R.m[3 * r + c] = E[4 * r + c];
    }
    P.p = v3(E[3], E[7], E[11]);
    return P;
}

__device__ __forceinline__ size_t brick_of(const GridDesc& g, int i, int j, int k) {
    return (size_t)(i >> 3) + (size_t)g.nbx * ((size_t)(j >> 3) + (size_t)g.nby * (size_t)(k >> 3));
}
__device__ __forceinline__ float brick_code(const GridDesc& g, size_t b, int i, int j, int k) {
    return __half2float(__ushort_as_half(__ldg(g.b16 + b * 512 + (i & 7) + 8 * (j & 7) + 64 * (k & 7))));
}
// A brick node's value: fmaf(scale, code, offset) in FP32 (the FP64 paths read it widened, so
// the two views are the same number and the FP64 pipe only widens it).
__device__ __forceinline__ float brick_value32(const GridDesc& g, int i, int j, int k) {
    const size_t b = brick_of(g, i, j, k);
    const float2 so = __ldg(g.bso + b);
    return fmaf(so.x, brick_code(g, b, i, j, k), so.y);
}
__device__ __forceinline__ double brick_value64(const GridDesc& g, int i, int j, int k) {
    return (double)brick_value32(g, i, j, k);
}

// The brick reads are kept out of line (results returned by value, in registers) so that the
// hot loops over the FP64 array and the FP32 cell-corner array stay as small as without bricks.
struct Corners32 {
    float c[8];
};
// Node offsets of a cell's 8 corners within one brick (corner order c000, c100, c010, c110, ...).
__device__ __forceinline__ int brick_corner_offset(int q) { return (q & 1) + 8 * ((q >> 1) & 1) + 64 * (q >> 2); }
// Whether cell (i, j, k)'s corners all lie in the brick of node (i, j, k) (about 2/3 of cells).
__device__ __forceinline__ bool cell_in_one_brick(int i, int j, int k) {
    return (i & 7) != 7 && (j & 7) != 7 && (k & 7) != 7;
}

static __device__ __noinline__ Corners32 brick_corners32(const GridDesc& g, int i, int j, int k) {
    Corners32 r;
    if (cell_in_one_brick(i, j, k)) {  // one scale/offset and eight codes of one brick
        const size_t b = brick_of(g, i, j, k);
        const float2 so = __ldg(g.bso + b);
        const unsigned short* cb = g.b16 + b * 512 + (i & 7) + 8 * (j & 7) + 64 * (k & 7);
#pragma unroll
        for (int q = 0; q < 8; ++q)
            r.c[q] = fmaf(so.x, __half2float(__ushort_as_half(__ldg(cb + brick_corner_offset(q)))), so.y);
        return r;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) r.c[q] = brick_value32(g, i + (q & 1), j + ((q >> 1) & 1), k + (q >> 2));
    return r;
}

static __device__ __noinline__ double brick_value64_cold(const GridDesc& g, int i, int j, int k) {
    return brick_value64(g, i, j, k);
}

__device__ __forceinline__ double grid_value(const GridDesc& g, int i, int j, int k) {
    if (g.b16) return brick_value64_cold(g, i, j, k);
    const size_t idx = (size_t)i + (size_t)g.ni * ((size_t)j + (size_t)g.nj * (size_t)k);
    if (g.v32) return (double)__ldg(g.v32 + idx);
    return __ldg(g.v64 + idx);
}

// The 8 corners of cell (i, j, k) from FP32 node values (storage 3), in cell-corner order.
__device__ __forceinline__ void node_corners32(const GridDesc& g, int i, int j, int k, float* c) {
    const size_t sj = (size_t)g.ni, sk = (size_t)g.ni * (size_t)g.nj;
    const float* b = g.v32 + (size_t)i + sj * (size_t)j + sk * (size_t)k;
    c[0] = __ldg(b);           c[1] = __ldg(b + 1);
    c[2] = __ldg(b + sj);      c[3] = __ldg(b + sj + 1);
    c[4] = __ldg(b + sk);      c[5] = __ldg(b + sk + 1);
    c[6] = __ldg(b + sk + sj); c[7] = __ldg(b + sk + sj + 1);
}

// The 8 corner values of cell (i, j, k), ordered c000, c100, c010, c110, c001, c101,
// c011, c111: FP32 (from the cell-corner array or the bricks) and FP64.
__device__ __forceinline__ void cell_corners32(const GridDesc& g, int i, int j, int k, float* c) {
    if (g.b16) {
        const Corners32 r = brick_corners32(g, i, j, k);
#pragma unroll
        for (int q = 0; q < 8; ++q) c[q] = r.c[q];
        return;
    }
    if (g.v32) {
        node_corners32(g, i, j, k, c);
        return;
    }
    const float4* cq = g.cells32 + 2 * ((size_t)i + (size_t)(g.ni - 1) * ((size_t)j + (size_t)(g.nj - 1) * k));
    const float4 lo = __ldg(cq), hi = __ldg(cq + 1);
    c[0] = lo.x; c[1] = lo.y; c[2] = lo.z; c[3] = lo.w;
    c[4] = hi.x; c[5] = hi.y; c[6] = hi.z; c[7] = hi.w;
}
// The cell-corner reads of FP64 / FP32 grids alone (no brick test), for code specialised on
// grids without bricks.
__device__ __forceinline__ void plain_corners32(const GridDesc& g, int i, int j, int k, float* c) {
    const float4* cq = g.cells32 + 2 * ((size_t)i + (size_t)(g.ni - 1) * ((size_t)j + (size_t)(g.nj - 1) * k));
    const float4 lo = __ldg(cq), hi = __ldg(cq + 1);
    c[0] = lo.x; c[1] = lo.y; c[2] = lo.z; c[3] = lo.w;
    c[4] = hi.x; c[5] = hi.y; c[6] = hi.z; c[7] = hi.w;
}
__device__ __forceinline__ void plain_corners64(const GridDesc& g, int i, int j, int k, double* c) {
    const size_t sj = (size_t)g.ni, sk = (size_t)g.ni * (size_t)g.nj;
    const size_t b = (size_t)i + sj * (size_t)j + sk * (size_t)k;
    c[0] = __ldg(g.v64 + b);           c[1] = __ldg(g.v64 + b + 1);
    c[2] = __ldg(g.v64 + b + sj);      c[3] = __ldg(g.v64 + b + sj + 1);
    c[4] = __ldg(g.v64 + b + sk);      c[5] = __ldg(g.v64 + b + sk + 1);
    c[6] = __ldg(g.v64 + b + sk + sj); c[7] = __ldg(g.v64 + b + sk + sj + 1);
}
__device__ __forceinline__ void cell_corners64(const GridDesc& g, int i, int j, int k, double* c) {
    if (g.b16) {
        const Corners32 r = brick_corners32(g, i, j, k);
#pragma unroll
        for (int q = 0; q < 8; ++q) c[q] = (double)r.c[q];
        return;
    }
    if (g.v32) {
        float f[8];
        node_corners32(g, i, j, k, f);
#pragma unroll
        for (int q = 0; q < 8; ++q) c[q] = (double)f[q];
        return;
    }
    const size_t sj = (size_t)g.ni, sk = (size_t)g.ni * (size_t)g.nj;
    const size_t b = (size_t)i + sj * (size_t)j + sk * (size_t)k;
    c[0] = __ldg(g.v64 + b);           c[1] = __ldg(g.v64 + b + 1);
    c[2] = __ldg(g.v64 + b + sj);      c[3] = __ldg(g.v64 + b + sj + 1);
    c[4] = __ldg(g.v64 + b + sk);      c[5] = __ldg(g.v64 + b + sk + 1);
    c[6] = __ldg(g.v64 + b + sk + sj); c[7] = __ldg(g.v64 + b + sk + sj + 1);
}

// FP64 arithmetic in the reference's operation order without FMA contraction.
// With these, the grid-frame point and query_SDF reproduce the reference's
// x86-64 (SSE2, no FMA) results bit for bit: same products, same sums, same
// IEEE division and rounding.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
// (1 - c) * a + c * b
__device__ __forceinline__ double lerp_ref(double c, double a, double b) {
    return add_rn(mul_rn(sub_rn(1.0, c), a), mul_rn(c, b));
}
// A v and A^T v, sums left to right
__device__ __forceinline__ V3 mul_ref(const M3& A, V3 v) {
    return {add_rn(add_rn(mul_rn(A.m[0], v.x), mul_rn(A.m[1], v.y)), mul_rn(A.m[2], v.z)),
            add_rn(add_rn(mul_rn(A.m[3], v.x), mul_rn(A.m[4], v.y)), mul_rn(A.m[5], v.z)),
            add_rn(add_rn(mul_rn(A.m[6], v.x), mul_rn(A.m[7], v.y)), mul_rn(A.m[8], v.z))};
}
__device__ __forceinline__ V3 mulT_ref(const M3& A, V3 v) {
    return {add_rn(add_rn(mul_rn(A.m[0], v.x), mul_rn(A.m[3], v.y)), mul_rn(A.m[6], v.z)),
            add_rn(add_rn(mul_rn(A.m[1], v.x), mul_rn(A.m[4], v.y)), mul_rn(A.m[7], v.z)),
            add_rn(add_rn(mul_rn(A.m[2], v.x), mul_rn(A.m[5], v.y)), mul_rn(A.m[8], v.z))};
}
// Contact point in world and in the SDF body's frame:
//   xw = R_A xi + p_A (CollisionDetection.cpp:136), x = R_B^T (xw - p_B) (BodySDFObj.cpp:211)
__device__ __forceinline__ V3 world_point(const M3& RA, V3 pA, V3 xi) {
    V3 r = mul_ref(RA, xi);
    return {add_rn(r.x, pA.x), add_rn(r.y, pA.y), add_rn(r.z, pA.z)};
}
__device__ __forceinline__ V3 grid_point(const M3& RB, V3 pB, V3 xw) {
    return mulT_ref(RB, v3(sub_rn(xw.x, pB.x), sub_rn(xw.y, pB.y), sub_rn(xw.z, pB.z)));
}

// Cell of a point inside the box: integer cell and fractional position,
// computed as the reference does ((x - min) / dx, floor, subtract).
struct Cell {
    int i, j, k;
    double u, v, w;
};
__device__ __forceinline__ Cell cell_of(const GridDesc& g, V3 x) {
    double ci = sub_rn(x.x, g.min_box[0]) / g.dx[0];
    double cj = sub_rn(x.y, g.min_box[1]) / g.dx[1];
    double ck = sub_rn(x.z, g.min_box[2]) / g.dx[2];
    Cell c;
    c.i = (int)floor(ci);
    c.j = (int)floor(cj);
    c.k = (int)floor(ck);
    c.u = sub_rn(ci, (double)c.i);
    c.v = sub_rn(cj, (double)c.j);
    c.w = sub_rn(ck, (double)c.k);
    return c;
}

// Trilinear interpolation at a cell position, the inside branch of
// BodySDFObj::query_SDF (BodySDFObj.cpp:130-155), in the reference's operation
// order.  Cell indices are clamped to the grid; the grid check at upload
// guarantees the reference's index arithmetic stays in range, so the clamp
// changes nothing.
__device__ __forceinline__ double trilinear_at(const GridDesc& g, Cell c) {
    int i = min(max(c.i, 0), g.ni - 1), j = min(max(c.j, 0), g.nj - 1), k = min(max(c.k, 0), g.nk - 1);
    int ip = (i == g.ni - 1) ? i : i + 1;
    int jp = (j == g.nj - 1) ? j : j + 1;
    int kp = (k == g.nk - 1) ? k : k + 1;
    double e[8];
    if (g.b16 && ip == i + 1 && jp == j + 1 && kp == k + 1) {  // FP16 bricks: the cell's corners in one read
        const Corners32 r = brick_corners32(g, i, j, k);
#pragma unroll
        for (int q = 0; q < 8; ++q) e[q] = (double)r.c[q];
    } else {
        e[0] = grid_value(g, i, j, k);   e[1] = grid_value(g, ip, j, k);
        e[2] = grid_value(g, i, jp, k);  e[3] = grid_value(g, ip, jp, k);
        e[4] = grid_value(g, i, j, kp);  e[5] = grid_value(g, ip, j, kp);
        e[6] = grid_value(g, i, jp, kp); e[7] = grid_value(g, ip, jp, kp);
    }
    double v00 = lerp_ref(c.u, e[0], e[1]);
    double v10 = lerp_ref(c.u, e[2], e[3]);
    double v01 = lerp_ref(c.u, e[4], e[5]);
    double v11 = lerp_ref(c.u, e[6], e[7]);
    double vk0 = lerp_ref(c.v, v00, v10);
    double vk1 = lerp_ref(c.v, v01, v11);
    return lerp_ref(c.w, vk0, vk1);
}
__device__ __forceinline__ double trilinear(const GridDesc& g, V3 x) { return trilinear_at(g, cell_of(g, x)); }

__device__ __forceinline__ bool in_box(const GridDesc& g, V3 x) {
    return x.x >= g.min_box[0] && x.x <= g.max_box[0] && x.y >= g.min_box[1] && x.y <= g.max_box[1] &&
           x.z >= g.min_box[2] && x.z <= g.max_box[2];
}

// BodySDFObj::query_SDF (BodySDFObj.cpp:123-174).
__device__ inline double query_sdf(const GridDesc& g, V3 x, bool outside_accurate) {
    if (in_box(g, x)) return trilinear(g, x);
    if (!outside_accurate) return (double)FLT_MAX;
    // distance to the box plus the value at the closest box point, :159-167
    V3 xb = v3(fmin(fmax(x.x, g.min_box[0]), g.max_box[0]), fmin(fmax(x.y, g.min_box[1]), g.max_box[1]),
               fmin(fmax(x.z, g.min_box[2]), g.max_box[2]));
    V3 dv = v3(sub_rn(x.x, xb.x), sub_rn(x.y, xb.y), sub_rn(x.z, xb.z));
    double n2 = add_rn(add_rn(mul_rn(dv.x, dv.x), mul_rn(dv.y, dv.y)), mul_rn(dv.z, dv.z));
    return add_rn(__dsqrt_rn(n2), trilinear(g, xb));
}

// Value, gradient and Hessian of the SDF at x (query_SDF / query_dSDF /
// query_ddSDF of the reference).  The value is always FP64.
template <typename T>
struct SdfJet {
    double v;      // query_SDF(x) (FLT_MAX outside the box)
    Vec3<T> g;     // query_dSDF(x)
    T h[6];        // query_ddSDF(x): xx, yy, zz, xy, xz, yz
};

constexpr double kFdEps = 1e-5;  // BodySDFObj.cpp:178,191

// Rarely executed exact paths (the 19-query FP64 stencil) are kept out of line so that
// the force kernel's hot loop stays compact in the instruction cache.
#ifndef SDFC_COLD
#define SDFC_COLD static __noinline__
#endif

// The reference's stencil (BodySDFObj.cpp:176-205), bit-identical in FP64.
__device__ SDFC_COLD void sdf_stencil(const GridDesc& g, V3 x, V3& grad, double* hess, bool want_hessian) {
    const double e = kFdEps, h = kFdEps / 2;
    double gp[3], gm[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        V3 xp = x, xm = x;
        if (a == 0) { xp.x = x.x + e; xm.x = x.x - e; }
        if (a == 1) { xp.y = x.y + e; xm.y = x.y - e; }
        if (a == 2) { xp.z = x.z + e; xm.z = x.z - e; }
        gp[a] = query_sdf(g, xp, true);
        gm[a] = query_sdf(g, xm, true);
    }
    grad = v3((gp[0] - gm[0]) / (2 * e), (gp[1] - gm[1]) / (2 * e), (gp[2] - gm[2]) / (2 * e));
    if (!want_hessian) return;
    double xs = query_sdf(g, x, true);
    const double ee = e * e;
#pragma unroll
    for (int a = 0; a < 3; ++a) hess[a] = sub_rn(add_rn(gp[a], gm[a]), mul_rn(2.0, xs)) / ee;
    const int pa[3] = {0, 0, 1}, pb[3] = {1, 2, 2};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        double c[3] = {x.x, x.y, x.z};
        double pp[3] = {c[0], c[1], c[2]}, mm[3] = {c[0], c[1], c[2]}, pm[3] = {c[0], c[1], c[2]},
               mp[3] = {c[0], c[1], c[2]};
        int a = pa[q], b = pb[q];
        pp[a] = c[a] + h; pp[b] = c[b] + h;
        mm[a] = c[a] - h; mm[b] = c[b] - h;
        pm[a] = c[a] + h; pm[b] = c[b] - h;
        mp[a] = c[a] - h; mp[b] = c[b] + h;
        double s = query_sdf(g, v3(pp[0], pp[1], pp[2]), true) + query_sdf(g, v3(mm[0], mm[1], mm[2]), true) -
                   query_sdf(g, v3(pm[0], pm[1], pm[2]), true) - query_sdf(g, v3(mp[0], mp[1], mp[2]), true);
        hess[3 + q] = s / ee;
    }
}

// sdf_stencil with its 19 queries spread over the lanes of one warp.  Every lane
// of the warp must call it with the same x (warp-uniform control flow, all 32
// lanes active).  Lane l < 19 evaluates one query point, the values are
// exchanged by shuffles and every lane combines them in sdf_stencil's operation
// order, so the results are bit-identical to sdf_stencil's.
__device__ SDFC_COLD void sdf_stencil_warp(const GridDesc& g, V3 x, V3& grad, double* hess, bool want_hessian,
                                        double& centre) {
    const int lane = threadIdx.x & 31;
    const double e = kFdEps, h = kFdEps / 2;
    double c[3] = {x.x, x.y, x.z};
    if (lane < 3) {  // gp[a]
        c[lane] = c[lane] + e;
    } else if (lane < 6) {  // gm[a]
        c[lane - 3] = c[lane - 3] - e;
    } else if (lane >= 7 && lane < 19) {  // mixed pair q: pp, mm, pm, mp
        const int q = (lane - 7) >> 2, kind = (lane - 7) & 3;
        const int a = q < 2 ? 0 : 1, b = q == 0 ? 1 : 2;
        const double ca = c[a], cb = c[b];
        c[a] = (kind == 0 || kind == 2) ? ca + h : ca - h;
        c[b] = (kind == 0 || kind == 3) ? cb + h : cb - h;
    }  // lane 6: the centre
    const double v = lane < 19 ? query_sdf(g, v3(c[0], c[1], c[2]), true) : 0.0;
    double gp[3], gm[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        gp[a] = __shfl_sync(0xffffffffu, v, a);
        gm[a] = __shfl_sync(0xffffffffu, v, 3 + a);
    }
    grad = v3((gp[0] - gm[0]) / (2 * e), (gp[1] - gm[1]) / (2 * e), (gp[2] - gm[2]) / (2 * e));
    const double xs = __shfl_sync(0xffffffffu, v, 6);
    centre = xs;
    if (!want_hessian) return;
    const double ee = e * e;
#pragma unroll
    for (int a = 0; a < 3; ++a) hess[a] = sub_rn(add_rn(gp[a], gm[a]), mul_rn(2.0, xs)) / ee;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double vpp = __shfl_sync(0xffffffffu, v, 7 + 4 * q), vmm = __shfl_sync(0xffffffffu, v, 8 + 4 * q);
        const double vpm = __shfl_sync(0xffffffffu, v, 9 + 4 * q), vmp = __shfl_sync(0xffffffffu, v, 10 + 4 * q);
        const double s = vpp + vmm - vpm - vmp;
        hess[3 + q] = s / ee;
    }
}

// True when the reference's stencil around x stays inside x's cell on every
// axis (no stencil point in another cell or outside the box, and the cell is
// not the clamped top cell).  The test keeps a margin of 2 eps from the
// faces, so a false "inside" cannot happen; a false "outside" only costs the
// (exact) stencil evaluation.
__device__ __forceinline__ bool stencil_in_cell(const GridDesc& g, const Cell& c) {
    const double m = 2.0 * kFdEps;
    return c.i >= 0 && c.j >= 0 && c.k >= 0 && c.i < g.ni - 1 && c.j < g.nj - 1 && c.k < g.nk - 1 &&
           c.u * g.dx[0] > m && (1.0 - c.u) * g.dx[0] > m && c.v * g.dx[1] > m && (1.0 - c.v) * g.dx[1] > m &&
           c.w * g.dx[2] > m && (1.0 - c.w) * g.dx[2] > m;
}

// stencil_only = true evaluates the reference's 26-query stencil for every
// point (bit-identical SDF derivatives); otherwise the analytic cell
// derivatives (in T) are used wherever the stencil stays inside one cell.
template <typename T>
__device__ inline void sdf_jet(const GridDesc& g, V3 x, SdfJet<T>& J, bool want_hessian, bool stencil_only) {
    if (in_box(g, x)) {
        Cell c = cell_of(g, x);
        J.v = trilinear_at(g, c);
        if (!stencil_only && stencil_in_cell(g, c)) {
            const T u = (T)c.u, v = (T)c.v, w = (T)c.w;
            const int i = c.i, j = c.j, k = c.k;
            T c000 = (T)grid_value(g, i, j, k), c100 = (T)grid_value(g, i + 1, j, k);
            T c010 = (T)grid_value(g, i, j + 1, k), c110 = (T)grid_value(g, i + 1, j + 1, k);
            T c001 = (T)grid_value(g, i, j, k + 1), c101 = (T)grid_value(g, i + 1, j, k + 1);
            T c011 = (T)grid_value(g, i, j + 1, k + 1), c111 = (T)grid_value(g, i + 1, j + 1, k + 1);
            T a00 = c100 - c000, a10 = c110 - c010, a01 = c101 - c001, a11 = c111 - c011;  // d/du
            T b0 = (1 - u) * c000 + u * c100, b1 = (1 - u) * c010 + u * c110;              // along v
            T b2 = (1 - u) * c001 + u * c101, b3 = (1 - u) * c011 + u * c111;
            T gu = (1 - v) * ((1 - w) * a00 + w * a01) + v * ((1 - w) * a10 + w * a11);
            T gv = (1 - w) * (b1 - b0) + w * (b3 - b2);
            T gw = ((1 - v) * b2 + v * b3) - ((1 - v) * b0 + v * b1);
            const T ix = (T)g.inv_dx[0], iy = (T)g.inv_dx[1], iz = (T)g.inv_dx[2];
            J.g = vec3<T>(gu * ix, gv * iy, gw * iz);
            if (want_hessian) {
                J.h[0] = J.h[1] = J.h[2] = T(0);
                J.h[3] = ((1 - w) * (a10 - a00) + w * (a11 - a01)) * (ix * iy);
                J.h[4] = ((1 - v) * (a01 - a00) + v * (a11 - a10)) * (ix * iz);
                J.h[5] = ((b3 - b2) - (b1 - b0)) * (iy * iz);
            }
            return;
        }
    } else {
        J.v = (double)FLT_MAX;
    }
    V3 gr;
    double hs[6];
    sdf_stencil(g, x, gr, hs, want_hessian);
    J.g = cast<T>(gr);
    if (want_hessian)
        for (int k = 0; k < 6; ++k) J.h[k] = (T)hs[k];
}

template <typename T>
__device__ __forceinline__ Vec3<T> hess_mul(const T* h, Vec3<T> v) {
    return {h[0] * v.x + h[3] * v.y + h[4] * v.z, h[3] * v.x + h[1] * v.y + h[5] * v.z,
            h[4] * v.x + h[5] * v.y + h[2] * v.z};
}

// ---------------------------------------------------------------- per-contact force
struct ContactParams {
    double kn, kt, mu, kd;  // kn, kt already scaled by scale * contact_scale (ForceGeneralSDFContact.cpp:155-156)
    float kn32, kt32, mu32, kd32;  // the same rounded to FP32 (the FP32 path's coefficients)
    bool friction;          // mu > eps (ForceGeneralSDFContact.cpp:199, 341)
};

constexpr double kFrictionEps = 1e-8;  // constants::eps, simulation/redmax/Utils.h:9

struct BodyState {
    Pose P;
    V3 w, v;  // phi = (w, v), body frame
};

// The FP32 fast path's map from the contact body's frame to the SDF grid:
// cell coordinates c = Rc xi + pc in FP64 (Rc = diag(1/dx) R_B^T R_A,
// pc = diag(1/dx) R_B^T (p_A - p_B) - org) and the grid-frame point in FP32.
struct CellMap {
    M3 Rc;
    V3 pc;
    Mat3<float> Rf;
    Vec3<float> pf;
    Vec3<float> of;  // -org in FP32 (cell coordinate = y / dx - org)
};

// Per-instance state of a pair as a force thread holds it: the FP64 poses and
// twists (exact path), their casts to the algebra type T, the coefficients,
// and the composite transform grid frame <- contact body frame (fast path).
template <typename T>
struct PairState {
    BodyState A, B;
    Mat3<T> R1, R2;
    Vec3<T> w1, v1, w2, v2;
    ContactParams cp;
    M3 RT;  // R_B^T R_A
    V3 pT;  // R_B^T (p_A - p_B)
    Mat3<T> Q;   // R_A^T R_B: body A's frame -> body B's, for body B's Jacobian columns
    CellMap cm;  // set by make_cell_map
};

template <typename T>
__device__ __forceinline__ void make_pair_state(const double* EA, const double* phiA, const double* EB,
                                                const double* phiB, const double* prm, PairState<T>& S) {
    S.A.P = load_pose(EA);
    S.B.P = load_pose(EB);
    S.A.w = v3(phiA[0], phiA[1], phiA[2]);
    S.A.v = v3(phiA[3], phiA[4], phiA[5]);
    S.B.w = v3(phiB[0], phiB[1], phiB[2]);
    S.B.v = v3(phiB[3], phiB[4], phiB[5]);
    S.R1 = cast<T>(S.A.P.R);
    S.R2 = cast<T>(S.B.P.R);
    S.w1 = cast<T>(S.A.w);
    S.v1 = cast<T>(S.A.v);
    S.w2 = cast<T>(S.B.w);
    S.v2 = cast<T>(S.B.v);
    S.cp.kn = prm[0] * prm[4] * prm[5];
    S.cp.kt = prm[1] * prm[4] * prm[5];
    S.cp.mu = prm[2];
    S.cp.kd = prm[3];
    S.cp.kn32 = (float)S.cp.kn;
    S.cp.kt32 = (float)S.cp.kt;
    S.cp.mu32 = (float)S.cp.mu;
    S.cp.kd32 = (float)S.cp.kd;
    S.cp.friction = S.cp.mu > kFrictionEps;
    S.RT = mul(transpose(S.B.P.R), S.A.P.R);
    S.pT = mulT(S.B.P.R, S.A.P.p - S.B.P.p);
    S.Q = cast<T>(transpose(S.RT));
}

// The pair's CellMap on grid g (after make_pair_state).
template <typename T>
__device__ __forceinline__ void make_cell_map(const GridDesc& g, PairState<T>& S) {
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) S.cm.Rc.m[3 * r + c] = S.RT.m[3 * r + c] * g.inv_dx[r];
        const double p = r == 0 ? S.pT.x : (r == 1 ? S.pT.y : S.pT.z);
        const double q = fma(p, g.inv_dx[r], -g.org[r]);
        if (r == 0) S.cm.pc.x = q; else if (r == 1) S.cm.pc.y = q; else S.cm.pc.z = q;
    }
    S.cm.Rf = cast<float>(S.RT);
    S.cm.pf = cast<float>(S.pT);
    S.cm.of = vec3<float>((float)-g.org[0], (float)-g.org[1], (float)-g.org[2]);
}

// Cell of an active contact for the FP32 throughput path: the grid-frame point
// through the composite FP64 transform and the cell coordinate by one FP64
// fused multiply-add per axis.  `ok` is false when the reference's derivative
// stencil (+-1e-5 per axis) could reach another cell or the clamped top cell;
// such contacts take the exact path.  The integer cell comes from the FP32
// coordinate: where it disagrees with the FP64 floor the FP64 fraction lies
// within FP32 round-off of a face, which `ok` rejects.  Active contacts lie
// inside the grid box (detection guarantees it), so no box test is needed.
struct FastCell {
    Vec3<float> xi32;  // the contact point in its body's frame (FP32)
    Vec3<float> y;  // grid-frame point (FP32)
    double ud, vd, wd;
    int i, j, k;
    bool ok;    // the reference's derivative stencil stays in the cell
    bool near;  // it crosses faces of the cell, within the grid's nodes (cross_face_terms applies)
    signed char dir[3];  // per axis: +1 / -1 when the stencil crosses the upper / lower face
};

template <typename T>
__device__ __forceinline__ FastCell fast_cell(const GridDesc& g, const CellMap& cm, V3 xi, Vec3<float> xf) {
    FastCell c;
    const M3& R = cm.Rc;
    const double cx = fma(R.m[0], xi.x, fma(R.m[1], xi.y, fma(R.m[2], xi.z, cm.pc.x)));
    const double cy = fma(R.m[3], xi.x, fma(R.m[4], xi.y, fma(R.m[5], xi.z, cm.pc.y)));
    const double cz = fma(R.m[6], xi.x, fma(R.m[7], xi.y, fma(R.m[8], xi.z, cm.pc.z)));
    c.xi32 = xf;
    c.y = mul(cm.Rf, xf) + cm.pf;
    // the cell from the FP32 point (any cell within FP32 round-off of the true one; where it
    // is not the FP64 coordinate's own cell the FP64 fraction below leaves [eps, 1 - eps] and
    // `ok` rejects the contact)
    c.i = (int)floorf(fmaf(c.y.x, g.finv_dx[0], cm.of.x));
    c.j = (int)floorf(fmaf(c.y.y, g.finv_dx[1], cm.of.y));
    c.k = (int)floorf(fmaf(c.y.z, g.finv_dx[2], cm.of.z));
    c.ud = cx - (double)c.i;
    c.vd = cy - (double)c.j;
    c.wd = cz - (double)c.k;
    // the stencil stays in the cell when every face is more than eps away
    // (a margin of 1.0001 eps absorbs the FP32 evaluation of this test)
    const float m = (float)(1.0001 * 1e-5);
    const float u = (float)c.ud, v = (float)c.vd, w = (float)c.wd;
    const bool inrange = c.i >= 0 && c.j >= 0 && c.k >= 0 && c.i < g.ni - 1 && c.j < g.nj - 1 && c.k < g.nk - 1;
    const float f[3] = {u, v, w};
    const int ci[3] = {c.i, c.j, c.k}, nn[3] = {g.ni, g.nj, g.nk};
    bool inside = true, near = inrange;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const bool up = (1.f - f[a]) * g.fdx[a] <= m, down = f[a] * g.fdx[a] <= m;
        inside = inside && !up && !down;
        c.dir[a] = up ? 1 : (down ? -1 : 0);
        // a face crossing needs the next layer of nodes, the point within its own cell, and a
        // cell wider than the stencil
        near = near && !(up && down) && f[a] >= 0.f && f[a] <= 1.f && (!up || ci[a] + 2 <= nn[a] - 1) &&
               (!down || ci[a] >= 1);
    }
    c.ok = inrange && inside;
    c.near = near && !inside;
    return c;
}

// A node's value as the FP32 paths read it: the FP32 node value, the FP16 brick decode, or the
// cell-corner array's copy (FP64 grids: its FP32 rounding).
__device__ __forceinline__ float node32(const GridDesc& g, int i, int j, int k) {
    if (g.b16) return brick_value32(g, i, j, k);
    const size_t idx = (size_t)i + (size_t)g.ni * ((size_t)j + (size_t)g.nj * (size_t)k);
    if (g.v32) return __ldg(g.v32 + idx);
    if (i < g.ni - 1 && j < g.nj - 1 && k < g.nk - 1)
        return __ldg(reinterpret_cast<const float*>(
            g.cells32 + 2 * ((size_t)i + (size_t)(g.ni - 1) * ((size_t)j + (size_t)(g.nj - 1) * k))));
    return (float)__ldg(g.v64 + idx);
}

// The reference's derivative stencil (BodySDFObj.cpp:176-205: gradient by central differences
// at +-eps, Hessian by second differences at +-eps and mixed ones at +-eps/2) where it crosses
// faces of the contact's cell, in closed form.  Along an axis the interpolant over two cells is
// the cell's multilinear polynomial plus r(t) D2, with r(t) the distance beyond the face (cell
// units) and D2 the nodes' second difference across it; in 3D the product of those 1D forms.  So
// the stencil's differences are the cell's analytic derivatives (computed by the caller) plus:
//   gradient a:  (r(t + d) - r(t - d)) M_a / (2 eps)
//   Hessian aa:  (r(t + d) + r(t - d)) M_a / eps^2
//   Hessian ab:  (dr_a 2 h_b dM_a/db + dr_b 2 h_a dM_b/da + dr_a dr_b M_ab) / eps^2
// with d = eps / dx, h = d / 2, dr = r(t + h) - r(t - h), M_a the second difference along a
// interpolated bilinearly at the point's other two coordinates, M_ab the product of the two
// second differences interpolated along the third.  The second differences are formed as
// differences of differences, (n0 - n1) - (n1 - n2): neighbouring node values are close, so the
// inner differences are exact or nearly so, where n0 - 2 n1 + n2 rounds at the larger value's
// exponent and the cancellation against n2 keeps that error (measured 1.75e-5 of the face terms on
// a curved grid, 5e-7 with the nested form).  The in-cell nodes come from the cell's FP32 corners
// already in registers, the others from the FP32 node reads (FP64 grids: their FP32 rounding, as
// the cell's own FP32 derivatives use).  The rest is products of small numbers, so FP32 keeps its
// relative precision where the FP64 differences of the reference cancel.  The distances beyond
// the faces come from the FP64 fractions (in FP64 where they are small, below).  Equal to the
// reference's stencil in exact arithmetic
// (checked against exact rational arithmetic on random cells).
struct FaceTerms {
    float g[3], h[6];
};
static __device__ __noinline__ FaceTerms cross_face_terms(const GridDesc& g, const FastCell& fc, Corners32 cc,
                                                          bool want_hessian) {
    const double fr[3] = {fc.ud, fc.vd, fc.wd};
    const int c0[3] = {fc.i, fc.j, fc.k};
    const float eps = (float)kFdEps;
    float t[3], rp[3], rm[3], hp[3], hm[3], hh[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        t[a] = (float)fr[a];
        hh[a] = 0.5f * eps * g.finv_dx[a];
        rp[a] = rm[a] = hp[a] = hm[a] = 0.f;  // r(t + d), r(t - d), r(t + h), r(t - h)
        if (fc.dir[a] != 0) {
            // the distances beyond the crossed face, r = d - (distance to the face) for the steps d
            // and d / 2: FP32 where r is at least d / 8, FP64 where it is smaller (the difference
            // cancels there, and FP32's absolute error 2^-24 d would be a large part of r)
            const float del = eps * g.finv_dx[a];
            const float dist = fc.dir[a] == 1 ? (float)(1.0 - fr[a]) : t[a];
            float r1 = del - dist, r2 = 0.5f * del - dist;
            const float lim = 0.125f * del;
            if ((r1 > -lim && r1 < lim) || (r2 > -lim && r2 < lim)) {
                const double d64 = kFdEps * g.inv_dx[a];
                const double off = fc.dir[a] == 1 ? fr[a] - 1.0 : -fr[a];
                r1 = (float)(d64 + off);
                r2 = (float)fma(0.5, d64, off);
            }
            r1 = fmaxf(r1, 0.f);
            r2 = fmaxf(r2, 0.f);
            if (fc.dir[a] == 1) {
                rp[a] = r1;
                hp[a] = r2;
            } else {
                rm[a] = r1;
                hm[a] = r2;
            }
        }
    }
    // the node at offsets o[0..2] (each in -1..2) from the cell's lowest corner
    auto node = [&](const int* o) -> float {
        if (o[0] >= 0 && o[0] <= 1 && o[1] >= 0 && o[1] <= 1 && o[2] >= 0 && o[2] <= 1)
            return cc.c[o[0] + 2 * o[1] + 4 * o[2]];
        return node32(g, c0[0] + o[0], c0[1] + o[1], c0[2] + o[2]);
    };
    // node offsets along axis a of the second difference across the crossed face: the node
    // beyond it, the face's node, the cell's other node
    auto across = [&](int a, int m) -> int { return fc.dir[a] == 1 ? 2 - m : m - 1; };
    // the second difference along axis a at offsets (ob, oc) of a's two other axes
    auto d2 = [&](int a, int ob, int oc) -> float {
        int o[3];
        o[a == 0 ? 1 : 0] = ob;
        o[a == 2 ? 1 : 2] = oc;
        float n[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            o[a] = across(a, m);
            n[m] = node(o);
        }
        return (n[0] - n[1]) - (n[1] - n[2]);
    };
    FaceTerms r;
    float Ma[3], dMa[3][2];  // M_a, and its derivatives along a's two other axes (cell units)
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        Ma[a] = dMa[a][0] = dMa[a][1] = 0.f;
        r.g[a] = 0.f;
        r.h[a] = 0.f;
        if (fc.dir[a] == 0) continue;
        const int b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;
        const float d00 = d2(a, 0, 0), d10 = d2(a, 1, 0), d01 = d2(a, 0, 1), d11 = d2(a, 1, 1);
        const float tb = t[b], tc = t[c];
        Ma[a] = (1.f - tc) * ((1.f - tb) * d00 + tb * d10) + tc * ((1.f - tb) * d01 + tb * d11);
        dMa[a][0] = (1.f - tc) * (d10 - d00) + tc * (d11 - d01);  // along b
        dMa[a][1] = (1.f - tb) * (d01 - d00) + tb * (d11 - d10);  // along c
        r.g[a] = (rp[a] - rm[a]) * Ma[a] / (2.f * eps);
        r.h[a] = (rp[a] + rm[a]) * Ma[a] / (eps * eps);
    }
    r.h[3] = r.h[4] = r.h[5] = 0.f;
    if (!want_hessian) return r;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int a = q < 2 ? 0 : 1, b = q == 0 ? 1 : 2, c = 3 - a - b;
        const float dra = hp[a] - hm[a], drb = hp[b] - hm[b];
        float s = 0.f;
        // dM_a along b: b is a's first other axis when b < c
        if (dra != 0.f) s += dra * 2.f * hh[b] * dMa[a][b < c ? 0 : 1];
        if (drb != 0.f) s += drb * 2.f * hh[a] * dMa[b][a < c ? 0 : 1];
        if (dra != 0.f && drb != 0.f) {
            float mab[2];
#pragma unroll
            for (int oc = 0; oc < 2; ++oc) {
                // the second difference along b of the second differences along a
                float e[3];
#pragma unroll
                for (int y = 0; y < 3; ++y) {
                    int o[3];
                    o[b] = across(b, y);
                    o[c] = oc;
                    float n[3];
#pragma unroll
                    for (int m = 0; m < 3; ++m) {
                        o[a] = across(a, m);
                        n[m] = node(o);
                    }
                    e[y] = (n[0] - n[1]) - (n[1] - n[2]);
                }
                mab[oc] = (e[0] - e[1]) - (e[1] - e[2]);
            }
            s += dra * drb * ((1.f - t[c]) * mab[0] + t[c] * mab[1]);
        }
        r.h[3 + q] = s / (eps * eps);
    }
    return r;
}

// A contact's grid-frame point and SDF jet from the exact path, computed ahead
// of contact_geometry by the whole warp (warp_exact_jets).
template <typename T>
struct ExactJet {
    V3 x;
    SdfJet<T> J;
    bool set;
};

// The exact path for the warp's contacts whose derivative stencil leaves their
// cell (`mine`): the reference-order grid point and depth, and the stencil
// derivatives with their 19 queries spread over the warp's lanes, one contact
// at a time, so that no lane walks a 19-query FP64 chain alone.  Must be called
// by all 32 lanes.  Results equal sdf_jet's on the exact path.
template <typename T>
__device__ inline void warp_exact_jets(const GridDesc& g, const PairState<T>& S, V3 xi, bool mine, bool want_hessian,
                                       ExactJet<T>& ej) {
    ej.set = false;
    V3 x = v3(0, 0, 0);
    bool stencil = false;
    if (mine) {
        x = grid_point(S.B.P.R, S.B.P.p, world_point(S.A.P.R, S.A.P.p, xi));
        // inside a cell the exact path takes the cell's own derivatives (sdf_jet)
        stencil = !(in_box(g, x) && stencil_in_cell(g, cell_of(g, x)));
    }
    unsigned m = __ballot_sync(0xffffffffu, stencil);
    const int lane = threadIdx.x & 31;
    while (m) {
        const int o = __ffs(m) - 1;
        m &= m - 1;
        const V3 xo = v3(__shfl_sync(0xffffffffu, x.x, o), __shfl_sync(0xffffffffu, x.y, o),
                         __shfl_sync(0xffffffffu, x.z, o));
        V3 gr;
        double hs[6], centre;
        sdf_stencil_warp(g, xo, gr, hs, want_hessian, centre);
        if (lane == o) {
            ej.set = true;
            ej.x = xo;
            ej.J.v = in_box(g, xo) ? centre : (double)FLT_MAX;
            ej.J.g = cast<T>(gr);
            for (int k = 0; k < 6; ++k) ej.J.h[k] = want_hessian ? (T)hs[k] : T(0);
        }
    }
}

// The contact point in the algebra type (from the FastCell's FP32 copy on the fast path).
template <typename T>
__device__ __forceinline__ Vec3<T> point_in(V3 xi, const FastCell* fc) {
    if constexpr (std::is_same<T, float>::value) {
        if (fc) return fc->xi32;
    }
    return cast<T>(xi);
}

// Grid-frame point, depth and SDF jet of one contact.
//   Exact path (T = double, the stencil mode, and contacts whose stencil
//   leaves the cell): the reference's operation order, bit-identical depth.
//   Fast path (T = float with a FastCell `fc` whose `ok` is set): the depth by
//   FP64 trilinear interpolation at the FastCell, the gradient / Hessian in
//   FP32; the depth then differs from the reference's by FP64 round-off only.
// x: the grid-frame point in the algebra type (on the fast path computed in FP32).
// `valid == false` marks a padding lane: the grid is not read and the result
// is discarded by the caller, but the lane still walks the same code so that
// warp collectives downstream see every lane.
// BR = false: specialised for grids without FP16 bricks (the caller guarantees it).
template <typename T, bool BR = true>
__device__ inline void contact_geometry(const GridDesc& g, const PairState<T>& S, V3 xi, const FastCell* fc,
                                        bool want_hessian, bool valid, bool stencil_only, Vec3<T>& x, double& d,
                                        SdfJet<T>& J, const ExactJet<T>* ej = nullptr) {
    if (!valid) {
        x = cast<T>(xi);
        d = -1.0;
        J.v = -1.0;
        J.g = vec3<T>(1, 0, 0);
        for (int k = 0; k < 6; ++k) J.h[k] = T(0);
        return;
    }
    if (ej && ej->set) {  // computed by the warp (warp_exact_jets)
        x = cast<T>(ej->x);
        J = ej->J;
        d = J.v + g.col_th;
        return;
    }
    if constexpr (std::is_same<T, float>::value) {
        if (fc && (fc->ok || fc->near) && !stencil_only) {
            const int i = fc->i, j = fc->j, k = fc->k;
            const double ud = fc->ud, vd = fc->vd, wd = fc->wd;
            double e[8];
            float cc[8];
            bool have32 = false;
            if constexpr (BR) {
                if (g.b16) {  // FP16 bricks: one decode serves both the depth (widened) and the derivatives
                    const Corners32 r = brick_corners32(g, i, j, k);
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        cc[q] = r.c[q];
                        e[q] = (double)cc[q];
                    }
                    have32 = true;
                } else if (g.v32) {  // FP32 node values: one set of loads serves both the depth and the derivatives
                    node_corners32(g, i, j, k, cc);
#pragma unroll
                    for (int q = 0; q < 8; ++q) e[q] = (double)cc[q];
                    have32 = true;
                } else {
                    cell_corners64(g, i, j, k, e);
                }
            } else {
                // (FP32 grids keep an FP64 copy: widening the FP32 corners here instead would put
                // eight conversions per contact on GB300's FP64 pipe, measured slower than the
                // eight FP64 gathers)
                plain_corners64(g, i, j, k, e);
            }
            const double e000 = e[0], e100 = e[1], e010 = e[2], e110 = e[3];
            const double e001 = e[4], e101 = e[5], e011 = e[6], e111 = e[7];
            const double q0 = fma(ud, e100 - e000, e000), q1 = fma(ud, e110 - e010, e010);
            const double q2 = fma(ud, e101 - e001, e001), q3 = fma(ud, e111 - e011, e011);
            const double r0 = fma(vd, q1 - q0, q0), r1 = fma(vd, q3 - q2, q2);
            J.v = fma(wd, r1 - r0, r0);
            x = fc->y;
            d = J.v + g.col_th;
            // FP32 analytic derivatives of the cell's interpolant
            const float u = (float)ud, v = (float)vd, w = (float)wd;
            if (!have32) {
                if constexpr (BR)
                    cell_corners32(g, i, j, k, cc);
                else
                    plain_corners32(g, i, j, k, cc);
            }
            const float c000 = cc[0], c100 = cc[1], c010 = cc[2], c110 = cc[3];
            const float c001 = cc[4], c101 = cc[5], c011 = cc[6], c111 = cc[7];
            const float a00 = c100 - c000, a10 = c110 - c010, a01 = c101 - c001, a11 = c111 - c011;
            const float b0 = fmaf(u, a00, c000), b1 = fmaf(u, a10, c010);
            const float b2 = fmaf(u, a01, c001), b3 = fmaf(u, a11, c011);
            const float gu = (1 - v) * ((1 - w) * a00 + w * a01) + v * ((1 - w) * a10 + w * a11);
            const float gv = (1 - w) * (b1 - b0) + w * (b3 - b2);
            const float gw = ((1 - v) * b2 + v * b3) - ((1 - v) * b0 + v * b1);
            const float ix = g.finv_dx[0], iy = g.finv_dx[1], iz = g.finv_dx[2];
            J.g = vec3<float>(gu * ix, gv * iy, gw * iz);
            if (want_hessian) {
                J.h[0] = J.h[1] = J.h[2] = 0.f;
                J.h[3] = ((1 - w) * (a10 - a00) + w * (a11 - a01)) * (ix * iy);
                J.h[4] = ((1 - v) * (a01 - a00) + v * (a11 - a10)) * (ix * iz);
                J.h[5] = ((b3 - b2) - (b1 - b0)) * (iy * iz);
            }
            if (fc->near) {  // the reference's stencil crosses faces: its extra terms in closed form
                Corners32 c8;
#pragma unroll
                for (int q = 0; q < 8; ++q) c8.c[q] = cc[q];
                const FaceTerms ft = cross_face_terms(g, *fc, c8, want_hessian);
                J.g = vec3<float>(J.g.x + ft.g[0], J.g.y + ft.g[1], J.g.z + ft.g[2]);
                if (want_hessian)
#pragma unroll
                    for (int q = 0; q < 6; ++q) J.h[q] += ft.h[q];
            }
            return;
        }
    }
    const V3 xe = grid_point(S.B.P.R, S.B.P.p, world_point(S.A.P.R, S.A.P.p, xi));
    sdf_jet(g, xe, J, want_hessian, stencil_only);
    x = cast<T>(xe);
    d = J.v + g.col_th;
}

// Penetration energy of one contact, e = kn d^2 / 2 with kn scaled as in the force law
// (ForceGeneralSDFContact.cpp:155-156) and d = SDF + col_th < 0 its depth, and its derivatives
// kn d dd/dq wrt the twist coordinates of body A (contact points) and body B (SDF), from the
// same jet as the force path: dd/dxw = R_B g, so for body A
//   w-rows: xi1 x (R_A^T R_B g),  v-rows: R_A^T R_B g,
// and for body B (dx/dq_B = [skew(x) | -I]):  w-rows: g x x,  v-rows: -g.
template <typename T>
struct ContactEnergy {
    double e;
    Vec3<T> aw, av, bw, bv;
};

template <typename T, bool BR = true>
__device__ inline ContactEnergy<T> contact_energy(const GridDesc& g, V3 xi1d, const PairState<T>& S, const FastCell* fc,
                                                  bool valid, bool stencil_only, const ExactJet<T>* ej = nullptr) {
    Vec3<T> x;
    double dd;
    SdfJet<T> J;
    contact_geometry<T, BR>(g, S, xi1d, fc, false, valid, stencil_only, x, dd, J, ej);
    ContactEnergy<T> E;
    const double kn = S.cp.kn;
    E.e = valid ? 0.5 * kn * dd * dd : 0.0;
    const T s = valid ? (T)(kn * dd) : T(0);
    const Vec3<T> gr = J.g;
    const Vec3<T> xi1 = point_in<T>(xi1d, fc);
    const Vec3<T> ga = mulT(S.R1, mul(S.R2, gr));
    E.av = s * ga;
    E.aw = s * cross(xi1, ga);
    E.bw = s * cross(gr, x);
    E.bv = -s * gr;
    return E;
}

// A coefficient in the algebra type: the FP64 value, or its FP32 rounding kept in ContactParams.
template <typename T>
__device__ __forceinline__ T fp_coef(double v, float v32) {
    if constexpr (std::is_same<T, float>::value)
        return v32;
    else
        return v;
}

// The force-law scalars s1 = -kn d + kd ddot d and sK = kn d - kd ddot d
// (ForceGeneralSDFContact.cpp:300, 328): in the reference's expression for the
// FP64 path, from the FP64 depth rounded once for the FP32 path.
template <typename T>
__device__ __forceinline__ void force_scalars(const ContactParams& cp, double dd, T ddot, T& s1, T& sK) {
    if constexpr (std::is_same<T, float>::value) {
        const float df = (float)dd;
        const float k = cp.kd32 * ddot - cp.kn32;
        s1 = df * k;
        sK = -s1;
    } else {
        s1 = -cp.kn * dd + cp.kd * ddot * dd;
        sK = cp.kn * dd - cp.kd * ddot * dd;
    }
}

// Static-friction test mu |fc| >= kt |tdot| - eps (ForceGeneralSDFContact.cpp:202, 365).
template <typename T>
__device__ __forceinline__ bool static_friction(const ContactParams& cp, T fc_norm, T tn) {
    if constexpr (std::is_same<T, float>::value)
        return cp.mu32 * fc_norm >= cp.kt32 * tn - (float)kFrictionEps;
    else
        return cp.mu * fc_norm >= cp.kt * tn - kFrictionEps;
}

// Value-only force of one active contact: fm = [Gamma1^T f1; Gamma2^T f2]
// (ForceGeneralSDFContact::computeForce, :147-219, with BodySDFObj::collision value form :239-274).
template <typename T>
struct ContactForce {
    Vec3<T> xi1, xi2, f1, f2;
};

template <typename T, bool BR = true>
__device__ inline ContactForce<T> contact_force(const GridDesc& g, V3 xi1d, const PairState<T>& S, const FastCell* fc,
                                                bool valid, bool stencil_only, const ExactJet<T>* ej = nullptr) {
    Vec3<T> x;
    double dd;
    SdfJet<T> J;
    contact_geometry<T, BR>(g, S, xi1d, fc, false, valid, stencil_only, x, dd, J, ej);
    const ContactParams& cp = S.cp;
    const Mat3<T>& R1 = S.R1;
    const Mat3<T>& R2 = S.R2;
    const Vec3<T> xi1 = point_in<T>(xi1d, fc);
    const Vec3<T> xw1d = mul(R1, cross(S.w1, xi1) + S.v1);  // R1 (skew(xi1)^T w1 + v1)
    const T gn = norm(J.g);
    const Vec3<T> e = vec3<T>(J.g.x / gn, J.g.y / gn, J.g.z / gn);
    const Vec3<T> n = mul(R2, e);
    const T d = (T)dd;
    const Vec3<T> xi2 = x - d * e;
    const Vec3<T> xdot = cross(x, S.w2) + mulT(R2, xw1d) - S.v2;
    const T ddot = dot(J.g, xdot);
    const Vec3<T> vw = xw1d - mul(R2, cross(S.w2, xi2) + S.v2);
    const Vec3<T> t = vw - dot(n, vw) * n;
    T s1, sK;
    force_scalars(cp, dd, ddot, s1, sK);
    const Vec3<T> rho1 = mulT(R1, n), rho2 = e;  // R2^T n = e
    ContactForce<T> F;
    F.xi1 = xi1;
    F.xi2 = xi2;
    F.f1 = s1 * rho1;
    F.f2 = sK * rho2;
    if (cp.friction) {
        const Vec3<T> c1 = cross(xi1, rho1);
        const T fc_norm = fabs(s1) * sqrt(dot(c1, c1) + dot(rho1, rho1));
        const T tn = norm(t);
        const Vec3<T> tau1 = mulT(R1, t), tau2 = mulT(R2, t);
        const T mu = fp_coef<T>(cp.mu, cp.mu32), kt = fp_coef<T>(cp.kt, cp.kt32);
        if (static_friction(cp, fc_norm, tn)) {
            F.f1 = F.f1 - kt * tau1;
            F.f2 = F.f2 + kt * tau2;
        } else {
            const T r = mu * fc_norm / tn;
            F.f1 = F.f1 - r * tau1;
            F.f2 = F.f2 + r * tau2;
        }
    }
    return F;
}

// Force plus Jacobian columns of one active contact
// (ForceGeneralSDFContact::computeForceWithDerivative, :221-447, with
// BodySDFObj::collision derivative form :278-377).
//
// sink.force(xi1, f1, xi2, f2) receives the force; then, for each of the 24
// columns c (0-5: dq1, 6-11: dq2 -> Km columns; 12-17: dphi1, 18-23: dphi2 ->
// Dm columns), sink.column(c, N1, N2, T2) receives the column's factors.
template <typename T, class Sink, bool BR = true>
__device__ inline void contact_force_jacobian(const GridDesc& g, V3 xi1d, const PairState<T>& S, const FastCell* fc,
                                              Sink& sink, bool valid, bool stencil_only,
                                              const ExactJet<T>* ej = nullptr, bool skip_q2 = false) {
    // collision, :292-310
    Vec3<T> x;
    double dd;
    SdfJet<T> J;
    contact_geometry<T, BR>(g, S, xi1d, fc, true, valid, stencil_only, x, dd, J, ej);
    const ContactParams& cp = S.cp;
    const Mat3<T>& R1 = S.R1;
    const Mat3<T>& R2 = S.R2;
    const Vec3<T>& w1 = S.w1;
    const Vec3<T>& v1 = S.v1;
    const Vec3<T>& w2 = S.w2;
    const Vec3<T>& v2 = S.v2;
    const Vec3<T> xi1 = point_in<T>(xi1d, fc);
    const T d = (T)dd;
    // kinematics of the contact point, :238-252
    const Vec3<T> u1 = cross(w1, xi1) + v1;  // skew(xi1)^T w1 + v1
    const Vec3<T> xw1d = mul(R1, u1);
    const Vec3<T> gr = J.g;
    const T gn = norm(gr);
    // FP32 path: the unit normal and de/dg through one reciprocal of |g|
    constexpr bool kRecip = std::is_same<T, float>::value;
    const T inv_gn = kRecip ? T(1) / gn : T(0);
    const Vec3<T> e = kRecip ? inv_gn * gr : vec3<T>(gr.x / gn, gr.y / gn, gr.z / gn);
    const Vec3<T> n = mul(R2, e);
    const Vec3<T> xi2 = x - d * e;
    const Vec3<T> xdot = cross(x, w2) + mulT(R2, xw1d) - v2;
    const T ddot = dot(gr, xdot);
    const Vec3<T> wxi = cross(w2, xi2) + v2;
    const Vec3<T> vw = xw1d - mul(R2, wxi);
    const T nvw = dot(n, vw);
    const Vec3<T> t = vw - nvw * n;

    // derivatives of the collision quantities wrt xw / xw_dot, :316-373
    Mat3<T> Hm;
    Hm.m[0] = J.h[0]; Hm.m[1] = J.h[3]; Hm.m[2] = J.h[4];
    Hm.m[3] = J.h[3]; Hm.m[4] = J.h[1]; Hm.m[5] = J.h[5];
    Hm.m[6] = J.h[4]; Hm.m[7] = J.h[5]; Hm.m[8] = J.h[2];
    Mat3<T> De;  // de/dg = (|g| I - g g^T / |g|) / |g|^2  (FP32 path: (I - e e^T) / |g|)
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            De.m[3 * r + c] = kRecip ? ((r == c ? T(1) : T(0)) - comp(e, r) * comp(e, c)) * inv_gn
                                     : (gn * (r == c ? T(1) : T(0)) - comp(gr, r) * comp(gr, c) / gn) / (gn * gn);
    const Mat3<T> de_dx = mul(De, Hm);
    const Mat3<T> R2T = transpose(R2);
    const Mat3<T> de_dxw = mul(de_dx, R2T);
    const Mat3<T> dn_dxw = mul(R2, de_dxw);
    const Vec3<T> dd_dxw = mul(R2, gr);  // row vector g^T R2^T
    Mat3<T> dxi2_dxw;  // R2^T - e dd_dxw^T - d de_dxw
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            dxi2_dxw.m[3 * r + c] = R2T.m[3 * r + c] - comp(e, r) * comp(dd_dxw, c) - d * de_dxw.m[3 * r + c];
    const Vec3<T> Hxdot = hess_mul(J.h, xdot);
    // dddot/dxw = (g^T skew(w2)^T + xdot^T H) R2^T, as a column vector R2 (w2 x g + H xdot)
    const Vec3<T> dddot_dxw = mul(R2, cross(w2, gr) + Hxdot);
    const Vec3<T> dddot_dxwd = dd_dxw;  // g^T R2^T
    Mat3<T> Sw;
    Sw.m[0] = 0; Sw.m[1] = -w2.z; Sw.m[2] = w2.y;
    Sw.m[3] = w2.z; Sw.m[4] = 0; Sw.m[5] = -w2.x;
    Sw.m[6] = -w2.y; Sw.m[7] = w2.x; Sw.m[8] = 0;
    const Mat3<T> R2Sw = mul(R2, Sw);
    const Mat3<T> dxw2d_dxw = mul(R2Sw, dxi2_dxw);  // dxw2dot/dxw = R2 skew(w2) dxi2_dxw
    // dtdot/dxw = -dxw2d_dxw - nvw dn_dxw - n (vw^T dn_dxw) + n n^T dxw2d_dxw
    const Vec3<T> vdn = mulT(dn_dxw, vw);
    const Vec3<T> ndx = mulT(dxw2d_dxw, n);
    Mat3<T> dt_dxw;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            dt_dxw.m[3 * r + c] = -dxw2d_dxw.m[3 * r + c] - nvw * dn_dxw.m[3 * r + c] - comp(n, r) * comp(vdn, c) +
                                  comp(n, r) * comp(ndx, c);
    // dtdot/dxw_dot = I - n n^T (applied as P v = v - n (n.v))

    // force-law scalars, :300-328 (the depth-dependent magnitudes from the FP64 depth)
    const T kn = fp_coef<T>(cp.kn, cp.kn32), kt = fp_coef<T>(cp.kt, cp.kt32), mu = fp_coef<T>(cp.mu, cp.mu32),
            kd = fp_coef<T>(cp.kd, cp.kd32);
    T s1, sK;
    force_scalars(cp, dd, ddot, s1, sK);
    const Vec3<T> rho1 = mulT(R1, n);
    const Vec3<T> rho2 = e;  // R2^T n
    const Vec3<T> xr1 = cross(xi1, rho1);
    Vec3<T> f1 = s1 * rho1, f2 = sK * rho2;

    const bool friction = cp.friction;
    T fc_norm = 0, tn = 0, ratio = 0;
    bool stat = true;
    Vec3<T> tau1 = vec3<T>(0, 0, 0), tau2 = vec3<T>(0, 0, 0);
    if (friction) {
        fc_norm = fabs(s1) * sqrt(dot(xr1, xr1) + dot(rho1, rho1));
        tn = norm(t);
        tau1 = mulT(R1, t);
        tau2 = mulT(R2, t);
        stat = static_friction(cp, fc_norm, tn);
        ratio = fc_norm / tn;
        if (stat) {
            f1 = f1 - kt * tau1;
            f2 = f2 + kt * tau2;
        } else {
            f1 = f1 - (mu * ratio) * tau1;
            f2 = f2 + (mu * ratio) * tau2;
        }
    }
    sink.force(xi1, f1, xi2, f2);
    // FP32 path: the friction columns' per-contact factors.  Sliding: al = cm (dfn - ratio dtn)
    // with cm = mu / tn, dfn = s1 (xr1.(xi1 x N1) + rho1.N1) / fc_norm, dtn = t.dt_j / tn, i.e.
    // al = fa (xr1.(xi1 x N1) + rho1.N1) - fb t.dt_j; static: al = 0, be = ga = kt.
    constexpr bool kFusedFriction = std::is_same<T, float>::value;
    const T cm = mu / tn;
    const T fa = stat ? T(0) : cm * s1 / fc_norm, fb = stat ? T(0) : cm * ratio / tn;
    const T be = stat ? kt : cm * fc_norm, ga = stat ? kt : mu * ratio;
    const T fr = fa * (dot(xr1, xr1) + dot(rho1, rho1));  // a Dm column's al per unit r
    const Mat3<T>& Q = S.Q;

    // One column's factors from its derivatives (dd_j, dddot_j, dn_j, dt_j, dxi2_j of the depth,
    // its rate, the normal, the tangential velocity and the body-B contact point along column c);
    // blk = c / 6 (0: dq1, 1: dq2 -> Km; 2: dphi1, 3: dphi2 -> Dm), j = c % 6, rot = j < 3.
    auto emit = [&](int c, int blk, bool rot, int j, T dd_j, T dddot_j, const Vec3<T>& dn_j, const Vec3<T>& dt_j,
                    const Vec3<T>& dxi2_j) {
        const bool kcol = blk < 2;  // Km column (dq) vs Dm column (dphi)
        Vec3<T> N1, N2, T2 = vec3<T>(0, 0, 0);
        if constexpr (kFusedFriction) {  // the FP32 path
            // body A's column first (without the terms of its own frame's rotation, N1p)
            Vec3<T> N1p;
            T r;
            if (kcol) {
                r = kn * dd_j - kd * dddot_j * d - kd * ddot * dd_j;
                N1p = -r * rho1 - sK * mulT(R1, dn_j);
                T2 = -sK * cross(rho2, dxi2_j);
            } else {
                r = kd * dddot_j * d;
                N1p = r * rho1;
            }
            if (friction) {
                // both regimes in one form, N1 -= al tau1 + be R1^T dt_j (+ ga tau1 x e_j), so that the
                // static and sliding contacts of a warp do not diverge (the sliding terms of the
                // reference form below, with cm = mu / tn distributed over the sum).  A Dm column
                // has N1 = r rho1, so there xr1.(xi1 x N1) + rho1.N1 = r (|xr1|^2 + |rho1|^2).
                T al;
                if (kcol) {
                    const Vec3<T> N1n = (blk == 0 && rot) ? N1p - sK * cross(rho1, unit<T>(j)) : N1p;
                    al = fa * (dot(xr1, cross(xi1, N1n)) + dot(rho1, N1n));
                } else {
                    al = fr * r;
                }
                al = al - fb * dot(t, dt_j);
                N1p = N1p - (al * tau1 + be * mulT(R1, dt_j));
                if (kcol) T2 = T2 - ga * cross(tau2, dxi2_j);
            }
            // the two bodies' world forces are opposite (R1 N1p = -R2 N2p): N2p = -Q^T N1p; then
            // each body's frame-rotation terms, (sK rho + ga tau) x e_j on body A's rotational
            // dq1 columns (subtracted) and body B's rotational dq2 columns (added)
            N2 = -mulT(Q, N1p);
            N1 = N1p;
            if (blk == 0 && rot) N1 = N1 - cross(sK * rho1 + ga * tau1, unit<T>(j));
            if (blk == 1 && rot) N2 = N2 + cross(sK * rho2 + ga * tau2, unit<T>(j));
            sink.column(c, N1, N2, T2);
            return;
        }
        // normal-force columns
        if (kcol) {
            T r = kn * dd_j - kd * dddot_j * d - kd * ddot * dd_j;
            N1 = -r * rho1 - sK * mulT(R1, dn_j);
            N2 = r * rho2 + sK * mulT(R2, dn_j);
            if (blk == 0 && rot) N1 = N1 - sK * cross(rho1, unit<T>(j));
            if (blk == 1 && rot) N2 = N2 + sK * cross(rho2, unit<T>(j));
            T2 = -sK * cross(rho2, dxi2_j);
        } else {
            T r = kd * dddot_j * d;
            N1 = r * rho1;
            N2 = -r * rho2;
        }
        if (friction) {
            // dfc_norm = fc1^T dfc1 / |fc1|, with dfc1 = Gamma1^T N1 and fc1 = s1 Gamma1^T rho1
            T dfn = s1 * (dot(xr1, cross(xi1, N1)) + dot(rho1, N1)) / fc_norm;
            T dtn = dot(t, dt_j) / tn;
            if (stat) {
                N1 = N1 - kt * mulT(R1, dt_j);
                N2 = N2 + kt * mulT(R2, dt_j);
                if (blk == 0 && rot) N1 = N1 - kt * cross(tau1, unit<T>(j));
                if (blk == 1 && rot) N2 = N2 + kt * cross(tau2, unit<T>(j));
                if (kcol) T2 = T2 - kt * cross(tau2, dxi2_j);
            } else {
                T cm = mu / tn;
                T s = dfn - ratio * dtn;
                N1 = N1 - cm * (s * tau1 + fc_norm * mulT(R1, dt_j));
                N2 = N2 + cm * (s * tau2 + fc_norm * mulT(R2, dt_j));
                if (blk == 0 && rot) N1 = N1 - (mu * ratio) * cross(tau1, unit<T>(j));
                if (blk == 1 && rot) N2 = N2 + (mu * ratio) * cross(tau2, unit<T>(j));
                if (kcol) T2 = T2 - (mu * ratio) * cross(tau2, dxi2_j);
            }
        }
        sink.column(c, N1, N2, T2);
    };
    const Vec3<T> zero3 = vec3<T>(0, 0, 0);

    // The column blocks run as separate loops, so that each block's intermediate matrices
    // die with its loop; each loop holds one copy of emit and of the sink's warp sums (the
    // kernel is sensitive to its code size).  dq1 and dphi1 go through the contact point:
    // dxw1/dq1 = [-R1 skew(xi1) | R1] = dxw1dot/dphi1, dxw1dot/dq1 = [-R1 skew(u1) | 0].
#pragma unroll 1
    for (int j = 0; j < 6; ++j) {  // dq1
        const Vec3<T> a = (j < 3) ? mul(R1, cross(unit<T>(j), xi1)) : col(R1, j - 3);
        const Vec3<T> b = (j < 3) ? mul(R1, cross(unit<T>(j), u1)) : vec3<T>(0, 0, 0);
        emit(j, 0, j < 3, j, dot(dd_dxw, a), dot(dddot_dxw, a) + dot(dddot_dxwd, b), mul(dn_dxw, a),
             mul(dt_dxw, a) + (b - dot(n, b) * n), mul(dxi2_dxw, a));
    }
    if (skip_q2) {
        // The dq2 columns of Km are derived by the caller (finalize_kernel) from the summed dq1
        // columns, and so are the dphi2 columns of Dm: the force depends on the velocities
        // through ddot and the relative velocity vw, and for a common world twist (rotation w
        // about the origin) of both bodies ddot is unchanged while vw gains
        // w x (xw1 - xw2) = w x (d n).  Hence Dm2 = -Dm1 Ad(E_A^{-1} E_B) + [C | 0], where
        // column j of C is the response to vw = d R2 (e_j x e) with ddot fixed (w = R2 e_j).
        // Iterations 0-5: the dphi1 columns; 6-8: C's columns, into the (unused) dq2
        // accumulators of Km.
#pragma unroll 1
        for (int j = 0; j < 9; ++j) {
            Vec3<T> dv;
            T dq;
            if (j < 6) {
                dv = (j < 3) ? mul(R1, cross(unit<T>(j), xi1)) : col(R1, j - 3);
                dq = dot(dddot_dxwd, dv);
            } else {
                dv = d * mul(R2, cross(unit<T>(j - 6), e));
                dq = T(0);
            }
            emit(j < 6 ? 12 + j : j, 2, false, j, T(0), dq, zero3, dv - dot(n, dv) * n, zero3);
        }
        return;
    }
    const Vec3<T> rxd = mulT(R2, xw1d);
#pragma unroll 1
    for (int j = 0; j < 6; ++j) {  // dq2: dx/dq2 = [skew(x) | -I]
        Vec3<T> dxj = (j < 3) ? cross(x, unit<T>(j)) : -unit<T>(j - 3);
        const T dd_j = dot(gr, dxj);
        Vec3<T> de_j = mul(de_dx, dxj);
        Vec3<T> dn_j = mul(R2, de_j);
        if (j < 3) dn_j = dn_j + mul(R2, cross(unit<T>(j), e));
        const Vec3<T> dxi2_j = dxj - dd_j * e - d * de_j;
        T dddot_j;
        if (j < 3) {
            // g^T(-Sw Sx + skew(R2^T xw_dot)) e_j + (H xdot)^T Sx e_j
            Vec3<T> sxe = cross(x, unit<T>(j));
            dddot_j = dot(gr, -cross(w2, sxe) + cross(rxd, unit<T>(j))) + dot(Hxdot, sxe);
        } else {
            dddot_j = dot(gr, cross(w2, unit<T>(j - 3))) - comp(Hxdot, j - 3);
        }
        // dxw2dot/dq2 = [-R2 skew(w2 x xi2 + v2) + R2 Sw dxi2_dq2.left | R2 Sw dxi2_dq2.right]
        Vec3<T> dxw2d_j = mul(R2Sw, dxi2_j);
        if (j < 3) dxw2d_j = dxw2d_j - mul(R2, cross(wxi, unit<T>(j)));
        // dtdot/dq2 = -dxw2d - nvw dn - n (vw.dn - n.dxw2d)
        const Vec3<T> dt_j = -dxw2d_j - nvw * dn_j - (dot(vw, dn_j) - dot(n, dxw2d_j)) * n;
        emit(6 + j, 1, j < 3, j, dd_j, dddot_j, dn_j, dt_j, dxi2_j);
    }
#pragma unroll 1
    for (int j = 0; j < 6; ++j) {  // dphi1
        const Vec3<T> a = (j < 3) ? mul(R1, cross(unit<T>(j), xi1)) : col(R1, j - 3);
        emit(12 + j, 2, j < 3, j, T(0), dot(dddot_dxwd, a), zero3, a - dot(n, a) * n, zero3);
    }
#pragma unroll 1
    for (int j = 0; j < 6; ++j) {  // dphi2
        T dddot_j;
        Vec3<T> q;
        if (j < 3) {
            dddot_j = dot(gr, cross(x, unit<T>(j)));
            q = mul(R2, cross(unit<T>(j), xi2));  // dxw2dot/dphi2 column R2 (e_j x xi2)
        } else {
            dddot_j = -comp(gr, j - 3);
            q = col(R2, j - 3);
        }
        emit(18 + j, 3, j < 3, j, T(0), dddot_j, zero3, -(q - dot(n, q) * n), zero3);
    }
}

}  // namespace sdfc
