// Signed distance grid of a closed triangle mesh on the GPU: sdfgen::make_level_set3
// (simulation/externals/sdfgen/makelevelset3.cpp:161-227) and the grid layout of
// BodySDFObj::precompute_SDF (simulation/redmax/Body/BodySDFObj.cpp:38-84), with results
// bit-identical to the reference's sequential FP32 code.
//
// The reference runs three phases; each maps to launches whose results do not depend on
// the order in which the GPU's threads run:
//
//   band       every triangle writes (distance, triangle) into the nodes of its bounding
//              box widened by exact_band, keeping the smaller distance; ties keep the lower
//              triangle index, which is what the reference's strict `d < phi` over triangles
//              in index order keeps.  Here each (node, triangle) pair is one thread and the
//              node keeps min over the packed key (distance bits << 32 | triangle): a
//              non-negative float's bits order like the float.  The same triangles count
//              their crossings of the grid's +i rays (one atomic add per crossing; sums are
//              order-free).  Work is cut into chunks of kLsChunk pairs, one warp each, so
//              that one large triangle spreads over many warps and small ones fill theirs.
//   sweeps     two passes of eight fast-sweeping orders.  In one order the node (i, j, k)
//              reads the closest triangle of its seven upwind neighbours, all of which come
//              earlier in the reference's loop.  One cooperative launch per order: a CTA per
//              k-plane walks the plane's diagonals, each diagonal's nodes in parallel, and
//              starts a diagonal only once the plane before it has passed that diagonal (a
//              bounded wait on a progress counter).  Each node sees exactly the neighbour
//              values the sequential loop would have shown it, so the result is the
//              sequential one.
//   sign       per grid row (j, k) the running crossing count's parity flips the sign
//              (one warp per row, parity prefix by ballot).
//
// Arithmetic: FP32 distances and FP64 grid coordinates as in the reference, which is
// compiled without contraction; this file is compiled with -fmad=false so that no
// multiply-add is fused either.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <climits>
#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

#include "sdfc.h"
#include "sdfc_internal.h"

namespace {

constexpr int kLsThreads = 128;   // threads per CTA of the band kernel
constexpr int kLsChunk = 256;     // (node, triangle) pairs per band warp
constexpr int kLsSweepThreads = 1024;  // 128 nodes of a diagonal per pass
constexpr int kLsMinSlab = 1;     // planes per sweep slab, at least
constexpr unsigned kNoTri = 0xffffffffu;

struct LsGrid {
    float ox, oy, oz;  // origin (node 0, 0, 0)
    float dx, dy, dz;
    int ni, nj, nk;
    __host__ __device__ size_t at(int i, int j, int k) const {
        return (size_t)i + (size_t)ni * ((size_t)j + (size_t)nj * (size_t)k);
    }
    // Vec3f gx(i*dx+origin[0], j*dy+origin[1], k*dz+origin[2])
    __device__ float3 node(int i, int j, int k) const {
        return make_float3((float)i * dx + ox, (float)j * dy + oy, (float)k * dz + oz);
    }
};

// Per-triangle band work (written by ls_plan_kernel).
struct LsPlan {
    int i0, j0, k0, ni, nj, nk;  // band box: first node and extents
    int cj0, ck0, cnj, cnk;      // crossing box in (j, k)
    long long first_chunk;
    int chunks;
};

__device__ __forceinline__ float3 ld_vert(const float* __restrict__ v, unsigned q) {
    return make_float3(v[3 * (size_t)q], v[3 * (size_t)q + 1], v[3 * (size_t)q + 2]);
}

__device__ __forceinline__ float3 f3sub(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float f3dot(float3 a, float3 b) {
    float d = a.x * b.x;
    d += a.y * b.y;
    d += a.z * b.z;
    return d;
}
// dist(a, b) of sdfgen vec.h: sqrt of the squared differences summed in index order
__device__ __forceinline__ float f3dist(float3 a, float3 b) {
    float d = (a.x - b.x) * (a.x - b.x);
    d += (a.y - b.y) * (a.y - b.y);
    d += (a.z - b.z) * (a.z - b.z);
    return sqrtf(d);
}
__device__ __forceinline__ float fmin_std(float a, float b) { return b < a ? b : a; }  // std::min

// point_segment_distance (makelevelset3.cpp:8-20).  The reference divides the float dot
// product by the float squared length in FP64 and rounds the quotient to float.  Double
// rounding of a quotient of floats through a format of p' >= 2p + 2 bits is innocuous
// (Figueroa, "When is double rounding innocuous?", 1995): the result is the correctly rounded
// float quotient, so one IEEE FP32 division gives the same bits without the FP64 unit.
__device__ float ls_seg(float3 x0, float3 x1, float3 x2) {
    const float3 dx = f3sub(x2, x1);
    const float m2 = f3dot(dx, dx);
    float s12 = __fdiv_rn(f3dot(f3sub(x2, x0), dx), m2);
    if (s12 < 0)
        s12 = 0;
    else if (s12 > 1)
        s12 = 1;
    const float t = 1 - s12;
    const float3 p = make_float3(s12 * x1.x + t * x2.x, s12 * x1.y + t * x2.y, s12 * x1.z + t * x2.z);
    return f3dist(x0, p);
}

// point_triangle_distance (makelevelset3.cpp:23-54)
__device__ float ls_tri(float3 x0, float3 x1, float3 x2, float3 x3) {
    const float3 x13 = f3sub(x1, x3), x23 = f3sub(x2, x3), x03 = f3sub(x0, x3);
    const float m13 = f3dot(x13, x13), m23 = f3dot(x23, x23), d = f3dot(x13, x23);
    const float den = m13 * m23 - d * d;
    const float invdet = 1.f / (den < 1e-30f ? 1e-30f : den);
    const float a = f3dot(x13, x03), b = f3dot(x23, x03);
    const float w23 = invdet * (m23 * a - d * b);
    const float w31 = invdet * (m13 * b - d * a);
    const float w12 = 1 - w23 - w31;
    if (w23 >= 0 && w31 >= 0 && w12 >= 0) {
        // w23*x1 + w31*x2 + w12*x3, summed left to right
        const float3 p = make_float3(w23 * x1.x + w31 * x2.x + w12 * x3.x, w23 * x1.y + w31 * x2.y + w12 * x3.y,
                                     w23 * x1.z + w31 * x2.z + w12 * x3.z);
        return f3dist(x0, p);
    }
    if (w23 > 0) return fmin_std(ls_seg(x0, x1, x2), ls_seg(x0, x1, x3));
    if (w31 > 0) return fmin_std(ls_seg(x0, x1, x2), ls_seg(x0, x2, x3));
    return fmin_std(ls_seg(x0, x1, x3), ls_seg(x0, x2, x3));
}

// orientation (makelevelset3.cpp:97-113): sign of the doubled area, ties broken by
// simulation of simplicity
__device__ int ls_orient(double x1, double y1, double x2, double y2, double& area) {
    area = y1 * x2 - x1 * y2;
    if (area > 0) return 1;
    if (area < 0) return -1;
    if (y2 > y1) return 1;
    if (y2 < y1) return -1;
    if (x1 > x2) return 1;
    if (x1 < x2) return -1;
    return 0;
}

// point_in_triangle_2d (makelevelset3.cpp:118-134)
__device__ bool ls_in_tri(double x0, double y0, double x1, double y1, double x2, double y2, double x3, double y3,
                          double& a, double& b, double& c) {
    x1 -= x0;
    x2 -= x0;
    x3 -= x0;
    y1 -= y0;
    y2 -= y0;
    y3 -= y0;
    const int sa = ls_orient(x2, y2, x3, y3, a);
    if (sa == 0) return false;
    const int sb = ls_orient(x3, y3, x1, y1, b);
    if (sb != sa) return false;
    const int sc = ls_orient(x1, y1, x2, y2, c);
    if (sc != sa) return false;
    const double sum = a + b + c;
    a /= sum;
    b /= sum;
    c /= sum;
    return true;
}

__device__ __forceinline__ int clampi(int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); }
// sdfgen::min / max of three: min(a1, min(a2, a3)) with std::min / std::max
__device__ __forceinline__ double dmin_std(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double dmax_std(double a, double b) { return a < b ? b : a; }
__device__ __forceinline__ double min3d(double a, double b, double c) { return dmin_std(a, dmin_std(b, c)); }
__device__ __forceinline__ double max3d(double a, double b, double c) { return dmax_std(a, dmax_std(b, c)); }

// The triangle's grid coordinates fi = ((double)x - origin) / dx per vertex.
struct TriGrid {
    double fi[3], fj[3], fk[3];
};

__device__ TriGrid tri_grid(const float* __restrict__ verts, const unsigned* __restrict__ tris, unsigned t,
                            const LsGrid& g) {
    TriGrid r;
    for (int m = 0; m < 3; ++m) {
        const float3 x = ld_vert(verts, tris[3 * (size_t)t + m]);
        r.fi[m] = ((double)x.x - g.ox) / g.dx;
        r.fj[m] = ((double)x.y - g.oy) / g.dy;
        r.fk[m] = ((double)x.z - g.oz) / g.dz;
    }
    return r;
}

__global__ void ls_init_kernel(unsigned long long* __restrict__ key, int* __restrict__ count, size_t n,
                               unsigned long long init_key) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        key[q] = init_key;
        count[q] = 0;
    }
}

// One thread per triangle: its band box and crossing box (makelevelset3.cpp:173-208),
// and its range of band chunks.
__global__ void ls_plan_kernel(const float* __restrict__ verts, const unsigned* __restrict__ tris, int nt, LsGrid g,
                               int band, LsPlan* __restrict__ plan, unsigned long long* __restrict__ total) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool valid = t < nt;
    const TriGrid c = tri_grid(verts, tris, valid ? (unsigned)t : 0u, g);
    LsPlan p;
    const int i0 = clampi((int)min3d(c.fi[0], c.fi[1], c.fi[2]) - band, 0, g.ni - 1);
    const int i1 = clampi((int)max3d(c.fi[0], c.fi[1], c.fi[2]) + band + 1, 0, g.ni - 1);
    const int j0 = clampi((int)min3d(c.fj[0], c.fj[1], c.fj[2]) - band, 0, g.nj - 1);
    const int j1 = clampi((int)max3d(c.fj[0], c.fj[1], c.fj[2]) + band + 1, 0, g.nj - 1);
    const int k0 = clampi((int)min3d(c.fk[0], c.fk[1], c.fk[2]) - band, 0, g.nk - 1);
    const int k1 = clampi((int)max3d(c.fk[0], c.fk[1], c.fk[2]) + band + 1, 0, g.nk - 1);
    p.i0 = i0;
    p.j0 = j0;
    p.k0 = k0;
    p.ni = i1 - i0 + 1;
    p.nj = j1 - j0 + 1;
    p.nk = k1 - k0 + 1;
    const int cj0 = clampi((int)ceil(min3d(c.fj[0], c.fj[1], c.fj[2])), 0, g.nj - 1);
    const int cj1 = clampi((int)floor(max3d(c.fj[0], c.fj[1], c.fj[2])), 0, g.nj - 1);
    const int ck0 = clampi((int)ceil(min3d(c.fk[0], c.fk[1], c.fk[2])), 0, g.nk - 1);
    const int ck1 = clampi((int)floor(max3d(c.fk[0], c.fk[1], c.fk[2])), 0, g.nk - 1);
    p.cj0 = cj0;
    p.ck0 = ck0;
    p.cnj = cj1 >= cj0 ? cj1 - cj0 + 1 : 0;
    p.cnk = ck1 >= ck0 ? ck1 - ck0 + 1 : 0;
    // with i0 <= i1 etc. always (clamped), the band box is never empty
    const long long work = (long long)p.ni * p.nj * p.nk + (long long)p.cnj * p.cnk;
    p.chunks = valid ? (int)((work + kLsChunk - 1) / kLsChunk) : 0;
    // the warp's chunk ranges: one atomic per warp, inclusive scan over the lanes
    long long incl = p.chunks;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    unsigned long long base = 0;
    if (lane == 31) base = atomicAdd(total, (unsigned long long)incl);
    base = __shfl_sync(0xffffffffu, base, 31);
    p.first_chunk = (long long)base + incl - p.chunks;
    if (valid) plan[t] = p;
}

// chunk -> triangle map (one thread per triangle writes its chunks)
__global__ void ls_chunk_map_kernel(const LsPlan* __restrict__ plan, int nt, int* __restrict__ chunk_tri) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const LsPlan p = plan[t];
    for (int c = 0; c < p.chunks; ++c) chunk_tri[p.first_chunk + c] = t;
}

// One warp per chunk of kLsChunk (node, triangle) pairs, kLsThreads / 32 chunks per CTA: band
// distances (makelevelset3.cpp:180-189) and crossing counts (makelevelset3.cpp:191-207).
__global__ void __launch_bounds__(kLsThreads) ls_band_kernel(const float* __restrict__ verts,
                                                             const unsigned* __restrict__ tris, LsGrid g,
                                                             const LsPlan* __restrict__ plan,
                                                             const int* __restrict__ chunk_tri,
                                                             unsigned long long* __restrict__ key,
                                                             int* __restrict__ count, float init,
                                                             long long chunks) {
    const long long chunk = (long long)blockIdx.x * (kLsThreads / 32) + (threadIdx.x >> 5);
    if (chunk >= chunks) return;
    const int t = chunk_tri[chunk];
    const LsPlan p = plan[t];
    const long long base = (chunk - p.first_chunk) * kLsChunk;
    const long long vol = (long long)p.ni * p.nj * p.nk;
    const long long work = vol + (long long)p.cnj * p.cnk;
    const unsigned q0 = tris[3 * (size_t)t], q1 = tris[3 * (size_t)t + 1], q2 = tris[3 * (size_t)t + 2];
    const float3 xp = ld_vert(verts, q0), xq = ld_vert(verts, q1), xr = ld_vert(verts, q2);
    for (int u = threadIdx.x & 31; u < kLsChunk; u += 32) {
        const long long w = base + u;
        if (w >= work) break;
        if (w < vol) {
            const int li = (int)(w % p.ni);
            const long long rest = w / p.ni;
            const int lj = (int)(rest % p.nj), lk = (int)(rest / p.nj);
            const int i = p.i0 + li, j = p.j0 + lj, k = p.k0 + lk;
            const float d = ls_tri(g.node(i, j, k), xp, xq, xr);
            if (d < init)  // also drops NaN, which never passes the reference's `d < phi`
                atomicMin(&key[g.at(i, j, k)], ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)t);
        } else {
            const long long v = w - vol;
            const int j = p.cj0 + (int)(v % p.cnj), k = p.ck0 + (int)(v / p.cnj);
            const TriGrid c = tri_grid(verts, tris, (unsigned)t, g);
            double a, b, cc;
            if (ls_in_tri((double)j, (double)k, c.fj[0], c.fk[0], c.fj[1], c.fk[1], c.fj[2], c.fk[2], a, b, cc)) {
                const double fi = a * c.fi[0] + b * c.fi[1] + cc * c.fi[2];
                const int iv = (int)ceil(fi);
                if (iv < 0)
                    atomicAdd(&count[g.at(0, j, k)], 1);
                else if (iv < g.ni)
                    atomicAdd(&count[g.at(iv, j, k)], 1);
            }
        }
    }
}

// key -> (phi, closest)
__global__ void ls_unpack_kernel(const unsigned long long* __restrict__ key, float* __restrict__ phi,
                                 int* __restrict__ closest, size_t n, float init) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long k = key[q];
        const unsigned t = (unsigned)(k & 0xffffffffu);
        if (t == kNoTri) {
            phi[q] = init;
            closest[q] = -1;
        } else {
            phi[q] = __uint_as_float((unsigned)(k >> 32));
            closest[q] = (int)t;
        }
    }
}

// Triangle vertices gathered per triangle, three float4 each: x1 y1 z1 x2 | y2 z2 x3 y3 | z3 - - -
__global__ void ls_soup_kernel(const float* __restrict__ verts, const unsigned* __restrict__ tris, int nt,
                               float4* __restrict__ soup) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nt) return;
    const float3 a = ld_vert(verts, tris[3 * (size_t)t]), b = ld_vert(verts, tris[3 * (size_t)t + 1]),
                 c = ld_vert(verts, tris[3 * (size_t)t + 2]);
    soup[3 * (size_t)t] = make_float4(a.x, a.y, a.z, b.x);
    soup[3 * (size_t)t + 1] = make_float4(b.y, b.z, c.x, c.y);
    soup[3 * (size_t)t + 2] = make_float4(c.z, 0.f, 0.f, 0.f);
}

__device__ __forceinline__ float ls_tri_soup(const float4* __restrict__ soup, int t, float3 x0) {
    const float4 a = __ldg(soup + 3 * (size_t)t), b = __ldg(soup + 3 * (size_t)t + 1),
                 c = __ldg(soup + 3 * (size_t)t + 2);
    return ls_tri(x0, make_float3(a.x, a.y, a.z), make_float3(a.w, b.x, b.y), make_float3(b.z, b.w, c.x));
}

// The sweep step of node (i, j, k) in order (di, dj, dk) (makelevelset3.cpp:75-94 with
// check_neighbour, :56-71), by a group of 8 lanes: lane e < 7 takes the reference's e-th
// neighbour, (i-di,j,k) (i,j-dj,k) (i-di,j-dj,k) (i,j,k-dk) (i-di,j,k-dk) (i,j-dj,k-dk)
// (i-di,j-dj,k-dk), i.e. offsets by the bits of e + 1.  The candidates' distances do not depend
// on phi, so the lanes evaluate them at once; the comparisons then run in the reference's
// order over shuffles.  A candidate equal to the node's own triangle or to an earlier
// candidate cannot pass `d < phi` (phi is at most that triangle's distance from the same
// node position, the same bits) and is not evaluated.
//
// Plane k and, unless prev_remote, plane k - dk belong to the calling CTA's slab: only it
// writes them during the launch, so plain (L1-cached) loads see its own stores.  A plane
// k - dk of another slab is read through L2 (ld.global.cg): its lines may sit in this SM's L1
// from before that slab finished them.  All 32 lanes of the warp call this (valid = false for
// lanes without a node).
__device__ __forceinline__ void ls_sweep_node8(const float4* __restrict__ soup, const LsGrid& g, float* phi,
                                               int* closest, bool valid, int i, int j, int k, int di, int dj,
                                               int dk, bool prev_remote) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, e = lane & 7, gbase = lane & ~7;
    const int f = e + 1;
    int ct = -1, own = -1;
    float phi0 = 0.f;
    size_t self = 0;
    if (valid) {
        self = g.at(i, j, k);
        own = closest[self];
        phi0 = phi[self];
        if (e < 7) {
            const size_t q = g.at(i - ((f & 1) ? di : 0), j - ((f & 2) ? dj : 0), k - ((f & 4) ? dk : 0));
            ct = (prev_remote && (f & 4)) ? __ldcg(closest + q) : closest[q];
        }
    }
    bool use = ct >= 0 && ct != own;
#pragma unroll
    for (int e2 = 0; e2 < 7; ++e2) {
        const int v = __shfl_sync(full, ct, gbase + e2);
        if (e2 < e && v == ct) use = false;
    }
    float d = use ? ls_tri_soup(soup, ct, g.node(i, j, k)) : INFINITY;
    // The reference's comparisons in order (replace when d < phi) keep the smallest distance and,
    // among equal ones, the earliest candidate, and keep the node's own only if no candidate is
    // strictly smaller: an arg-min over the 8 lanes ordered by (distance, lane), then one test.
    // Unused candidates carry +inf (a used NaN distance never passes `d < phi`: it is dropped
    // too, as the ordered tree below would otherwise rank it).
    if (d != d) d = INFINITY;
    int at = e;
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        const float d2 = __shfl_xor_sync(full, d, o);
        const int a2 = __shfl_xor_sync(full, at, o);
        if (d2 < d || (d2 == d && a2 < at)) {
            d = d2;
            at = a2;
        }
    }
    const int best_ct = __shfl_sync(full, ct, gbase + at);
    if (valid && e == 0 && d < phi0) {
        phi[self] = d;
        closest[self] = best_ct;
    }
}

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Bound on the polls of one wait (each at least ~0.3 us): about a second.
constexpr long kLsSpinLimit = 1L << 22;
// Polls without sleeping first (a plane usually waits for one diagonal of its neighbour).
constexpr long kLsSpinFast = 1L << 12;

// One sweep order over slabs of planes.  With sweep-relative indices (a, b, c) (a = i - 1 for
// di > 0, ni - 2 - i for di < 0, likewise b, c), CTA s owns the planes c in [s P, s P + P) and
// walks the slab's diagonals M = a + b + (c - s P) in order, each diagonal's nodes in parallel,
// a __syncthreads between diagonals.  Node (a, b, c) reads nodes of plane c on diagonals M - 1,
// M - 2 and of plane c - 1 on M - 1, M - 2, M - 3: for the slab's first plane those lie in slab
// s - 1, on its diagonals up to M + P - 1, so the slab starts diagonal M once progress[s - 1]
// (slab s - 1's finished diagonals) reaches M + P.  Every node therefore reads what the
// reference's loop (c, b, a ascending) would have shown it.  Needs all CTAs resident
// (cooperative launch); every wait is bounded: after spin_limit polls the CTA sets *err and
// returns, and the others see *err and return.  need_extra (0 in use) is added to every awaited
// progress value: a test sets it beyond any slab's diagonals so that every wait runs out.
__global__ void __launch_bounds__(kLsSweepThreads, 1) ls_sweep_slabs_kernel(const float4* __restrict__ soup,
                                                                       LsGrid g, float* phi, int* closest, int di,
                                                                       int dj, int dk, int P, int* progress,
                                                                       int* err, long spin_limit, int need_extra) {
    __shared__ int s_seen;
    const int A = g.ni - 2, B = g.nj - 2, planes = g.nk - 1;
    const int s = blockIdx.x;
    const int c0 = s * P;
    if (c0 >= planes) return;
    const int np = min(P, planes - c0);
    const int steps = A + B + np;       // diagonals of this slab
    const int prev_steps = A + B + P;   // diagonals of slab s - 1 (always a full slab)
    const bool signal = c0 + np < planes;
    int seen = s == 0 ? INT_MAX : 0;
    for (int M = 0; M < steps; ++M) {
        const int need = min(M + P, prev_steps) + need_extra;
        if (seen < need) {  // uniform over the CTA
            if (threadIdx.x == 0) {
                int v;
                long it = 0;
                while ((v = ld_acquire_gpu(progress + s - 1)) < need) {
                    if (ld_acquire_gpu(err) != 0) {
                        v = -1;
                        break;
                    }
                    if (++it > spin_limit) {
                        atomicExch(err, 1);
                        v = -1;
                        break;
                    }
                    if (it > kLsSpinFast) __nanosleep(64);  // back off only on long waits
                }
                s_seen = v;
            }
            __syncthreads();
            seen = s_seen;
            if (seen < 0) return;
        }
        // nodes of diagonal M: planes cl in [cl_lo, cl_hi], in each a in [a_lo, a_hi]; a group
        // of 8 lanes per node, kLsSweepThreads / 8 nodes per pass
        const int cl_lo = max(0, M - A - B), cl_hi = min(np - 1, M);
        int total = 0;
        for (int cl = cl_lo; cl <= cl_hi; ++cl) {
            const int m = M - cl;
            total += min(A, m) - max(0, m - B) + 1;
        }
        for (int base = 0; base < total; base += kLsSweepThreads / 8) {
            const int t = base + (int)(threadIdx.x >> 3);
            int cl = cl_lo, a = -1;
            if (t < total) {
                int rest = t;
                for (; cl <= cl_hi; ++cl) {
                    const int m = M - cl;
                    const int a_lo = max(0, m - B), cnt = min(A, m) - a_lo + 1;
                    if (rest < cnt) {
                        a = a_lo + rest;
                        break;
                    }
                    rest -= cnt;
                }
            }
            const bool valid = a >= 0;
            const int b = M - cl - a;
            const int c = c0 + cl;
            const int i = di > 0 ? a + 1 : g.ni - 2 - a;
            const int j = dj > 0 ? b + 1 : g.nj - 2 - b;
            const int k = dk > 0 ? c + 1 : g.nk - 2 - c;
            ls_sweep_node8(soup, g, phi, closest, valid, i, j, k, di, dj, dk, cl == 0 && s > 0);
        }
        __syncthreads();
        if (signal && threadIdx.x == 0) st_release_gpu(progress + s, M + 1);
    }
}

// One warp per row (j, k): negate where the running crossing count is odd
// (makelevelset3.cpp:214-226).
__global__ void ls_sign_kernel(float* __restrict__ phi, const int* __restrict__ count, LsGrid g, int rows) {
    const int lane = threadIdx.x & 31;
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (row >= rows) return;
    const size_t base = (size_t)row * g.ni;
    unsigned carry = 0;
    for (int i0 = 0; i0 < g.ni; i0 += 32) {
        const int i = i0 + lane;
        const unsigned odd = i < g.ni ? (unsigned)(count[base + i] & 1) : 0u;
        const unsigned bal = __ballot_sync(0xffffffffu, odd);
        const unsigned upto = bal & (0xffffffffu >> (31 - lane));
        const unsigned par = (carry + __popc(upto)) & 1u;
        if (i < g.ni && par) phi[base + i] = -phi[base + i];
        carry = (carry + __popc(bal)) & 1u;
    }
}

int ls_check(sdfc_context* ctx, int nv, const unsigned* tris_host, int nt, int ni, int nj, int nk, int band) {
    if (nv < 0 || nt < 0 || ni < 1 || nj < 1 || nk < 1 || band < 0)
        return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "make_level_set3: bad sizes");
    if ((double)ni * nj * nk > 4.0e9)
        return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "make_level_set3: grid too large");
    if (tris_host)
        for (size_t q = 0; q < 3 * (size_t)nt; ++q)
            if (tris_host[q] >= (unsigned)nv)
                return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "make_level_set3: vertex index out of range");
    return SDFC_OK;
}

// The level set from device arrays, on the context's stream.
int ls_run(sdfc_context* ctx, const float* d_verts, const unsigned* d_tris, int nt, const float origin[3], float dx,
           float dy, float dz, int ni, int nj, int nk, int band, float* d_phi, cudaStream_t st) {
    const LsGrid g{origin[0], origin[1], origin[2], dx, dy, dz, ni, nj, nk};
    const size_t n = (size_t)ni * nj * nk;
    // phi.assign((ni+nj+nk)*(dx+dy+dz))
    const float init = (float)(ni + nj + nk) * (dx + dy + dz);
    // an untouched node's key: above every (distance, triangle) key, its triangle field kNoTri
    const unsigned long long init_key = ~0ull;
    unsigned long long* d_key = nullptr;
    int* d_count = nullptr;
    int* d_closest = nullptr;
    LsPlan* d_plan = nullptr;
    unsigned long long* d_total = nullptr;
    int* d_chunk_tri = nullptr;
    float4* d_soup = nullptr;
    int* d_progress = nullptr;
    int rc = SDFC_OK;
    auto cleanup = [&]() {
        for (void* p : {(void*)d_key, (void*)d_count, (void*)d_closest, (void*)d_plan, (void*)d_total,
                        (void*)d_chunk_tri, (void*)d_soup, (void*)d_progress})
            if (p) cudaFreeAsync(p, st);
    };
#define LS_TRY(call)                                                                                          \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess) {                                                                              \
            cleanup();                                                                                        \
            return sdfc_impl::fail(ctx, SDFC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
        }                                                                                                     \
    } while (0)
    LS_TRY(cudaMallocAsync((void**)&d_key, sizeof(unsigned long long) * n, st));
    LS_TRY(cudaMallocAsync((void**)&d_count, sizeof(int) * n, st));
    LS_TRY(cudaMallocAsync((void**)&d_closest, sizeof(int) * n, st));
    LS_TRY(cudaMallocAsync((void**)&d_plan, sizeof(LsPlan) * std::max(nt, 1), st));
    LS_TRY(cudaMallocAsync((void**)&d_total, sizeof(unsigned long long), st));
    LS_TRY(cudaMemsetAsync(d_total, 0, sizeof(unsigned long long), st));
    const int fill_blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)sdfc::device_sm_count() * 16);
    ls_init_kernel<<<fill_blocks, 256, 0, st>>>(d_key, d_count, n, init_key);
    LS_TRY(cudaGetLastError());
    unsigned long long total = 0;
    if (nt > 0) {
        ls_plan_kernel<<<(nt + 127) / 128, 128, 0, st>>>(d_verts, d_tris, nt, g, band, d_plan, d_total);
        LS_TRY(cudaGetLastError());
        LS_TRY(cudaMemcpyAsync(&total, d_total, sizeof(total), cudaMemcpyDeviceToHost, st));
        LS_TRY(cudaStreamSynchronize(st));
    }
    if (total > (unsigned long long)INT32_MAX) {
        cleanup();
        return sdfc_impl::fail(ctx, SDFC_ERR_CAPACITY, "make_level_set3: band work exceeds 2^31 chunks");
    }
    if (total > 0) {
        LS_TRY(cudaMallocAsync((void**)&d_chunk_tri, sizeof(int) * total, st));
        ls_chunk_map_kernel<<<(nt + 127) / 128, 128, 0, st>>>(d_plan, nt, d_chunk_tri);
        LS_TRY(cudaGetLastError());
        const unsigned band_blocks = (unsigned)((total + kLsThreads / 32 - 1) / (kLsThreads / 32));
        ls_band_kernel<<<band_blocks, kLsThreads, 0, st>>>(d_verts, d_tris, g, d_plan, d_chunk_tri, d_key,
                                                           d_count, init, (long long)total);
        LS_TRY(cudaGetLastError());
    }
    ls_unpack_kernel<<<fill_blocks, 256, 0, st>>>(d_key, d_phi, d_closest, n, init);
    LS_TRY(cudaGetLastError());
    if (ni >= 2 && nj >= 2 && nk >= 2 && nt > 0) {
        static const int dirs[8][3] = {{1, 1, 1},  {-1, -1, -1}, {1, 1, -1},  {-1, -1, 1},
                                       {1, -1, 1}, {-1, 1, -1},  {1, -1, -1}, {-1, 1, 1}};
        const int planes = nk - 1;
        LS_TRY(cudaMallocAsync((void**)&d_soup, sizeof(float4) * 3 * (size_t)nt, st));
        LS_TRY(cudaMallocAsync((void**)&d_progress, sizeof(int) * ((size_t)planes + 1), st));
        int* d_err = d_progress + planes;
        LS_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
        ls_soup_kernel<<<(nt + 127) / 128, 128, 0, st>>>(d_verts, d_tris, nt, d_soup);
        LS_TRY(cudaGetLastError());
        int dev = 0, sms = 0, per_sm = 0;
        LS_TRY(cudaGetDevice(&dev));
        LS_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        LS_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ls_sweep_slabs_kernel, kLsSweepThreads, 0));
        if (per_sm < 1) {
            cleanup();
            return sdfc_impl::fail(ctx, SDFC_ERR_CUDA, "make_level_set3: sweep kernel cannot be resident");
        }
        // slabs of P planes, one CTA each, all resident
        const int capacity = sms * per_sm;
        const char* slab_env = std::getenv("SDFC_LS_SLAB");  // tuning knob: planes per slab
        const int min_slab = slab_env ? std::max(1, std::atoi(slab_env)) : kLsMinSlab;
        const int P = std::max(min_slab, (planes + capacity - 1) / capacity);
        const int slabs = (planes + P - 1) / P;
        LsGrid gg = g;
        float* a_phi = d_phi;
        int* a_closest = d_closest;
        int aP = P;
        // SDFC_TEST_EXPIRE_SWEEP_WAITS (tests of the failure path only): every wait awaits a
        // progress no slab reaches and gives up after a short spin, so the call must report it
        long spin_limit = kLsSpinLimit;
        int need_extra = 0;
        if (std::getenv("SDFC_TEST_EXPIRE_SWEEP_WAITS")) {
            spin_limit = 1000;
            need_extra = 1 << 30;
        }
        for (int pass = 0; pass < 2; ++pass)
            for (int s = 0; s < 8; ++s) {
                int di = dirs[s][0], dj = dirs[s][1], dk = dirs[s][2];
                LS_TRY(cudaMemsetAsync(d_progress, 0, sizeof(int) * planes, st));
                void* args[] = {(void*)&d_soup, (void*)&gg, (void*)&a_phi,  (void*)&a_closest,
                                (void*)&di,     (void*)&dj, (void*)&dk,     (void*)&aP,
                                (void*)&d_progress, (void*)&d_err, (void*)&spin_limit, (void*)&need_extra};
                LS_TRY(cudaLaunchCooperativeKernel((const void*)ls_sweep_slabs_kernel, dim3(slabs),
                                                   dim3(kLsSweepThreads), args, 0, st));
            }
        int h_err = 0;
        LS_TRY(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
        LS_TRY(cudaStreamSynchronize(st));
        if (h_err) {
            cleanup();
            return sdfc_impl::fail(ctx, SDFC_ERR_CUDA, "make_level_set3: a sweep wait timed out");
        }
    }
    const int rows = nj * nk;
    ls_sign_kernel<<<(rows + 7) / 8, 256, 0, st>>>(d_phi, d_count, g, rows);
    LS_TRY(cudaGetLastError());
    cleanup();
#undef LS_TRY
    return rc;
}

}  // namespace

extern "C" {

int sdfc_make_level_set3_device(sdfc_context* ctx, const float* d_verts, int nv, const unsigned* d_tris, int nt,
                                const float origin[3], float dx, float dy, float dz, int ni, int nj, int nk,
                                int exact_band, float* d_phi, void* stream) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (!origin || (!d_phi) || (nt > 0 && (!d_verts || !d_tris)))
        return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "make_level_set3: null pointer");
    int rc = ls_check(ctx, nv, nullptr, nt, ni, nj, nk, exact_band);
    if (rc) return rc;
    if ((rc = sdfc_impl::use_device(ctx))) return rc;
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return ls_run(ctx, d_verts, d_tris, nt, origin, dx, dy, dz, ni, nj, nk, exact_band, d_phi, st);
}

int sdfc_make_level_set3(sdfc_context* ctx, const float* verts, int nv, const unsigned* tris, int nt,
                         const float origin[3], float dx, float dy, float dz, int ni, int nj, int nk, int exact_band,
                         float* phi) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (!origin || !phi || (nt > 0 && (!verts || !tris)))
        return sdfc_impl::fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "make_level_set3: null pointer");
    int rc = ls_check(ctx, nv, tris, nt, ni, nj, nk, exact_band);
    if (rc) return rc;
    if ((rc = sdfc_impl::use_device(ctx))) return rc;
    cudaStream_t st = ctx->stream;
    const size_t n = (size_t)ni * nj * nk;
    float* d_v = nullptr;
    unsigned* d_t = nullptr;
    float* d_phi = nullptr;
    auto release = [&]() {
        for (void* p : {(void*)d_v, (void*)d_t, (void*)d_phi})
            if (p) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
    };
#define LSH_TRY(call)                                                                                         \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess) {                                                                              \
            release();                                                                                        \
            return sdfc_impl::fail(ctx, SDFC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
        }                                                                                                     \
    } while (0)
    LSH_TRY(cudaMallocAsync((void**)&d_v, sizeof(float) * 3 * (size_t)std::max(nv, 1), st));
    LSH_TRY(cudaMallocAsync((void**)&d_t, sizeof(unsigned) * 3 * (size_t)std::max(nt, 1), st));
    LSH_TRY(cudaMallocAsync((void**)&d_phi, sizeof(float) * n, st));
    if (nv > 0) LSH_TRY(cudaMemcpyAsync(d_v, verts, sizeof(float) * 3 * (size_t)nv, cudaMemcpyHostToDevice, st));
    if (nt > 0) LSH_TRY(cudaMemcpyAsync(d_t, tris, sizeof(unsigned) * 3 * (size_t)nt, cudaMemcpyHostToDevice, st));
    rc = ls_run(ctx, d_v, d_t, nt, origin, dx, dy, dz, ni, nj, nk, exact_band, d_phi, st);
    if (rc) {
        release();
        return rc;
    }
    LSH_TRY(cudaMemcpyAsync(phi, d_phi, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    LSH_TRY(cudaStreamSynchronize(st));
    release();
#undef LSH_TRY
    return SDFC_OK;
}

int sdfc_sdf_grid_layout(const double* V, int nv, double dx, int res, int shape[3], double min_box[3],
                         double max_box[3], double spacing[3], float origin_f[3]) {
    if (!V || nv < 1 || res < 1 || !(dx > 0) || !shape || !min_box || !max_box || !spacing)
        return SDFC_ERR_INVALID_ARGUMENT;
    // min_box / max_box: sdfgen::update_minmax over the float vertices in order
    // (simulation/externals/sdfgen/util.h:140-144).  Its `else if` skips the max test for a
    // vertex that lowered the min, so the first vertex never raises the max and the box can
    // miss extreme vertices; the reference's grid is that box, kept as is.
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    double bmn[3], bmx[3];  // Body::_bounding_box of the FP64 vertices
    for (int a = 0; a < 3; ++a) bmn[a] = bmx[a] = V[a];
    for (int v = 0; v < nv; ++v)
        for (int a = 0; a < 3; ++a) {
            const double x = V[3 * (size_t)v + a];
            const float xf = (float)x;
            if (xf < mn[a])
                mn[a] = xf;
            else if (xf > mx[a])
                mx[a] = xf;
            bmn[a] = std::min(bmn[a], x);
            bmx[a] = std::max(bmx[a], x);
        }
    double h[3];
    for (int a = 0; a < 3; ++a) h[a] = std::min(dx, (bmx[a] - bmn[a]) / res);
    for (int a = 0; a < 3; ++a) {
        const float unit = (float)h[a];
        mn[a] -= 1.0f * unit;  // padding = 1
        mx[a] += 1.0f * unit;
    }
    for (int a = 0; a < 3; ++a) {
        const float num = (mx[a] - mn[a]) + (float)(0.5 * h[a]);
        const float q = num / (float)h[a];
        if (!(q >= 0) || q > 4.0e9f) return SDFC_ERR_INVALID_ARGUMENT;
        shape[a] = (int)((unsigned)q + 1u);
        min_box[a] = (double)mn[a];
        max_box[a] = (double)mx[a];
        spacing[a] = h[a];
        if (origin_f) origin_f[a] = mn[a];
    }
    return SDFC_OK;
}

}  // extern "C"
