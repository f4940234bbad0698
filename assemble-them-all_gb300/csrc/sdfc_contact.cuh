// Device-side point-vs-SDF contact math for sm_103a.
//
// Restates, for one active contact, the reference redmax computation
//   BodySDFObj::collision              simulation/redmax/Body/BodySDFObj.cpp:239-377
//   ForceGeneralSDFContact::computeForce[WithDerivative](contacts, ...)
//                                      simulation/redmax/Force/ForceGeneralSDFContact.cpp:147-447
// in FP64, but organised for a GPU thread:
//   * the SDF gradient / Hessian are the analytic derivatives of the trilinear
//     interpolant of the point's cell.  Inside a cell these equal the
//     reference's central differences (step 1e-5, BodySDFObj.cpp:176-205) up to
//     FP64 round-off; when any stencil point of those differences leaves the
//     cell or the box, the exact 26-query stencil is evaluated instead, so the
//     result follows the reference in every case;
//   * every 6x6 block of Km/Dm is written as Gamma^T N (Gamma = [skew(xi)^T, I],
//     simulation/redmax/Utils.h:196): the body-A rows of the contact's Jacobian
//     columns are [xi1 x N1_j; N1_j] and the body-B rows are
//     [xi2 x N2_j + T2_j; N2_j], with N1_j, N2_j, T2_j 3-vectors per column j.
//     The 24 columns (q1, q2, phi1, phi2) are produced one at a time and handed
//     to a sink, so a thread never holds a 12x12 block.
#pragma once

#include <cfloat>
#include <cstdint>

namespace sdfc {

// ---------------------------------------------------------------- small vectors
struct V3 {
    double x, y, z;
};
__device__ __forceinline__ V3 v3(double a, double b, double c) { return {a, b, c}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double norm(V3 a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ double comp(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
__device__ __forceinline__ V3 unit(int k) { return {k == 0 ? 1.0 : 0.0, k == 1 ? 1.0 : 0.0, k == 2 ? 1.0 : 0.0}; }

// 3x3 row-major
struct M3 {
    double m[9];
};
__device__ __forceinline__ V3 mul(const M3& A, V3 v) {
    return {A.m[0] * v.x + A.m[1] * v.y + A.m[2] * v.z, A.m[3] * v.x + A.m[4] * v.y + A.m[5] * v.z,
            A.m[6] * v.x + A.m[7] * v.y + A.m[8] * v.z};
}
__device__ __forceinline__ V3 mulT(const M3& A, V3 v) {  // A^T v
    return {A.m[0] * v.x + A.m[3] * v.y + A.m[6] * v.z, A.m[1] * v.x + A.m[4] * v.y + A.m[7] * v.z,
            A.m[2] * v.x + A.m[5] * v.y + A.m[8] * v.z};
}
__device__ __forceinline__ V3 col(const M3& A, int c) { return {A.m[c], A.m[3 + c], A.m[6 + c]}; }
__device__ __forceinline__ M3 mul(const M3& A, const M3& B) {
    M3 C;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            C.m[3 * r + c] = A.m[3 * r] * B.m[c] + A.m[3 * r + 1] * B.m[3 + c] + A.m[3 * r + 2] * B.m[6 + c];
    return C;
}
__device__ __forceinline__ M3 transpose(const M3& A) {
    return {{A.m[0], A.m[3], A.m[6], A.m[1], A.m[4], A.m[7], A.m[2], A.m[5], A.m[8]}};
}

// ---------------------------------------------------------------- grids and poses
// An SDF grid as the reference's BodySDFObj holds it (BodySDFObj.h:13-16), values
// indexed [i + ni*(j + nj*k)] (simulation/externals/sdfgen/array3.h:70-79).
struct GridDesc {
    int ni, nj, nk;
    int storage;  // 0 = FP64 values, 1 = FP32 values
    double min_box[3], max_box[3], dx[3];
    double col_th;
    const double* v64;   // storage 0
    const float* v32;    // FP32 copy: always present (prefilter); the values for storage 1
    float fmin[3], fmax[3], finv_dx[3];  // FP32 prefilter constants
    float lip;        // bound on |grad| of the interpolant over the grid
    float vmax;       // max |value|
};

struct PointsDesc {
    int n;
    int storage;       // 0 = FP64 SoA, 1 = FP32 SoA
    const float* x32;  // FP32 SoA copy (x[n], y[n], z[n]); exact when storage == 1
    const double* x64; // FP64 SoA (storage 0 only)
    float radius;      // max |xi|
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

__device__ __forceinline__ double grid_value(const GridDesc& g, int i, int j, int k) {
    size_t idx = (size_t)i + (size_t)g.ni * ((size_t)j + (size_t)g.nj * (size_t)k);
    return g.storage == 0 ? g.v64[idx] : (double)__ldg(g.v32 + idx);
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

// Trilinear interpolation of the cell containing x (x inside the box), the
// inside branch of BodySDFObj::query_SDF (BodySDFObj.cpp:130-155), in the
// reference's operation order.  Cell indices are clamped to the grid; the
// grid check at upload guarantees the reference's index arithmetic stays in
// range, so the clamp changes nothing.
__device__ __forceinline__ double trilinear(const GridDesc& g, V3 x) {
    double ci = sub_rn(x.x, g.min_box[0]) / g.dx[0];
    double cj = sub_rn(x.y, g.min_box[1]) / g.dx[1];
    double ck = sub_rn(x.z, g.min_box[2]) / g.dx[2];
    int i = (int)floor(ci), j = (int)floor(cj), k = (int)floor(ck);
    ci = sub_rn(ci, (double)i);
    cj = sub_rn(cj, (double)j);
    ck = sub_rn(ck, (double)k);
    i = min(max(i, 0), g.ni - 1);
    j = min(max(j, 0), g.nj - 1);
    k = min(max(k, 0), g.nk - 1);
    int ip = (i == g.ni - 1) ? i : i + 1;
    int jp = (j == g.nj - 1) ? j : j + 1;
    int kp = (k == g.nk - 1) ? k : k + 1;
    double v00 = lerp_ref(ci, grid_value(g, i, j, k), grid_value(g, ip, j, k));
    double v10 = lerp_ref(ci, grid_value(g, i, jp, k), grid_value(g, ip, jp, k));
    double v01 = lerp_ref(ci, grid_value(g, i, j, kp), grid_value(g, ip, j, kp));
    double v11 = lerp_ref(ci, grid_value(g, i, jp, kp), grid_value(g, ip, jp, kp));
    double vk0 = lerp_ref(cj, v00, v10);
    double vk1 = lerp_ref(cj, v01, v11);
    return lerp_ref(ck, vk0, vk1);
}

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

// Value, gradient and Hessian of the SDF at x, following the reference's
// query_SDF / query_dSDF / query_ddSDF.  Returns the value query_SDF(x, false).
struct SdfJet {
    double v;      // query_SDF(x) (FLT_MAX outside the box)
    V3 g;          // query_dSDF(x)
    double h[6];   // query_ddSDF(x): xx, yy, zz, xy, xz, yz
    bool stencil;  // true when the exact 26-query stencil was used
};

constexpr double kFdEps = 1e-5;  // BodySDFObj.cpp:178,191

__device__ __forceinline__ bool same_cell(double xa, double mn, double mx, double dx, int cell, int n) {
    // The FD stencil point xa stays inside the box and in `cell` (and `cell`
    // is not the clamped top cell).
    if (!(xa >= mn && xa <= mx)) return false;
    int c = (int)floor((xa - mn) / dx);
    return c == cell && cell < n - 1;
}

__device__ inline void sdf_stencil(const GridDesc& g, V3 x, SdfJet& J, bool want_hessian) {
    // Exact reference stencil, BodySDFObj.cpp:176-205.
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
    J.g = v3((gp[0] - gm[0]) / (2 * e), (gp[1] - gm[1]) / (2 * e), (gp[2] - gm[2]) / (2 * e));
    J.stencil = true;
    if (!want_hessian) return;
    double xs = query_sdf(g, x, true);
    const double ee = e * e;
#pragma unroll
    for (int a = 0; a < 3; ++a) J.h[a] = sub_rn(add_rn(gp[a], gm[a]), mul_rn(2.0, xs)) / ee;
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
        J.h[3 + q] = s / ee;
    }
}

// stencil_only = true evaluates the reference's 26-query stencil for every
// point (bit-identical SDF derivatives); otherwise the analytic cell
// derivatives are used wherever the stencil stays inside one cell.
__device__ inline void sdf_jet(const GridDesc& g, V3 x, SdfJet& J, bool want_hessian, bool stencil_only = false) {
    J.v = query_sdf(g, x, false);
    if (!stencil_only && in_box(g, x)) {
        double cx = (x.x - g.min_box[0]) / g.dx[0];
        double cy = (x.y - g.min_box[1]) / g.dx[1];
        double cz = (x.z - g.min_box[2]) / g.dx[2];
        int i = (int)floor(cx), j = (int)floor(cy), k = (int)floor(cz);
        const double e = kFdEps;
        bool interior = same_cell(x.x + e, g.min_box[0], g.max_box[0], g.dx[0], i, g.ni) &&
                        same_cell(x.x - e, g.min_box[0], g.max_box[0], g.dx[0], i, g.ni) &&
                        same_cell(x.y + e, g.min_box[1], g.max_box[1], g.dx[1], j, g.nj) &&
                        same_cell(x.y - e, g.min_box[1], g.max_box[1], g.dx[1], j, g.nj) &&
                        same_cell(x.z + e, g.min_box[2], g.max_box[2], g.dx[2], k, g.nk) &&
                        same_cell(x.z - e, g.min_box[2], g.max_box[2], g.dx[2], k, g.nk);
        if (interior) {
            // analytic derivatives of the cell's trilinear interpolant
            double u = cx - i, v = cy - j, w = cz - k;
            double c000 = grid_value(g, i, j, k), c100 = grid_value(g, i + 1, j, k);
            double c010 = grid_value(g, i, j + 1, k), c110 = grid_value(g, i + 1, j + 1, k);
            double c001 = grid_value(g, i, j, k + 1), c101 = grid_value(g, i + 1, j, k + 1);
            double c011 = grid_value(g, i, j + 1, k + 1), c111 = grid_value(g, i + 1, j + 1, k + 1);
            double a00 = c100 - c000, a10 = c110 - c010, a01 = c101 - c001, a11 = c111 - c011;  // d/du
            double b0 = (1 - u) * c000 + u * c100, b1 = (1 - u) * c010 + u * c110;              // along v
            double b2 = (1 - u) * c001 + u * c101, b3 = (1 - u) * c011 + u * c111;
            double gu = (1 - v) * ((1 - w) * a00 + w * a01) + v * ((1 - w) * a10 + w * a11);
            double gv = (1 - w) * (b1 - b0) + w * (b3 - b2);
            double gw = ((1 - v) * b2 + v * b3) - ((1 - v) * b0 + v * b1);
            J.g = v3(gu / g.dx[0], gv / g.dx[1], gw / g.dx[2]);
            if (want_hessian) {
                J.h[0] = J.h[1] = J.h[2] = 0.0;
                J.h[3] = ((1 - w) * (a10 - a00) + w * (a11 - a01)) / (g.dx[0] * g.dx[1]);
                J.h[4] = ((1 - v) * (a01 - a00) + v * (a11 - a10)) / (g.dx[0] * g.dx[2]);
                J.h[5] = ((b3 - b2) - (b1 - b0)) / (g.dx[1] * g.dx[2]);
            }
            J.stencil = false;
            return;
        }
    }
    sdf_stencil(g, x, J, want_hessian);
}

__device__ __forceinline__ V3 hess_mul(const double* h, V3 v) {
    return {h[0] * v.x + h[3] * v.y + h[4] * v.z, h[3] * v.x + h[1] * v.y + h[5] * v.z,
            h[4] * v.x + h[5] * v.y + h[2] * v.z};
}

// ---------------------------------------------------------------- per-contact force
struct ContactParams {
    double kn, kt, mu, kd;  // kn, kt already scaled by scale * contact_scale (ForceGeneralSDFContact.cpp:155-156)
};

constexpr double kFrictionEps = 1e-8;  // constants::eps, simulation/redmax/Utils.h:9

struct BodyState {
    Pose P;
    V3 w, v;  // phi = (w, v), body frame
};

// Value-only force of one active contact: fm = [Gamma1^T f1; Gamma2^T f2]
// (ForceGeneralSDFContact::computeForce, :147-219, with BodySDFObj::collision value form :239-274).
struct ContactForce {
    V3 xi1, xi2, f1, f2;
};

// `valid == false` marks a padding lane: the grid is not read and the result is
// discarded by the caller, but the lane still walks the same code so that warp
// collectives downstream see every lane.
__device__ __forceinline__ void jet_or_pad(const GridDesc& g, V3 x, SdfJet& J, bool want_hessian, bool valid,
                                           bool stencil_only) {
    if (valid) {
        sdf_jet(g, x, J, want_hessian, stencil_only);
    } else {
        J.v = -1.0;
        J.g = v3(1.0, 0.0, 0.0);
        for (int k = 0; k < 6; ++k) J.h[k] = 0.0;
        J.stencil = false;
    }
}

__device__ inline ContactForce contact_force(const GridDesc& g, V3 xi1, const BodyState& A, const BodyState& B,
                                      const ContactParams& cp, bool valid = true, bool stencil_only = false) {
    V3 xw1 = world_point(A.P.R, A.P.p, xi1);
    V3 u1 = cross(A.w, xi1) + A.v;  // skew(xi1)^T w1 + v1
    V3 xw1d = mul(A.P.R, u1);
    V3 x = grid_point(B.P.R, B.P.p, xw1);
    SdfJet J;
    jet_or_pad(g, x, J, false, valid, stencil_only);
    double d = J.v + g.col_th;
    double gn = norm(J.g);
    V3 e = v3(J.g.x / gn, J.g.y / gn, J.g.z / gn);
    V3 n = mul(B.P.R, e);
    V3 xi2 = x - d * e;
    V3 xdot = cross(x, B.w) + mulT(B.P.R, xw1d) - B.v;
    double ddot = dot(J.g, xdot);
    V3 xw2d = mul(B.P.R, cross(B.w, xi2) + B.v);
    V3 vw = xw1d - xw2d;
    V3 t = vw - dot(n, vw) * n;
    double s1 = -cp.kn * d + cp.kd * ddot * d;
    double sK = cp.kn * d - cp.kd * ddot * d;
    V3 rho1 = mulT(A.P.R, n), rho2 = e;  // R2^T n = e
    ContactForce F;
    F.xi1 = xi1;
    F.xi2 = xi2;
    F.f1 = s1 * rho1;
    F.f2 = sK * rho2;
    if (cp.mu > kFrictionEps) {
        V3 c1 = cross(xi1, rho1);
        double fc_norm = fabs(s1) * sqrt(dot(c1, c1) + dot(rho1, rho1));
        double tn = norm(t);
        V3 tau1 = mulT(A.P.R, t), tau2 = mulT(B.P.R, t);
        if (cp.mu * fc_norm >= cp.kt * tn - kFrictionEps) {
            F.f1 = F.f1 - cp.kt * tau1;
            F.f2 = F.f2 + cp.kt * tau2;
        } else {
            double r = cp.mu * fc_norm / tn;
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
template <class Sink>
__device__ inline void contact_force_jacobian(const GridDesc& g, V3 xi1, const BodyState& A, const BodyState& B,
                                       const ContactParams& cp, Sink& sink, bool valid = true,
                                       bool stencil_only = false) {
    const M3& R1 = A.P.R;
    const M3& R2 = B.P.R;
    // kinematics of the contact point, :238-252
    V3 xw1 = world_point(R1, A.P.p, xi1);
    V3 u1 = cross(A.w, xi1) + A.v;
    V3 xw1d = mul(R1, u1);
    // collision, :292-310
    V3 x = grid_point(R2, B.P.p, xw1);
    SdfJet J;
    jet_or_pad(g, x, J, true, valid, stencil_only);
    const double d = J.v + g.col_th;
    const V3 gr = J.g;
    const double gn = norm(gr);
    const V3 e = v3(gr.x / gn, gr.y / gn, gr.z / gn);
    const V3 n = mul(R2, e);
    const V3 xi2 = x - d * e;
    const V3 xdot = cross(x, B.w) + mulT(R2, xw1d) - B.v;
    const double ddot = dot(gr, xdot);
    const V3 wxi = cross(B.w, xi2) + B.v;
    const V3 xw2d = mul(R2, wxi);
    const V3 vw = xw1d - xw2d;
    const double nvw = dot(n, vw);
    const V3 t = vw - nvw * n;

    // derivatives of the collision quantities wrt xw / xw_dot, :316-373
    // de/dx = (I - e e^T) H / |g|
    M3 Hm;
    Hm.m[0] = J.h[0]; Hm.m[1] = J.h[3]; Hm.m[2] = J.h[4];
    Hm.m[3] = J.h[3]; Hm.m[4] = J.h[1]; Hm.m[5] = J.h[5];
    Hm.m[6] = J.h[4]; Hm.m[7] = J.h[5]; Hm.m[8] = J.h[2];
    M3 De;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            De.m[3 * r + c] = (gn * (r == c ? 1.0 : 0.0) - comp(gr, r) * comp(gr, c) / gn) / (gn * gn);
    const M3 de_dx = mul(De, Hm);
    const M3 R2T = transpose(R2);
    const M3 de_dxw = mul(de_dx, R2T);
    const M3 dn_dxw = mul(R2, de_dxw);
    const V3 dd_dxw = mul(R2, gr);  // row vector g^T R2^T
    // dxi2/dxw = R2^T - e dd_dxw^T - d de_dxw
    M3 dxi2_dxw;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            dxi2_dxw.m[3 * r + c] = R2T.m[3 * r + c] - comp(e, r) * comp(dd_dxw, c) - d * de_dxw.m[3 * r + c];
    const V3 Hxdot = hess_mul(J.h, xdot);
    // dddot/dxw = (g^T skew(w2)^T + xdot^T H) R2^T ; as a column vector R2 (skew(w2) g + H xdot)
    const V3 dddot_dxw = mul(R2, cross(B.w, gr) + Hxdot);
    const V3 dddot_dxwd = dd_dxw;  // g^T R2^T
    // dxw2dot/dxw = R2 skew(w2) dxi2_dxw
    M3 Sw;
    Sw.m[0] = 0; Sw.m[1] = -B.w.z; Sw.m[2] = B.w.y;
    Sw.m[3] = B.w.z; Sw.m[4] = 0; Sw.m[5] = -B.w.x;
    Sw.m[6] = -B.w.y; Sw.m[7] = B.w.x; Sw.m[8] = 0;
    const M3 R2Sw = mul(R2, Sw);
    const M3 dxw2d_dxw = mul(R2Sw, dxi2_dxw);
    // dtdot/dxw = -dxw2d_dxw - nvw dn_dxw - n (vw^T dn_dxw) + n n^T dxw2d_dxw
    const V3 vdn = mulT(dn_dxw, vw);
    const V3 ndx = mulT(dxw2d_dxw, n);
    M3 dt_dxw;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            dt_dxw.m[3 * r + c] = -dxw2d_dxw.m[3 * r + c] - nvw * dn_dxw.m[3 * r + c] - comp(n, r) * comp(vdn, c) +
                                  comp(n, r) * comp(ndx, c);
    // dtdot/dxw_dot = I - n n^T (applied as P v = v - n (n.v))

    // force-law scalars, :300-328
    const double kn = cp.kn, kt = cp.kt, mu = cp.mu, kd = cp.kd;
    const double s1 = -kn * d + kd * ddot * d;
    const double sK = kn * d - kd * ddot * d;
    const V3 rho1 = mulT(R1, n);
    const V3 rho2 = e;
    const V3 xr1 = cross(xi1, rho1);
    V3 f1 = s1 * rho1, f2 = sK * rho2;

    const bool friction = mu > kFrictionEps;
    double fc_norm = 0.0, tn = 0.0, ratio = 0.0;
    bool stat = true;
    V3 tau1 = v3(0, 0, 0), tau2 = v3(0, 0, 0);
    if (friction) {
        fc_norm = fabs(s1) * sqrt(dot(xr1, xr1) + dot(rho1, rho1));
        tn = norm(t);
        tau1 = mulT(R1, t);
        tau2 = mulT(R2, t);
        stat = mu * fc_norm >= kt * tn - kFrictionEps;
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

    // q2-column ingredients (collision derivatives wrt the SDF body's pose)
    //   dx_dq2 = [skew(x) | -I]
    //   dn_dq2[:,j] = R2 de_dx dx_dq2[:,j] (+ R2 (e_j x e), j<3)
    //   dddot_dq2 (row) = g^T(-Sw Sx + skew(R2^T xw_dot)) + (H xdot)^T Sx | g^T Sw - (H xdot)^T
    const V3 rxd = mulT(R2, xw1d);

#pragma unroll 1
    for (int c = 0; c < 24; ++c) {
        const int blk = c / 6, j = c % 6;
        const bool kcol = blk < 2;  // Km column (dq) vs Dm column (dphi)
        double dd_j = 0.0, dddot_j = 0.0;
        V3 dn_j = v3(0, 0, 0), dt_j = v3(0, 0, 0), dxi2_j = v3(0, 0, 0);
        if (blk == 0 || blk == 2) {
            // through the contact point: dxw1/dq1 = [-R1 skew(xi1) | R1] = dxw1dot/dphi1,
            // dxw1dot/dq1 = [-R1 skew(u1) | 0]
            V3 a = (j < 3) ? mul(R1, cross(unit(j), xi1)) : col(R1, j - 3);  // -R1 skew(xi1) e_j = R1 (e_j x xi1)
            if (blk == 0) {
                V3 b = (j < 3) ? mul(R1, cross(unit(j), u1)) : v3(0, 0, 0);
                dd_j = dot(dd_dxw, a);
                dddot_j = dot(dddot_dxw, a) + dot(dddot_dxwd, b);
                dn_j = mul(dn_dxw, a);
                dt_j = mul(dt_dxw, a) + (b - dot(n, b) * n);
                dxi2_j = mul(dxi2_dxw, a);
            } else {
                dddot_j = dot(dddot_dxwd, a);
                dt_j = a - dot(n, a) * n;
            }
        } else if (blk == 1) {
            // dx_dq2 column
            V3 dxj = (j < 3) ? cross(unit(j), x) : -unit(j - 3);  // skew(x) e_j = x x e_j = -(e_j x x)
            if (j < 3) dxj = -dxj;
            dd_j = dot(gr, dxj);
            V3 de_j = mul(de_dx, dxj);
            dn_j = mul(R2, de_j);
            if (j < 3) dn_j = dn_j + mul(R2, cross(unit(j), e));
            dxi2_j = dxj - dd_j * e - d * de_j;
            if (j < 3) {
                // g^T(-Sw Sx + skew(rxd)) e_j + (H xdot)^T Sx e_j
                V3 sxe = cross(x, unit(j));  // Sx e_j
                dddot_j = dot(gr, -cross(B.w, sxe) + cross(rxd, unit(j))) + dot(Hxdot, sxe);
            } else {
                dddot_j = dot(gr, cross(B.w, unit(j - 3))) - comp(Hxdot, j - 3);
            }
            // dxw2dot/dq2 = [-R2 skew(w2 x xi2 + v2) + R2 Sw dxi2_dq2.left | R2 Sw dxi2_dq2.right]
            V3 dxw2d_j = mul(R2Sw, dxi2_j);
            if (j < 3) dxw2d_j = dxw2d_j - mul(R2, cross(wxi, unit(j)));
            // dtdot/dq2 = -dxw2d - nvw dn - n (vw.dn - n.dxw2d)
            dt_j = -dxw2d_j - nvw * dn_j - (dot(vw, dn_j) - dot(n, dxw2d_j)) * n;
        } else {  // blk == 3: dphi2
            if (j < 3) {
                V3 sxe = cross(x, unit(j));
                dddot_j = dot(gr, sxe);
                // dxw2dot/dphi2 col = R2 (e_j x xi2); dtdot = -(I - nn^T) that
                V3 q = mul(R2, cross(unit(j), xi2));
                dt_j = -(q - dot(n, q) * n);
            } else {
                dddot_j = -comp(gr, j - 3);
                V3 q = col(R2, j - 3);
                dt_j = -(q - dot(n, q) * n);
            }
        }

        // normal-force columns
        V3 N1, N2, T2 = v3(0, 0, 0);
        if (kcol) {
            double r = kn * dd_j - kd * dddot_j * d - kd * ddot * dd_j;
            N1 = -r * rho1 - sK * mulT(R1, dn_j);
            N2 = r * rho2 + sK * mulT(R2, dn_j);
            if (blk == 0 && j < 3) N1 = N1 - sK * cross(rho1, unit(j));
            if (blk == 1 && j < 3) N2 = N2 + sK * cross(rho2, unit(j));
            T2 = -sK * cross(rho2, dxi2_j);
        } else {
            double r = kd * dddot_j * d;
            N1 = r * rho1;
            N2 = -r * rho2;
        }
        if (friction) {
            // dfc_norm = fc1^T dfc1 / |fc1|, with dfc1 = Gamma1^T N1 and fc1 = s1 Gamma1^T rho1
            double dfn = s1 * (dot(xr1, cross(xi1, N1)) + dot(rho1, N1)) / fc_norm;
            double dtn = dot(t, dt_j) / tn;
            if (stat) {
                N1 = N1 - kt * mulT(R1, dt_j);
                N2 = N2 + kt * mulT(R2, dt_j);
                if (blk == 0 && j < 3) N1 = N1 - kt * cross(tau1, unit(j));
                if (blk == 1 && j < 3) N2 = N2 + kt * cross(tau2, unit(j));
                if (kcol) T2 = T2 - kt * cross(tau2, dxi2_j);
            } else {
                double cm = mu / tn;
                double s = dfn - ratio * dtn;
                N1 = N1 - cm * (s * tau1 + fc_norm * mulT(R1, dt_j));
                N2 = N2 + cm * (s * tau2 + fc_norm * mulT(R2, dt_j));
                if (blk == 0 && j < 3) N1 = N1 - (mu * ratio) * cross(tau1, unit(j));
                if (blk == 1 && j < 3) N2 = N2 + (mu * ratio) * cross(tau2, unit(j));
                if (kcol) T2 = T2 - (mu * ratio) * cross(tau2, dxi2_j);
            }
        }
        sink.column(c, N1, N2, T2);
    }
}

}  // namespace sdfc
