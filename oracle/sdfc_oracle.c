/*
 * ORACLE — test infrastructure, not the product.
 *
 * A plain-C, FP64, single-threaded restatement of the reference redmax
 * point-vs-SDF contact path (Assemble-Them-All, simulation/redmax).  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it, and
 * only to check or time against; the product never links or calls it.
 *
 * Parity of this restatement is pinned against the reference itself: the
 * reference sources are compiled by oracle/ref/Makefile into a harness
 * library, and tests/golden/ holds vectors generated from it
 * (tests/golden/make_golden.py).
 *
 * Conventions (same as the reference):
 *   - 3x3 / 3x6 / 6x6 matrices are row-major double arrays.
 *   - A pose E is a 4x4 row-major homogeneous matrix [R p; 0 1].
 *   - A body velocity phi = (w, v) is expressed in the body frame.
 *   - The SDF grid is indexed a[i + ni*(j + nj*k)]
 *     (simulation/externals/sdfgen/array3.h:70-79).
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared (no FMA contraction, so the
 * arithmetic matches the reference's x86-64 SSE2 build on every host).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "sdfc_oracle.h"

/* constants::eps in simulation/redmax/Utils.h:9 */
#define ORC_FRICTION_EPS 1e-8
/* FD step of query_dSDF / query_ddSDF, simulation/redmax/Body/BodySDFObj.cpp:178,191 */
#define ORC_FD_EPS 1e-5

/* ------------------------------------------------------------------ small linear algebra */
static void m3_transpose(const double* a, double* t) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) t[3 * c + r] = a[3 * r + c];
}
static void m3_mul(const double* a, const double* b, double* c) { /* c = a b (3x3) */
    double t[9];
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) {
            double s = 0.0;
            for (int j = 0; j < 3; ++j) s += a[3 * r + j] * b[3 * j + k];
            t[3 * r + k] = s;
        }
    memcpy(c, t, sizeof t);
}
static void m3_vec(const double* a, const double* v, double* out) {
    double t[3];
    for (int r = 0; r < 3; ++r) t[r] = a[3 * r] * v[0] + a[3 * r + 1] * v[1] + a[3 * r + 2] * v[2];
    memcpy(out, t, sizeof t);
}
static void m3t_vec(const double* a, const double* v, double* out) { /* a^T v */
    double t[3];
    for (int c = 0; c < 3; ++c) t[c] = a[c] * v[0] + a[3 + c] * v[1] + a[6 + c] * v[2];
    memcpy(out, t, sizeof t);
}
static void skew3(const double* v, double* s) { /* math::skew, simulation/redmax/Utils.h:25-31 */
    s[0] = 0.0;   s[1] = -v[2]; s[2] = v[1];
    s[3] = v[2];  s[4] = 0.0;   s[5] = -v[0];
    s[6] = -v[1]; s[7] = v[0];  s[8] = 0.0;
}
static void cross3(const double* a, const double* b, double* c) {
    double t[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    memcpy(c, t, sizeof t);
}
static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double norm3(const double* a) { return sqrt(dot3(a, a)); }
static void pose_split(const double* E, double* R, double* p) {
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) R[3 * r + c] = E[4 * r + c];
        p[r] = E[4 * r + 3];
    }
}
/* generic dense: C(m x n) = A(m x k) B(k x n), all row-major */
static void mm(const double* A, const double* B, double* C, int m, int k, int n) {
    double* t = (double*)malloc(sizeof(double) * (size_t)m * n);
    for (int r = 0; r < m; ++r)
        for (int c = 0; c < n; ++c) {
            double s = 0.0;
            for (int j = 0; j < k; ++j) s += A[r * k + j] * B[j * n + c];
            t[r * n + c] = s;
        }
    memcpy(C, t, sizeof(double) * (size_t)m * n);
    free(t);
}
/* GTRT = gamma(xi)^T R^T (6x3): rows 0-2 skew(xi) R^T, rows 3-5 R^T.
 * gamma(xi) = [skew(xi)^T, I], simulation/redmax/Utils.h:196-201 */
static void gtrt_of(const double* xi, const double* R, double* G) {
    double S[9], RT[9], SRT[9];
    skew3(xi, S);
    m3_transpose(R, RT);
    m3_mul(S, RT, SRT);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            G[3 * r + c] = SRT[3 * r + c];
            G[3 * (r + 3) + c] = RT[3 * r + c];
        }
}
/* Gamma^T M for M (3 x n): rows 0-2 skew(xi) M, rows 3-5 M (6 x n) */
static void gammaT_mul(const double* xi, const double* M, int n, double* out) {
    double S[9];
    skew3(xi, S);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < n; ++c) {
            out[r * n + c] = S[3 * r] * M[c] + S[3 * r + 1] * M[n + c] + S[3 * r + 2] * M[2 * n + c];
            out[(r + 3) * n + c] = M[r * n + c];
        }
}

/* ------------------------------------------------------------------ SDF queries */

/* BodySDFObj::query_SDF, simulation/redmax/Body/BodySDFObj.cpp:123-174 */
double orc_query_sdf(const orc_grid* g, const double* x, int outside_accurate) {
    int inside = 1;
    for (int i = 0; i < 3; ++i) inside = inside && x[i] >= g->min_box[i] && x[i] <= g->max_box[i];
    if (inside) {
        double ci = (x[0] - g->min_box[0]) / g->dx[0];
        double cj = (x[1] - g->min_box[1]) / g->dx[1];
        double ck = (x[2] - g->min_box[2]) / g->dx[2];
        int i = (int)floor(ci), j = (int)floor(cj), k = (int)floor(ck);
        ci = ci - i;
        cj = cj - j;
        ck = ck - k;
        int ni = g->ni, nj = g->nj, nk = g->nk;
        int ip = (i == ni - 1) ? i : i + 1; /* top-boundary clamp, :138-140 */
        int jp = (j == nj - 1) ? j : j + 1;
        int kp = (k == nk - 1) ? k : k + 1;
#define A3(a, b, c) g->v[(size_t)(a) + (size_t)ni * ((size_t)(b) + (size_t)nj * (size_t)(c))]
        double v00 = (1 - ci) * A3(i, j, k) + ci * A3(ip, j, k);
        double v10 = (1 - ci) * A3(i, jp, k) + ci * A3(ip, jp, k);
        double v01 = (1 - ci) * A3(i, j, kp) + ci * A3(ip, j, kp);
        double v11 = (1 - ci) * A3(i, jp, kp) + ci * A3(ip, jp, kp);
#undef A3
        double vk0 = (1 - cj) * v00 + cj * v10;
        double vk1 = (1 - cj) * v01 + cj * v11;
        return (1 - ck) * vk0 + ck * vk1;
    }
    if (outside_accurate) {
        double xb[3], dv[3];
        for (int i = 0; i < 3; ++i) {
            double t = x[i] > g->min_box[i] ? x[i] : g->min_box[i];
            xb[i] = t < g->max_box[i] ? t : g->max_box[i];
            dv[i] = x[i] - xb[i];
        }
        return norm3(dv) + orc_query_sdf(g, xb, 0);
    }
    return (double)FLT_MAX;
}

/* BodySDFObj::query_dSDF, :176-187 (central differences of the interpolant) */
void orc_query_dsdf(const orc_grid* g, const double* x, double* v) {
    const double eps = ORC_FD_EPS;
    for (int a = 0; a < 3; ++a) {
        double xp[3] = {x[0], x[1], x[2]}, xm[3] = {x[0], x[1], x[2]};
        xp[a] = x[a] + eps;
        xm[a] = x[a] - eps;
        v[a] = orc_query_sdf(g, xp, 1) - orc_query_sdf(g, xm, 1);
    }
    for (int a = 0; a < 3; ++a) v[a] /= (2 * eps);
}

/* BodySDFObj::query_ddSDF, :189-205 (FD Hessian, half steps on mixed terms) */
void orc_query_ddsdf(const orc_grid* g, const double* x, double* H) {
    const double eps = ORC_FD_EPS, h = ORC_FD_EPS / 2;
    double xs = orc_query_sdf(g, x, 1);
    for (int a = 0; a < 3; ++a) {
        double xp[3] = {x[0], x[1], x[2]}, xm[3] = {x[0], x[1], x[2]};
        xp[a] = x[a] + eps;
        xm[a] = x[a] - eps;
        H[4 * a] = orc_query_sdf(g, xp, 1) + orc_query_sdf(g, xm, 1) - 2 * xs;
    }
    static const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int q = 0; q < 3; ++q) {
        int a = pairs[q][0], b = pairs[q][1];
        double pp[3] = {x[0], x[1], x[2]}, mm_[3] = {x[0], x[1], x[2]};
        double pm[3] = {x[0], x[1], x[2]}, mp[3] = {x[0], x[1], x[2]};
        pp[a] = x[a] + h; pp[b] = x[b] + h;
        mm_[a] = x[a] - h; mm_[b] = x[b] - h;
        pm[a] = x[a] + h; pm[b] = x[b] - h;
        mp[a] = x[a] - h; mp[b] = x[b] + h;
        double s = orc_query_sdf(g, pp, 1) + orc_query_sdf(g, mm_, 1) - orc_query_sdf(g, pm, 1) -
                   orc_query_sdf(g, mp, 1);
        H[3 * a + b] = s;
        H[3 * b + a] = s;
    }
    for (int i = 0; i < 9; ++i) H[i] /= (eps * eps);
}

/* BodySDFObj::distance, :207-213 */
double orc_distance(const orc_grid* g, const double* E_B, const double* xw) {
    double R[9], p[3], d[3], x[3];
    pose_split(E_B, R, p);
    for (int i = 0; i < 3; ++i) d[i] = xw[i] - p[i];
    m3t_vec(R, d, x);
    return orc_query_sdf(g, x, 0) + g->col_th;
}

/* ------------------------------------------------------------------ contact query */

/* BodySDFObj::collision, value form :239-274 and derivative form :278-377.
 * out layout is documented in sdfc_oracle.h (ORC_COLLISION_*). */
void orc_collision(const orc_grid* g, const double* E_B, const double* phi_B, const double* xw,
                   const double* xw_dot, int want_deriv, double* out) {
    double R2[9], p2[3], R2T[9];
    pose_split(E_B, R2, p2);
    m3_transpose(R2, R2T);
    const double* w2 = phi_B;
    const double* v2 = phi_B + 3;
    double x[3], tmp[3];
    for (int i = 0; i < 3; ++i) tmp[i] = xw[i] - p2[i];
    m3_vec(R2T, tmp, x);

    double d = orc_query_sdf(g, x, 0) + g->col_th;
    double dd_dx[3];
    orc_query_dsdf(g, x, dd_dx);
    double gn = norm3(dd_dx);
    double e[3] = {dd_dx[0] / gn, dd_dx[1] / gn, dd_dx[2] / gn};
    double n[3];
    m3_vec(R2, e, n);
    double xi2[3] = {x[0] - d * e[0], x[1] - d * e[1], x[2] - d * e[2]};
    double Sw[9], SwT[9], xdot[3], a1[3], a2[3];
    skew3(w2, Sw);
    m3_transpose(Sw, SwT);
    m3_vec(SwT, x, a1);
    m3_vec(R2T, xw_dot, a2);
    for (int i = 0; i < 3; ++i) xdot[i] = a1[i] + a2[i] - v2[i];
    double ddot = dot3(dd_dx, xdot);
    double wxi[3], xw2_dot[3], vw[3];
    cross3(w2, xi2, wxi);
    for (int i = 0; i < 3; ++i) wxi[i] += v2[i];
    m3_vec(R2, wxi, xw2_dot);
    for (int i = 0; i < 3; ++i) vw[i] = xw_dot[i] - xw2_dot[i];
    double P[9]; /* I - n n^T */
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) P[3 * r + c] = (r == c ? 1.0 : 0.0) - n[r] * n[c];
    double tdot[3];
    m3_vec(P, vw, tdot);

    out[0] = d;
    memcpy(out + 1, n, sizeof n);
    out[4] = ddot;
    memcpy(out + 5, tdot, sizeof tdot);
    memcpy(out + 8, xi2, sizeof xi2);
    if (!want_deriv) return;

    double* dd_dxw = out + ORC_C_DD_DXW;
    double* dd_dq2 = out + ORC_C_DD_DQ2;
    double* dn_dxw = out + ORC_C_DN_DXW;
    double* dn_dq2 = out + ORC_C_DN_DQ2;
    double* dddot_dxw = out + ORC_C_DDDOT_DXW;
    double* dddot_dxwdot = out + ORC_C_DDDOT_DXWDOT;
    double* dddot_dq2 = out + ORC_C_DDDOT_DQ2;
    double* dddot_dphi2 = out + ORC_C_DDDOT_DPHI2;
    double* dtdot_dxw = out + ORC_C_DTDOT_DXW;
    double* dtdot_dxwdot = out + ORC_C_DTDOT_DXWDOT;
    double* dtdot_dq2 = out + ORC_C_DTDOT_DQ2;
    double* dtdot_dphi2 = out + ORC_C_DTDOT_DPHI2;
    double* dxi2_dxw = out + ORC_C_DXI2_DXW;
    double* dxi2_dq2 = out + ORC_C_DXI2_DQ2;

    /* x: dx_dxw = R2^T, dx_dw2 = skew(x), dx_dv2 = -I   (:317-319) */
    double Sx[9];
    skew3(x, Sx);
    /* d (:322-324) */
    { /* row vectors r^T M: r_c = sum_j r_j M[j][c] */
        for (int c = 0; c < 3; ++c) {
            dd_dxw[c] = dd_dx[0] * R2T[c] + dd_dx[1] * R2T[3 + c] + dd_dx[2] * R2T[6 + c];
            dd_dq2[c] = dd_dx[0] * Sx[c] + dd_dx[1] * Sx[3 + c] + dd_dx[2] * Sx[6 + c];
            dd_dq2[3 + c] = -dd_dx[c];
        }
    }
    /* n (:327-344) */
    double de_ddd[9];
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c)
            de_ddd[3 * i + c] = (gn * (i == c ? 1.0 : 0.0) - dd_dx[i] * dd_dx[c] / gn) / (gn * gn);
    double Hs[9], de_dx[9], de_dxw[9], de_dw2[9], de_dv2[9];
    orc_query_ddsdf(g, x, Hs);
    m3_mul(de_ddd, Hs, de_dx);
    m3_mul(de_dx, R2T, de_dxw);
    m3_mul(de_dx, Sx, de_dw2);
    for (int i = 0; i < 9; ++i) de_dv2[i] = -de_dx[i];
    m3_mul(R2, de_dxw, dn_dxw);
    {
        double A[9], B[9];
        m3_mul(R2, de_dw2, A);
        m3_mul(R2, de_dv2, B);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                dn_dq2[6 * r + c] = A[3 * r + c];
                dn_dq2[6 * r + 3 + c] = B[3 * r + c];
            }
        for (int c = 0; c < 3; ++c) { /* += R2 skew(e_c) e */
            double ec[3] = {0, 0, 0}, Se[9], t[3], u[3];
            ec[c] = 1.0;
            skew3(ec, Se);
            m3_vec(Se, e, t);
            m3_vec(R2, t, u);
            for (int r = 0; r < 3; ++r) dn_dq2[6 * r + c] += u[r];
        }
    }
    /* xi2 (:347-349) */
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            dxi2_dxw[3 * r + c] = R2T[3 * r + c] - e[r] * dd_dxw[c] - d * de_dxw[3 * r + c];
            dxi2_dq2[6 * r + c] = Sx[3 * r + c] - e[r] * dd_dq2[c] - d * de_dw2[3 * r + c];
            dxi2_dq2[6 * r + 3 + c] = -(r == c ? 1.0 : 0.0) - e[r] * dd_dq2[3 + c] - d * de_dv2[3 * r + c];
        }
    /* ddot (:352-357) */
    {
        double r1[3], r2[3], t1[3];
        for (int c = 0; c < 3; ++c) {
            r1[c] = dd_dx[0] * SwT[c] + dd_dx[1] * SwT[3 + c] + dd_dx[2] * SwT[6 + c];
            r2[c] = xdot[0] * Hs[c] + xdot[1] * Hs[3 + c] + xdot[2] * Hs[6 + c];
            t1[c] = r1[c] + r2[c];
        }
        for (int c = 0; c < 3; ++c) {
            dddot_dxw[c] = t1[0] * R2T[c] + t1[1] * R2T[3 + c] + t1[2] * R2T[6 + c];
            dddot_dxwdot[c] = dd_dx[0] * R2T[c] + dd_dx[1] * R2T[3 + c] + dd_dx[2] * R2T[6 + c];
        }
        double SwSx[9], M1[9], Srx[9], rx[3], xH[3];
        m3_mul(Sw, Sx, SwSx);
        m3_vec(R2T, xw_dot, rx);
        skew3(rx, Srx);
        for (int i = 0; i < 9; ++i) M1[i] = -SwSx[i] + Srx[i];
        for (int c = 0; c < 3; ++c) xH[c] = r2[c];
        for (int c = 0; c < 3; ++c) {
            double a = dd_dx[0] * M1[c] + dd_dx[1] * M1[3 + c] + dd_dx[2] * M1[6 + c];
            double b = xH[0] * Sx[c] + xH[1] * Sx[3 + c] + xH[2] * Sx[6 + c];
            dddot_dq2[c] = a + b;
            double a2_ = dd_dx[0] * Sw[c] + dd_dx[1] * Sw[3 + c] + dd_dx[2] * Sw[6 + c];
            dddot_dq2[3 + c] = a2_ - xH[c];
            dddot_dphi2[c] = dd_dx[0] * Sx[c] + dd_dx[1] * Sx[3 + c] + dd_dx[2] * Sx[6 + c];
            dddot_dphi2[3 + c] = -dd_dx[c];
        }
    }
    /* xw2_dot (:360-369) */
    double dxw2_dxw[9], dxw2_dq2[18], dxw2_dphi2[18];
    {
        double R2Sw[9];
        m3_mul(R2, Sw, R2Sw);
        m3_mul(R2Sw, dxi2_dxw, dxw2_dxw);
        double wxv[3], S1[9], A[9];
        cross3(w2, xi2, wxv);
        for (int i = 0; i < 3; ++i) wxv[i] += v2[i];
        skew3(wxv, S1);
        m3_mul(R2, S1, A);
        double L[9], Rr[9], Bl[9], Br[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                L[3 * r + c] = dxi2_dq2[6 * r + c];
                Rr[3 * r + c] = dxi2_dq2[6 * r + 3 + c];
            }
        m3_mul(R2Sw, L, Bl);
        m3_mul(R2Sw, Rr, Br);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                dxw2_dq2[6 * r + c] = -A[3 * r + c] + Bl[3 * r + c];
                dxw2_dq2[6 * r + 3 + c] = Br[3 * r + c];
            }
        for (int c = 0; c < 3; ++c) {
            double ec[3] = {0, 0, 0}, Se[9], t[3], u[3];
            ec[c] = 1.0;
            skew3(ec, Se);
            m3_vec(Se, xi2, t);
            m3_vec(R2, t, u);
            for (int r = 0; r < 3; ++r) dxw2_dphi2[6 * r + c] = u[r];
        }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) dxw2_dphi2[6 * r + 3 + c] = R2[3 * r + c];
    }
    /* tdot (:372-376) */
    {
        double nvw = dot3(n, vw);
        double vdn[3]; /* vw^T dn_dxw */
        for (int c = 0; c < 3; ++c) vdn[c] = vw[0] * dn_dxw[c] + vw[1] * dn_dxw[3 + c] + vw[2] * dn_dxw[6 + c];
        double NN[9], NNx[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) NN[3 * r + c] = n[r] * n[c];
        m3_mul(NN, dxw2_dxw, NNx);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
                dtdot_dxw[3 * r + c] = -dxw2_dxw[3 * r + c] - nvw * dn_dxw[3 * r + c] - n[r] * vdn[c] + NNx[3 * r + c];
        /* (I - n n^T)(I - 0) */
        memcpy(dtdot_dxwdot, P, sizeof P);
        for (int c = 0; c < 6; ++c) {
            double vd = vw[0] * dn_dq2[c] + vw[1] * dn_dq2[6 + c] + vw[2] * dn_dq2[12 + c];
            double nd = n[0] * dxw2_dq2[c] + n[1] * dxw2_dq2[6 + c] + n[2] * dxw2_dq2[12 + c];
            for (int r = 0; r < 3; ++r)
                dtdot_dq2[6 * r + c] = -dxw2_dq2[6 * r + c] - nvw * dn_dq2[6 * r + c] - n[r] * (vd - nd);
        }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 6; ++c)
                dtdot_dphi2[6 * r + c] =
                    -(P[3 * r] * dxw2_dphi2[c] + P[3 * r + 1] * dxw2_dphi2[6 + c] + P[3 * r + 2] * dxw2_dphi2[12 + c]);
    }
}

/* ------------------------------------------------------------------ detection */

/* collision_detection_general_SDF, simulation/redmax/CollisionDetection/CollisionDetection.cpp:124-147.
 * Writes the ids of points with distance < 0 in ascending order; returns their count. */
int orc_detect(const orc_grid* g, const double* E_A, const double* E_B, const double* pts, int n, int* ids,
               double* dist_out) {
    double RA[9], pA[3];
    pose_split(E_A, RA, pA);
    int cnt = 0;
    for (int i = 0; i < n; ++i) {
        double xw[3];
        m3_vec(RA, pts + 3 * i, xw);
        for (int k = 0; k < 3; ++k) xw[k] += pA[k];
        double d = orc_distance(g, E_B, xw);
        if (dist_out) dist_out[i] = d;
        if (d < 0.) {
            if (ids) ids[cnt] = i;
            ++cnt;
        }
    }
    return cnt;
}

/* ------------------------------------------------------------------ forces */

static void contact_kinematics(const double* E_A, const double* phi_A, const double* xi1, double* xw1,
                               double* xw1_dot) {
    /* ForceGeneralSDFContact.cpp:158-160 / :238-240 */
    double R1[9], p1[3], S[9], ST[9], t[3];
    pose_split(E_A, R1, p1);
    m3_vec(R1, xi1, xw1);
    for (int k = 0; k < 3; ++k) xw1[k] += p1[k];
    skew3(xi1, S);
    m3_transpose(S, ST);
    m3_vec(ST, phi_A, t);
    for (int k = 0; k < 3; ++k) t[k] += phi_A[3 + k];
    m3_vec(R1, t, xw1_dot);
}

/* ForceGeneralSDFContact::computeForce(contacts, fm), :147-219 */
static void force_value(const orc_grid* g, const double* E_A, const double* phi_A, const double* E_B,
                        const double* phi_B, const orc_params* prm, const double* pts, const int* ids,
                        int n_active, double* fm) {
    double R1[9], p1[3], R2[9], p2[3];
    pose_split(E_A, R1, p1);
    pose_split(E_B, R2, p2);
    const double kn = prm->kn * prm->scale * prm->contact_scale;
    const double kt = prm->kt * prm->scale * prm->contact_scale;
    memset(fm, 0, sizeof(double) * 12);
    for (int c = 0; c < n_active; ++c) {
        const double* xi1 = pts + 3 * ids[c];
        double xw1[3], xw1_dot[3], q[ORC_COLLISION_VALUE];
        contact_kinematics(E_A, phi_A, xi1, xw1, xw1_dot);
        orc_collision(g, E_B, phi_B, xw1, xw1_dot, 0, q);
        double d = q[0], *n = q + 1, ddot = q[4], *tdot = q + 5, *xi2 = q + 8;
        double G1[18], G2[18], ni1[6], ni2[6];
        gtrt_of(xi1, R1, G1);
        gtrt_of(xi2, R2, G2);
        mm(G1, n, ni1, 6, 3, 1);
        mm(G2, n, ni2, 6, 3, 1);
        double fc1[6];
        double s1 = -kn * d + prm->damping * ddot * d;
        double s2 = kn * d - prm->damping * ddot * d;
        for (int k = 0; k < 6; ++k) {
            fc1[k] = s1 * ni1[k];
            fm[k] += fc1[k];
            fm[6 + k] += s2 * ni2[k];
        }
        double fc_norm = 0.0;
        for (int k = 0; k < 6; ++k) fc_norm += fc1[k] * fc1[k];
        fc_norm = sqrt(fc_norm);
        double tdot_norm = norm3(tdot);
        if (prm->mu > ORC_FRICTION_EPS) {
            double Gt1[6], Gt2[6];
            mm(G1, tdot, Gt1, 6, 3, 1);
            mm(G2, tdot, Gt2, 6, 3, 1);
            int stat = prm->mu * fc_norm >= kt * tdot_norm - ORC_FRICTION_EPS;
            double c1 = stat ? -kt : -prm->mu * fc_norm / tdot_norm;
            double c2 = stat ? kt : prm->mu * fc_norm / tdot_norm;
            for (int k = 0; k < 6; ++k) {
                fm[k] += c1 * Gt1[k];
                fm[6 + k] += c2 * Gt2[k];
            }
        }
    }
}

/* (6 x 3) * (3 x 6) helper */
static void m63_m36(const double* A, const double* B, double* C) { mm(A, B, C, 6, 3, 6); }
/* block (rb, cb) of a 12x12 row-major matrix, add 6x6 (or 6x3 when ncol == 3) scaled */
static void add_block(double* M12, int rb, int cb, const double* B, int ncol, double s) {
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < ncol; ++c) M12[(rb + r) * 12 + cb + c] += s * B[r * ncol + c];
}
/* tmp.col(j) = dGamma2_dq(j)^T * w for dGamma2_dq(j) = sum_k dGamma2_dxi2(k) * dxi2_dq(k, j).
 * dGamma2_dxi2(k) is the 3x6 derivative of gamma(xi2) wrt xi2_k (:275-279); only its
 * left 3x3 (skew(xi2)^T part) is nonzero: d(skew(xi)^T)/dxi_k = skew(e_k)^T. */
static void dgamma_T_w(const double* dxi2_dq, const double* w, double* tmp) {
    /* dGamma(j)^T w (6-vector): top 3 = (sum_k dxi2_dq(k,j) skew(e_k)^T)^T w = sum_k dxi2_dq(k,j) skew(e_k) w */
    memset(tmp, 0, sizeof(double) * 36);
    for (int j = 0; j < 6; ++j)
        for (int k = 0; k < 3; ++k) {
            double ek[3] = {0, 0, 0}, Se[9], t[3];
            ek[k] = 1.0;
            skew3(ek, Se);
            m3_vec(Se, w, t);
            double s = dxi2_dq[6 * k + j];
            for (int r = 0; r < 3; ++r) tmp[r * 6 + j] += s * t[r];
        }
}

/* ForceGeneralSDFContact::computeForceWithDerivative(contacts, fm, Km, Dm), :221-447 */
static void force_deriv(const orc_grid* g, const double* E_A, const double* phi_A, const double* E_B,
                        const double* phi_B, const orc_params* prm, const double* pts, const int* ids,
                        int n_active, double* fm, double* Km, double* Dm) {
    double R1[9], p1[3], R2[9], p2[3], R1T[9], R2T[9];
    pose_split(E_A, R1, p1);
    pose_split(E_B, R2, p2);
    m3_transpose(R1, R1T);
    m3_transpose(R2, R2T);
    const double kn = prm->kn * prm->scale * prm->contact_scale;
    const double kt = prm->kt * prm->scale * prm->contact_scale;
    const double kd = prm->damping, mu = prm->mu;
    memset(fm, 0, sizeof(double) * 12);
    memset(Km, 0, sizeof(double) * 144);
    memset(Dm, 0, sizeof(double) * 144);
    for (int c = 0; c < n_active; ++c) {
        const double* xi1 = pts + 3 * ids[c];
        double xw1[3], xw1_dot[3];
        contact_kinematics(E_A, phi_A, xi1, xw1, xw1_dot);
        /* dxw1_dq1, dxw1dot_dq1, dxw1dot_dphi1 (3x6), :242-252 */
        double S1[9], S1T[9], A[9], dxw1_dq1[18], dxw1dot_dq1[18], dxw1dot_dphi1[18];
        skew3(xi1, S1);
        m3_transpose(S1, S1T);
        m3_mul(R1, S1, A);
        double inner[3], Sinner[9], B[9], C[9];
        m3_vec(S1T, phi_A, inner);
        for (int k = 0; k < 3; ++k) inner[k] += phi_A[3 + k];
        skew3(inner, Sinner);
        m3_mul(R1, Sinner, B);
        m3_mul(R1, S1T, C);
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) {
                dxw1_dq1[6 * r + k] = -A[3 * r + k];
                dxw1_dq1[6 * r + 3 + k] = R1[3 * r + k];
                dxw1dot_dq1[6 * r + k] = -B[3 * r + k];
                dxw1dot_dq1[6 * r + 3 + k] = 0.0;
                dxw1dot_dphi1[6 * r + k] = C[3 * r + k];
                dxw1dot_dphi1[6 * r + 3 + k] = R1[3 * r + k];
            }
        double q[ORC_COLLISION_DERIV];
        orc_collision(g, E_B, phi_B, xw1, xw1_dot, 1, q);
        double d = q[0], *n = q + 1, ddot = q[4], *tdot = q + 5, *xi2 = q + 8;
        const double* dd_dxw1 = q + ORC_C_DD_DXW;
        const double* dd_dq2 = q + ORC_C_DD_DQ2;
        const double* dn_dxw1 = q + ORC_C_DN_DXW;
        const double* dn_dq2 = q + ORC_C_DN_DQ2;
        const double* dddot_dxw1 = q + ORC_C_DDDOT_DXW;
        const double* dddot_dxw1dot = q + ORC_C_DDDOT_DXWDOT;
        const double* dddot_dq2 = q + ORC_C_DDDOT_DQ2;
        const double* dddot_dphi2 = q + ORC_C_DDDOT_DPHI2;
        const double* dtdot_dxw1 = q + ORC_C_DTDOT_DXW;
        const double* dtdot_dxw1dot = q + ORC_C_DTDOT_DXWDOT;
        const double* dtdot_dq2 = q + ORC_C_DTDOT_DQ2;
        const double* dtdot_dphi2 = q + ORC_C_DTDOT_DPHI2;
        const double* dxi2_dxw1 = q + ORC_C_DXI2_DXW;
        const double* dxi2_dq2 = q + ORC_C_DXI2_DQ2;

        double dxi2_dq1[18];
        mm(dxi2_dxw1, dxw1_dq1, dxi2_dq1, 3, 3, 6);

        double G1[18], G2[18], ni1[6], ni2[6];
        gtrt_of(xi1, R1, G1);
        gtrt_of(xi2, R2, G2);
        mm(G1, n, ni1, 6, 3, 1);
        mm(G2, n, ni2, 6, 3, 1);

        /* contact force on the contact body, :300-325 */
        double s1 = -kn * d + kd * ddot * d;
        double fc1[6];
        for (int k = 0; k < 6; ++k) {
            fc1[k] = s1 * ni1[k];
            fm[k] += fc1[k];
        }
        double dd_dq1[6], dddot_dq1[6], dn_dq1[18], dddot_dphi1[6], dtdot_dq1[18], dtdot_dphi1[18];
        mm(dd_dxw1, dxw1_dq1, dd_dq1, 1, 3, 6);
        {
            double a[6], b[6];
            mm(dddot_dxw1, dxw1_dq1, a, 1, 3, 6);
            mm(dddot_dxw1dot, dxw1dot_dq1, b, 1, 3, 6);
            for (int k = 0; k < 6; ++k) dddot_dq1[k] = a[k] + b[k];
        }
        mm(dn_dxw1, dxw1_dq1, dn_dq1, 3, 3, 6);
        mm(dddot_dxw1dot, dxw1dot_dphi1, dddot_dphi1, 1, 3, 6);
        {
            double a[18], b[18];
            mm(dtdot_dxw1, dxw1_dq1, a, 3, 3, 6);
            mm(dtdot_dxw1dot, dxw1dot_dq1, b, 3, 3, 6);
            for (int k = 0; k < 18; ++k) dtdot_dq1[k] = a[k] + b[k];
        }
        mm(dtdot_dxw1dot, dxw1dot_dphi1, dtdot_dphi1, 3, 3, 6);

        const double sK = kn * d - kd * ddot * d;
        double row_q1[6], row_q2[6];
        for (int k = 0; k < 6; ++k) {
            row_q1[k] = kn * dd_dq1[k] - kd * dddot_dq1[k] * d - kd * ddot * dd_dq1[k];
            row_q2[k] = kn * dd_dq2[k] - kd * dddot_dq2[k] * d - kd * ddot * dd_dq2[k];
        }
        double dfc1_dq1[36], dfc1_dq2[36], dfc1_dphi1[36], dfc1_dphi2[36];
        {
            double GD1[36], GD2[36];
            m63_m36(G1, dn_dq1, GD1);
            m63_m36(G1, dn_dq2, GD2);
            for (int r = 0; r < 6; ++r)
                for (int cc = 0; cc < 6; ++cc) {
                    dfc1_dq1[6 * r + cc] = -ni1[r] * row_q1[cc] - sK * GD1[6 * r + cc];
                    dfc1_dq2[6 * r + cc] = -ni1[r] * row_q2[cc] - sK * GD2[6 * r + cc];
                    dfc1_dphi1[6 * r + cc] = ni1[r] * kd * dddot_dphi1[cc] * d;
                    dfc1_dphi2[6 * r + cc] = ni1[r] * kd * dddot_dphi2[cc] * d;
                }
            /* dfc1_dq1.leftCols(3) -= sK * Gamma1^T skew(R1^T n) */
            double rn[3], Srn[9], GS[18];
            m3_vec(R1T, n, rn);
            skew3(rn, Srn);
            gammaT_mul(xi1, Srn, 3, GS);
            for (int r = 0; r < 6; ++r)
                for (int cc = 0; cc < 3; ++cc) dfc1_dq1[6 * r + cc] -= sK * GS[3 * r + cc];
        }
        add_block(Km, 0, 0, dfc1_dq1, 6, 1.0);
        add_block(Km, 0, 6, dfc1_dq2, 6, 1.0);
        add_block(Dm, 0, 0, dfc1_dphi1, 6, 1.0);
        add_block(Dm, 0, 6, dfc1_dphi2, 6, 1.0);

        /* contact force on the SDF body, :328-349 */
        for (int k = 0; k < 6; ++k) fm[6 + k] += sK * ni2[k];
        {
            double rn2[3], tmp1[36], tmp2[36], GD1[36], GD2[36];
            m3_vec(R2T, n, rn2);
            dgamma_T_w(dxi2_dq1, rn2, tmp1);
            dgamma_T_w(dxi2_dq2, rn2, tmp2);
            m63_m36(G2, dn_dq1, GD1);
            m63_m36(G2, dn_dq2, GD2);
            double b10[36], b11[36];
            for (int r = 0; r < 6; ++r)
                for (int cc = 0; cc < 6; ++cc) {
                    b10[6 * r + cc] = ni2[r] * row_q1[cc] + sK * (tmp1[6 * r + cc] + GD1[6 * r + cc]);
                    b11[6 * r + cc] = ni2[r] * row_q2[cc] + sK * (tmp2[6 * r + cc] + GD2[6 * r + cc]);
                }
            add_block(Km, 6, 0, b10, 6, 1.0);
            add_block(Km, 6, 6, b11, 6, 1.0);
            double Srn[9], GS[18];
            skew3(rn2, Srn);
            gammaT_mul(xi2, Srn, 3, GS);
            add_block(Km, 6, 6, GS, 3, sK);
            double e10[36], e11[36];
            for (int r = 0; r < 6; ++r)
                for (int cc = 0; cc < 6; ++cc) {
                    e10[6 * r + cc] = ni2[r] * kd * dddot_dphi1[cc] * d;
                    e11[6 * r + cc] = ni2[r] * kd * dddot_dphi2[cc] * d;
                }
            add_block(Dm, 6, 0, e10, 6, -1.0);
            add_block(Dm, 6, 6, e11, 6, -1.0);
        }

        /* friction, :352-445 */
        if (mu > ORC_FRICTION_EPS) {
            double fc_norm = 0.0;
            for (int k = 0; k < 6; ++k) fc_norm += fc1[k] * fc1[k];
            fc_norm = sqrt(fc_norm);
            double tdot_norm = norm3(tdot);
            double dfn_dq1[6], dfn_dq2[6], dfn_dphi1[6], dfn_dphi2[6];
            double dtn_dq1[6], dtn_dq2[6], dtn_dphi1[6], dtn_dphi2[6];
            for (int cc = 0; cc < 6; ++cc) {
                double a = 0, b = 0, e = 0, f = 0;
                for (int r = 0; r < 6; ++r) {
                    a += fc1[r] * dfc1_dq1[6 * r + cc];
                    b += fc1[r] * dfc1_dq2[6 * r + cc];
                    e += fc1[r] * dfc1_dphi1[6 * r + cc];
                    f += fc1[r] * dfc1_dphi2[6 * r + cc];
                }
                dfn_dq1[cc] = (1. / fc_norm) * a;
                dfn_dq2[cc] = (1. / fc_norm) * b;
                dfn_dphi1[cc] = (1. / fc_norm) * e;
                dfn_dphi2[cc] = (1. / fc_norm) * f;
                double a2 = 0, b2 = 0, e2 = 0, f2 = 0;
                for (int r = 0; r < 3; ++r) {
                    a2 += tdot[r] * dtdot_dq1[6 * r + cc];
                    b2 += tdot[r] * dtdot_dq2[6 * r + cc];
                    e2 += tdot[r] * dtdot_dphi1[6 * r + cc];
                    f2 += tdot[r] * dtdot_dphi2[6 * r + cc];
                }
                dtn_dq1[cc] = (1. / tdot_norm) * a2;
                dtn_dq2[cc] = (1. / tdot_norm) * b2;
                dtn_dphi1[cc] = (1. / tdot_norm) * e2;
                dtn_dphi2[cc] = (1. / tdot_norm) * f2;
            }
            int stat = mu * fc_norm >= kt * tdot_norm - ORC_FRICTION_EPS;
            double Gt1[6], Gt2[6];
            mm(G1, tdot, Gt1, 6, 3, 1);
            mm(G2, tdot, Gt2, 6, 3, 1);
            double rt1[3], rt2[3];
            m3_vec(R1T, tdot, rt1);
            m3_vec(R2T, tdot, rt2);
            if (stat) {
                for (int k = 0; k < 6; ++k) fm[k] += -kt * Gt1[k];
                double X[36];
                m63_m36(G1, dtdot_dq1, X);
                add_block(Km, 0, 0, X, 6, -kt);
                double Srt[9], GS[18];
                skew3(rt1, Srt);
                gammaT_mul(xi1, Srt, 3, GS);
                add_block(Km, 0, 0, GS, 3, -kt);
                m63_m36(G1, dtdot_dq2, X);
                add_block(Km, 0, 6, X, 6, -kt);
                m63_m36(G1, dtdot_dphi1, X);
                add_block(Dm, 0, 0, X, 6, -kt);
                m63_m36(G1, dtdot_dphi2, X);
                add_block(Dm, 0, 6, X, 6, -kt);
            } else {
                double ratio = fc_norm / tdot_norm;
                for (int k = 0; k < 6; ++k) fm[k] += -mu * ratio * Gt1[k];
                /* -mu/|t| * G1 * (t dfn - |f|/|t| t dtn + |f| dtdot) */
                const double* dfn[4] = {dfn_dq1, dfn_dq2, dfn_dphi1, dfn_dphi2};
                const double* dtn[4] = {dtn_dq1, dtn_dq2, dtn_dphi1, dtn_dphi2};
                const double* dtd[4] = {dtdot_dq1, dtdot_dq2, dtdot_dphi1, dtdot_dphi2};
                for (int w = 0; w < 4; ++w) {
                    double Mx[18], X[36];
                    for (int r = 0; r < 3; ++r)
                        for (int cc = 0; cc < 6; ++cc)
                            Mx[6 * r + cc] = tdot[r] * dfn[w][cc] - ratio * tdot[r] * dtn[w][cc] + fc_norm * dtd[w][6 * r + cc];
                    m63_m36(G1, Mx, X);
                    double* M = (w < 2) ? Km : Dm;
                    add_block(M, 0, (w % 2) ? 6 : 0, X, 6, -mu / tdot_norm);
                }
                double v3[3] = {ratio * rt1[0], ratio * rt1[1], ratio * rt1[2]}, Sv[9], GS[18];
                skew3(v3, Sv);
                gammaT_mul(xi1, Sv, 3, GS);
                add_block(Km, 0, 0, GS, 3, -mu);
            }
            /* SDF body */
            double tmp1[36], tmp2[36];
            dgamma_T_w(dxi2_dq1, rt2, tmp1);
            dgamma_T_w(dxi2_dq2, rt2, tmp2);
            if (stat) {
                for (int k = 0; k < 6; ++k) fm[6 + k] += kt * Gt2[k];
                double X[36];
                m63_m36(G2, dtdot_dq1, X);
                add_block(Km, 6, 0, X, 6, kt);
                add_block(Km, 6, 0, tmp1, 6, kt);
                m63_m36(G2, dtdot_dq2, X);
                add_block(Km, 6, 6, X, 6, kt);
                add_block(Km, 6, 6, tmp2, 6, kt);
                double Srt[9], GS[18];
                skew3(rt2, Srt);
                gammaT_mul(xi2, Srt, 3, GS);
                add_block(Km, 6, 6, GS, 3, kt);
                m63_m36(G2, dtdot_dphi1, X);
                add_block(Dm, 6, 0, X, 6, kt);
                m63_m36(G2, dtdot_dphi2, X);
                add_block(Dm, 6, 6, X, 6, kt);
            } else {
                double ratio = fc_norm / tdot_norm;
                for (int k = 0; k < 6; ++k) fm[6 + k] += mu * ratio * Gt2[k];
                const double* dfn[4] = {dfn_dq1, dfn_dq2, dfn_dphi1, dfn_dphi2};
                const double* dtn[4] = {dtn_dq1, dtn_dq2, dtn_dphi1, dtn_dphi2};
                const double* dtd[4] = {dtdot_dq1, dtdot_dq2, dtdot_dphi1, dtdot_dphi2};
                for (int w = 0; w < 4; ++w) {
                    double Mx[18], X[36];
                    for (int r = 0; r < 3; ++r)
                        for (int cc = 0; cc < 6; ++cc)
                            Mx[6 * r + cc] = tdot[r] * dfn[w][cc] - tdot[r] * ratio * dtn[w][cc] + fc_norm * dtd[w][6 * r + cc];
                    m63_m36(G2, Mx, X);
                    double* M = (w < 2) ? Km : Dm;
                    add_block(M, 6, (w % 2) ? 6 : 0, X, 6, mu / tdot_norm);
                }
                add_block(Km, 6, 0, tmp1, 6, mu * ratio);
                add_block(Km, 6, 6, tmp2, 6, mu * ratio);
                double v3[3] = {ratio * rt2[0], ratio * rt2[1], ratio * rt2[2]}, Sv[9], GS[18];
                skew3(v3, Sv);
                gammaT_mul(xi2, Sv, 3, GS);
                add_block(Km, 6, 6, GS, 3, mu);
            }
        }
    }
}

/* ForceGeneralSDFContact::computeForce / computeForceWithDerivative public
 * wrappers (:46-105): detection, then the per-contact sums for the pair. */
int orc_pair_eval(const orc_grid* g, const double* pts, int n_pts, const double* E_A, const double* phi_A,
                  const double* E_B, const double* phi_B, const orc_params* prm, int want_deriv, double* fm,
                  double* Km, double* Dm, int* ids) {
    int own = (ids == NULL);
    if (own) ids = (int*)malloc(sizeof(int) * (size_t)(n_pts > 0 ? n_pts : 1));
    int n_active = orc_detect(g, E_A, E_B, pts, n_pts, ids, NULL);
    if (want_deriv)
        force_deriv(g, E_A, phi_A, E_B, phi_B, prm, pts, ids, n_active, fm, Km, Dm);
    else
        force_value(g, E_A, phi_A, E_B, phi_B, prm, pts, ids, n_active, fm);
    if (own) free(ids);
    return n_active;
}

/* ------------------------------------------------------------------ BDF1 of one translational mover */

/* Joint::update (Q = [I q; 0 1], E_pj = E_pj0 Q; JointTranslational.cpp:9-40,
 * Joint.cpp) then Body::update (E_0i = E_0j E_ji, phi = Ad(E_ij) S_j qdot;
 * Body.cpp:138-156).  For the translational joint S_j = [0; I], so
 * phi = (0, R_ji^T qdot). */
void orc_mover_pose(const orc_mover* m, const double* q, const double* qdot, double* E0i, double* phi) {
    double Q[16] = {1, 0, 0, q[0], 0, 1, 0, q[1], 0, 0, 1, q[2], 0, 0, 0, 1};
    double E0j[16];
    mm(m->E_pj0, Q, E0j, 4, 4, 4);
    mm(E0j, m->E_ji, E0i, 4, 4, 4);
    double Rji[9], pji[3];
    pose_split(m->E_ji, Rji, pji);
    double v[3];
    m3t_vec(Rji, qdot, v);
    phi[0] = phi[1] = phi[2] = 0.0;
    phi[3] = v[0];
    phi[4] = v[1];
    phi[5] = v[2];
}

/* Simulation::evaluate_g_BDF1 / evaluate_g_with_derivatives_BDF1 (Simulation.cpp:1081-1165)
 * with Simulation::computeMatrices (:379-503) specialised to one translational mover:
 * J = Ad(E_ij) S_j = [0; R_ji^T] is constant, so Jdot = dJ/dq = 0, M = J^T Mm J,
 * f = J^T fm + fr, K = J^T Km J + Kr, D = J^T Dm J + Dr.  fm is the mover's gravity
 * and external force (Body::computeMaximalForce, Body.cpp:247-271; its Coriolis term
 * only has angular rows, which J^T drops) plus every contact's mover block. */
void orc_bdf1_eval(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q0, const double* qdot0,
                   const double* q1, double* g, double* H) {
    orc_bdf1_eval_full(m, pairs, n_pairs, q0, qdot0, q1, g, H, NULL, NULL);
}

void orc_bdf1_eval_full(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q0,
                        const double* qdot0, const double* q1, double* g, double* H, double* M_out,
                        double* D_out) {
    const double h = m->h;
    double qd1[3], E0i[16], phi[6], R0i[9], p0i[3], Rji[9], pji[3];
    for (int k = 0; k < 3; ++k) qd1[k] = (q1[k] - q0[k]) / h;
    orc_mover_pose(m, q1, qd1, E0i, phi);
    pose_split(E0i, R0i, p0i);
    pose_split(m->E_ji, Rji, pji);
    /* linear rows of fm for the mover: gravity + external */
    double fl[3], Kll[9] = {0}, Dll[9] = {0}, mg[3], ft[3];
    for (int k = 0; k < 3; ++k) mg[k] = m->mass * m->gravity[k];
    m3t_vec(R0i, mg, fl);
    m3t_vec(R0i, m->f_ext + 3, ft);
    for (int k = 0; k < 3; ++k) fl[k] += m->inertia[3 + k] * ft[k];
    const double zero6[6] = {0, 0, 0, 0, 0, 0};
    for (int c = 0; c < n_pairs; ++c) {
        const orc_pair* P = pairs + c;
        double fm[12], Km[144], Dm[144];
        const double *EA, *phiA, *EB, *phiB;
        if (P->mover_is_contact) {
            EA = E0i; phiA = phi; EB = P->E_fixed; phiB = zero6;
        } else {
            EA = P->E_fixed; phiA = zero6; EB = E0i; phiB = phi;
        }
        orc_pair_eval(P->grid, P->pts, P->n_pts, EA, phiA, EB, phiB, &P->prm, H != NULL, fm, Km, Dm, NULL);
        const int o = P->mover_is_contact ? 0 : 6;
        for (int r = 0; r < 3; ++r) {
            fl[r] += fm[o + 3 + r];
            if (H)
                for (int s = 0; s < 3; ++s) {
                    Kll[3 * r + s] += Km[(o + 3 + r) * 12 + o + 3 + s];
                    Dll[3 * r + s] += Dm[(o + 3 + r) * 12 + o + 3 + s];
                }
        }
    }
    /* reduced: f = R_ji fl + fr; M = R_ji diag(m) R_ji^T */
    double f[3], M[9], Md[9] = {0};
    m3_vec(Rji, fl, f);
    for (int k = 0; k < 3; ++k) f[k] += -m->joint_stiffness * (q1[k] - m->q_rest[k]) - m->joint_damping * qd1[k];
    for (int k = 0; k < 3; ++k) Md[4 * k] = m->inertia[3 + k];
    double RjiT[9], T[9];
    m3_transpose(Rji, RjiT);
    m3_mul(Rji, Md, T);
    m3_mul(T, RjiT, M);
    double dq[3];
    for (int k = 0; k < 3; ++k) dq[k] = q1[k] - q0[k] - h * qdot0[k];
    double Mdq[3];
    m3_vec(M, dq, Mdq);
    for (int k = 0; k < 3; ++k) g[k] = Mdq[k] - h * h * f[k];
    if (H) {
        double K[9], D[9];
        m3_mul(Rji, Kll, T);
        m3_mul(T, RjiT, K);
        m3_mul(Rji, Dll, T);
        m3_mul(T, RjiT, D);
        for (int k = 0; k < 3; ++k) {
            K[4 * k] -= m->joint_stiffness;
            D[4 * k] -= m->joint_damping;
        }
        for (int k = 0; k < 9; ++k) H[k] = M[k] - h * h * K[k] - h * D[k];
        if (D_out) memcpy(D_out, D, sizeof D);
    }
    if (M_out) memcpy(M_out, M, sizeof M);
}

/* 3x3 solve by Gaussian elimination with partial pivoting (the algorithm of Eigen's
 * PartialPivLU used by Simulation::newton, Simulation.cpp:1028). */
static void solve3(const double* A_in, const double* b_in, double* x) {
    double A[9], b[3];
    memcpy(A, A_in, sizeof A);
    memcpy(b, b_in, sizeof b);
    for (int c = 0; c < 3; ++c) {
        int p = c;
        for (int r = c + 1; r < 3; ++r)
            if (fabs(A[3 * r + c]) > fabs(A[3 * p + c])) p = r;
        if (p != c) {
            for (int k = 0; k < 3; ++k) {
                double t = A[3 * c + k];
                A[3 * c + k] = A[3 * p + k];
                A[3 * p + k] = t;
            }
            double t = b[c];
            b[c] = b[p];
            b[p] = t;
        }
        for (int r = c + 1; r < 3; ++r) {
            double l = A[3 * r + c] / A[3 * c + c];
            for (int k = c; k < 3; ++k) A[3 * r + k] -= l * A[3 * c + k];
            b[r] -= l * b[c];
        }
    }
    for (int r = 2; r >= 0; --r) {
        double s = b[r];
        for (int k = r + 1; k < 3; ++k) s -= A[3 * r + k] * x[k];
        x[r] = s / A[3 * r + r];
    }
}

/* Simulation::integration_BDF1 (Simulation.cpp:1248-1270) with Simulation::newton
 * (:999-1079): tolerance 1e-8 on |g|, at most max(20 ndof, 100) iterations, backtracking
 * line search halving alpha up to 20 times, 3 consecutive line-search failures stop. */
int orc_bdf1_step(const orc_mover* m, const orc_pair* pairs, int n_pairs, double* q, double* qdot, int* iters,
                  int* evals) {
    const double h = m->h, tol = 1e-8;
    const int max_iter = 100, max_ls = 20, max_strike = 3;
    double q0[3], qd0[3], x[3];
    for (int k = 0; k < 3; ++k) {
        q0[k] = q[k];
        qd0[k] = qdot[k];
        x[k] = q0[k] + h * qd0[k];
    }
    int converged = 0, strike = 0, it = 0, ev = 0;
    for (; it < max_iter; ++it) {
        double g[3], H[9], dx[3], mg[3];
        orc_bdf1_eval(m, pairs, n_pairs, q0, qd0, x, g, H);
        ++ev;
        for (int k = 0; k < 3; ++k) mg[k] = -g[k];
        solve3(H, mg, dx);
        const double gnorm = norm3(g);
        double alpha = 1.0, gn[3] = {0, 0, 0};
        int ok = 0;
        for (int trial = 0; trial < max_ls; ++trial, alpha *= 0.5) {
            double xt[3] = {x[0] + alpha * dx[0], x[1] + alpha * dx[1], x[2] + alpha * dx[2]};
            orc_bdf1_eval(m, pairs, n_pairs, q0, qd0, xt, gn, NULL);
            ++ev;
            if (norm3(gn) < gnorm) {
                ok = 1;
                break;
            }
        }
        if (ok) {
            strike = 0;
        } else if (++strike >= max_strike) {
            break;
        }
        for (int k = 0; k < 3; ++k) x[k] = x[k] + alpha * dx[k];
        if (norm3(gn) < tol) {
            converged = 1;
            break;
        }
    }
    for (int k = 0; k < 3; ++k) {
        qdot[k] = (x[k] - q0[k]) / h;
        q[k] = x[k];
    }
    if (iters) *iters = it + (converged ? 1 : 0);
    if (evals) *evals = ev;
    return converged;
}

/* ------------------------------------------------------------------ adjoint of the BDF1 rollout */

/* Partial-pivoting LU of a 3x3 (PA = LU, L unit lower, stored in one array) and the
 * solve of A^T z = y with those factors (Eigen's PartialPivLU::transpose().solve, which
 * the reference calls at Simulation.cpp:1587): U^T w = y, L^T u = w, z = P^T u. */
static void lu3(const double* A_in, double* LU, int* perm) {
    memcpy(LU, A_in, 9 * sizeof(double));
    for (int k = 0; k < 3; ++k) perm[k] = k;
    for (int c = 0; c < 3; ++c) {
        int p = c;
        for (int r = c + 1; r < 3; ++r)
            if (fabs(LU[3 * r + c]) > fabs(LU[3 * p + c])) p = r;
        if (p != c) {
            for (int k = 0; k < 3; ++k) {
                double t = LU[3 * c + k];
                LU[3 * c + k] = LU[3 * p + k];
                LU[3 * p + k] = t;
            }
            int t = perm[c];
            perm[c] = perm[p];
            perm[p] = t;
        }
        for (int r = c + 1; r < 3; ++r) {
            LU[3 * r + c] /= LU[3 * c + c];
            for (int k = c + 1; k < 3; ++k) LU[3 * r + k] -= LU[3 * r + c] * LU[3 * c + k];
        }
    }
}

static void lu3_solve_transposed(const double* LU, const int* perm, const double* y, double* z) {
    double w[3], u[3];
    for (int r = 0; r < 3; ++r) { /* U^T w = y */
        double s = y[r];
        for (int k = 0; k < r; ++k) s -= LU[3 * k + r] * w[k];
        w[r] = s / LU[3 * r + r];
    }
    for (int r = 2; r >= 0; --r) { /* L^T u = w */
        double s = w[r];
        for (int k = r + 1; k < 3; ++k) s -= LU[3 * k + r] * u[k];
        u[r] = s;
    }
    for (int r = 0; r < 3; ++r) z[perm[r]] = u[r];
}

/* Simulation::backward_BDF1 (Simulation.cpp:1559-1634) for one translational mover, with
 * the per-step H, M, D that the reference saves after each converged step
 * (integration_BDF1, :1262-1269, evaluating evaluate_g_with_derivatives_BDF1 at q_k with
 * qdot_k = (q_k - q_{k-1}) / h) recomputed here from the trajectory q_his[0..T].
 * df_dq[T x 3] is dL/dq_k for k = 1..T.  Outputs dL/dq_0, dL/dqdot_0 and, beyond the
 * reference, dL/df_ext (world-frame external force: the torque rows are 0 because the
 * translational joint's J has no angular part): df_ext's direct term in f is
 * R_ji diag(m) R_0i^T fe, so dL/dfe = h^2 R_0i diag(m) R_ji^T sum_k z_k. */
void orc_bdf1_backward(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q_his,
                       const double* qdot0, int T, const double* df_dq, double* df_dq0, double* df_dqdot0,
                       double* df_dfext) {
    const double h = m->h;
    double* Ms = (double*)calloc((size_t)(T > 0 ? T : 1) * 27, sizeof(double));
    double* Ds = Ms + 9 * (size_t)(T > 0 ? T : 1);
    double* Hs = Ds + 9 * (size_t)(T > 0 ? T : 1);
    double* z = (double*)calloc((size_t)(T > 0 ? T : 1) * 3, sizeof(double));
    for (int k = 1; k <= T; ++k) { /* the saved step data */
        double qd_prev[3], g[3];
        const double* qp = q_his + 3 * (k - 1);
        if (k == 1) {
            memcpy(qd_prev, qdot0, sizeof qd_prev);
        } else {
            for (int c = 0; c < 3; ++c) qd_prev[c] = (qp[c] - q_his[3 * (k - 2) + c]) / h;
        }
        orc_bdf1_eval_full(m, pairs, n_pairs, qp, qd_prev, q_his + 3 * k, g, Hs + 9 * (k - 1), Ms + 9 * (k - 1),
                           Ds + 9 * (k - 1));
    }
    for (int k = T - 1; k >= 0; --k) { /* z_k for step k + 1 */
        double y[3], t[3], LU[9];
        int perm[3];
        for (int c = 0; c < 3; ++c) y[c] = df_dq[3 * k + c];
        if (k < T - 1) {
            double A[9];
            for (int c = 0; c < 9; ++c) A[c] = -2.0 * Ms[9 * (k + 1) + c] + h * Ds[9 * (k + 1) + c];
            m3t_vec(A, z + 3 * (k + 1), t);
            for (int c = 0; c < 3; ++c) y[c] -= t[c];
        }
        if (k < T - 2) {
            m3t_vec(Ms + 9 * (k + 2), z + 3 * (k + 2), t);
            for (int c = 0; c < 3; ++c) y[c] -= t[c];
        }
        lu3(Hs + 9 * k, LU, perm);
        lu3_solve_transposed(LU, perm, y, z + 3 * k);
    }
    double g0[3] = {0, 0, 0}, gd0[3] = {0, 0, 0}, t[3];
    if (T > 0) {
        double A[9], B[9];
        for (int c = 0; c < 9; ++c) {
            A[c] = -Ms[c] + h * Ds[c];
            B[c] = -h * Ms[c];
        }
        m3t_vec(A, z, t);
        for (int c = 0; c < 3; ++c) g0[c] -= t[c];
        m3t_vec(B, z, t);
        for (int c = 0; c < 3; ++c) gd0[c] -= t[c];
    }
    if (T > 1) {
        m3t_vec(Ms + 9, z + 3, t);
        for (int c = 0; c < 3; ++c) g0[c] -= t[c];
    }
    if (df_dq0) memcpy(df_dq0, g0, sizeof g0);
    if (df_dqdot0) memcpy(df_dqdot0, gd0, sizeof gd0);
    if (df_dfext) {
        double zs[3] = {0, 0, 0}, E0i[16], phi[6], R0i[9], p0i[3], Rji[9], pji[3], v[3], w[3];
        for (int k = 0; k < T; ++k)
            for (int c = 0; c < 3; ++c) zs[c] += z[3 * k + c];
        orc_mover_pose(m, q_his, qdot0, E0i, phi); /* R_0i is the same at every q */
        pose_split(E0i, R0i, p0i);
        pose_split(m->E_ji, Rji, pji);
        m3t_vec(Rji, zs, v);
        for (int c = 0; c < 3; ++c) v[c] *= m->inertia[3 + c];
        m3_vec(R0i, v, w);
        for (int c = 0; c < 3; ++c) {
            df_dfext[c] = 0.0;
            df_dfext[3 + c] = h * h * w[c];
        }
    }
    free(Ms);
    free(z);
}
