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

/* Simulation::get_body_distance (rm/Simulation.cpp:276-296): the `from` body's mesh vertices to
 * world by get_body_vertices (:252-264), then the `to` body's distance() (BodySDFObj.cpp:207-213),
 * minimised.  get_body_vertices evaluates (R2 * v + p2).eval() with a Matrix3 R2; in the reference's
 * x86-64 build Eigen computes rows 0 and 1 of R2 * v as one SSE2 packet, ((r0 v0 + r1 v1) + r2 v2),
 * and row 2 by its unrolled scalar reduction, r0 v0 + (r1 v1 + r2 v2); both are kept.  d_out
 * (optional) receives every vertex's distance. */
double orc_body_distance(const orc_grid* g, const double* E_from, const double* E_to, const double* V, int n,
                         double* d_out) {
    double R[9], p[3];
    pose_split(E_from, R, p);
    double m = INFINITY;
    for (int i = 0; i < n; ++i) {
        const double* v = V + 3 * i;
        double xw[3];
        xw[0] = (R[0] * v[0] + R[1] * v[1]) + R[2] * v[2];
        xw[1] = (R[3] * v[0] + R[4] * v[1]) + R[5] * v[2];
        xw[2] = R[6] * v[0] + (R[7] * v[1] + R[8] * v[2]);
        for (int k = 0; k < 3; ++k) xw[k] += p[k];
        const double d = orc_distance(g, E_to, xw);
        if (d_out) d_out[i] = d;
        if (d < m) m = d;
    }
    return m;
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

/* Sum over the pair's active contacts of the norm of each contact's own 12-vector (its term of
 * fm, ForceGeneralSDFContact::computeForce(contacts), ForceGeneralSDFContact.cpp:147-219, for the
 * contact alone).  Where the contacts' forces cancel in fm (a peg pressed all round into a bore),
 * this is the scale against which the error of fm is meaningful.  Not in the reference. */
double orc_pair_force_norm_sum(const orc_grid* g, const double* pts, int n_pts, const double* E_A,
                               const double* phi_A, const double* E_B, const double* phi_B, const orc_params* prm) {
    int* ids = (int*)malloc(sizeof(int) * (size_t)(n_pts > 0 ? n_pts : 1));
    const int n_active = orc_detect(g, E_A, E_B, pts, n_pts, ids, NULL);
    double total = 0.0, f[12];
    for (int c = 0; c < n_active; ++c) {
        force_value(g, E_A, phi_A, E_B, phi_B, prm, pts, ids + c, 1, f);
        double s = 0.0;
        for (int k = 0; k < 12; ++k) s += f[k] * f[k];
        total += sqrt(s);
    }
    free(ids);
    return total;
}

/* ------------------------------------------------------------------ penetration energy */

/* Penetration energy of a pair: the sum over its active contacts (orc_detect) of kn d^2 / 2,
 * kn scaled as in the force law (ForceGeneralSDFContact.cpp:155-156), and its gradient wrt the
 * twists of A then B (w, v each): kn d dd/dq with dd/dxw = R_B g (g = query_dSDF at the
 * grid-frame point, BodySDFObj.cpp:176-187), dxw/dq_A = [-R_A skew(xi) | R_A],
 * dx/dq_B = [skew(x) | -I].  The reference has no energy; this is the definition the GPU's
 * energy mode computes, on the reference's own distance and gradient. */
double orc_pair_energy(const orc_grid* g, const double* pts, int n_pts, const double* E_A, const double* E_B,
                       const orc_params* prm, double* dE) {
    int* ids = (int*)malloc(sizeof(int) * (size_t)(n_pts > 0 ? n_pts : 1));
    double* dist = (double*)malloc(sizeof(double) * (size_t)(n_pts > 0 ? n_pts : 1));
    const int na = orc_detect(g, E_A, E_B, pts, n_pts, ids, dist);
    const double kn = prm->kn * prm->scale * prm->contact_scale;
    double RA[9], pA[3], RB[9], pB[3];
    pose_split(E_A, RA, pA);
    pose_split(E_B, RB, pB);
    double e = 0.0;
    for (int k = 0; k < 12; ++k) dE[k] = 0.0;
    for (int c = 0; c < na; ++c) {
        const double* xi = pts + 3 * (size_t)ids[c];
        double xw[3], t[3], x[3], gr[3], w[3], ga[3], aw[3], bw[3];
        m3_vec(RA, xi, xw);
        for (int k = 0; k < 3; ++k) t[k] = xw[k] + pA[k] - pB[k];
        m3t_vec(RB, t, x);
        const double d = dist[ids[c]]; /* orc_detect writes distances by point index */
        orc_query_dsdf(g, x, gr);
        m3_vec(RB, gr, w);
        m3t_vec(RA, w, ga);
        cross3(xi, ga, aw);
        cross3(gr, x, bw);
        const double s = kn * d;
        e += 0.5 * kn * d * d;
        for (int k = 0; k < 3; ++k) {
            dE[k] += s * aw[k];
            dE[3 + k] += s * ga[k];
            dE[6 + k] += s * bw[k];
            dE[9 + k] -= s * gr[k];
        }
    }
    free(ids);
    free(dist);
    return e;
}

/* ------------------------------------------------------------------ BDF1 of one moving part */

/* ---- translational joint (3 dof) */

static void trans_pose(const orc_mover* m, const double* q, const double* qdot, double* E0i, double* phi) {
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
static void trans_eval_full(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q0,
                            const double* qdot0, const double* q1, double* g, double* H, double* M_out,
                            double* D_out) {
    const double h = m->h;
    double qd1[3], E0i[16], phi[6], R0i[9], p0i[3], Rji[9], pji[3];
    for (int k = 0; k < 3; ++k) qd1[k] = (q1[k] - q0[k]) / h;
    trans_pose(m, q1, qd1, E0i, phi);
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

/* ---- free joint with exponential rotation coordinates (6 dof: q = (p, r)) */

/* small dense helpers (row-major) */
static void mz(double* a, int n) { memset(a, 0, sizeof(double) * (size_t)n); }
static void m3_add(const double* a, const double* b, double* c) {
    for (int k = 0; k < 9; ++k) c[k] = a[k] + b[k];
}
static void m3_scale(const double* a, double s, double* c) {
    for (int k = 0; k < 9; ++k) c[k] = a[k] * s;
}
static void m3_tmul(const double* a, const double* b, double* c) { /* c = a^T b */
    double at[9];
    m3_transpose(a, at);
    m3_mul(at, b, c);
}
static void unskew3(const double* a, double* v) { /* math::unskew, rm/Utils.h:45-51 */
    v[0] = a[7];
    v[1] = a[2];
    v[2] = a[3];
}
static void skew_of_cross(const double* a, const double* b, double* S) { /* skew(a x b) */
    double c[3];
    cross3(a, b, c);
    skew3(c, S);
}

/* math::exp(Vector3): Rodrigues' formula (rm/Utils.h:108-124). */
static void so3_exp(const double* w_in, double* R) {
    double wl = norm3(w_in);
    mz(R, 9);
    R[0] = R[4] = R[8] = 1.0;
    if (wl > 1e-12) {
        const double wx = w_in[0] / wl, wy = w_in[1] / wl, wz = w_in[2] / wl;
        const double c = cos(wl), s = sin(wl), c1 = 1.0 - c;
        R[0] = c + wx * wx * c1;
        R[1] = -wz * s + wx * wy * c1;
        R[2] = wy * s + wx * wz * c1;
        R[3] = wz * s + wx * wy * c1;
        R[4] = c + wy * wy * c1;
        R[5] = -wx * s + wy * wz * c1;
        R[6] = -wy * s + wx * wz * c1;
        R[7] = wx * s + wy * wz * c1;
        R[8] = c + wz * wz * c1;
    }
}

/* The rotation part of the joint and its derivatives (JointSphericalExp::update,
 * rm/Joint/JointSphericalExp.cpp:13-190): R = exp(r), Rdot, T (body angular velocity =
 * T rdot), Tdot, and their derivatives wrt r.  With d = 1 / |r|^2,
 * A_j = (r_j [r] + [r x (I - R) e_j]) d and dR/dr_j = A_j R. */
typedef struct {
    double R[9], Rdot[9], T[9], Tdot[9];
    double dR[3][9], dRdot[3][9], dT[3][9], dTdot[3][9];
} orc_rot;

static void rot_update(const double* q, const double* qd, orc_rot* o) {
    double e[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    if (norm3(q) < 1e-9) { /* |q| < math::eps: the first-order expansion about R = I */
        mz(o->R, 9);
        o->R[0] = o->R[4] = o->R[8] = 1.0;
        mz(o->Rdot, 9);
        for (int j = 0; j < 3; ++j) {
            double S[9];
            skew3(e[j], S);
            memcpy(o->dR[j], S, sizeof S);
            for (int k = 0; k < 9; ++k) o->Rdot[k] += S[k] * qd[j];
        }
        mz(o->T, 9);
        o->T[0] = o->T[4] = o->T[8] = 1.0;
        for (int j = 0; j < 3; ++j) {
            double P[9], v[3];
            m3_tmul(o->Rdot, o->dR[j], P);
            unskew3(P, v);
            for (int r = 0; r < 3; ++r) o->Tdot[3 * r + j] = v[r];
        }
        for (int k = 0; k < 3; ++k)
            for (int j = 0; j < 3; ++j) {
                double P[9], v[3];
                m3_tmul(o->dR[k], o->dR[j], P);
                unskew3(P, v);
                for (int r = 0; r < 3; ++r) o->dT[k][3 * r + j] = v[r];
            }
        /* this branch sets neither dRdot nor dTdot (JointSphericalExp.cpp:43-58); the free
         * joint reads them as zero (their values before any rotation was ever evaluated) */
        for (int k = 0; k < 3; ++k) {
            mz(o->dRdot[k], 9);
            mz(o->dTdot[k], 9);
        }
        return;
    }
    so3_exp(q, o->R);
    const double q2 = dot3(q, q), d = 1.0 / q2;
    const double qqd = dot3(q, qd);
    double A[3][9], B[3][9], C[3][9], Ad[3][9], Bd[3][9], Cd[3][9], v[3][3];
    double Sq[9], Sqd[9];
    skew3(q, Sq);
    skew3(qd, Sqd);
    for (int j = 0; j < 3; ++j) {
        for (int r = 0; r < 3; ++r) v[j][r] = e[j][r] - o->R[3 * r + j]; /* (I - R) e_j */
        skew_of_cross(q, v[j], C[j]);
        m3_scale(Sq, q[j], B[j]);
        double BC[9];
        m3_add(B[j], C[j], BC);
        m3_scale(BC, d, A[j]);
        m3_mul(A[j], o->R, o->dR[j]);
    }
    mz(o->Rdot, 9);
    for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 9; ++k) o->Rdot[k] += o->dR[j][k] * qd[j];
    const double ddot = -2.0 * qqd / (q2 * q2);
    for (int j = 0; j < 3; ++j) {
        double a[3], b[3], Rde[3], w[3];
        cross3(qd, v[j], a);
        for (int r = 0; r < 3; ++r) Rde[r] = o->Rdot[3 * r + j];
        cross3(q, Rde, b);
        for (int r = 0; r < 3; ++r) w[r] = a[r] - b[r];
        skew3(w, Cd[j]);
        for (int k = 0; k < 9; ++k) Bd[j][k] = qd[j] * Sq[k] + q[j] * Sqd[k];
        for (int k = 0; k < 9; ++k) Ad[j][k] = (Bd[j][k] + Cd[j][k]) * d + (B[j][k] + C[j][k]) * ddot;
    }
    double dd_dq[3], dddot_dq[3], dA[3][3][9], dB[3][3][9], dC[3][3][9]; /* [j][k] */
    for (int k = 0; k < 3; ++k) {
        dd_dq[k] = -2.0 * q[k] / (q2 * q2);
        for (int j = 0; j < 3; ++j) {
            double Sek[9];
            skew3(e[k], Sek);
            for (int t = 0; t < 9; ++t) dB[j][k][t] = q[j] * Sek[t] + (j == k ? Sq[t] : 0.0);
            double c1[9], dRe[3], c2v[3], c2[9];
            skew_of_cross(e[k], v[j], c1);
            for (int r = 0; r < 3; ++r) dRe[r] = o->dR[k][3 * r + j];
            cross3(q, dRe, c2v);
            for (int r = 0; r < 3; ++r) c2v[r] = -c2v[r];
            skew3(c2v, c2);
            m3_add(c1, c2, dC[j][k]);
            for (int t = 0; t < 9; ++t) dA[j][k][t] = (dB[j][k][t] + dC[j][k][t]) * d + (B[j][t] + C[j][t]) * dd_dq[k];
        }
    }
    for (int k = 0; k < 3; ++k) { /* dRdot/dq_k = sum_j (dA_jk R + A_j dR_k) qd_j */
        mz(o->dRdot[k], 9);
        for (int j = 0; j < 3; ++j) {
            double P1[9], P2[9];
            m3_mul(dA[j][k], o->R, P1);
            m3_mul(A[j], o->dR[k], P2);
            for (int t = 0; t < 9; ++t) o->dRdot[k][t] += (P1[t] + P2[t]) * qd[j];
        }
    }
    double dAd[3][3][9];
    for (int k = 0; k < 3; ++k) {
        dddot_dq[k] = (-2.0 * qd[k] * q2 + 8.0 * qqd * q[k]) / (q2 * q2 * q2);
        for (int j = 0; j < 3; ++j) {
            double Sek[9], dBd[9], dCd[9], a[3], b[3], c[3], dRe[3], Rde[3], dRde[3], w[3];
            skew3(e[k], Sek);
            for (int t = 0; t < 9; ++t) dBd[t] = qd[j] * Sek[t] + (j == k ? Sqd[t] : 0.0);
            for (int r = 0; r < 3; ++r) {
                dRe[r] = o->dR[k][3 * r + j];
                Rde[r] = o->Rdot[3 * r + j];
                dRde[r] = o->dRdot[k][3 * r + j];
            }
            cross3(qd, dRe, a);
            cross3(e[k], Rde, b);
            cross3(q, dRde, c);
            for (int r = 0; r < 3; ++r) w[r] = -a[r] - b[r] - c[r];
            skew3(w, dCd);
            for (int t = 0; t < 9; ++t)
                dAd[j][k][t] = (dBd[t] + dCd[t]) * d + (Bd[j][t] + Cd[j][t]) * dd_dq[k] +
                               (dB[j][k][t] + dC[j][k][t]) * ddot + (B[j][t] + C[j][t]) * dddot_dq[k];
        }
    }
    double Rt[9], Rdt[9];
    m3_transpose(o->R, Rt);
    m3_transpose(o->Rdot, Rdt);
    for (int j = 0; j < 3; ++j) {
        double P[9], P1[9], P2[9], P3[9], t1[9], w[3];
        m3_mul(Rt, o->dR[j], P);
        unskew3(P, w);
        for (int r = 0; r < 3; ++r) o->T[3 * r + j] = w[r];
        /* Tdot_j = unskew(Rdot^T A_j R + R^T Adot_j R + R^T A_j Rdot) */
        m3_mul(Rdt, A[j], t1);
        m3_mul(t1, o->R, P1);
        m3_mul(Rt, Ad[j], t1);
        m3_mul(t1, o->R, P2);
        m3_mul(Rt, A[j], t1);
        m3_mul(t1, o->Rdot, P3);
        for (int t = 0; t < 9; ++t) P[t] = P1[t] + P2[t] + P3[t];
        unskew3(P, w);
        for (int r = 0; r < 3; ++r) o->Tdot[3 * r + j] = w[r];
        for (int k = 0; k < 3; ++k) {
            double d2R[9], Q1[9], Q2[9], dRkt[9], dRdkt[9], S[9], u[3];
            m3_mul(dA[j][k], o->R, Q1);
            m3_mul(A[j], o->dR[k], Q2);
            for (int t = 0; t < 9; ++t) d2R[t] = Q1[t] + Q2[t];
            m3_transpose(o->dR[k], dRkt);
            m3_transpose(o->dRdot[k], dRdkt);
            /* dT_k col j = unskew(dR_k^T dR_j + R^T d2R_jk) */
            m3_mul(dRkt, o->dR[j], Q1);
            m3_mul(Rt, d2R, Q2);
            for (int t = 0; t < 9; ++t) S[t] = Q1[t] + Q2[t];
            unskew3(S, u);
            for (int r = 0; r < 3; ++r) o->dT[k][3 * r + j] = u[r];
            /* dTdot_k col j: the derivative of Tdot_j's three products wrt q_k */
            const double* terms[9][3] = {
                {dRdkt, A[j], o->R},     {Rdt, dA[j][k], o->R},  {Rdt, A[j], o->dR[k]},
                {dRkt, Ad[j], o->R},     {Rt, dAd[j][k], o->R},  {Rt, Ad[j], o->dR[k]},
                {dRkt, A[j], o->Rdot},   {Rt, dA[j][k], o->Rdot}, {Rt, A[j], o->dRdot[k]}};
            mz(S, 9);
            for (int q3 = 0; q3 < 9; ++q3) {
                double X[9], Y[9];
                m3_mul(terms[q3][0], terms[q3][1], X);
                m3_mul(X, terms[q3][2], Y);
                for (int t = 0; t < 9; ++t) S[t] += Y[t];
            }
            unskew3(S, u);
            for (int r = 0; r < 3; ++r) o->dTdot[k][3 * r + j] = u[r];
        }
    }
}

/* T only (JointSphericalExp::inner_update, :192-235), for the reparameterisation. */
static void rot_T(const double* q, double* T) {
    const double zero[3] = {0, 0, 0};
    orc_rot o;
    rot_update(q, zero, &o);
    memcpy(T, o.T, sizeof o.T);
}

/* 6x6 helpers */
static void m6_mul(const double* a, const double* b, double* c) { mm(a, b, c, 6, 6, 6); }
static void m6_transpose(const double* a, double* t) {
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) t[6 * c + r] = a[6 * r + c];
}
static void m6_vec(const double* a, const double* v, double* out) {
    for (int r = 0; r < 6; ++r) {
        double s = 0.0;
        for (int c = 0; c < 6; ++c) s += a[6 * r + c] * v[c];
        out[r] = s;
    }
}
static void m6t_vec(const double* a, const double* v, double* out) {
    for (int c = 0; c < 6; ++c) {
        double s = 0.0;
        for (int r = 0; r < 6; ++r) s += a[6 * r + c] * v[r];
        out[c] = s;
    }
}
/* math::Ad(E) (rm/Utils.h:85-94): [R 0; [p] R  R] */
static void adjoint6(const double* E, double* A) {
    double R[9], p[3], S[9], SR[9];
    pose_split(E, R, p);
    skew3(p, S);
    m3_mul(S, R, SR);
    mz(A, 36);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            A[6 * r + c] = R[3 * r + c];
            A[6 * (r + 3) + c] = SR[3 * r + c];
            A[6 * (r + 3) + c + 3] = R[3 * r + c];
        }
}
static void pose_inverse(const double* E, double* Ei) {
    double R[9], p[3];
    pose_split(E, R, p);
    mz(Ei, 16);
    for (int r = 0; r < 3; ++r) {
        double s = 0.0;
        for (int c = 0; c < 3; ++c) {
            Ei[4 * r + c] = R[3 * c + r];
            s += R[3 * c + r] * p[c];
        }
        Ei[4 * r + 3] = -s;
    }
    Ei[15] = 1.0;
}

/* Kinematics of the free body: JointFree3DExp::update (rm/Joint/JointFree3DExp.cpp:13-99),
 * Joint::update (rm/Joint/Joint.cpp:93-121: E_pj = E_pj0 Q), Body::update (Body.cpp:138-156:
 * E_0i = E_0j E_ji, phi = Ad(E_ij) phi_j) and Robot::computeJointJacobianWithDerivative for a
 * joint attached to the world (rm/Robot.cpp:687-704): J = Ad(E_ij) S_j, Jdot = Ad(E_ij) S_j_dot,
 * dJ/dq_k = Ad(E_ij) dS_j/dq_k, dJdot/dq_k = Ad(E_ij) dS_j_dot/dq_k. */
typedef struct {
    double E0i[16], phi[6];
    double J[36], Jdot[36], dJ[6][36], dJdot[6][36];
} orc_free_kin;

static void free_kinematics(const orc_mover* m, const double* q, const double* qd, orc_free_kin* k) {
    orc_rot o;
    rot_update(q + 3, qd + 3, &o);
    double S[36], Sd[36], dS[6][36], dSd[6][36];
    mz(S, 36);
    mz(Sd, 36);
    for (int i = 0; i < 6; ++i) {
        mz(dS[i], 36);
        mz(dSd[i], 36);
    }
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            S[6 * r + 3 + c] = o.T[3 * r + c];          /* angular rows, rotation columns */
            S[6 * (r + 3) + c] = o.R[3 * c + r];        /* linear rows, translation columns: R^T */
            Sd[6 * r + 3 + c] = o.Tdot[3 * r + c];
            Sd[6 * (r + 3) + c] = o.Rdot[3 * c + r];
            for (int i = 0; i < 3; ++i) {
                dS[3 + i][6 * r + 3 + c] = o.dT[i][3 * r + c];
                dS[3 + i][6 * (r + 3) + c] = o.dR[i][3 * c + r];
                dSd[3 + i][6 * r + 3 + c] = o.dTdot[i][3 * r + c];
                dSd[3 + i][6 * (r + 3) + c] = o.dRdot[i][3 * c + r];
            }
        }
    double Q[16], Eij[16], Aij[36], E0j[16];
    mz(Q, 16);
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) Q[4 * r + c] = o.R[3 * r + c];
        Q[4 * r + 3] = q[r];
    }
    Q[15] = 1.0;
    mm(m->E_pj0, Q, E0j, 4, 4, 4);
    mm(E0j, m->E_ji, k->E0i, 4, 4, 4);
    pose_inverse(m->E_ji, Eij);
    adjoint6(Eij, Aij);
    m6_mul(Aij, S, k->J);
    m6_mul(Aij, Sd, k->Jdot);
    for (int i = 0; i < 6; ++i) {
        m6_mul(Aij, dS[i], k->dJ[i]);
        m6_mul(Aij, dSd[i], k->dJdot[i]);
    }
    m6_vec(k->J, qd, k->phi);
}

/* Body::computeMaximalForceWithDerivative (rm/Body/Body.cpp:275-330): Coriolis
 * ad(phi)^T (I phi), gravity R_0i^T m g, external I .* R_0i^T f_ext, with Km (wrt the body
 * twist coordinates) and Dm (wrt phi); added to fm[6], Km[36], Dm[36]. */
static void free_body_force(const orc_mover* m, const double* E0i, const double* phi, double* fm, double* Km,
                            double* Dm) {
    double R0i[9], p0i[3], fg[3], mg[3], fh[3], ft[3];
    pose_split(E0i, R0i, p0i);
    const double* I = m->inertia;
    double adT[36], Sw[9], Sv[9];
    skew3(phi, Sw);
    skew3(phi + 3, Sv);
    mz(adT, 36); /* ad(phi)^T = [Sw^T Sv^T; 0 Sw^T] */
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            adT[6 * r + c] = Sw[3 * c + r];
            adT[6 * r + c + 3] = Sv[3 * c + r];
            adT[6 * (r + 3) + c + 3] = Sw[3 * c + r];
        }
    double Iphi[6], fc[6];
    for (int k = 0; k < 6; ++k) Iphi[k] = I[k] * phi[k];
    m6_vec(adT, Iphi, fc);
    for (int k = 0; k < 3; ++k) mg[k] = m->mass * m->gravity[k];
    m3t_vec(R0i, mg, fg);
    m3t_vec(R0i, m->f_ext, fh);
    m3t_vec(R0i, m->f_ext + 3, ft);
    for (int k = 0; k < 3; ++k) {
        fm[k] += fc[k] + I[k] * fh[k];
        fm[3 + k] += fc[3 + k] + fg[k] + I[3 + k] * ft[k];
    }
    if (!Km) return;
    double S[9];
    skew3(fg, S);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Km[6 * (3 + r) + c] += S[3 * r + c];
    double Sh[9], St[9];
    skew3(fh, Sh);
    skew3(ft, St);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            Km[6 * r + c] += Sh[3 * r + c] * I[r];
            Km[6 * (3 + r) + c] += St[3 * r + c] * I[3 + r];
        }
    for (int c = 0; c < 6; ++c)
        for (int r = 0; r < 6; ++r) Dm[6 * r + c] += adT[6 * r + c] * I[c];
    double Iw[3] = {I[0] * phi[0], I[1] * phi[1], I[2] * phi[2]};
    double mv[3] = {I[3] * phi[3], I[4] * phi[4], I[5] * phi[5]};
    double e[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int j = 0; j < 3; ++j) {
        double a[3], b[3];
        cross3(e[j], Iw, a);
        cross3(e[j], mv, b);
        for (int r = 0; r < 3; ++r) {
            Dm[6 * r + j] -= a[r];
            Dm[6 * r + 3 + j] -= b[r];
            Dm[6 * (3 + r) + j] -= b[r];
        }
    }
}

/* One evaluation of the free mover at (q1, qdot1 = (q1 - q0) / h): g, H, M, D of
 * Simulation::evaluate_g[_with_derivatives]_BDF1 (Simulation.cpp:1081-1165) with
 * Simulation::computeMatrices (:422-503) for a single body:
 *   M = J^T Mm J, f = J^T fm - J^T Mm Jdot qdot + fr,
 *   dM/dq_k = dJ_k^T Mm J + (dJ_k^T Mm J)^T,
 *   K = Kqvv + Kr + J^T Km J + J^T Dm (dJ/dq qdot) + [dJ_k^T fm]_k,
 *   D = -J^T Mm Jdot - J^T Mm (dJ/dq qdot) + Dr + J^T Dm J,
 *   H = M - h^2 K - h D + [dM/dq_k (q1 - q0 - h qdot0)]_k.
 * Optional outputs: H, M, D (36 each) and J, E0i for the adjoint. */
static void free_eval_full(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q0,
                           const double* qdot0, const double* q1, double* g, double* H, double* M_out, double* D_out,
                           double* J_out, double* E0i_out) {
    const double h = m->h;
    const int want = H != NULL || D_out != NULL;
    double qd1[6];
    for (int k = 0; k < 6; ++k) qd1[k] = (q1[k] - q0[k]) / h;
    orc_free_kin kin;
    free_kinematics(m, q1, qd1, &kin);
    double fm[6] = {0}, Km[36] = {0}, Dm[36] = {0};
    free_body_force(m, kin.E0i, kin.phi, fm, want ? Km : NULL, Dm);
    const double zero6[6] = {0, 0, 0, 0, 0, 0};
    for (int c = 0; c < n_pairs; ++c) {
        const orc_pair* P = pairs + c;
        double pf[12], pK[144], pD[144];
        const double *EA, *phiA, *EB, *phiB;
        if (P->mover_is_contact) {
            EA = kin.E0i; phiA = kin.phi; EB = P->E_fixed; phiB = zero6;
        } else {
            EA = P->E_fixed; phiA = zero6; EB = kin.E0i; phiB = kin.phi;
        }
        orc_pair_eval(P->grid, P->pts, P->n_pts, EA, phiA, EB, phiB, &P->prm, want, pf, pK, pD, NULL);
        const int o = P->mover_is_contact ? 0 : 6;
        for (int r = 0; r < 6; ++r) {
            fm[r] += pf[o + r];
            if (want)
                for (int s = 0; s < 6; ++s) {
                    Km[6 * r + s] += pK[(o + r) * 12 + o + s];
                    Dm[6 * r + s] += pD[(o + r) * 12 + o + s];
                }
        }
    }
    const double* Mm = m->inertia;
    double MmJ[36], JT[36], M[36], MmJdot[36], JTMmJdot[36], fqvv[6], f[6], t6[6];
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) {
            MmJ[6 * r + c] = kin.J[6 * r + c] * Mm[r];
            MmJdot[6 * r + c] = kin.Jdot[6 * r + c] * Mm[r];
        }
    m6_transpose(kin.J, JT);
    m6_mul(JT, MmJ, M);
    m6_mul(JT, MmJdot, JTMmJdot); /* J^T Mm Jdot */
    m6_vec(JTMmJdot, qd1, fqvv);
    m6t_vec(kin.J, fm, t6);
    for (int k = 0; k < 6; ++k) {
        const double fr = -m->joint_stiffness * (q1[k] - m->q_rest[k]) - m->joint_damping * qd1[k];
        f[k] = t6[k] - fqvv[k] + fr;
    }
    double dq[6], Mdq[6];
    for (int k = 0; k < 6; ++k) dq[k] = q1[k] - q0[k] - h * qdot0[k];
    m6_vec(M, dq, Mdq);
    for (int k = 0; k < 6; ++k) g[k] = Mdq[k] - h * h * f[k];
    if (M_out) memcpy(M_out, M, sizeof M);
    if (J_out) memcpy(J_out, kin.J, sizeof kin.J);
    if (E0i_out) memcpy(E0i_out, kin.E0i, sizeof kin.E0i);
    if (!want) return;
    double dJq[36]; /* column k = dJ_k qdot */
    for (int k = 0; k < 6; ++k) {
        double v[6];
        m6_vec(kin.dJ[k], qd1, v);
        for (int r = 0; r < 6; ++r) dJq[6 * r + k] = v[r];
    }
    double JTMm[36], Dqvv[36], X[36], MmJdq[6], K[36], D[36], JTDm[36], Y[36];
    m6_transpose(MmJ, JTMm);
    m6_mul(JTMm, dJq, X);
    for (int t = 0; t < 36; ++t) Dqvv[t] = -JTMmJdot[t] - X[t];
    double MmJdotqd[6];
    m6_vec(MmJdot, qd1, MmJdotqd);
    m6_mul(JT, Dm, JTDm);
    double JTKm[36], JTKmJ[36];
    m6_mul(JT, Km, JTKm);
    m6_mul(JTKm, kin.J, JTKmJ);
    m6_mul(JTDm, dJq, Y);
    for (int t = 0; t < 36; ++t) K[t] = JTKmJ[t] + Y[t];
    for (int k = 0; k < 6; ++k) {
        double a[6], b[6], c[6], dJdq[6];
        m6t_vec(kin.dJ[k], MmJdotqd, a);  /* dJ_k^T Mm Jdot qdot */
        m6_vec(kin.dJdot[k], qd1, dJdq);  /* dJdot_k qdot */
        m6_vec(JTMm, dJdq, b);
        m6t_vec(kin.dJ[k], fm, c);        /* dJ_k^T fm */
        (void)MmJdq;
        for (int r = 0; r < 6; ++r) K[6 * r + k] += -a[r] - b[r] + c[r];
        K[6 * k + k] -= m->joint_stiffness;
    }
    double JTDmJ[36];
    m6_mul(JTDm, kin.J, JTDmJ);
    for (int t = 0; t < 36; ++t) D[t] = Dqvv[t] + JTDmJ[t];
    for (int k = 0; k < 6; ++k) D[6 * k + k] -= m->joint_damping;
    if (D_out) memcpy(D_out, D, sizeof D);
    if (H) {
        for (int t = 0; t < 36; ++t) H[t] = M[t] - h * h * K[t] - h * D[t];
        for (int k = 0; k < 6; ++k) {
            double T1[36], T2[36], dMk[36], v[6];
            m6_transpose(kin.dJ[k], T1);
            m6_mul(T1, MmJ, T2);
            m6_transpose(T2, T1);
            for (int t = 0; t < 36; ++t) dMk[t] = T2[t] + T1[t];
            m6_vec(dMk, dq, v);
            for (int r = 0; r < 6; ++r) H[6 * r + k] += v[r];
        }
    }
}

/* ---- dispatch on the joint */

static int mover_ndof(const orc_mover* m) { return m->ndof == 6 ? 6 : 3; }

void orc_mover_pose(const orc_mover* m, const double* q, const double* qdot, double* E0i, double* phi) {
    if (mover_ndof(m) == 3) {
        trans_pose(m, q, qdot, E0i, phi);
        return;
    }
    orc_free_kin kin;
    free_kinematics(m, q, qdot, &kin);
    memcpy(E0i, kin.E0i, sizeof kin.E0i);
    memcpy(phi, kin.phi, sizeof kin.phi);
}

void orc_bdf1_eval_full(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q0,
                        const double* qdot0, const double* q1, double* g, double* H, double* M, double* D) {
    if (mover_ndof(m) == 3)
        trans_eval_full(m, pairs, n_pairs, q0, qdot0, q1, g, H, M, D);
    else
        free_eval_full(m, pairs, n_pairs, q0, qdot0, q1, g, H, M, D, NULL, NULL);
}

void orc_bdf1_eval(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q0, const double* qdot0,
                   const double* q1, double* g, double* H) {
    orc_bdf1_eval_full(m, pairs, n_pairs, q0, qdot0, q1, g, H, NULL, NULL);
}

/* Partial-pivoting LU (PA = LU, L unit lower in the same array) of an n x n matrix, n <= 6: the
 * algorithm of Eigen's PartialPivLU used by Simulation::newton (:1028) and stored for the
 * adjoint (:1267). */
static void lu_n(const double* A_in, int n, double* LU, int* perm) {
    memcpy(LU, A_in, sizeof(double) * (size_t)(n * n));
    for (int k = 0; k < n; ++k) perm[k] = k;
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(LU[n * r + c]) > fabs(LU[n * p + c])) p = r;
        if (p != c) {
            for (int k = 0; k < n; ++k) {
                double t = LU[n * c + k];
                LU[n * c + k] = LU[n * p + k];
                LU[n * p + k] = t;
            }
            int t = perm[c];
            perm[c] = perm[p];
            perm[p] = t;
        }
        for (int r = c + 1; r < n; ++r) {
            LU[n * r + c] /= LU[n * c + c];
            for (int k = c + 1; k < n; ++k) LU[n * r + k] -= LU[n * r + c] * LU[n * c + k];
        }
    }
}

/* A x = b with the factors */
static void lu_solve_n(const double* LU, const int* perm, int n, const double* b, double* x) {
    double y[6];
    for (int r = 0; r < n; ++r) {
        double s = b[perm[r]];
        for (int k = 0; k < r; ++k) s -= LU[n * r + k] * y[k];
        y[r] = s;
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = y[r];
        for (int k = r + 1; k < n; ++k) s -= LU[n * r + k] * x[k];
        x[r] = s / LU[n * r + r];
    }
}

/* A^T z = y with the factors: U^T w = y, L^T u = w, z = P^T u */
static void lu_solve_transposed_n(const double* LU, const int* perm, int n, const double* y, double* z) {
    double w[6], u[6];
    for (int r = 0; r < n; ++r) {
        double s = y[r];
        for (int k = 0; k < r; ++k) s -= LU[n * k + r] * w[k];
        w[r] = s / LU[n * r + r];
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = w[r];
        for (int k = r + 1; k < n; ++k) s -= LU[n * k + r] * u[k];
        u[r] = s;
    }
    for (int r = 0; r < n; ++r) z[perm[r]] = u[r];
}

/* Gaussian elimination with partial pivoting, the 3-dof solve of the Newton step (the same
 * operations as lu_n + lu_solve_n, in the order the translational restatement pinned). */
static void solve_newton(const double* A_in, const double* b_in, int n, double* x) {
    double A[36], b[6];
    memcpy(A, A_in, sizeof(double) * (size_t)(n * n));
    memcpy(b, b_in, sizeof(double) * (size_t)n);
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(A[n * r + c]) > fabs(A[n * p + c])) p = r;
        if (p != c) {
            for (int k = 0; k < n; ++k) {
                double t = A[n * c + k];
                A[n * c + k] = A[n * p + k];
                A[n * p + k] = t;
            }
            double t = b[c];
            b[c] = b[p];
            b[p] = t;
        }
        for (int r = c + 1; r < n; ++r) {
            double l = A[n * r + c] / A[n * c + c];
            for (int k = c; k < n; ++k) A[n * r + k] -= l * A[n * c + k];
            b[r] -= l * b[c];
        }
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = b[r];
        for (int k = r + 1; k < n; ++k) s -= A[n * r + k] * x[k];
        x[r] = s / A[n * r + r];
    }
}

static double norm_n(const double* v, int n) {
    double s = 0.0;
    for (int k = 0; k < n; ++k) s += v[k] * v[k];
    return sqrt(s);
}

/* JointSphericalExp::reparam (rm/Joint/JointSphericalExp.cpp:237-266), called by
 * Simulation::forward after every step (Simulation.cpp:955-957): a rotation vector longer
 * than 1.5 pi is shortened by 2 pi and its rate mapped so the body's angular velocity stays. */
static void free_reparam(double* q, double* qd) {
    double* r = q + 3;
    double rn = norm3(r);
    if (rn <= 1.5 * M_PI) return;
    double S0[9], S1[9], w[3], LU[9];
    int perm[3];
    rot_T(r, S0);
    while (rn > 1.5 * M_PI) {
        const double s = 1.0 - 2.0 * M_PI / rn;
        for (int k = 0; k < 3; ++k) r[k] *= s;
        rn = norm3(r);
    }
    rot_T(r, S1);
    m3_vec(S0, qd + 3, w);
    lu_n(S1, 3, LU, perm);
    lu_solve_n(LU, perm, 3, w, qd + 3);
}

/* Simulation::integration_BDF1 (Simulation.cpp:1248-1270) with Simulation::newton
 * (:999-1079): tolerance 1e-8 on |g|, at most max(20 ndof, 100) iterations, backtracking
 * line search halving alpha up to 20 times, 3 consecutive line-search failures stop; then the
 * free joint's reparameterisation (:955-957). */
int orc_bdf1_step(const orc_mover* m, const orc_pair* pairs, int n_pairs, double* q, double* qdot, int* iters,
                  int* evals) {
    const int n = mover_ndof(m);
    const double h = m->h, tol = m->newton_tol > 0.0 ? m->newton_tol : 1e-8;
    const int max_iter = 20 * n > 100 ? 20 * n : 100, max_ls = 20, max_strike = 3;
    double q0[6], qd0[6], x[6];
    for (int k = 0; k < n; ++k) {
        q0[k] = q[k];
        qd0[k] = qdot[k];
        x[k] = q0[k] + h * qd0[k];
    }
    int converged = 0, strike = 0, it = 0, ev = 0;
    for (; it < max_iter; ++it) {
        double g[6], H[36], dx[6], mg[6];
        orc_bdf1_eval(m, pairs, n_pairs, q0, qd0, x, g, H);
        ++ev;
        for (int k = 0; k < n; ++k) mg[k] = -g[k];
        solve_newton(H, mg, n, dx);
        const double gnorm = norm_n(g, n);
        double alpha = 1.0, gn[6] = {0, 0, 0, 0, 0, 0};
        int ok = 0;
        for (int trial = 0; trial < max_ls; ++trial, alpha *= 0.5) {
            double xt[6];
            for (int k = 0; k < n; ++k) xt[k] = x[k] + alpha * dx[k];
            orc_bdf1_eval(m, pairs, n_pairs, q0, qd0, xt, gn, NULL);
            ++ev;
            if (norm_n(gn, n) < gnorm) {
                ok = 1;
                break;
            }
        }
        if (ok) {
            strike = 0;
        } else if (++strike >= max_strike) {
            break;
        }
        for (int k = 0; k < n; ++k) x[k] = x[k] + alpha * dx[k];
        if (norm_n(gn, n) < tol) {
            converged = 1;
            break;
        }
    }
    for (int k = 0; k < n; ++k) {
        qdot[k] = (x[k] - q0[k]) / h;
        q[k] = x[k];
    }
    if (n == 6) free_reparam(q, qdot);
    if (iters) *iters = it + (converged ? 1 : 0);
    if (evals) *evals = ev;
    return converged;
}

/* ------------------------------------------------------------------ adjoint of the BDF1 rollout */

/* Simulation::backward_BDF1 (Simulation.cpp:1559-1634) for one moving part, with the per-step
 * H, M, D that the reference saves after each converged step (integration_BDF1, :1262-1269:
 * evaluate_g_with_derivatives_BDF1 at q_k with qdot_k = (q_k - q_{k-1}) / h) recomputed here from
 * the trajectory q_his[0..T] (the reparameterisation is not differentiated, as in the reference).
 * df_dq[T x n] is dL/dq_k for k = 1..T.  Outputs dL/dq_0, dL/dqdot_0 and, beyond the reference,
 * dL/df_ext: the external force enters step k's f as J_k^T diag(I) blkdiag(R_0i^T, R_0i^T) f_ext
 * (Body.cpp:288-289), so dL/df_ext = h^2 sum_k blkdiag(R_0i, R_0i) diag(I) J_k z_k.  (For the
 * translational joint J = [0; R_ji^T], which leaves the torque rows 0.) */
void orc_bdf1_backward(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q_his,
                       const double* qdot0, int T, const double* df_dq, double* df_dq0, double* df_dqdot0,
                       double* df_dfext) {
    const int n = mover_ndof(m), nn = n * n;
    const double h = m->h;
    const size_t TT = (size_t)(T > 0 ? T : 1);
    double* Ms = (double*)calloc(TT * (3 * (size_t)nn + 6), sizeof(double));
    double* Ds = Ms + nn * TT;
    double* Hs = Ds + nn * TT;
    double* U = Hs + nn * TT; /* per step: blkdiag(R_0i) diag(I) J applied to z, filled below */
    double* z = (double*)calloc(TT * (size_t)n, sizeof(double));
    double* Js = (double*)calloc(TT * 36, sizeof(double));
    double* Rs = (double*)calloc(TT * 9, sizeof(double));
    for (int k = 1; k <= T; ++k) { /* the saved step data */
        double qd_prev[6], g[6];
        const double* qp = q_his + n * (k - 1);
        if (k == 1) {
            memcpy(qd_prev, qdot0, sizeof(double) * (size_t)n);
        } else {
            for (int c = 0; c < n; ++c) qd_prev[c] = (qp[c] - q_his[n * (k - 2) + c]) / h;
        }
        double* Hk = Hs + nn * (size_t)(k - 1);
        double* Mk = Ms + nn * (size_t)(k - 1);
        double* Dk = Ds + nn * (size_t)(k - 1);
        if (n == 3) {
            trans_eval_full(m, pairs, n_pairs, qp, qd_prev, q_his + 3 * k, g, Hk, Mk, Dk);
            double E0i[16], phi[6], p0i[3], Rji[9], pji[3];
            double qd1[3];
            for (int c = 0; c < 3; ++c) qd1[c] = (q_his[3 * k + c] - qp[c]) / h;
            trans_pose(m, q_his + 3 * k, qd1, E0i, phi);
            pose_split(E0i, Rs + 9 * (size_t)(k - 1), p0i);
            pose_split(m->E_ji, Rji, pji);
            double* J = Js + 36 * (size_t)(k - 1); /* 6 x 3: [0; R_ji^T] */
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) J[3 * (3 + r) + c] = Rji[3 * c + r];
        } else {
            double E0i[16], p0i[3];
            free_eval_full(m, pairs, n_pairs, qp, qd_prev, q_his + 6 * k, g, Hk, Mk, Dk, Js + 36 * (size_t)(k - 1),
                           E0i);
            pose_split(E0i, Rs + 9 * (size_t)(k - 1), p0i);
        }
    }
    for (int k = T - 1; k >= 0; --k) { /* z_k for step k + 1 */
        double y[6], LU[36];
        int perm[6];
        for (int c = 0; c < n; ++c) y[c] = df_dq[n * k + c];
        if (k < T - 1) {
            const double* M1 = Ms + nn * (size_t)(k + 1);
            const double* D1 = Ds + nn * (size_t)(k + 1);
            for (int c = 0; c < n; ++c)
                for (int r = 0; r < n; ++r) y[c] -= (-2.0 * M1[n * r + c] + h * D1[n * r + c]) * z[n * (k + 1) + r];
        }
        if (k < T - 2) {
            const double* M2 = Ms + nn * (size_t)(k + 2);
            for (int c = 0; c < n; ++c)
                for (int r = 0; r < n; ++r) y[c] -= M2[n * r + c] * z[n * (k + 2) + r];
        }
        lu_n(Hs + nn * (size_t)k, n, LU, perm);
        lu_solve_transposed_n(LU, perm, n, y, z + n * k);
    }
    double g0[6] = {0}, gd0[6] = {0};
    if (T > 0)
        for (int c = 0; c < n; ++c)
            for (int r = 0; r < n; ++r) {
                g0[c] -= (-Ms[n * r + c] + h * Ds[n * r + c]) * z[r];
                gd0[c] -= (-h * Ms[n * r + c]) * z[r];
            }
    if (T > 1)
        for (int c = 0; c < n; ++c)
            for (int r = 0; r < n; ++r) g0[c] -= Ms[nn + n * r + c] * z[n + r];
    if (df_dq0) memcpy(df_dq0, g0, sizeof(double) * (size_t)n);
    if (df_dqdot0) memcpy(df_dqdot0, gd0, sizeof(double) * (size_t)n);
    if (df_dfext) {
        double acc[6] = {0};
        for (int k = 0; k < T; ++k) {
            const double* J = Js + 36 * (size_t)k; /* 6 x n */
            const double* R = Rs + 9 * (size_t)k;
            double Jz[6], w[3], v[3];
            for (int r = 0; r < 6; ++r) {
                double s = 0.0;
                for (int c = 0; c < n; ++c) s += J[n * r + c] * z[n * k + c];
                Jz[r] = s * m->inertia[r];
            }
            m3_vec(R, Jz, w);
            m3_vec(R, Jz + 3, v);
            for (int c = 0; c < 3; ++c) {
                acc[c] += w[c];
                acc[3 + c] += v[c];
            }
        }
        for (int c = 0; c < 6; ++c) df_dfext[c] = h * h * acc[c];
    }
    (void)U;
    free(Ms);
    free(z);
    free(Js);
    free(Rs);
}

/* ------------------------------------------------------------------ mesh -> SDF grid */

/* sdfgen::make_level_set3 (simulation/externals/sdfgen/makelevelset3.cpp:161-227), the grid
 * builder of BodySDFObj::precompute_SDF (rm/Body/BodySDFObj.cpp:38-84), in FP32 with its operation
 * order (vec.h: sums in index order; compiled without contraction).  Sequential, like the
 * reference; the GPU runs the same arithmetic with the sweeps as diagonal wavefronts. */
typedef struct {
    float v[3];
} ov3;

static ov3 ov_sub(ov3 a, ov3 b) {
    ov3 r = {{a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]}};
    return r;
}
static ov3 ov_scale(float s, ov3 a) {
    ov3 r = {{s * a.v[0], s * a.v[1], s * a.v[2]}};
    return r;
}
static ov3 ov_add(ov3 a, ov3 b) {
    ov3 r = {{a.v[0] + b.v[0], a.v[1] + b.v[1], a.v[2] + b.v[2]}};
    return r;
}
static float ov_dot(ov3 a, ov3 b) {
    float d = a.v[0] * b.v[0];
    d += a.v[1] * b.v[1];
    d += a.v[2] * b.v[2];
    return d;
}
static float ov_mag2(ov3 a) { return ov_dot(a, a); }
static float ov_dist(ov3 a, ov3 b) {
    float d = (a.v[0] - b.v[0]) * (a.v[0] - b.v[0]);
    d += (a.v[1] - b.v[1]) * (a.v[1] - b.v[1]);
    d += (a.v[2] - b.v[2]) * (a.v[2] - b.v[2]);
    return sqrtf(d);
}
static float ofmin(float a, float b) { return b < a ? b : a; }  /* std::min */

static float seg_dist(ov3 x0, ov3 x1, ov3 x2) { /* point_segment_distance */
    ov3 dx = ov_sub(x2, x1);
    double m2 = (double)ov_mag2(dx);
    float s12 = (float)((double)ov_dot(ov_sub(x2, x0), dx) / m2);
    if (s12 < 0)
        s12 = 0;
    else if (s12 > 1)
        s12 = 1;
    return ov_dist(x0, ov_add(ov_scale(s12, x1), ov_scale(1 - s12, x2)));
}

static float tri_dist(ov3 x0, ov3 x1, ov3 x2, ov3 x3) { /* point_triangle_distance */
    ov3 x13 = ov_sub(x1, x3), x23 = ov_sub(x2, x3), x03 = ov_sub(x0, x3);
    float m13 = ov_mag2(x13), m23 = ov_mag2(x23), d = ov_dot(x13, x23);
    float den = m13 * m23 - d * d;
    float invdet = 1.f / (den < 1e-30f ? 1e-30f : den); /* max(den, 1e-30f) */
    float a = ov_dot(x13, x03), b = ov_dot(x23, x03);
    float w23 = invdet * (m23 * a - d * b);
    float w31 = invdet * (m13 * b - d * a);
    float w12 = 1 - w23 - w31;
    if (w23 >= 0 && w31 >= 0 && w12 >= 0)
        return ov_dist(x0, ov_add(ov_add(ov_scale(w23, x1), ov_scale(w31, x2)), ov_scale(w12, x3)));
    if (w23 > 0) return ofmin(seg_dist(x0, x1, x2), seg_dist(x0, x1, x3));
    if (w31 > 0) return ofmin(seg_dist(x0, x1, x2), seg_dist(x0, x2, x3));
    return ofmin(seg_dist(x0, x1, x3), seg_dist(x0, x2, x3));
}

static int orient2(double x1, double y1, double x2, double y2, double* area) { /* orientation, SOS */
    *area = y1 * x2 - x1 * y2;
    if (*area > 0) return 1;
    if (*area < 0) return -1;
    if (y2 > y1) return 1;
    if (y2 < y1) return -1;
    if (x1 > x2) return 1;
    if (x1 < x2) return -1;
    return 0;
}

static int in_tri_2d(double x0, double y0, double x1, double y1, double x2, double y2, double x3, double y3,
                     double* a, double* b, double* c) { /* point_in_triangle_2d */
    x1 -= x0; x2 -= x0; x3 -= x0;
    y1 -= y0; y2 -= y0; y3 -= y0;
    int sa = orient2(x2, y2, x3, y3, a);
    if (sa == 0) return 0;
    int sb = orient2(x3, y3, x1, y1, b);
    if (sb != sa) return 0;
    int sc = orient2(x1, y1, x2, y2, c);
    if (sc != sa) return 0;
    double sum = *a + *b + *c;
    *a /= sum;
    *b /= sum;
    *c /= sum;
    return 1;
}

static int oclampi(int a, int lo, int hi) { return a < lo ? lo : (a > hi ? hi : a); }
/* sdfgen::min / max of three: min(a1, min(a2, a3)) with std::min(a, b) = b < a ? b : a and
 * std::max(a, b) = a < b ? b : a */
static double omin3(double a, double b, double c) { double m = c < b ? c : b; return m < a ? m : a; }
static double omax3(double a, double b, double c) { double m = b < c ? c : b; return a < m ? m : a; }

void orc_make_level_set3(const float* verts, int nv, const unsigned* tris, int nt, const float* origin, float dx,
                         float dy, float dz, int ni, int nj, int nk, int band, float* phi) {
    (void)nv;
    const size_t n = (size_t)ni * nj * nk;
    int* closest = (int*)malloc(sizeof(int) * n);
    int* count = (int*)calloc(n, sizeof(int));
    const float init = (float)(ni + nj + nk) * (dx + dy + dz);
#define OIX(i, j, k) ((size_t)(i) + (size_t)ni * ((size_t)(j) + (size_t)nj * (size_t)(k)))
    for (size_t q = 0; q < n; ++q) {
        phi[q] = init;
        closest[q] = -1;
    }
    ov3 o = {{origin[0], origin[1], origin[2]}};
    for (int t = 0; t < nt; ++t) {
        unsigned p = tris[3 * t], q = tris[3 * t + 1], r = tris[3 * t + 2];
        ov3 xp = {{verts[3 * p], verts[3 * p + 1], verts[3 * p + 2]}};
        ov3 xq = {{verts[3 * q], verts[3 * q + 1], verts[3 * q + 2]}};
        ov3 xr = {{verts[3 * r], verts[3 * r + 1], verts[3 * r + 2]}};
        double fip = ((double)xp.v[0] - o.v[0]) / dx, fjp = ((double)xp.v[1] - o.v[1]) / dy,
               fkp = ((double)xp.v[2] - o.v[2]) / dz;
        double fiq = ((double)xq.v[0] - o.v[0]) / dx, fjq = ((double)xq.v[1] - o.v[1]) / dy,
               fkq = ((double)xq.v[2] - o.v[2]) / dz;
        double fir = ((double)xr.v[0] - o.v[0]) / dx, fjr = ((double)xr.v[1] - o.v[1]) / dy,
               fkr = ((double)xr.v[2] - o.v[2]) / dz;
        int i0 = oclampi((int)omin3(fip, fiq, fir) - band, 0, ni - 1),
            i1 = oclampi((int)omax3(fip, fiq, fir) + band + 1, 0, ni - 1);
        int j0 = oclampi((int)omin3(fjp, fjq, fjr) - band, 0, nj - 1),
            j1 = oclampi((int)omax3(fjp, fjq, fjr) + band + 1, 0, nj - 1);
        int k0 = oclampi((int)omin3(fkp, fkq, fkr) - band, 0, nk - 1),
            k1 = oclampi((int)omax3(fkp, fkq, fkr) + band + 1, 0, nk - 1);
        for (int k = k0; k <= k1; ++k)
            for (int j = j0; j <= j1; ++j)
                for (int i = i0; i <= i1; ++i) {
                    ov3 gx = {{(float)i * dx + o.v[0], (float)j * dy + o.v[1], (float)k * dz + o.v[2]}};
                    float d = tri_dist(gx, xp, xq, xr);
                    if (d < phi[OIX(i, j, k)]) {
                        phi[OIX(i, j, k)] = d;
                        closest[OIX(i, j, k)] = t;
                    }
                }
        j0 = oclampi((int)ceil(omin3(fjp, fjq, fjr)), 0, nj - 1);
        j1 = oclampi((int)floor(omax3(fjp, fjq, fjr)), 0, nj - 1);
        k0 = oclampi((int)ceil(omin3(fkp, fkq, fkr)), 0, nk - 1);
        k1 = oclampi((int)floor(omax3(fkp, fkq, fkr)), 0, nk - 1);
        for (int k = k0; k <= k1; ++k)
            for (int j = j0; j <= j1; ++j) {
                double a, b, c;
                if (in_tri_2d(j, k, fjp, fkp, fjq, fkq, fjr, fkr, &a, &b, &c)) {
                    double fi = a * fip + b * fiq + c * fir;
                    int iv = (int)ceil(fi);
                    if (iv < 0)
                        ++count[OIX(0, j, k)];
                    else if (iv < ni)
                        ++count[OIX(iv, j, k)];
                }
            }
    }
    static const int dirs[8][3] = {{1, 1, 1}, {-1, -1, -1}, {1, 1, -1}, {-1, -1, 1},
                                   {1, -1, 1}, {-1, 1, -1}, {1, -1, -1}, {-1, 1, 1}};
    for (int pass = 0; pass < 2; ++pass)
        for (int s = 0; s < 8; ++s) {
            const int di = dirs[s][0], dj = dirs[s][1], dk = dirs[s][2];
            const int ia = di > 0 ? 1 : ni - 2, ib = di > 0 ? ni : -1;
            const int ja = dj > 0 ? 1 : nj - 2, jb = dj > 0 ? nj : -1;
            const int ka = dk > 0 ? 1 : nk - 2, kb = dk > 0 ? nk : -1;
            for (int k = ka; k != kb; k += dk)
                for (int j = ja; j != jb; j += dj)
                    for (int i = ia; i != ib; i += di) {
                        ov3 gx = {{(float)i * dx + o.v[0], (float)j * dy + o.v[1], (float)k * dz + o.v[2]}};
                        const int nb[7][3] = {{i - di, j, k},      {i, j - dj, k},      {i - di, j - dj, k},
                                              {i, j, k - dk},      {i - di, j, k - dk}, {i, j - dj, k - dk},
                                              {i - di, j - dj, k - dk}};
                        for (int m = 0; m < 7; ++m) { /* check_neighbour */
                            const int ct = closest[OIX(nb[m][0], nb[m][1], nb[m][2])];
                            if (ct >= 0) {
                                unsigned p = tris[3 * ct], q = tris[3 * ct + 1], r = tris[3 * ct + 2];
                                ov3 xp = {{verts[3 * p], verts[3 * p + 1], verts[3 * p + 2]}};
                                ov3 xq = {{verts[3 * q], verts[3 * q + 1], verts[3 * q + 2]}};
                                ov3 xr = {{verts[3 * r], verts[3 * r + 1], verts[3 * r + 2]}};
                                float d = tri_dist(gx, xp, xq, xr);
                                if (d < phi[OIX(i, j, k)]) {
                                    phi[OIX(i, j, k)] = d;
                                    closest[OIX(i, j, k)] = ct;
                                }
                            }
                        }
                    }
        }
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj; ++j) {
            int total = 0;
            for (int i = 0; i < ni; ++i) {
                total += count[OIX(i, j, k)];
                if (total % 2 == 1) phi[OIX(i, j, k)] = -phi[OIX(i, j, k)];
            }
        }
#undef OIX
    free(closest);
    free(count);
}
