// The free3d-exp reduced system of sdfc_joint.cuh (rot_update, free_system) computed by one warp
// per scene.  The one-thread version is a chain of small matrix products, about 15k dependent
// FP64 operations per Newton evaluation; a batched BDF1 round waits for its slowest scene, so
// that chain's latency bounds every round.  Here each step of the same computation fills one
// shared-memory array, the lanes splitting its entries, with every entry's expression written
// as in the one-thread version (same operands, same order), and a __syncwarp between steps.
#pragma once

#include "sdfc_joint.cuh"

namespace sdfc_joint {

// Per-entry forms of the 3x3 / 6x6 products of sdfc_joint.cuh.
__device__ __forceinline__ double e_mul3(const double* a, const double* b, int r, int s) {
    return a[3 * r] * b[s] + a[3 * r + 1] * b[3 + s] + a[3 * r + 2] * b[6 + s];
}
__device__ __forceinline__ double e_tmul3(const double* a, const double* b, int r, int s) {  // (a^T b)_rs
    return a[r] * b[s] + a[3 + r] * b[3 + s] + a[6 + r] * b[6 + s];
}
__device__ __forceinline__ double e_mul6(const double* a, const double* b, int r, int s) {
    double v = 0.0;
    for (int k = 0; k < 6; ++k) v += a[6 * r + k] * b[6 * k + s];
    return v;
}
__device__ __forceinline__ double e_tmul6(const double* a, const double* b, int r, int s) {
    double v = 0.0;
    for (int k = 0; k < 6; ++k) v += a[6 * k + r] * b[6 * k + s];
    return v;
}
__device__ __forceinline__ double e_mv6(const double* a, const double* x, int r) {
    double v = 0.0;
    for (int k = 0; k < 6; ++k) v += a[6 * r + k] * x[k];
    return v;
}
__device__ __forceinline__ double e_tmv6(const double* a, const double* x, int r) {
    double v = 0.0;
    for (int k = 0; k < 6; ++k) v += a[6 * k + r] * x[k];
    return v;
}

// One warp's scratch (shared memory).  Index conventions: [j][t] = 9 j + t,
// [j][k][t] = 9 (3 j + k) + t, [k][j][t] = 9 (3 k + j) + t.
struct FreeWarp {
    // rot_update
    double R[9], Rdot[9], T[9], Tdot[9];
    double dR[27], dRdot[27], dT[27], dTdot[27];  // [k][t]
    double A[27], BC[27], Ad[27], BCd[27];        // [j][t]
    double X1[27], X2[27], X3[27];                // [j][t]
    double dA[81], dBC[81];                       // [j][k][t]
    double dAd[81], d2R[81];                      // [k][j][t]
    double TX[729];                               // [k][j][m][t]
    // free_system
    double Aij[36], S[36], Sd[36], J[36], Jd[36], E0j[16], E0i[16];
    double phi[6], fm[6], f[6], dq[6], g[6], MmJdqd[6], MmJdq[6];
    double MmJ[36], MmJd[36], M[36], JTMmJd[36];
    double Km[36], Dm[36], X[36], Y[36], K[36], Dd[36], H[36], dJq[36];
    double dS[108], dSd[108], dJ[108], dJd[108];  // [k - 3][36]
    double dJdq[18], dJdqv[18], dMcols[18];       // [k - 3][6]
    // contact sums and scene inputs
    double fmc[6], Kmc[36], Dmc[36];
};

#define SDFC_WFOR(t, n) for (int t = (int)(threadIdx.x & 31); t < (n); t += 32)

// the entry of a 3x3 product that unskew reads for row r of the column: (a21, a02, a10)
__device__ __forceinline__ int unskew_entry(int r) { return r == 0 ? 7 : (r == 1 ? 2 : 3); }

// rot_update by one warp (same arithmetic).
__device__ inline void rot_update_w(const double* q, const double* qd, bool deriv, FreeWarp& w) {
    const int lane = threadIdx.x & 31;
    const double E[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    if (norm3(q) < 1e-9) {  // first-order branch about R = I: rare, run by lane 0
        if (lane == 0) {
            Rot o;
            rot_update(q, qd, deriv, o);
            for (int t = 0; t < 9; ++t) {
                w.R[t] = o.R[t];
                w.Rdot[t] = o.Rdot[t];
                w.T[t] = o.T[t];
                w.Tdot[t] = o.Tdot[t];
                for (int k = 0; k < 3; ++k) {
                    w.dR[9 * k + t] = o.dR[k][t];
                    w.dRdot[9 * k + t] = o.dRdot[k][t];
                    w.dT[9 * k + t] = o.dT[k][t];
                    w.dTdot[9 * k + t] = o.dTdot[k][t];
                }
            }
        }
        __syncwarp();
        return;
    }
    double Rl[9];
    so3_exp(q, Rl);
    if (lane < 9) w.R[lane] = Rl[lane];
    const double q2 = dot3(q, q), d = 1.0 / q2, qqd = dot3(q, qd);
    double Sq[9], Sqd[9];
    skew(q, Sq);
    skew(qd, Sqd);
    SDFC_WFOR(t, 27) {
        const int j = t / 9, k = t % 9;
        double vj[3], C[9];
        for (int r = 0; r < 3; ++r) vj[r] = E[j][r] - Rl[3 * r + j];
        skew_cross(q, vj, C);
        const double bc = q[j] * Sq[k] + C[k];
        w.BC[t] = bc;
        w.A[t] = bc * d;
    }
    __syncwarp();
    SDFC_WFOR(t, 27) { w.dR[t] = e_mul3(&w.A[9 * (t / 9)], w.R, (t % 9) / 3, t % 3); }
    __syncwarp();
    SDFC_WFOR(k, 9) {
        double v = 0.0;
        for (int j = 0; j < 3; ++j) v += w.dR[9 * j + k] * qd[j];
        w.Rdot[k] = v;
    }
    __syncwarp();
    const double ddot = -2.0 * qqd / (q2 * q2);
    SDFC_WFOR(t, 27) {
        const int j = t / 9, k = t % 9;
        double vj[3], a[3], b[3], Rde[3], wv[3], Cd[9];
        for (int r = 0; r < 3; ++r) {
            vj[r] = E[j][r] - Rl[3 * r + j];
            Rde[r] = w.Rdot[3 * r + j];
        }
        cross(qd, vj, a);
        cross(q, Rde, b);
        for (int r = 0; r < 3; ++r) wv[r] = a[r] - b[r];
        skew(wv, Cd);
        const double bcd = qd[j] * Sq[k] + q[j] * Sqd[k] + Cd[k];
        w.BCd[t] = bcd;
        w.Ad[t] = bcd * d + w.BC[t] * ddot;
    }
    __syncwarp();
    // T column j = unskew(R^T dR_j); Tdot column j = unskew(Rdot^T A_j R + R^T Ad_j R + R^T A_j Rdot)
    SDFC_WFOR(t, 90) {
        if (t < 9) {
            const int j = t / 3, r = t % 3, e = unskew_entry(r);
            w.T[3 * r + j] = e_tmul3(w.R, &w.dR[9 * j], e / 3, e % 3);
        } else {
            const int u = t - 9, which = u / 27, jj = (u % 27) / 9, e = u % 9;
            if (which == 0)
                w.X1[9 * jj + e] = e_tmul3(w.Rdot, &w.A[9 * jj], e / 3, e % 3);
            else if (which == 1)
                w.X2[9 * jj + e] = e_tmul3(w.R, &w.Ad[9 * jj], e / 3, e % 3);
            else
                w.X3[9 * jj + e] = e_tmul3(w.R, &w.A[9 * jj], e / 3, e % 3);
        }
    }
    __syncwarp();
    SDFC_WFOR(t, 9) {
        const int j = t / 3, r = t % 3, e = unskew_entry(r);
        double s = e_mul3(&w.X1[9 * j], w.R, e / 3, e % 3);
        s += e_mul3(&w.X2[9 * j], w.R, e / 3, e % 3);
        s += e_mul3(&w.X3[9 * j], w.Rdot, e / 3, e % 3);
        w.Tdot[3 * r + j] = s;
    }
    __syncwarp();
    if (!deriv) return;
    double dd_dq[3];
    for (int k = 0; k < 3; ++k) dd_dq[k] = -2.0 * q[k] / (q2 * q2);
    SDFC_WFOR(u, 81) {  // [j][k][t]
        const int j = u / 27, k = (u / 9) % 3, t = u % 9;
        double vj[3], Sek[9], c1[9], c2[9], dRe[3], cv[3];
        for (int r = 0; r < 3; ++r) vj[r] = E[j][r] - Rl[3 * r + j];
        skew(E[k], Sek);
        skew_cross(E[k], vj, c1);
        for (int r = 0; r < 3; ++r) dRe[r] = w.dR[9 * k + 3 * r + j];
        cross(q, dRe, cv);
        for (int r = 0; r < 3; ++r) cv[r] = -cv[r];
        skew(cv, c2);
        const double dbc = q[j] * Sek[t] + (j == k ? Sq[t] : 0.0) + c1[t] + c2[t];
        w.dBC[u] = dbc;
        w.dA[u] = dbc * d + w.BC[9 * j + t] * dd_dq[k];
    }
    __syncwarp();
    SDFC_WFOR(u, 27) {  // dRdot[k][t]
        const int k = u / 9, t = u % 9;
        double v = 0.0;
        for (int j = 0; j < 3; ++j) {
            const double p1 = e_mul3(&w.dA[9 * (3 * j + k)], w.R, t / 3, t % 3);
            const double p2 = e_mul3(&w.A[9 * j], &w.dR[9 * k], t / 3, t % 3);
            v += (p1 + p2) * qd[j];
        }
        w.dRdot[u] = v;
    }
    __syncwarp();
    SDFC_WFOR(u, 81) {  // [k][j][t]: dAd and d2R
        const int k = u / 27, j = (u / 9) % 3, t = u % 9;
        const double dddot = (-2.0 * qd[k] * q2 + 8.0 * qqd * q[k]) / (q2 * q2 * q2);
        double Sek[9], dCd[9], a[3], b[3], c[3], dRe[3], Rde[3], dRde[3], wv[3];
        skew(E[k], Sek);
        for (int r = 0; r < 3; ++r) {
            dRe[r] = w.dR[9 * k + 3 * r + j];
            Rde[r] = w.Rdot[3 * r + j];
            dRde[r] = w.dRdot[9 * k + 3 * r + j];
        }
        cross(qd, dRe, a);
        cross(E[k], Rde, b);
        cross(q, dRde, c);
        for (int r = 0; r < 3; ++r) wv[r] = -a[r] - b[r] - c[r];
        skew(wv, dCd);
        const double dbcd = qd[j] * Sek[t] + (j == k ? Sqd[t] : 0.0) + dCd[t];
        w.dAd[u] = dbcd * d + w.BCd[9 * j + t] * dd_dq[k] + w.dBC[9 * (3 * j + k) + t] * ddot +
                   w.BC[9 * j + t] * dddot;
        double x = e_mul3(&w.dA[9 * (3 * j + k)], w.R, t / 3, t % 3);
        x += e_mul3(&w.A[9 * j], &w.dR[9 * k], t / 3, t % 3);
        w.d2R[u] = x;
    }
    __syncwarp();
    // dTdot's nine triple products: first factors (f0^T-style products), [k][j][m][t]
    SDFC_WFOR(u, 729) {
        const int kj = u / 81, m = (u / 9) % 9, e = u % 9, k = kj / 3, j = kj % 3;
        const double* Aj = &w.A[9 * j];
        const double* dAjk = &w.dA[9 * (3 * j + k)];
        const double* dRk = &w.dR[9 * k];
        const double* f0;
        const double* f1;
        switch (m) {
            case 0: f0 = &w.dRdot[9 * k]; f1 = Aj; break;
            case 1: f0 = w.Rdot; f1 = dAjk; break;
            case 2: f0 = w.Rdot; f1 = Aj; break;
            case 3: f0 = dRk; f1 = &w.Ad[9 * j]; break;
            case 4: f0 = w.R; f1 = &w.dAd[9 * kj]; break;
            case 5: f0 = w.R; f1 = &w.Ad[9 * j]; break;
            case 6: f0 = dRk; f1 = Aj; break;
            case 7: f0 = w.R; f1 = dAjk; break;
            default: f0 = w.R; f1 = Aj; break;
        }
        w.TX[u] = e_tmul3(f0, f1, e / 3, e % 3);
    }
    __syncwarp();
    SDFC_WFOR(u, 54) {
        if (u < 27) {  // dT[k] column j = unskew(dR_k^T dR_j + R^T d2R)
            const int k = u / 9, j = (u / 3) % 3, r = u % 3, e = unskew_entry(r);
            double s = e_tmul3(&w.dR[9 * k], &w.dR[9 * j], e / 3, e % 3);
            s += e_tmul3(w.R, &w.d2R[9 * (3 * k + j)], e / 3, e % 3);
            w.dT[9 * k + 3 * r + j] = s;
        } else {  // dTdot[k] column j
            const int v = u - 27, k = v / 9, j = (v / 3) % 3, r = v % 3, e = unskew_entry(r);
            const double* f2[9] = {w.R, w.R, &w.dR[9 * k], w.R, w.R, &w.dR[9 * k], w.Rdot, w.Rdot, &w.dRdot[9 * k]};
            double s = 0.0;
            for (int m = 0; m < 9; ++m) s += e_mul3(&w.TX[81 * (3 * k + j) + 9 * m], f2[m], e / 3, e % 3);
            w.dTdot[9 * k + 3 * r + j] = s;
        }
    }
    __syncwarp();
}

// free_system by one warp: g (and with deriv H) of the free body into w.g, w.H; w.M always.
__device__ inline void free_system_w(const FreeBody& m, const double* fe, const double* q0, const double* qd0,
                                     const double* q1, bool deriv, FreeWarp& w) {
    const int lane = threadIdx.x & 31;
    const double h = m.h;
    double qd1[6];
    for (int k = 0; k < 6; ++k) qd1[k] = (q1[k] - q0[k]) / h;
    rot_update_w(q1 + 3, qd1 + 3, deriv, w);
    const double* I = m.inertia;
    // Ad(E_ij), S_j, Sdot_j
    SDFC_WFOR(t, 108) {
        if (t < 36) {
            const int r = t / 6, c = t % 6;
            double a = 0.0;
            if (r < 3 && c < 3) {
                a = m.E_ji[4 * c + r];
            } else if (r >= 3 && c >= 3) {
                a = m.E_ji[4 * (c - 3) + (r - 3)];
            } else if (r >= 3) {
                double Rt[9], pi[3], Sk[9];
                for (int rr = 0; rr < 3; ++rr)
                    for (int cc = 0; cc < 3; ++cc) Rt[3 * rr + cc] = m.E_ji[4 * cc + rr];
                for (int rr = 0; rr < 3; ++rr)
                    pi[rr] = -(Rt[3 * rr] * m.E_ji[3] + Rt[3 * rr + 1] * m.E_ji[7] + Rt[3 * rr + 2] * m.E_ji[11]);
                skew(pi, Sk);
                double v = 0.0;
                for (int k = 0; k < 3; ++k) v += Sk[3 * (r - 3) + k] * Rt[3 * k + c];
                a = v;
            }
            w.Aij[t] = a;
        } else {
            const int u = t - 36, which = u / 36, e = u % 36, r = e / 6, c = e % 6;
            const double* Tm = which ? w.Tdot : w.T;
            const double* Rm = which ? w.Rdot : w.R;
            double v = 0.0;
            if (r < 3 && c >= 3) v = Tm[3 * r + (c - 3)];
            if (r >= 3 && c < 3) v = Rm[3 * c + (r - 3)];
            (which ? w.Sd : w.S)[e] = v;
        }
    }
    __syncwarp();
    // J = Ad S, Jdot = Ad Sdot; E_0j = E_pj0 Q
    SDFC_WFOR(t, 88) {
        if (t < 72) {
            const int which = t / 36, e = t % 36;
            (which ? w.Jd : w.J)[e] = e_mul6(w.Aij, which ? w.Sd : w.S, e / 6, e % 6);
        } else {
            const int e = t - 72, r = e / 4, c = e % 4;
            double s = 0.0;
            for (int k = 0; k < 4; ++k) {
                const double qv = k < 3 ? (c < 3 ? w.R[3 * k + c] : q1[k]) : (c == 3 ? 1.0 : 0.0);
                s += m.E_pj0[4 * r + k] * qv;
            }
            w.E0j[e] = s;
        }
    }
    __syncwarp();
    SDFC_WFOR(t, 22) {
        if (t < 16) {
            const int r = t / 4, c = t % 4;
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += w.E0j[4 * r + k] * m.E_ji[4 * k + c];
            w.E0i[t] = s;
        } else {
            w.phi[t - 16] = e_mv6(w.J, qd1, t - 16);
        }
    }
    __syncwarp();
    // body forces + contacts (all lanes hold the small vectors), MmJ, MmJdot
    double fm[6];
    {
        const double* phi = w.phi;
        double Sw[9], Sv[9], adT[36], Iphi[6], fc[6], fg[3], fh[3], ft[3], R0i[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) R0i[3 * r + c] = w.E0i[4 * r + c];
        skew(phi, Sw);
        skew(phi + 3, Sv);
        zero(adT, 36);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                adT[6 * r + c] = Sw[3 * c + r];
                adT[6 * r + c + 3] = Sv[3 * c + r];
                adT[6 * (r + 3) + c + 3] = Sw[3 * c + r];
            }
        for (int k = 0; k < 6; ++k) Iphi[k] = I[k] * phi[k];
        mv6(adT, Iphi, fc);
        for (int r = 0; r < 3; ++r) {
            fg[r] = fh[r] = ft[r] = 0.0;
            for (int c = 0; c < 3; ++c) {
                fg[r] += R0i[3 * c + r] * (m.mass * m.gravity[c]);
                fh[r] += R0i[3 * c + r] * fe[c];
                ft[r] += R0i[3 * c + r] * fe[3 + c];
            }
        }
        for (int k = 0; k < 3; ++k) {
            fm[k] = fc[k] + I[k] * fh[k] + w.fmc[k];
            fm[3 + k] = fc[3 + k] + fg[k] + I[3 + k] * ft[k] + w.fmc[3 + k];
        }
        if (lane < 6) w.fm[lane] = fm[lane];
        if (deriv) {  // Km, Dm of the body
            double Sg[9], Sh[9], St[9];
            skew(fg, Sg);
            skew(fh, Sh);
            skew(ft, St);
            const double Iw[3] = {I[0] * phi[0], I[1] * phi[1], I[2] * phi[2]};
            const double mv[3] = {I[3] * phi[3], I[4] * phi[4], I[5] * phi[5]};
            SDFC_WFOR(t, 72) {
                const int e = t % 36, r = e / 6, c = e % 6;
                if (t < 36) {
                    double v = w.Kmc[e];
                    if (r >= 3 && c < 3) {
                        v += Sg[3 * (r - 3) + c];
                        v += St[3 * (r - 3) + c] * I[r];
                    } else if (r < 3 && c < 3) {
                        v += Sh[3 * r + c] * I[r];
                    }
                    w.Km[e] = v;
                } else {
                    double v = w.Dmc[e];
                    v += adT[e] * I[c];
                    double a[3], b[3];
                    const double E[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
                    if (r < 3 && c < 3) {
                        cross(E[c], Iw, a);
                        v -= a[r];
                    } else if (r < 3) {
                        cross(E[c - 3], mv, b);
                        v -= b[r];
                    } else if (c < 3) {
                        cross(E[c], mv, b);
                        v -= b[r - 3];
                    }
                    w.Dm[e] = v;
                }
            }
        }
    }
    SDFC_WFOR(t, 72) {
        const int e = t % 36, r = e / 6;
        if (t < 36)
            w.MmJ[e] = w.J[e] * I[r];
        else
            w.MmJd[e] = w.Jd[e] * I[r];
    }
    __syncwarp();
    // M = J^T Mm J, J^T Mm Jdot; with deriv also J^T Km, J^T Dm
    SDFC_WFOR(t, deriv ? 144 : 72) {
        const int which = t / 36, e = t % 36, r = e / 6, c = e % 6;
        if (which == 0)
            w.M[e] = e_tmul6(w.J, w.MmJ, r, c);
        else if (which == 1)
            w.JTMmJd[e] = e_tmul6(w.J, w.MmJd, r, c);
        else if (which == 2)
            w.X[e] = e_tmul6(w.J, w.Km, r, c);
        else
            w.Y[e] = e_tmul6(w.J, w.Dm, r, c);
    }
    __syncwarp();
    SDFC_WFOR(t, 6) {  // f, dq
        const double fq = e_mv6(w.JTMmJd, qd1, t);
        const double t6 = e_tmv6(w.J, fm, t);
        w.f[t] = t6 - fq - m.Kr * q1[t] - m.Dr * qd1[t];
        w.dq[t] = q1[t] - q0[t] - h * qd0[t];
    }
    __syncwarp();
    SDFC_WFOR(t, 6) { w.g[t] = e_mv6(w.M, w.dq, t) - h * h * w.f[t]; }
    if (!deriv) {
        __syncwarp();
        return;
    }
    // K = J^T Km J, D = J^T Dm J - J^T Mm Jdot, dS_k, dSdot_k, MmJdot qdot, MmJ dq
    SDFC_WFOR(t, 72 + 216 + 12) {
        if (t < 72) {
            const int which = t / 36, e = t % 36;
            if (which == 0)
                w.K[e] = e_mul6(w.X, w.J, e / 6, e % 6);
            else
                w.Dd[e] = e_mul6(w.Y, w.J, e / 6, e % 6) - w.JTMmJd[e];
        } else if (t < 288) {
            const int u = t - 72, which = u / 108, kk = (u % 108) / 36, e = u % 36, r = e / 6, c = e % 6;
            double v = 0.0;
            if (which == 0) {
                if (r < 3 && c >= 3) v = w.dT[9 * kk + 3 * r + (c - 3)];
                if (r >= 3 && c < 3) v = w.dR[9 * kk + 3 * c + (r - 3)];
                w.dS[36 * kk + e] = v;
            } else {
                if (r < 3 && c >= 3) v = w.dTdot[9 * kk + 3 * r + (c - 3)];
                if (r >= 3 && c < 3) v = w.dRdot[9 * kk + 3 * c + (r - 3)];
                w.dSd[36 * kk + e] = v;
            }
        } else {
            const int u = t - 288;
            if (u < 6)
                w.MmJdqd[u] = e_mv6(w.MmJd, qd1, u);
            else
                w.MmJdq[u - 6] = e_mv6(w.MmJ, w.dq, u - 6);
        }
    }
    __syncwarp();
    SDFC_WFOR(t, 216) {  // dJ_k = Ad dS_k, dJdot_k = Ad dSdot_k
        const int which = t / 108, u = t % 108, kk = u / 36, e = u % 36;
        if (which == 0)
            w.dJ[u] = e_mul6(w.Aij, &w.dS[36 * kk], e / 6, e % 6);
        else
            w.dJd[u] = e_mul6(w.Aij, &w.dSd[36 * kk], e / 6, e % 6);
    }
    __syncwarp();
    SDFC_WFOR(t, 54) {  // dJ_k qdot (column k of dJq), dJdot_k qdot, dJ_k dq * I
        const int which = t / 18, kk = (t % 18) / 6, r = t % 6;
        const double* dJk = &w.dJ[36 * kk];
        if (which == 0)
            w.dJq[6 * r + 3 + kk] = e_mv6(dJk, qd1, r);
        else if (which == 1)
            w.dJdq[6 * kk + r] = e_mv6(&w.dJd[36 * kk], qd1, r);
        else
            w.dJdqv[6 * kk + r] = e_mv6(dJk, w.dq, r) * I[r];
    }
    SDFC_WFOR(t, 18) {  // the rotation columns k = 3..5 of dJq are written above; the others are zero
        const int r = t / 3, c = t % 3;
        w.dJq[6 * r + c] = 0.0;
    }
    __syncwarp();
    SDFC_WFOR(t, 36) {  // column k = 3..5 terms of K and dM/dq_k dq
        const int which = t / 18, kk = (t % 18) / 6, r = t % 6;
        const double* dJk = &w.dJ[36 * kk];
        if (which == 0) {
            const double a = e_tmv6(dJk, w.MmJdqd, r);
            const double b = e_tmv6(w.MmJ, &w.dJdq[6 * kk], r);
            const double c = e_tmv6(dJk, w.fm, r);
            w.K[6 * r + 3 + kk] += -a - b + c;
        } else {
            const double u = e_tmv6(dJk, w.MmJdq, r);
            const double v = e_tmv6(w.J, &w.dJdqv[6 * kk], r);
            w.dMcols[6 * kk + r] = u + v;
        }
    }
    __syncwarp();
    SDFC_WFOR(t, 72) {  // + J^T Dm dJq (into K), - J^T Mm dJq (into D)
        const int which = t / 36, e = t % 36;
        if (which == 0)
            w.X[e] = e_mul6(w.Y, w.dJq, e / 6, e % 6);
        else
            w.S[e] = e_tmul6(w.MmJ, w.dJq, e / 6, e % 6);  // S is free again
    }
    __syncwarp();
    SDFC_WFOR(e, 36) {
        const int r = e / 6, c = e % 6;
        double k = w.K[e] + w.X[e];
        double dd = w.Dd[e] - w.S[e];
        if (r == c) {
            k -= m.Kr;
            dd -= m.Dr;
        }
        double hv = w.M[e] - h * h * k - h * dd;
        if (c >= 3) hv += w.dMcols[6 * (c - 3) + r];
        w.H[e] = hv;
    }
    __syncwarp();
}

#undef SDFC_WFOR

}  // namespace sdfc_joint
