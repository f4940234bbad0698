// Kinematics and reduced dynamics of one moving part on a free3d-exp joint (6 dof:
// q = (p, r), translation and exponential rotation coordinates), FP64, one thread per scene.
//
// Restates, for a single body attached to the world:
//   JointSphericalExp::update / inner_update / reparam (simulation/redmax/Joint/JointSphericalExp.cpp:13-266),
//   JointFree3DExp::update (simulation/redmax/Joint/JointFree3DExp.cpp:13-99),
//   Joint::update, Body::update (rm/Joint/Joint.cpp:93-121, rm/Body/Body.cpp:138-156),
//   Robot::computeJointJacobianWithDerivative (rm/Robot.cpp:687-704): J = Ad(E_ij) S_j, ...,
//   Body::computeMaximalForceWithDerivative (rm/Body/Body.cpp:275-330),
//   Simulation::computeMatrices with derivatives (rm/Simulation.cpp:422-503) and the BDF1 g, H
//   (:1094-1165).
// Matrices are row-major double arrays.
#pragma once

#include <cuda_runtime.h>

namespace sdfc_joint {

constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ void zero(double* a, int n) {
    for (int k = 0; k < n; ++k) a[k] = 0.0;
}
__device__ __forceinline__ void mul3(const double* a, const double* b, double* c) {
    for (int r = 0; r < 3; ++r)
        for (int s = 0; s < 3; ++s) c[3 * r + s] = a[3 * r] * b[s] + a[3 * r + 1] * b[3 + s] + a[3 * r + 2] * b[6 + s];
}
__device__ __forceinline__ void tmul3(const double* a, const double* b, double* c) {  // a^T b
    for (int r = 0; r < 3; ++r)
        for (int s = 0; s < 3; ++s) c[3 * r + s] = a[r] * b[s] + a[3 + r] * b[3 + s] + a[6 + r] * b[6 + s];
}
__device__ __forceinline__ void skew(const double* v, double* S) {
    S[0] = 0.0;   S[1] = -v[2]; S[2] = v[1];
    S[3] = v[2];  S[4] = 0.0;   S[5] = -v[0];
    S[6] = -v[1]; S[7] = v[0];  S[8] = 0.0;
}
__device__ __forceinline__ void cross(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ double norm3(const double* a) { return sqrt(dot3(a, a)); }
__device__ __forceinline__ void unskew(const double* a, double* v) {  // (a21, a02, a10)
    v[0] = a[7];
    v[1] = a[2];
    v[2] = a[3];
}
__device__ __forceinline__ void skew_cross(const double* a, const double* b, double* S) {
    double c[3];
    cross(a, b, c);
    skew(c, S);
}
__device__ __forceinline__ void set_col3(double* M, int j, const double* v) {
    M[j] = v[0];
    M[3 + j] = v[1];
    M[6 + j] = v[2];
}

// Rodrigues' formula (math::exp(Vector3), rm/Utils.h:108-124)
__device__ inline void so3_exp(const double* w, double* R) {
    const double wl = norm3(w);
    zero(R, 9);
    R[0] = R[4] = R[8] = 1.0;
    if (wl > 1e-12) {
        const double x = w[0] / wl, y = w[1] / wl, z = w[2] / wl;
        double s, c;
        sincos(wl, &s, &c);
        const double c1 = 1.0 - c;
        R[0] = c + x * x * c1;  R[1] = -z * s + x * y * c1; R[2] = y * s + x * z * c1;
        R[3] = z * s + x * y * c1; R[4] = c + y * y * c1;  R[5] = -x * s + y * z * c1;
        R[6] = -y * s + x * z * c1; R[7] = x * s + y * z * c1; R[8] = c + z * z * c1;
    }
}

// The rotation, its rate, T (body angular velocity = T rdot), Tdot and, with `deriv`,
// their derivatives wrt r.  d = 1/|r|^2, A_j = (r_j [r] + [r x (I - R) e_j]) d, dR/dr_j = A_j R.
struct Rot {
    double R[9], Rdot[9], T[9], Tdot[9];
    double dR[3][9], dRdot[3][9], dT[3][9], dTdot[3][9];
};

__device__ inline void rot_update(const double* q, const double* qd, bool deriv, Rot& o) {
    const double E[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    if (norm3(q) < 1e-9) {  // first-order branch about R = I (|q| < math::eps)
        zero(o.R, 9);
        o.R[0] = o.R[4] = o.R[8] = 1.0;
        zero(o.Rdot, 9);
        for (int j = 0; j < 3; ++j) {
            skew(E[j], o.dR[j]);
            for (int k = 0; k < 9; ++k) o.Rdot[k] += o.dR[j][k] * qd[j];
        }
        zero(o.T, 9);
        o.T[0] = o.T[4] = o.T[8] = 1.0;
        for (int j = 0; j < 3; ++j) {
            double P[9], v[3];
            tmul3(o.Rdot, o.dR[j], P);
            unskew(P, v);
            set_col3(o.Tdot, j, v);
        }
        if (deriv)
            for (int k = 0; k < 3; ++k) {
                for (int j = 0; j < 3; ++j) {
                    double P[9], v[3];
                    tmul3(o.dR[k], o.dR[j], P);
                    unskew(P, v);
                    set_col3(o.dT[k], j, v);
                }
                // the reference's branch leaves these unset; they read as zero there
                zero(o.dRdot[k], 9);
                zero(o.dTdot[k], 9);
            }
        return;
    }
    so3_exp(q, o.R);
    const double q2 = dot3(q, q), d = 1.0 / q2, qqd = dot3(q, qd);
    double A[3][9], BC[3][9], Ad[3][9], BCd[3][9], v[3][3], Sq[9], Sqd[9];
    skew(q, Sq);
    skew(qd, Sqd);
    for (int j = 0; j < 3; ++j) {
        for (int r = 0; r < 3; ++r) v[j][r] = E[j][r] - o.R[3 * r + j];
        double C[9];
        skew_cross(q, v[j], C);
        for (int k = 0; k < 9; ++k) {
            BC[j][k] = q[j] * Sq[k] + C[k];
            A[j][k] = BC[j][k] * d;
        }
        mul3(A[j], o.R, o.dR[j]);
    }
    zero(o.Rdot, 9);
    for (int j = 0; j < 3; ++j)
        for (int k = 0; k < 9; ++k) o.Rdot[k] += o.dR[j][k] * qd[j];
    const double ddot = -2.0 * qqd / (q2 * q2);
    for (int j = 0; j < 3; ++j) {
        double a[3], b[3], Rde[3], w[3], Cd[9];
        cross(qd, v[j], a);
        for (int r = 0; r < 3; ++r) Rde[r] = o.Rdot[3 * r + j];
        cross(q, Rde, b);
        for (int r = 0; r < 3; ++r) w[r] = a[r] - b[r];
        skew(w, Cd);
        for (int k = 0; k < 9; ++k) {
            BCd[j][k] = qd[j] * Sq[k] + q[j] * Sqd[k] + Cd[k];
            Ad[j][k] = BCd[j][k] * d + BC[j][k] * ddot;
        }
    }
    double Rt[9], Rdt[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            Rt[3 * r + c] = o.R[3 * c + r];
            Rdt[3 * r + c] = o.Rdot[3 * c + r];
        }
    for (int j = 0; j < 3; ++j) {
        double P[9], X[9], S[9], w[3];
        mul3(Rt, o.dR[j], P);
        unskew(P, w);
        set_col3(o.T, j, w);
        mul3(Rdt, A[j], X);
        mul3(X, o.R, S);
        mul3(Rt, Ad[j], X);
        mul3(X, o.R, P);
        for (int k = 0; k < 9; ++k) S[k] += P[k];
        mul3(Rt, A[j], X);
        mul3(X, o.Rdot, P);
        for (int k = 0; k < 9; ++k) S[k] += P[k];
        unskew(S, w);
        set_col3(o.Tdot, j, w);
    }
    if (!deriv) return;
    // derivatives of A_j and Adot_j wrt q_k, then of Rdot, T, Tdot
    double dA[3][3][9], dBC[3][3][9];  // [j][k]
    double dd_dq[3];
    for (int k = 0; k < 3; ++k) {
        dd_dq[k] = -2.0 * q[k] / (q2 * q2);
        for (int j = 0; j < 3; ++j) {
            double Sek[9], c1[9], c2[9], dRe[3], cv[3];
            skew(E[k], Sek);
            skew_cross(E[k], v[j], c1);
            for (int r = 0; r < 3; ++r) dRe[r] = o.dR[k][3 * r + j];
            cross(q, dRe, cv);
            for (int r = 0; r < 3; ++r) cv[r] = -cv[r];
            skew(cv, c2);
            for (int t = 0; t < 9; ++t) {
                dBC[j][k][t] = q[j] * Sek[t] + (j == k ? Sq[t] : 0.0) + c1[t] + c2[t];
                dA[j][k][t] = dBC[j][k][t] * d + BC[j][t] * dd_dq[k];
            }
        }
    }
    for (int k = 0; k < 3; ++k) {
        zero(o.dRdot[k], 9);
        for (int j = 0; j < 3; ++j) {
            double P1[9], P2[9];
            mul3(dA[j][k], o.R, P1);
            mul3(A[j], o.dR[k], P2);
            for (int t = 0; t < 9; ++t) o.dRdot[k][t] += (P1[t] + P2[t]) * qd[j];
        }
    }
    for (int k = 0; k < 3; ++k) {
        const double dddot = (-2.0 * qd[k] * q2 + 8.0 * qqd * q[k]) / (q2 * q2 * q2);
        double dRkt[9], dRdkt[9];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                dRkt[3 * r + c] = o.dR[k][3 * c + r];
                dRdkt[3 * r + c] = o.dRdot[k][3 * c + r];
            }
        for (int j = 0; j < 3; ++j) {
            double Sek[9], dCd[9], a[3], b[3], c[3], dRe[3], Rde[3], dRde[3], w[3], dAd[9];
            skew(E[k], Sek);
            for (int r = 0; r < 3; ++r) {
                dRe[r] = o.dR[k][3 * r + j];
                Rde[r] = o.Rdot[3 * r + j];
                dRde[r] = o.dRdot[k][3 * r + j];
            }
            cross(qd, dRe, a);
            cross(E[k], Rde, b);
            cross(q, dRde, c);
            for (int r = 0; r < 3; ++r) w[r] = -a[r] - b[r] - c[r];
            skew(w, dCd);
            for (int t = 0; t < 9; ++t) {
                const double dBCd = qd[j] * Sek[t] + (j == k ? Sqd[t] : 0.0) + dCd[t];
                dAd[t] = dBCd * d + BCd[j][t] * dd_dq[k] + dBC[j][k][t] * ddot + BC[j][t] * dddot;
            }
            // dT_k col j = unskew(dR_k^T dR_j + R^T (dA_jk R + A_j dR_k))
            double d2R[9], P[9], S[9], X[9], u[3];
            mul3(dA[j][k], o.R, d2R);
            mul3(A[j], o.dR[k], P);
            for (int t = 0; t < 9; ++t) d2R[t] += P[t];
            mul3(dRkt, o.dR[j], S);
            mul3(Rt, d2R, P);
            for (int t = 0; t < 9; ++t) S[t] += P[t];
            unskew(S, u);
            set_col3(o.dT[k], j, u);
            // dTdot_k col j: derivative of (Rdot^T A_j R + R^T Adot_j R + R^T A_j Rdot)
            const double* f[9][3] = {{dRdkt, A[j], o.R},    {Rdt, dA[j][k], o.R},  {Rdt, A[j], o.dR[k]},
                                     {dRkt, Ad[j], o.R},    {Rt, dAd, o.R},        {Rt, Ad[j], o.dR[k]},
                                     {dRkt, A[j], o.Rdot},  {Rt, dA[j][k], o.Rdot}, {Rt, A[j], o.dRdot[k]}};
            zero(S, 9);
            for (int m = 0; m < 9; ++m) {
                mul3(f[m][0], f[m][1], X);
                mul3(X, f[m][2], P);
                for (int t = 0; t < 9; ++t) S[t] += P[t];
            }
            unskew(S, u);
            set_col3(o.dTdot[k], j, u);
        }
    }
}

// 6x6 helpers
__device__ __forceinline__ void mul6(const double* a, const double* b, double* c) {
    for (int r = 0; r < 6; ++r)
        for (int s = 0; s < 6; ++s) {
            double v = 0.0;
            for (int k = 0; k < 6; ++k) v += a[6 * r + k] * b[6 * k + s];
            c[6 * r + s] = v;
        }
}
__device__ __forceinline__ void tmul6(const double* a, const double* b, double* c) {  // a^T b
    for (int r = 0; r < 6; ++r)
        for (int s = 0; s < 6; ++s) {
            double v = 0.0;
            for (int k = 0; k < 6; ++k) v += a[6 * k + r] * b[6 * k + s];
            c[6 * r + s] = v;
        }
}
__device__ __forceinline__ void mv6(const double* a, const double* x, double* y) {
    for (int r = 0; r < 6; ++r) {
        double v = 0.0;
        for (int k = 0; k < 6; ++k) v += a[6 * r + k] * x[k];
        y[r] = v;
    }
}
__device__ __forceinline__ void tmv6(const double* a, const double* x, double* y) {  // a^T x
    for (int r = 0; r < 6; ++r) {
        double v = 0.0;
        for (int k = 0; k < 6; ++k) v += a[6 * k + r] * x[k];
        y[r] = v;
    }
}

// Ad(E_ij) for E_ij = E_ji^{-1}: [R^T 0; [-R^T p] R^T  R^T] with (R, p) of E_ji
__device__ inline void adjoint_inverse(const double* Eji, double* A) {
    double Rt[9], pi[3], S[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) Rt[3 * r + c] = Eji[4 * c + r];
    for (int r = 0; r < 3; ++r) pi[r] = -(Rt[3 * r] * Eji[3] + Rt[3 * r + 1] * Eji[7] + Rt[3 * r + 2] * Eji[11]);
    skew(pi, S);
    zero(A, 36);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            A[6 * r + c] = Rt[3 * r + c];
            A[6 * (r + 3) + c + 3] = Rt[3 * r + c];
            double v = 0.0;
            for (int k = 0; k < 3; ++k) v += S[3 * r + k] * Rt[3 * k + c];
            A[6 * (r + 3) + c] = v;
        }
}

__device__ __forceinline__ void mat4_mul(const double* A, const double* B, double* C) {
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += A[4 * r + k] * B[4 * k + c];
            C[4 * r + c] = s;
        }
}

// Pose and twist of the body (Joint::update, Body::update): E_0i = E_pj0 [R p; 0 1] E_ji,
// phi = Ad(E_ij) S_j qdot with S_j qdot = (T rdot, R^T pdot).
__device__ inline void free_pose(const double* E_pj0, const double* E_ji, const double* q, const double* qd,
                                 double* E0i, double* phi) {
    Rot o;
    rot_update(q + 3, qd + 3, false, o);
    double Q[16], E0j[16];
    zero(Q, 16);
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) Q[4 * r + c] = o.R[3 * r + c];
        Q[4 * r + 3] = q[r];
    }
    Q[15] = 1.0;
    mat4_mul(E_pj0, Q, E0j);
    mat4_mul(E0j, E_ji, E0i);
    double pj[6], A[36];
    for (int r = 0; r < 3; ++r) {
        pj[r] = o.T[3 * r] * qd[3] + o.T[3 * r + 1] * qd[4] + o.T[3 * r + 2] * qd[5];
        pj[3 + r] = o.R[r] * qd[0] + o.R[3 + r] * qd[1] + o.R[6 + r] * qd[2];
    }
    adjoint_inverse(E_ji, A);
    mv6(A, pj, phi);
}

// J = Ad(E_ij) S_j (6 x 6, row-major) of the free body at q: body twist = J qdot.
__device__ inline void free_jacobian(const double* E_ji, const double* q, double* J) {
    const double zero3[3] = {0.0, 0.0, 0.0};
    Rot o;
    rot_update(q + 3, zero3, false, o);
    double A[36], S[36];
    adjoint_inverse(E_ji, A);
    zero(S, 36);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            S[6 * r + 3 + c] = o.T[3 * r + c];
            S[6 * (r + 3) + c] = o.R[3 * c + r];
        }
    mul6(A, S, J);
}

// The reduced system of the free body at (q1, qd1) from the summed mover blocks of the
// contacts (fmc[6], Kmc[36], Dmc[36], wrt the body twist).  Outputs g (with q0, qdot0) and,
// with `deriv`, H and D; always M; J and R_0i for the adjoint if asked.
struct FreeBody {
    double mass, inertia[6], E_pj0[16], E_ji[16], gravity[3], h, Kr, Dr;
};

__device__ inline void free_system(const FreeBody& m, const double* fe, const double* q0, const double* qd0,
                                   const double* q1, const double* fmc, const double* Kmc, const double* Dmc,
                                   bool deriv, double* g, double* H, double* M, double* D, double* J_out,
                                   double* R0i_out) {
    const double h = m.h;
    double qd1[6];
    for (int k = 0; k < 6; ++k) qd1[k] = (q1[k] - q0[k]) / h;
    Rot o;
    rot_update(q1 + 3, qd1 + 3, deriv, o);
    // S_j, S_j_dot (and derivatives) -> J = Ad(E_ij) S_j, ...
    double Aij[36], S[36], J[36], Jd[36];
    adjoint_inverse(m.E_ji, Aij);
    zero(S, 36);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            S[6 * r + 3 + c] = o.T[3 * r + c];
            S[6 * (r + 3) + c] = o.R[3 * c + r];
        }
    mul6(Aij, S, J);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            S[6 * r + 3 + c] = o.Tdot[3 * r + c];
            S[6 * (r + 3) + c] = o.Rdot[3 * c + r];
        }
    mul6(Aij, S, Jd);
    // pose and twist
    double Q[16], E0j[16], E0i[16], R0i[9], phi[6];
    zero(Q, 16);
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) Q[4 * r + c] = o.R[3 * r + c];
        Q[4 * r + 3] = q1[r];
    }
    Q[15] = 1.0;
    mat4_mul(m.E_pj0, Q, E0j);
    mat4_mul(E0j, m.E_ji, E0i);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R0i[3 * r + c] = E0i[4 * r + c];
    mv6(J, qd1, phi);
    // body forces (Body::computeMaximalForceWithDerivative) + contacts
    const double* I = m.inertia;
    double fm[6], Km[36], Dm[36];
    double Sw[9], Sv[9], adT[36], Iphi[6], fc[6];
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
    double fg[3], fh[3], ft[3];
    for (int r = 0; r < 3; ++r) {
        fg[r] = fh[r] = ft[r] = 0.0;
        for (int c = 0; c < 3; ++c) {
            fg[r] += R0i[3 * c + r] * (m.mass * m.gravity[c]);
            fh[r] += R0i[3 * c + r] * fe[c];
            ft[r] += R0i[3 * c + r] * fe[3 + c];
        }
    }
    for (int k = 0; k < 3; ++k) {
        fm[k] = fc[k] + I[k] * fh[k] + fmc[k];
        fm[3 + k] = fc[3 + k] + fg[k] + I[3 + k] * ft[k] + fmc[3 + k];
    }
    // M = J^T Mm J, fqvv = -J^T Mm Jdot qdot, f = J^T fm + fqvv + fr
    double MmJ[36], MmJd[36], JTMmJd[36], t6[6], fq[6], f[6];
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) {
            MmJ[6 * r + c] = J[6 * r + c] * I[r];
            MmJd[6 * r + c] = Jd[6 * r + c] * I[r];
        }
    tmul6(J, MmJ, M);
    tmul6(J, MmJd, JTMmJd);
    mv6(JTMmJd, qd1, fq);
    tmv6(J, fm, t6);
    for (int k = 0; k < 6; ++k) f[k] = t6[k] - fq[k] - m.Kr * q1[k] - m.Dr * qd1[k];
    double dq[6], Mdq[6];
    for (int k = 0; k < 6; ++k) dq[k] = q1[k] - q0[k] - h * qd0[k];
    mv6(M, dq, Mdq);
    for (int k = 0; k < 6; ++k) g[k] = Mdq[k] - h * h * f[k];
    if (J_out)
        for (int k = 0; k < 36; ++k) J_out[k] = J[k];
    if (R0i_out)
        for (int k = 0; k < 9; ++k) R0i_out[k] = R0i[k];
    if (!deriv) return;
    // Km, Dm of the body
    for (int k = 0; k < 36; ++k) {
        Km[k] = Kmc[k];
        Dm[k] = Dmc[k];
    }
    {
        double Sg[9], Sh[9], St[9];
        skew(fg, Sg);
        skew(fh, Sh);
        skew(ft, St);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                Km[6 * (3 + r) + c] += Sg[3 * r + c];
                Km[6 * r + c] += Sh[3 * r + c] * I[r];
                Km[6 * (3 + r) + c] += St[3 * r + c] * I[3 + r];
            }
        for (int c = 0; c < 6; ++c)
            for (int r = 0; r < 6; ++r) Dm[6 * r + c] += adT[6 * r + c] * I[c];
        const double Iw[3] = {I[0] * phi[0], I[1] * phi[1], I[2] * phi[2]};
        const double mv[3] = {I[3] * phi[3], I[4] * phi[4], I[5] * phi[5]};
        const double E[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int j = 0; j < 3; ++j) {
            double a[3], b[3];
            cross(E[j], Iw, a);
            cross(E[j], mv, b);
            for (int r = 0; r < 3; ++r) {
                Dm[6 * r + j] -= a[r];
                Dm[6 * r + 3 + j] -= b[r];
                Dm[6 * (3 + r) + j] -= b[r];
            }
        }
    }
    // dJ_k, dJdot_k (nonzero for the rotation coordinates k = 3..5 only)
    double dJq[36];  // column k = dJ_k qdot
    double K[36], Dd[36], X[36], Y[36];
    zero(dJq, 36);
    double MmJdqd[6];
    mv6(MmJd, qd1, MmJdqd);
    // K = J^T Km J (+ the rest below), D = J^T Dm J - J^T Mm Jdot (+ ...)
    tmul6(J, Km, X);
    mul6(X, J, K);
    tmul6(J, Dm, Y);  // J^T Dm, kept in Y
    mul6(Y, J, Dd);
    for (int k = 0; k < 36; ++k) Dd[k] -= JTMmJd[k];
    double dMcols[6][6];  // column k of H from dM/dq_k (q1 - q0 - h qdot0)
    for (int k = 0; k < 6; ++k)
        for (int r = 0; r < 6; ++r) dMcols[k][r] = 0.0;
    for (int k = 3; k < 6; ++k) {
        double dS[36], dSd[36], dJ[36], dJd[36];
        zero(dS, 36);
        zero(dSd, 36);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                dS[6 * r + 3 + c] = o.dT[k - 3][3 * r + c];
                dS[6 * (r + 3) + c] = o.dR[k - 3][3 * c + r];
                dSd[6 * r + 3 + c] = o.dTdot[k - 3][3 * r + c];
                dSd[6 * (r + 3) + c] = o.dRdot[k - 3][3 * c + r];
            }
        mul6(Aij, dS, dJ);
        mul6(Aij, dSd, dJd);
        double col[6], a[6], b[6], c[6], dJdq[6];
        mv6(dJ, qd1, col);
        for (int r = 0; r < 6; ++r) dJq[6 * r + k] = col[r];
        tmv6(dJ, MmJdqd, a);          // dJ_k^T Mm Jdot qdot
        mv6(dJd, qd1, dJdq);          // dJdot_k qdot
        tmv6(MmJ, dJdq, b);           // J^T Mm dJdot_k qdot
        tmv6(dJ, fm, c);              // dJ_k^T fm
        for (int r = 0; r < 6; ++r) K[6 * r + k] += -a[r] - b[r] + c[r];
        // dM/dq_k dq = (dJ_k^T Mm J + J^T Mm dJ_k) dq
        double MmJdq[6], dJdqv[6], u[6], w[6];
        mv6(MmJ, dq, MmJdq);
        tmv6(dJ, MmJdq, u);
        mv6(dJ, dq, dJdqv);
        for (int r = 0; r < 6; ++r) dJdqv[r] *= I[r];
        tmv6(J, dJdqv, w);
        for (int r = 0; r < 6; ++r) dMcols[k][r] = u[r] + w[r];
    }
    // + J^T Dm dJq - J^T Mm dJq, joint stiffness / damping
    mul6(Y, dJq, X);
    for (int k = 0; k < 36; ++k) K[k] += X[k];
    tmul6(MmJ, dJq, X);
    for (int k = 0; k < 36; ++k) Dd[k] -= X[k];
    for (int k = 0; k < 6; ++k) {
        K[6 * k + k] -= m.Kr;
        Dd[6 * k + k] -= m.Dr;
    }
    if (D)
        for (int k = 0; k < 36; ++k) D[k] = Dd[k];
    if (H) {
        for (int k = 0; k < 36; ++k) H[k] = M[k] - h * h * K[k] - h * Dd[k];
        for (int k = 0; k < 6; ++k)
            for (int r = 0; r < 6; ++r) H[6 * r + k] += dMcols[k][r];
    }
}

// JointSphericalExp::reparam for the rotation block of (q, qdot) (applied after each step).
__device__ inline void free_reparam(double* q, double* qd) {
    double* r = q + 3;
    double rn = norm3(r);
    if (rn <= 1.5 * kPi) return;
    const double zero3[3] = {0.0, 0.0, 0.0};
    Rot o0, o1;
    rot_update(r, zero3, false, o0);
    for (int it = 0; it < 64 && rn > 1.5 * kPi; ++it) {
        const double s = 1.0 - 2.0 * kPi / rn;
        for (int k = 0; k < 3; ++k) r[k] *= s;
        rn = norm3(r);
    }
    rot_update(r, zero3, false, o1);
    double w[3], A[9], b[3];
    for (int k = 0; k < 3; ++k) w[k] = o0.T[3 * k] * qd[3] + o0.T[3 * k + 1] * qd[4] + o0.T[3 * k + 2] * qd[5];
    // qd_r = T1^{-1} T0 qd_r by Gaussian elimination with partial pivoting
    for (int k = 0; k < 9; ++k) A[k] = o1.T[k];
    for (int k = 0; k < 3; ++k) b[k] = w[k];
    for (int c = 0; c < 3; ++c) {
        int p = c;
        for (int rr = c + 1; rr < 3; ++rr)
            if (fabs(A[3 * rr + c]) > fabs(A[3 * p + c])) p = rr;
        if (p != c) {
            for (int k = 0; k < 3; ++k) {
                const double t = A[3 * c + k];
                A[3 * c + k] = A[3 * p + k];
                A[3 * p + k] = t;
            }
            const double t = b[c];
            b[c] = b[p];
            b[p] = t;
        }
        for (int rr = c + 1; rr < 3; ++rr) {
            const double l = A[3 * rr + c] / A[3 * c + c];
            for (int k = c; k < 3; ++k) A[3 * rr + k] -= l * A[3 * c + k];
            b[rr] -= l * b[c];
        }
    }
    for (int rr = 2; rr >= 0; --rr) {
        double s = b[rr];
        for (int k = rr + 1; k < 3; ++k) s -= A[3 * rr + k] * qd[3 + k];
        qd[3 + rr] = s / A[3 * rr + rr];
    }
}

}  // namespace sdfc_joint
