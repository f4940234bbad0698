// Batched implicit-Euler (BDF1) steps of planner scenes; see include/sdfc.h.
//
// Restates, per scene, redmax's Simulation::integration_BDF1 + Simulation::newton
// (simulation/redmax/Simulation.cpp:999-1079, 1248-1270) with the reduced system of
// Simulation::computeMatrices (:379-503) for one mover on a joint to the world:
//   * translational (simulation/redmax/Joint/JointTranslational.cpp:9-40): J = Ad(E_ij) S_j =
//     [0; R_ji^T] is constant, so M = J^T Mm J, f = J^T fm + fr, K = J^T Km J + Kr,
//     D = J^T Dm J + Dr;
//   * free3d-exp (simulation/redmax/Joint/JointFree3DExp.cpp): the full system with the
//     configuration-dependent J, in sdfc_joint.cuh.
//
// Every scene runs the reference's Newton iteration as a small state machine;
// one "round" gives every unfinished scene exactly one force evaluation (with
// derivatives at a Newton point, value-only at a line-search trial), and a scene
// whose step ends goes on to its next step of the same sdfc_sim_step call in the
// next round (end_step), so a round is one batched evaluation of all contact pairs
// plus two tiny kernels:
//   sim_pose_kernel    per pair: the mover's pose / twist at the scene's current
//                      point, the pair's inputs and request (skip/value/derivative)
//   (batched evaluation of every requested pair)
//   sim_newton_kernel  per scene: g (and H), the 3x3 FP64 solve, line-search
//                      bookkeeping, convergence.
#include <cuda_runtime.h>

#include <cstdlib>

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "sdfc_internal.h"
#include "sdfc_joint.cuh"
#include "sdfc_joint_warp.cuh"

using sdfc_impl::dev_alloc;
using sdfc_impl::fail;
using sdfc_impl::use_device;

namespace {

constexpr double kTol = 1e-8;     // Simulation.cpp:1008 (default of MoverDev::tol)
constexpr int kMaxLineSearch = 20;  // :1011
constexpr int kMaxStrike = 3;     // :1014

enum Phase : int { kNewton = 0, kLine = 1, kDone = 2 };

constexpr int kMaxDof = 6;

// Threads per block of the per-scene kernels (Newton update, adjoint step).  Each scene's
// FP64 work runs on one thread; small blocks spread the scenes over all SMs so that no SM's
// FP64 pipe carries more than a few of them.
#ifndef SDFC_SCENE_THREADS
#define SDFC_SCENE_THREADS 32
#endif
constexpr int kSceneThreads = SDFC_SCENE_THREADS;

struct MoverDev {
    double mass, inertia[6], E_pj0[16], E_ji[16], gravity[3], h, Kr, Dr;
    double tol;  // Newton tolerance on |g| (the reference's 1e-8 unless set)
    int max_iter;
    int ndof;  // 3: translational, 6: free3d-exp
};

struct SceneState {
    double q0[kMaxDof], qd0[kMaxDof], x[kMaxDof], dx[kMaxDof], xt[kMaxDof];
    double gnorm, alpha;
    int phase, iter, trial, strike, converged;
    int step;  // steps this scene has finished in the current sdfc_sim_step call
    int nev;   // evaluations in its current step
};

// Evaluations one scene may spend on one step: the reference's Newton stops after max_iter
// iterations of at most 1 + 20 evaluations (Simulation.cpp:1009-1054); past this a step ends at
// its current iterate, unconverged (a bound that the stopping rules reach first).
constexpr int kMaxEvalsPerStep = 120 * (1 + kMaxLineSearch) + 2;

// Per sdfc_sim_step call, read by the Newton kernels (device memory, so that the captured round
// graphs stay valid across calls): the steps every scene takes, the recording row of the call's
// first step and the recorded trajectory (null when recording is off).
struct SimCtl {
    int target, rec_base;
    double* qhis;
};

__device__ inline sdfc_joint::FreeBody free_body(const MoverDev& m) {
    sdfc_joint::FreeBody b;
    b.mass = m.mass;
    for (int k = 0; k < 6; ++k) b.inertia[k] = m.inertia[k];
    for (int k = 0; k < 16; ++k) {
        b.E_pj0[k] = m.E_pj0[k];
        b.E_ji[k] = m.E_ji[k];
    }
    for (int k = 0; k < 3; ++k) b.gravity[k] = m.gravity[k];
    b.h = m.h;
    b.Kr = m.Kr;
    b.Dr = m.Dr;
    return b;
}

__device__ __forceinline__ void mat4_mul(const double* A, const double* B, double* C) {
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += A[4 * r + k] * B[4 * k + c];
            C[4 * r + c] = s;
        }
}

// Joint::update (E_pj = E_pj0 Q, Q = [I q; 0 1]) and Body::update (E_0i = E_0j E_ji,
// phi = Ad(E_ij) S_j qdot = (0, R_ji^T qdot)); Joint.cpp, Body.cpp:138-156.
__device__ void trans_pose(const MoverDev& m, const double* q, const double* qd, double* E0i, double* phi) {
    const double Q[16] = {1, 0, 0, q[0], 0, 1, 0, q[1], 0, 0, 1, q[2], 0, 0, 0, 1};
    double E0j[16];
    mat4_mul(m.E_pj0, Q, E0j);
    mat4_mul(E0j, m.E_ji, E0i);
    phi[0] = phi[1] = phi[2] = 0.0;
    for (int r = 0; r < 3; ++r) phi[3 + r] = m.E_ji[r] * qd[0] + m.E_ji[4 + r] * qd[1] + m.E_ji[8 + r] * qd[2];
}

__device__ void mover_pose(const MoverDev& m, const double* q, const double* qd, double* E0i, double* phi) {
    if (m.ndof == 6)
        sdfc_joint::free_pose(m.E_pj0, m.E_ji, q, qd, E0i, phi);
    else
        trans_pose(m, q, qd, E0i, phi);
}

__global__ void sim_begin_kernel(int n, int nd, const MoverDev* __restrict__ mover, const double* __restrict__ q,
                                 const double* __restrict__ qd, SceneState* __restrict__ st, int* remaining) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) *remaining = n;
    if (i >= n) return;
    SceneState s;
    const double h = mover[i].h;
    for (int k = 0; k < kMaxDof; ++k) s.q0[k] = s.qd0[k] = s.x[k] = s.dx[k] = s.xt[k] = 0.0;
    for (int k = 0; k < nd; ++k) {
        s.q0[k] = q[(size_t)nd * i + k];
        s.qd0[k] = qd[(size_t)nd * i + k];
        s.x[k] = s.q0[k] + h * s.qd0[k];  // initial guess, Simulation.cpp:1256
        s.dx[k] = s.xt[k] = 0.0;
    }
    s.gnorm = 0.0;
    s.alpha = 1.0;
    s.phase = kNewton;
    s.iter = s.trial = s.strike = s.converged = 0;
    s.step = s.nev = 0;
    st[i] = s;
}

// Poses of pair k (mover posed by its scene's current iterate) into evaluation slot j.  One
// compiled copy serves the full and the compacted rounds, so both pose a scene with the same
// arithmetic (inlined into each kernel, the joint's multiply-adds could contract differently).
__device__ __noinline__ void pose_pair(int k, int j, const int* __restrict__ pair_inst, const int* __restrict__ role,
                                 const double* __restrict__ E_fixed, const MoverDev* __restrict__ mover,
                                 const SceneState* __restrict__ st, double* __restrict__ EA, double* __restrict__ phiA,
                                 double* __restrict__ EB, double* __restrict__ phiB, int* __restrict__ mode) {
    const int i = pair_inst[k];
    const SceneState& s = st[i];
    if (s.phase == kDone) {
        mode[j] = 0;
        return;
    }
    const MoverDev& m = mover[i];
    const double* p = s.phase == kNewton ? s.x : s.xt;
    double qd[kMaxDof], E0i[16], phi[6];
    for (int c = 0; c < m.ndof; ++c) qd[c] = (p[c] - s.q0[c]) / m.h;
    mover_pose(m, p, qd, E0i, phi);
    double *Em = role[k] ? EA + 16 * (size_t)j : EB + 16 * (size_t)j;
    double *pm = role[k] ? phiA + 6 * (size_t)j : phiB + 6 * (size_t)j;
    double *Ef = role[k] ? EB + 16 * (size_t)j : EA + 16 * (size_t)j;
    double *pf = role[k] ? phiB + 6 * (size_t)j : phiA + 6 * (size_t)j;
    for (int c = 0; c < 16; ++c) {
        Em[c] = E0i[c];
        Ef[c] = E_fixed[16 * (size_t)k + c];
    }
    for (int c = 0; c < 6; ++c) {
        pm[c] = phi[c];
        pf[c] = 0.0;
    }
    mode[j] = s.phase == kNewton ? 2 : 1;
}

__global__ void sim_pose_kernel(int n_pairs, const int* __restrict__ pair_inst, const int* __restrict__ role,
                                const double* __restrict__ E_fixed, const MoverDev* __restrict__ mover,
                                const SceneState* __restrict__ st, double* __restrict__ EA, double* __restrict__ phiA,
                                double* __restrict__ EB, double* __restrict__ phiB, int* __restrict__ mode) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_pairs) return;
    pose_pair(k, k, pair_inst, role, E_fixed, mover, st, EA, phiA, EB, phiB, mode);
}

// ---------------------------------------------------------------- compacted rounds
//
// A batched Newton round waits for its slowest scene, and late in a step only a few scenes
// still iterate.  The Newton kernels append every scene that stays active, its pairs and their
// detection tiles to the next round's lists (double-buffered by round parity; order does not
// matter: every pair is evaluated on its own).  A compacted round evaluates only the listed
// pairs, in slots j = 0..count-1 of arrays sized for a capacity bucket chosen on the host from
// the active count it reads between rounds (the count only falls within a step); slots past the
// count are masked (mode 0), and tiles past the tile count point at the last slot, which is
// always masked.

struct CompactLists {
    int* cnt;  // scenes, pairs, tiles
    int* scene;
    int* pair;
    sdfc::InstanceDesc* inst;
    int* tile;
};

// Appends scene i (still iterating) to the next round's lists.
__device__ inline void append_active(int i, const int* __restrict__ pair_begin,
                                     const sdfc::InstanceDesc* __restrict__ inst_full, CompactLists nx) {
    const int k0 = pair_begin[i], k1 = pair_begin[i + 1];
    int nt = 0;
    for (int k = k0; k < k1; ++k) nt += inst_full[k].ntiles;
    const int js = atomicAdd(nx.cnt + 0, 1);
    nx.scene[js] = i;
    int jp = atomicAdd(nx.cnt + 1, k1 - k0);
    int tb = atomicAdd(nx.cnt + 2, nt);
    for (int k = k0; k < k1; ++k, ++jp) {
        sdfc::InstanceDesc d = inst_full[k];
        d.tile0 = tb;
        nx.pair[jp] = k;
        nx.inst[jp] = d;
        for (int t = 0; t < d.ntiles; ++t) nx.tile[tb + t] = jp;
        tb += d.ntiles;
    }
}

// Slots 0..Bp-1 of a compacted round: the listed pairs' poses and coefficients, masked slots
// past the count; tiles past the tile count mapped to the masked last slot.
__global__ void sim_pose_compact_kernel(int Bp, int Bt, const int* __restrict__ cnt, const int* __restrict__ pair_list,
                                        int* __restrict__ tile_c, const int* __restrict__ pair_inst,
                                        const int* __restrict__ role, const double* __restrict__ E_fixed,
                                        const double* __restrict__ prm, const MoverDev* __restrict__ mover,
                                        const SceneState* __restrict__ st, double* __restrict__ EA,
                                        double* __restrict__ phiA, double* __restrict__ EB, double* __restrict__ phiB,
                                        double* __restrict__ prm_c, int* __restrict__ mode) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < Bp) {
        if (t >= cnt[1]) {
            mode[t] = 0;
            return;
        }
        const int k = pair_list[t];
        for (int c = 0; c < 6; ++c) prm_c[6 * (size_t)t + c] = prm[6 * (size_t)k + c];
        pose_pair(k, t, pair_inst, role, E_fixed, mover, st, EA, phiA, EB, phiB, mode);
    } else if (t < Bp + Bt) {
        const int tt = t - Bp;
        if (tt >= cnt[2]) tile_c[tt] = Bp - 1;
    }
}

// The compacted round's results back to the pairs' rows (fm always; Km, Dm where requested).
__global__ void sim_scatter_kernel(const int* __restrict__ cnt, const int* __restrict__ pair_list,
                                   const int* __restrict__ mode_c, const double* __restrict__ fm_c,
                                   const double* __restrict__ Km_c, const double* __restrict__ Dm_c,
                                   const int* __restrict__ nact_c, const int* __restrict__ status_c,
                                   double* __restrict__ fm, double* __restrict__ Km, double* __restrict__ Dm,
                                   int* __restrict__ nact, int* __restrict__ status) {
    const int j = blockIdx.x;
    if (j >= cnt[1]) return;
    const int k = pair_list[j];
    const bool deriv = mode_c[j] == 2;
    for (int e = threadIdx.x; e < 300; e += blockDim.x) {
        if (e < 12)
            fm[12 * (size_t)k + e] = fm_c[12 * (size_t)j + e];
        else if (deriv && e < 156)
            Km[144 * (size_t)k + e - 12] = Km_c[144 * (size_t)j + e - 12];
        else if (deriv)
            Dm[144 * (size_t)k + e - 156] = Dm_c[144 * (size_t)j + e - 156];
    }
    if (threadIdx.x == 0) {
        nact[k] = nact_c[j];
        status[k] = status_c[j];
    }
}

// n x n solve (n <= 6) by Gaussian elimination with partial pivoting (the algorithm of
// the reference's PartialPivLU, Simulation.cpp:1028).
__device__ void solve_n(const double* A_in, const double* b_in, int n, double* x) {
    double A[kMaxDof * kMaxDof], b[kMaxDof];
    for (int k = 0; k < n * n; ++k) A[k] = A_in[k];
    for (int k = 0; k < n; ++k) b[k] = b_in[k];
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(A[n * r + c]) > fabs(A[n * p + c])) p = r;
        if (p != c) {
            for (int k = 0; k < n; ++k) {
                const double t = A[n * c + k];
                A[n * c + k] = A[n * p + k];
                A[n * p + k] = t;
            }
            const double t = b[c];
            b[c] = b[p];
            b[p] = t;
        }
        for (int r = c + 1; r < n; ++r) {
            const double l = A[n * r + c] / A[n * c + c];
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

__device__ __forceinline__ double norm_n(const double* v, int n) {
    double s = v[0] * v[0];
    for (int k = 1; k < n; ++k) s += v[k] * v[k];
    return sqrt(s);
}

// The free mover's contact sums: the mover's 6-row block of every pair's fm, Km, Dm.
__device__ void free_contact_sums(int k0, int k1, const int* __restrict__ role, const double* __restrict__ fm,
                                  const double* __restrict__ Km, const double* __restrict__ Dm, bool deriv,
                                  double* fmc, double* Kmc, double* Dmc) {
    for (int r = 0; r < 6; ++r) fmc[r] = 0.0;
    for (int r = 0; r < 36; ++r) Kmc[r] = Dmc[r] = 0.0;
    for (int k = k0; k < k1; ++k) {
        const int o = role[k] ? 0 : 6;
        for (int r = 0; r < 6; ++r) {
            fmc[r] += fm[12 * (size_t)k + o + r];
            if (deriv)
                for (int c = 0; c < 6; ++c) {
                    Kmc[6 * r + c] += Km[144 * (size_t)k + (o + r) * 12 + o + c];
                    Dmc[6 * r + c] += Dm[144 * (size_t)k + (o + r) * 12 + o + c];
                }
        }
    }
}

// The translational mover's g (and H) at p (SceneState point): reduced system of the
// contacts' linear rows, gravity and external force.
__device__ void trans_system(const MoverDev& m, const double* __restrict__ fe, const SceneState& s, const double* p,
                             int k0, int k1, const int* __restrict__ role, const double* __restrict__ fm,
                             const double* __restrict__ Km, const double* __restrict__ Dm, bool newton, double* g,
                             double* H) {
    const double h = m.h;
    double qd[3], E0i[16], phi[6];
    for (int c = 0; c < 3; ++c) qd[c] = (p[c] - s.q0[c]) / h;
    trans_pose(m, p, qd, E0i, phi);
    // fm (linear rows) of the mover: gravity and external force (Body.cpp:247-271) + contacts
    double fl[3], Kll[9] = {0}, Dll[9] = {0};
    for (int r = 0; r < 3; ++r) {
        double gr = 0.0, e = 0.0;
        for (int c = 0; c < 3; ++c) {
            gr += E0i[4 * c + r] * (m.mass * m.gravity[c]);
            e += E0i[4 * c + r] * fe[3 + c];
        }
        fl[r] = gr + m.inertia[3 + r] * e;
    }
    for (int k = k0; k < k1; ++k) {
        const int o = role[k] ? 0 : 6;
        for (int r = 0; r < 3; ++r) {
            fl[r] += fm[12 * (size_t)k + o + 3 + r];
            if (newton)
                for (int c = 0; c < 3; ++c) {
                    Kll[3 * r + c] += Km[144 * (size_t)k + (o + 3 + r) * 12 + o + 3 + c];
                    Dll[3 * r + c] += Dm[144 * (size_t)k + (o + 3 + r) * 12 + o + 3 + c];
                }
        }
    }
    // reduced system: f = R_ji fl + fr, M = R_ji diag(m) R_ji^T
    double R[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) R[3 * r + c] = m.E_ji[4 * r + c];
    double f[3], M[9];
    for (int r = 0; r < 3; ++r) {
        f[r] = R[3 * r] * fl[0] + R[3 * r + 1] * fl[1] + R[3 * r + 2] * fl[2];
        f[r] += -m.Kr * p[r] - m.Dr * qd[r];
        for (int c = 0; c < 3; ++c)
            M[3 * r + c] = R[3 * r] * m.inertia[3] * R[3 * c] + R[3 * r + 1] * m.inertia[4] * R[3 * c + 1] +
                           R[3 * r + 2] * m.inertia[5] * R[3 * c + 2];
    }
    double dq[3];
    for (int k = 0; k < 3; ++k) dq[k] = p[k] - s.q0[k] - h * s.qd0[k];
    for (int r = 0; r < 3; ++r) g[r] = M[3 * r] * dq[0] + M[3 * r + 1] * dq[1] + M[3 * r + 2] * dq[2] - h * h * f[r];
    if (!newton) return;
    // H = M - h^2 K - h D, K = R Kll R^T - Kr I, D = R Dll R^T - Dr I
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            double K = 0.0, D = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    K += R[3 * r + a] * Kll[3 * a + b] * R[3 * c + b];
                    D += R[3 * r + a] * Dll[3 * a + b] * R[3 * c + b];
                }
            if (r == c) {
                K -= m.Kr;
                D -= m.Dr;
            }
            H[3 * r + c] = M[3 * r + c] - h * h * K - h * D;
        }
}

// Ends scene i's step at its current iterate: q = x, qdot = (x - q0) / h, the free joint's
// rotation vector reparameterised (Simulation::forward, Simulation.cpp:955-957), the step's
// convergence flag and, when recording, its trajectory row.  When the call has more steps for
// the scene, starts the next one from that state as sim_begin_kernel does and returns true: a
// scene does not wait for the other scenes between the steps of one call (scenes are independent
// and each evaluation's result depends on its own inputs alone, so the trajectories are the ones
// the scenes take when every step waits for all of them).
__device__ bool end_step(int i, int n, const MoverDev& m, const SimCtl& c, double* __restrict__ q,
                         double* __restrict__ qd, int* __restrict__ conv, SceneState& s) {
    const int nd = m.ndof;
    double x[kMaxDof], v[kMaxDof];
    for (int k = 0; k < nd; ++k) {
        x[k] = s.x[k];
        v[k] = (s.x[k] - s.q0[k]) / m.h;
    }
    if (nd == 6) sdfc_joint::free_reparam(x, v);
    for (int k = 0; k < nd; ++k) {
        q[(size_t)nd * i + k] = x[k];
        qd[(size_t)nd * i + k] = v[k];
    }
    conv[i] = s.converged;
    ++s.step;
    if (c.qhis)
        for (int k = 0; k < nd; ++k) c.qhis[(size_t)nd * n * (c.rec_base + s.step) + (size_t)nd * i + k] = x[k];
    if (s.step >= c.target) return false;
    for (int k = 0; k < kMaxDof; ++k) s.q0[k] = s.qd0[k] = s.x[k] = s.dx[k] = s.xt[k] = 0.0;
    for (int k = 0; k < nd; ++k) {
        s.q0[k] = x[k];
        s.qd0[k] = v[k];
        s.x[k] = s.q0[k] + m.h * s.qd0[k];
    }
    s.gnorm = 0.0;
    s.alpha = 1.0;
    s.phase = kNewton;
    s.iter = s.trial = s.strike = s.converged = 0;
    s.nev = 0;
    return true;
}

__global__ void sim_newton_kernel(int n, const int* __restrict__ pair_begin, const int* __restrict__ role,
                                  const MoverDev* __restrict__ mover, const double* __restrict__ f_ext,
                                  const double* __restrict__ fm, const double* __restrict__ Km,
                                  const double* __restrict__ Dm, SceneState* __restrict__ st, int* remaining,
                                  unsigned long long* evaluations, const int* __restrict__ scene_list,
                                  const int* __restrict__ scene_cnt, const sdfc::InstanceDesc* __restrict__ inst_full,
                                  CompactLists nx, const SimCtl* __restrict__ ctl, double* __restrict__ q,
                                  double* __restrict__ qd, int* __restrict__ conv) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (scene_list) {
        if (i >= *scene_cnt) return;
        i = scene_list[i];
    } else if (i >= n) {
        return;
    }
    SceneState s = st[i];
    if (s.phase == kDone) return;
    atomicAdd(evaluations, 1ull);  // [0]: all scenes; [1 + i]: scene i (this thread's alone)
    evaluations[1 + i] += 1ull;
    const MoverDev& m = mover[i];
    const int nd = m.ndof;
    const bool newton = s.phase == kNewton;
    const double* p = newton ? s.x : s.xt;
    const double* fe = f_ext + 6 * (size_t)i;
    double g[kMaxDof], H[kMaxDof * kMaxDof];
    if (nd == 6) {
        double fmc[6], Kmc[36], Dmc[36], M[36];
        free_contact_sums(pair_begin[i], pair_begin[i + 1], role, fm, Km, Dm, newton, fmc, Kmc, Dmc);
        sdfc_joint::free_system(free_body(m), fe, s.q0, s.qd0, p, fmc, Kmc, Dmc, newton, g, newton ? H : nullptr, M,
                                nullptr, nullptr, nullptr);
    } else {
        trans_system(m, fe, s, p, pair_begin[i], pair_begin[i + 1], role, fm, Km, Dm, newton, g, H);
    }
    bool done = false;
    if (newton) {
        double mg[kMaxDof];
        for (int k = 0; k < nd; ++k) mg[k] = -g[k];
        solve_n(H, mg, nd, s.dx);
        s.gnorm = norm_n(g, nd);
        s.alpha = 1.0;
        s.trial = 0;
        for (int k = 0; k < nd; ++k) s.xt[k] = s.x[k] + s.dx[k];
        s.phase = kLine;
    } else {
        const double gn = norm_n(g, nd);
        bool step_done = false;
        if (gn < s.gnorm) {  // line search succeeded
            s.strike = 0;
            for (int k = 0; k < nd; ++k) s.x[k] = s.xt[k];
            step_done = true;
        } else if (++s.trial < kMaxLineSearch) {
            s.alpha *= 0.5;
            for (int k = 0; k < nd; ++k) s.xt[k] = s.x[k] + s.alpha * s.dx[k];
        } else {  // 20 failures: alpha = 0.5^20
            s.alpha *= 0.5;
            if (++s.strike >= kMaxStrike) {
                done = true;  // stops before the update, Simulation.cpp:1052-1054
            } else {
                for (int k = 0; k < nd; ++k) s.x[k] = s.x[k] + s.alpha * s.dx[k];
                step_done = true;
            }
        }
        if (step_done) {
            ++s.iter;
            if (gn < m.tol) {
                s.converged = 1;
                done = true;
            } else if (s.iter >= m.max_iter) {
                done = true;
            } else {
                s.phase = kNewton;
            }
        }
    }
    if (!done && ++s.nev >= kMaxEvalsPerStep) done = true;
    if (done && !end_step(i, n, m, *ctl, q, qd, conv, s)) {
        s.phase = kDone;
        atomicSub(remaining, 1);
    } else if (nx.cnt) {
        append_active(i, pair_begin, inst_full, nx);
    }
    st[i] = s;
}

// sim_newton_kernel for free3d-exp movers with one warp per scene (one scene per CTA): the
// contact sums and the reduced system are spread over the lanes (sdfc_joint_warp.cuh), lane 0
// runs the 6x6 solve and the line-search bookkeeping as sim_newton_kernel does.
__global__ void __launch_bounds__(32) sim_newton_free_warp_kernel(
    int n, const int* __restrict__ pair_begin, const int* __restrict__ role, const MoverDev* __restrict__ mover,
    const double* __restrict__ f_ext, const double* __restrict__ fm, const double* __restrict__ Km,
    const double* __restrict__ Dm, SceneState* __restrict__ st, int* remaining, unsigned long long* evaluations,
    const int* __restrict__ scene_list, const int* __restrict__ scene_cnt,
    const sdfc::InstanceDesc* __restrict__ inst_full, CompactLists nx, const SimCtl* __restrict__ ctl,
    double* __restrict__ q, double* __restrict__ qd, int* __restrict__ conv) {
    __shared__ sdfc_joint::FreeWarp w;
    int i = blockIdx.x;
    const int lane = threadIdx.x;
    if (scene_list) {
        if (i >= *scene_cnt) return;
        i = scene_list[i];
    } else if (i >= n) {
        return;
    }
    SceneState s = st[i];
    if (s.phase == kDone) return;  // uniform over the warp
    if (lane == 0) {
        atomicAdd(evaluations, 1ull);
        evaluations[1 + i] += 1ull;
    }
    const MoverDev& m = mover[i];
    const bool newton = s.phase == kNewton;
    const double* p = newton ? s.x : s.xt;
    // contact sums: the mover's 6-row block of every pair's fm, Km, Dm
    const int k0 = pair_begin[i], k1 = pair_begin[i + 1];
    for (int t = lane; t < 78; t += 32) {
        if (t >= 6 && !newton) break;
        double v = 0.0;
        for (int k = k0; k < k1; ++k) {
            const int o = role[k] ? 0 : 6;
            if (t < 6) {
                v += fm[12 * (size_t)k + o + t];
            } else {
                const int e = (t - 6) % 36, r = e / 6, c = e % 6;
                const double* src = t < 42 ? Km : Dm;
                v += src[144 * (size_t)k + (o + r) * 12 + o + c];
            }
        }
        if (t < 6)
            w.fmc[t] = v;
        else if (t < 42)
            w.Kmc[t - 6] = v;
        else
            w.Dmc[t - 42] = v;
    }
    __syncwarp();
    sdfc_joint::free_system_w(free_body(m), f_ext + 6 * (size_t)i, s.q0, s.qd0, p, newton, w);
    if (lane != 0) return;
    const int nd = 6;
    double g[6];
    for (int k = 0; k < 6; ++k) g[k] = w.g[k];
    bool done = false;
    if (newton) {
        double mg[kMaxDof], H[36];
        for (int k = 0; k < 36; ++k) H[k] = w.H[k];
        for (int k = 0; k < nd; ++k) mg[k] = -g[k];
        solve_n(H, mg, nd, s.dx);
        s.gnorm = norm_n(g, nd);
        s.alpha = 1.0;
        s.trial = 0;
        for (int k = 0; k < nd; ++k) s.xt[k] = s.x[k] + s.dx[k];
        s.phase = kLine;
    } else {
        const double gn = norm_n(g, nd);
        bool step_done = false;
        if (gn < s.gnorm) {
            s.strike = 0;
            for (int k = 0; k < nd; ++k) s.x[k] = s.xt[k];
            step_done = true;
        } else if (++s.trial < kMaxLineSearch) {
            s.alpha *= 0.5;
            for (int k = 0; k < nd; ++k) s.xt[k] = s.x[k] + s.alpha * s.dx[k];
        } else {
            s.alpha *= 0.5;
            if (++s.strike >= kMaxStrike) {
                done = true;
            } else {
                for (int k = 0; k < nd; ++k) s.x[k] = s.x[k] + s.alpha * s.dx[k];
                step_done = true;
            }
        }
        if (step_done) {
            ++s.iter;
            if (gn < m.tol) {
                s.converged = 1;
                done = true;
            } else if (s.iter >= m.max_iter) {
                done = true;
            } else {
                s.phase = kNewton;
            }
        }
    }
    if (!done && ++s.nev >= kMaxEvalsPerStep) done = true;
    if (done && !end_step(i, n, m, *ctl, q, qd, conv, s)) {
        s.phase = kDone;
        atomicSub(remaining, 1);
    } else if (nx.cnt) {
        append_active(i, pair_begin, inst_full, nx);
    }
    st[i] = s;
}

// ---------------------------------------------------------------- adjoint (backward_BDF1)
//
// Simulation::backward_BDF1 (Simulation.cpp:1559-1634) needs, per step k, the H, M and
// D that integration_BDF1 saves after convergence (:1262-1269): one derivative
// evaluation at (q_k, qdot_k = (q_k - q_{k-1}) / h).  Here the forward keeps only the
// trajectory q_0..q_T and the backward recomputes each step's H, D in reverse order,
// one batched evaluation per step, while it runs the recursion
//   z_k = H_k^{-T} (dL/dq_k - (-2M + h D_{k+1})^T z_{k+1} - M^T z_{k+2}).
// (The free joint's reparameterisation between steps is not differentiated, as in the
// reference.)

struct AdjState {
    double z1[kMaxDof], z2[kMaxDof];                       // z_{k+1}, z_{k+2}
    double D1[kMaxDof * kMaxDof], M1[kMaxDof * kMaxDof];   // D_{k+1}, M_{k+1}
    double M2[kMaxDof * kMaxDof];                          // M_{k+2}
    double acc[6];  // sum over steps of blkdiag(R_0i) diag(I) J z (the external force's gradient / h^2)
};

__global__ void adj_begin_kernel(int n, int T, AdjState* __restrict__ adj, int* __restrict__ t_dev) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        t_dev[0] = T;  // step being differentiated
        t_dev[1] = T;  // horizon
    }
    if (i >= n) return;
    AdjState a;
    for (int c = 0; c < kMaxDof; ++c) a.z1[c] = a.z2[c] = 0.0;
    for (int c = 0; c < kMaxDof * kMaxDof; ++c) a.D1[c] = a.M1[c] = a.M2[c] = 0.0;
    for (int c = 0; c < 6; ++c) a.acc[c] = 0.0;
    adj[i] = a;
}

// Pose of every pair at step t of the recorded trajectory (q_his is step-major:
// q_his[(t * n + scene) * nd + c]).
__global__ void adj_pose_kernel(int n_pairs, int n, int nd, const int* __restrict__ pair_inst,
                                const int* __restrict__ role, const double* __restrict__ E_fixed,
                                const MoverDev* __restrict__ mover, const double* __restrict__ q_his,
                                const int* __restrict__ t_dev, double* __restrict__ EA, double* __restrict__ phiA,
                                double* __restrict__ EB, double* __restrict__ phiB) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = t_dev[0];
    if (k >= n_pairs || t < 1) return;
    const int i = pair_inst[k];
    const MoverDev& m = mover[i];
    const double* q = q_his + (size_t)nd * ((size_t)t * n + i);
    const double* qp = q_his + (size_t)nd * ((size_t)(t - 1) * n + i);
    double qd[kMaxDof], E0i[16], phi[6];
    for (int c = 0; c < nd; ++c) qd[c] = (q[c] - qp[c]) / m.h;  // end_step's qdot
    mover_pose(m, q, qd, E0i, phi);
    double *Em = role[k] ? EA + 16 * (size_t)k : EB + 16 * (size_t)k;
    double *pm = role[k] ? phiA + 6 * (size_t)k : phiB + 6 * (size_t)k;
    double *Ef = role[k] ? EB + 16 * (size_t)k : EA + 16 * (size_t)k;
    double *pf = role[k] ? phiB + 6 * (size_t)k : phiA + 6 * (size_t)k;
    for (int c = 0; c < 16; ++c) {
        Em[c] = E0i[c];
        Ef[c] = E_fixed[16 * (size_t)k + c];
    }
    for (int c = 0; c < 6; ++c) {
        pm[c] = phi[c];
        pf[c] = 0.0;
    }
}

// Partial-pivoting LU of an n x n matrix (n <= 6) and the solve of A^T z = y with it
// (Eigen's PartialPivLU::transpose().solve, Simulation.cpp:1587): U^T w = y, L^T u = w,
// z = P^T u.
__device__ void lu_solve_transposed(const double* A, int n, const double* y, double* z) {
    double LU[kMaxDof * kMaxDof], w[kMaxDof], u[kMaxDof];
    int perm[kMaxDof];
    for (int k = 0; k < n * n; ++k) LU[k] = A[k];
    for (int k = 0; k < n; ++k) perm[k] = k;
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (fabs(LU[n * r + c]) > fabs(LU[n * p + c])) p = r;
        if (p != c) {
            for (int k = 0; k < n; ++k) {
                const double t = LU[n * c + k];
                LU[n * c + k] = LU[n * p + k];
                LU[n * p + k] = t;
            }
            const int t = perm[c];
            perm[c] = perm[p];
            perm[p] = t;
        }
        for (int r = c + 1; r < n; ++r) {
            LU[n * r + c] /= LU[n * c + c];
            for (int k = c + 1; k < n; ++k) LU[n * r + k] -= LU[n * r + c] * LU[n * c + k];
        }
    }
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

// One reverse step per scene.  At t = 1 it also writes the scene's gradients
// (:1590-1614): gout[18 i ..] = dL/dq0[nd] at 0, dL/dqdot0[nd] at 6, dL/df_ext[6] at 12.
// The external force enters step t's f as J^T diag(I) blkdiag(R_0i^T, R_0i^T) f_ext
// (Body.cpp:288-289), so dL/df_ext = h^2 sum_t blkdiag(R_0i) diag(I) J z_t.
__global__ void adj_step_kernel(int n, int nd, const int* __restrict__ pair_begin, const int* __restrict__ role,
                                const MoverDev* __restrict__ mover, const double* __restrict__ f_ext,
                                const double* __restrict__ fm, const double* __restrict__ Km,
                                const double* __restrict__ Dm, const double* __restrict__ q_his,
                                const double* __restrict__ qd0_rec, const double* __restrict__ df_dq,
                                const double* __restrict__ gE_his, const double* __restrict__ df_dE,
                                const int* __restrict__ t_dev, AdjState* __restrict__ adj, double* __restrict__ gout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = t_dev[0], T = t_dev[1];
    if (i >= n || t < 1) return;
    const MoverDev& m = mover[i];
    const double h = m.h;
    const double* q1 = q_his + (size_t)nd * ((size_t)t * n + i);
    const double* q0 = q_his + (size_t)nd * ((size_t)(t - 1) * n + i);
    double qd0[kMaxDof];
    for (int c = 0; c < nd; ++c)
        qd0[c] = t >= 2 ? (q0[c] - q_his[(size_t)nd * ((size_t)(t - 2) * n + i) + c]) / h : qd0_rec[(size_t)nd * i + c];
    double M[36], D[36], H[36], J[36], R0i[9];  // J is 6 x nd
    if (nd == 6) {
        double fmc[6], Kmc[36], Dmc[36], g[6];
        free_contact_sums(pair_begin[i], pair_begin[i + 1], role, fm, Km, Dm, true, fmc, Kmc, Dmc);
        sdfc_joint::free_system(free_body(m), f_ext + 6 * (size_t)i, q0, qd0, q1, fmc, Kmc, Dmc, true, g, H, M, D, J,
                                R0i);
    } else {
        double Kll[9] = {0}, Dll[9] = {0}, R[9];
        for (int k = pair_begin[i]; k < pair_begin[i + 1]; ++k) {
            const int o = role[k] ? 0 : 6;
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) {
                    Kll[3 * r + c] += Km[144 * (size_t)k + (o + 3 + r) * 12 + o + 3 + c];
                    Dll[3 * r + c] += Dm[144 * (size_t)k + (o + 3 + r) * 12 + o + 3 + c];
                }
        }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) R[3 * r + c] = m.E_ji[4 * r + c];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                M[3 * r + c] = R[3 * r] * m.inertia[3] * R[3 * c] + R[3 * r + 1] * m.inertia[4] * R[3 * c + 1] +
                               R[3 * r + 2] * m.inertia[5] * R[3 * c + 2];
                double K = 0.0, Dv = 0.0;
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        K += R[3 * r + a] * Kll[3 * a + b] * R[3 * c + b];
                        Dv += R[3 * r + a] * Dll[3 * a + b] * R[3 * c + b];
                    }
                if (r == c) {
                    K -= m.Kr;
                    Dv -= m.Dr;
                }
                D[3 * r + c] = Dv;
                H[3 * r + c] = M[3 * r + c] - h * h * K - h * Dv;
            }
        // J = [0; R_ji^T] (6 x 3); R_0i = R_pj0 R_ji does not depend on q
        for (int r = 0; r < 6; ++r)
            for (int c = 0; c < 3; ++c) J[3 * r + c] = r < 3 ? 0.0 : R[3 * c + (r - 3)];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c)
                R0i[3 * r + c] = m.E_pj0[4 * r] * R[c] + m.E_pj0[4 * r + 1] * R[3 + c] + m.E_pj0[4 * r + 2] * R[6 + c];
    }
    AdjState a = adj[i];
    double y[kMaxDof];
    for (int c = 0; c < nd; ++c) y[c] = df_dq[((size_t)i * T + (t - 1)) * nd + c];
    if (gE_his)  // dL/dE_total times dE_t/dq_t (step t's energy at its end state)
        for (int c = 0; c < nd; ++c) y[c] += df_dE[i] * gE_his[((size_t)(t - 1) * n + i) * nd + c];
    if (t < T)  // step t + 1: dg/dq_t = -2 M_{t+1} + h D_{t+1}
        for (int c = 0; c < nd; ++c)
            for (int r = 0; r < nd; ++r) y[c] -= (-2.0 * a.M1[nd * r + c] + h * a.D1[nd * r + c]) * a.z1[r];
    if (t < T - 1)  // step t + 2: dg/dq_t = M_{t+2}
        for (int c = 0; c < nd; ++c)
            for (int r = 0; r < nd; ++r) y[c] -= a.M2[nd * r + c] * a.z2[r];
    double z[kMaxDof];
    lu_solve_transposed(H, nd, y, z);
    {
        double Jz[6];
        for (int r = 0; r < 6; ++r) {
            double v = 0.0;
            for (int c = 0; c < nd; ++c) v += J[nd * r + c] * z[c];
            Jz[r] = v * m.inertia[r];
        }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                a.acc[r] += R0i[3 * r + c] * Jz[c];
                a.acc[3 + r] += R0i[3 * r + c] * Jz[3 + c];
            }
    }
    if (t == 1) {
        double* go = gout + 18 * (size_t)i;
        for (int c = 0; c < nd; ++c) {
            double g0 = 0.0, gd0 = 0.0;
            for (int r = 0; r < nd; ++r) {
                g0 -= (-M[nd * r + c] + h * D[nd * r + c]) * z[r];  // step 1
                if (T > 1) g0 -= a.M1[nd * r + c] * a.z1[r];           // step 2
                gd0 -= (-h * M[nd * r + c]) * z[r];
            }
            go[c] = g0;
            go[6 + c] = gd0;
        }
        for (int c = 0; c < 6; ++c) go[12 + c] = h * h * a.acc[c];
    }
    for (int c = 0; c < nd; ++c) {
        a.z2[c] = a.z1[c];
        a.z1[c] = z[c];
    }
    for (int c = 0; c < nd * nd; ++c) {
        a.M2[c] = a.M1[c];
        a.M1[c] = M[c];
        a.D1[c] = D[c];
    }
    adj[i] = a;
}

__global__ void adj_advance_kernel(int* t_dev) { t_dev[0] -= 1; }

// ---------------------------------------------------------------- penetration energy of the steps
//
// With energy recording on, every recorded step also evaluates each pair's penetration energy
// at the step's end state (sdfc_batch_energy) and reduces it per scene: E_t and its gradient
// wrt the joint coordinates, J^T dE/dq_m (the mover's twist block of each pair).

__global__ void energy_pose_kernel(int n_pairs, int nd, const int* __restrict__ pair_inst,
                                   const int* __restrict__ role, const double* __restrict__ E_fixed,
                                   const MoverDev* __restrict__ mover, const double* __restrict__ q,
                                   const double* __restrict__ qd, double* __restrict__ EA, double* __restrict__ phiA,
                                   double* __restrict__ EB, double* __restrict__ phiB) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_pairs) return;
    const int i = pair_inst[k];
    double E0i[16], phi[6];
    mover_pose(mover[i], q + (size_t)nd * i, qd + (size_t)nd * i, E0i, phi);
    double *Em = role[k] ? EA + 16 * (size_t)k : EB + 16 * (size_t)k;
    double *pm = role[k] ? phiA + 6 * (size_t)k : phiB + 6 * (size_t)k;
    double *Ef = role[k] ? EB + 16 * (size_t)k : EA + 16 * (size_t)k;
    double *pf = role[k] ? phiB + 6 * (size_t)k : phiA + 6 * (size_t)k;
    for (int c = 0; c < 16; ++c) {
        Em[c] = E0i[c];
        Ef[c] = E_fixed[16 * (size_t)k + c];
    }
    for (int c = 0; c < 6; ++c) {
        pm[c] = phi[c];
        pf[c] = 0.0;
    }
}

__global__ void energy_reduce_kernel(int n, int nd, const int* __restrict__ pair_begin, const int* __restrict__ role,
                                     const MoverDev* __restrict__ mover, const double* __restrict__ q,
                                     const double* __restrict__ e_pair, const double* __restrict__ dE_pair,
                                     double* __restrict__ E_out, double* __restrict__ g_out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const MoverDev& m = mover[i];
    double e = 0.0, dm[6] = {0, 0, 0, 0, 0, 0};
    for (int k = pair_begin[i]; k < pair_begin[i + 1]; ++k) {
        e += e_pair[k];
        const int o = role[k] ? 0 : 6;
        for (int c = 0; c < 6; ++c) dm[c] += dE_pair[12 * (size_t)k + o + c];
    }
    E_out[i] = e;
    double* g = g_out + (size_t)nd * i;
    if (nd == 6) {
        double J[36];
        sdfc_joint::free_jacobian(m.E_ji, q + 6 * (size_t)i, J);
        for (int c = 0; c < 6; ++c) {
            double v = 0.0;
            for (int r = 0; r < 6; ++r) v += J[6 * r + c] * dm[r];
            g[c] = v;
        }
    } else {  // J = [0; R_ji^T]: g = R_ji dE/dv
        for (int r = 0; r < 3; ++r) g[r] = m.E_ji[4 * r] * dm[3] + m.E_ji[4 * r + 1] * dm[4] + m.E_ji[4 * r + 2] * dm[5];
    }
}

}  // namespace

struct sdfc_sim {
    sdfc_context* ctx = nullptr;
    int n = 0, n_pairs = 0;
    int nd = 3;  // joint dofs of every mover (3 translational, 6 free3d-exp)
    // free3d-exp Newton updates on one thread per scene instead of one warp (SDFC_FREE_NEWTON_THREAD
    // set when the simulation is created; for comparing the two)
    bool free_thread = false;
    sdfc_batch* batch = nullptr;
    std::vector<int> order;  // sorted pair k -> caller's pair index
    MoverDev* d_mover = nullptr;
    SceneState* d_state = nullptr;
    double *d_q = nullptr, *d_qd = nullptr, *d_fext = nullptr;
    int *d_pair_inst = nullptr, *d_role = nullptr, *d_pair_begin = nullptr;
    double* d_Efixed = nullptr;
    double *d_EA = nullptr, *d_phiA = nullptr, *d_EB = nullptr, *d_phiB = nullptr, *d_prm = nullptr;
    int* d_mode = nullptr;
    double *d_fm = nullptr, *d_Km = nullptr, *d_Dm = nullptr;
    int *d_nact = nullptr, *d_status = nullptr, *d_conv = nullptr, *d_remaining = nullptr;
    unsigned long long* d_evals = nullptr;
    int* h_remaining = nullptr;
    long long rounds = 0;
    // the per-call control block (device copy read by the Newton kernels, pinned host staging)
    SimCtl* d_ctl = nullptr;
    SimCtl* h_ctl = nullptr;
    // SDFC_SIM_LOCKSTEP set at creation: every step waits for all scenes (one step per round
    // loop, as the scenes of one sdfc_sim_step call otherwise do not; for comparing the two)
    bool lockstep = false;
    double* d_qzero = nullptr;  // zero joint velocities (the energy evaluations' poses)
    std::vector<void*> allocations;
    // one Newton round (pose, batched evaluation, Newton update) as a CUDA graph per round
    // parity, captured at the first step and after a precision change
    cudaGraphExec_t round_exec[2] = {nullptr, nullptr};
    // compacted rounds: the next round's lists ([2] by parity; counts d_cnt[3 parity + 0..2]:
    // scenes, pairs, tiles), compact evaluation arrays, and one graph per capacity bucket and parity
    int parity = 0;
    int max_pairs_scene = 0, max_tiles_scene = 0;
    int* d_cnt = nullptr;
    int* d_scene_list[2] = {nullptr, nullptr};
    int* d_pair_list[2] = {nullptr, nullptr};
    sdfc::InstanceDesc* d_inst_c[2] = {nullptr, nullptr};
    int* d_tile_c[2] = {nullptr, nullptr};
    double *d_EA_c = nullptr, *d_phiA_c = nullptr, *d_EB_c = nullptr, *d_phiB_c = nullptr, *d_prm_c = nullptr;
    int* d_mode_c = nullptr;
    double *d_fm_c = nullptr, *d_Km_c = nullptr, *d_Dm_c = nullptr;
    int *d_nact_c = nullptr, *d_status_c = nullptr;
    std::vector<int> buckets;  // scene capacities, decreasing
    std::vector<cudaGraphExec_t> compact_exec;  // [2 b + parity]
    long long compact_rounds = 0;
    cudaStream_t capture_stream = nullptr;
    // adjoint: the recorded trajectory (step-major, (record_cap + 1) x n x 3), qdot_0,
    // dL/dq (n x T x 3), per-scene recursion state, gradients, reverse step counter
    int record_cap = 0, recorded = 0;
    double *d_qhis = nullptr, *d_qd0rec = nullptr, *d_dfdq = nullptr;
    size_t dfdq_cap = 0;
    AdjState* d_adj = nullptr;
    double* d_gout = nullptr;
    int* d_t = nullptr;
    cudaGraphExec_t back_exec = nullptr;
    // penetration energy per recorded step (step-major, record_cap x n) and its joint-space
    // gradient (record_cap x n x nd); per-pair energies of one evaluation; dL/dE per scene
    int energy_on = 0;
    double *d_Ehis = nullptr, *d_gEhis = nullptr, *d_epair = nullptr, *d_dEpair = nullptr, *d_dfdE = nullptr;
    std::vector<MoverDev> movers;  // host copy (tolerance updates)
};

namespace sdfc_impl {

void free_sim(sdfc_sim* s) {
    if (!s) return;
    for (cudaGraphExec_t& g : s->round_exec)
        if (g) cudaGraphExecDestroy(g);
    for (cudaGraphExec_t g : s->compact_exec)
        if (g) cudaGraphExecDestroy(g);
    if (s->back_exec) cudaGraphExecDestroy(s->back_exec);
    if (s->capture_stream) cudaStreamDestroy(s->capture_stream);
    cudaFree(s->d_qhis);
    cudaFree(s->d_qd0rec);
    cudaFree(s->d_dfdq);
    cudaFree(s->d_Ehis);
    cudaFree(s->d_gEhis);
    for (void* p : s->allocations) cudaFree(p);
    if (s->h_remaining) cudaFreeHost(s->h_remaining);
    if (s->h_ctl) cudaFreeHost(s->h_ctl);
    if (s->batch) sdfc_impl::free_batch(s->batch);
    delete s;
}

}  // namespace sdfc_impl

namespace {

using sdfc_impl::free_sim;

template <class T>
int alloc(sdfc_sim* s, T** p, size_t count) {
    void* v = nullptr;
    int rc = dev_alloc(s->ctx, &v, sizeof(T) * std::max<size_t>(count, 1));
    if (rc) return rc;
    s->allocations.push_back(v);
    *p = (T*)v;
    return SDFC_OK;
}

}  // namespace

extern "C" {

int sdfc_sim_create(sdfc_context* ctx, int n, const sdfc_mover* movers, int n_pairs, const sdfc_scene_pair* pairs,
                    sdfc_sim** out) {
    if (!ctx) return SDFC_ERR_INVALID_ARGUMENT;
    if (n <= 0 || !movers || n_pairs < 0 || (n_pairs > 0 && !pairs) || !out)
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_create: bad argument");
    for (int i = 0; i < n; ++i) {
        if (movers[i].joint != SDFC_JOINT_TRANSLATIONAL && movers[i].joint != SDFC_JOINT_FREE3D_EXP)
            return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_create: unknown joint type");
        if (movers[i].joint != movers[0].joint)
            return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_create: all movers of a sim share one joint type");
        if (!(movers[i].h > 0.0)) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_create: time step must be > 0");
    }
    const int nd = movers[0].joint == SDFC_JOINT_FREE3D_EXP ? 6 : 3;
    for (int k = 0; k < n_pairs; ++k)
        if (pairs[k].instance < 0 || pairs[k].instance >= n)
            return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_create: pair instance out of range");
    int rc = use_device(ctx);
    if (rc) return rc;
    auto* s = new sdfc_sim();
    s->ctx = ctx;
    s->n = n;
    s->n_pairs = n_pairs;
    s->nd = nd;
    s->free_thread = std::getenv("SDFC_FREE_NEWTON_THREAD") != nullptr;
    s->lockstep = std::getenv("SDFC_SIM_LOCKSTEP") != nullptr;
    // pairs grouped by scene (stable), so each scene's pairs are contiguous
    s->order.resize(n_pairs);
    std::iota(s->order.begin(), s->order.end(), 0);
    std::stable_sort(s->order.begin(), s->order.end(),
                     [&](int a, int b) { return pairs[a].instance < pairs[b].instance; });
    std::vector<int> pts(n_pairs), grd(n_pairs), inst(n_pairs), role(n_pairs), begin(n + 1, 0);
    std::vector<double> Ef(16 * (size_t)n_pairs), prm(6 * (size_t)n_pairs);
    for (int k = 0; k < n_pairs; ++k) {
        const sdfc_scene_pair& P = pairs[s->order[k]];
        pts[k] = P.points;
        grd[k] = P.grid;
        inst[k] = P.instance;
        role[k] = P.mover_is_contact ? 1 : 0;
        std::memcpy(&Ef[16 * (size_t)k], P.E_fixed, sizeof(double) * 16);
        const double pr[6] = {P.params.kn, P.params.kt, P.params.mu, P.params.damping, P.params.scale,
                              P.params.contact_scale};
        std::memcpy(&prm[6 * (size_t)k], pr, sizeof pr);
        begin[P.instance + 1]++;
    }
    for (int i = 0; i < n; ++i) begin[i + 1] += begin[i];
    std::vector<MoverDev> md(n);
    for (int i = 0; i < n; ++i) {
        const sdfc_mover& m = movers[i];
        MoverDev d{};
        d.mass = m.mass;
        std::memcpy(d.inertia, m.inertia, sizeof d.inertia);
        std::memcpy(d.E_pj0, m.E_pj0, sizeof d.E_pj0);
        std::memcpy(d.E_ji, m.E_ji, sizeof d.E_ji);
        std::memcpy(d.gravity, m.gravity, sizeof d.gravity);
        d.h = m.h;
        d.Kr = m.joint_stiffness;
        d.Dr = m.joint_damping;
        d.max_iter = std::max(20 * nd, 100);  // Simulation.cpp:1009
        d.ndof = nd;
        d.tol = kTol;
        md[i] = d;
    }
    if (n_pairs > 0 && (rc = sdfc_impl::batch_create(ctx, n_pairs, pts.data(), grd.data(), &s->batch))) {
        delete s;
        return rc;
    }
    if ((rc = alloc(s, &s->d_mover, n)) || (rc = alloc(s, &s->d_state, n)) || (rc = alloc(s, &s->d_q, (size_t)nd * n)) ||
        (rc = alloc(s, &s->d_qd, (size_t)nd * n)) || (rc = alloc(s, &s->d_fext, 6 * (size_t)n)) ||
        (rc = alloc(s, &s->d_pair_inst, n_pairs)) || (rc = alloc(s, &s->d_role, n_pairs)) ||
        (rc = alloc(s, &s->d_pair_begin, n + 1)) || (rc = alloc(s, &s->d_Efixed, 16 * (size_t)n_pairs)) ||
        (rc = alloc(s, &s->d_EA, 16 * (size_t)n_pairs)) || (rc = alloc(s, &s->d_phiA, 6 * (size_t)n_pairs)) ||
        (rc = alloc(s, &s->d_EB, 16 * (size_t)n_pairs)) || (rc = alloc(s, &s->d_phiB, 6 * (size_t)n_pairs)) ||
        (rc = alloc(s, &s->d_prm, 6 * (size_t)n_pairs)) || (rc = alloc(s, &s->d_mode, n_pairs)) ||
        (rc = alloc(s, &s->d_fm, 12 * (size_t)n_pairs)) || (rc = alloc(s, &s->d_Km, 144 * (size_t)n_pairs)) ||
        (rc = alloc(s, &s->d_Dm, 144 * (size_t)n_pairs)) || (rc = alloc(s, &s->d_nact, n_pairs)) ||
        (rc = alloc(s, &s->d_status, n_pairs)) || (rc = alloc(s, &s->d_conv, n)) ||
        (rc = alloc(s, &s->d_remaining, 1)) || (rc = alloc(s, &s->d_evals, (size_t)n + 1)) || (rc = alloc(s, &s->d_adj, n)) ||
        (rc = alloc(s, &s->d_gout, 18 * (size_t)n)) || (rc = alloc(s, &s->d_t, 2)) ||
        (rc = alloc(s, &s->d_epair, n_pairs)) || (rc = alloc(s, &s->d_dEpair, 12 * (size_t)n_pairs)) ||
        (rc = alloc(s, &s->d_dfdE, n)) || (rc = alloc(s, &s->d_ctl, 1)) || (rc = alloc(s, &s->d_qzero, (size_t)nd * n))) {
        free_sim(s);
        return rc;
    }
    if (cudaMallocHost((void**)&s->h_remaining, sizeof(int)) != cudaSuccess ||
        cudaMallocHost((void**)&s->h_ctl, sizeof(SimCtl)) != cudaSuccess) {
        free_sim(s);
        return fail(ctx, SDFC_ERR_CUDA, "sim_create: cudaMallocHost failed");
    }
    // compacted rounds: per-scene maxima of pairs and tiles, capacity buckets n/4, n/16, ...
    if (n_pairs > 0) {
        for (int i = 0; i < n; ++i) {
            int tiles = 0;
            for (int k = begin[i]; k < begin[i + 1]; ++k) tiles += s->batch->inst[k].ntiles;
            s->max_pairs_scene = std::max(s->max_pairs_scene, begin[i + 1] - begin[i]);
            s->max_tiles_scene = std::max(s->max_tiles_scene, tiles);
        }
        // SDFC_SIM_NO_COMPACT set at creation: full rounds only (for comparing the two)
        const bool compact = std::getenv("SDFC_SIM_NO_COMPACT") == nullptr;
        for (int b = n / 4; compact && b >= 1; b /= 4) {
            const long long Bp = (long long)b * s->max_pairs_scene + 1, Bt = (long long)b * s->max_tiles_scene;
            if (Bp <= n_pairs && Bt <= s->batch->total_tiles) s->buckets.push_back(b);
            if (b < 8) break;
        }
        s->compact_exec.assign(2 * s->buckets.size(), nullptr);
        const int tt = std::max(s->batch->total_tiles, 1);
        if ((rc = alloc(s, &s->d_cnt, 6)) || (rc = alloc(s, &s->d_scene_list[0], n)) ||
            (rc = alloc(s, &s->d_scene_list[1], n)) || (rc = alloc(s, &s->d_pair_list[0], n_pairs)) ||
            (rc = alloc(s, &s->d_pair_list[1], n_pairs)) || (rc = alloc(s, &s->d_inst_c[0], n_pairs + 1)) ||
            (rc = alloc(s, &s->d_inst_c[1], n_pairs + 1)) || (rc = alloc(s, &s->d_tile_c[0], tt)) ||
            (rc = alloc(s, &s->d_tile_c[1], tt)) || (rc = alloc(s, &s->d_EA_c, 16 * (size_t)(n_pairs + 1))) ||
            (rc = alloc(s, &s->d_phiA_c, 6 * (size_t)(n_pairs + 1))) ||
            (rc = alloc(s, &s->d_EB_c, 16 * (size_t)(n_pairs + 1))) ||
            (rc = alloc(s, &s->d_phiB_c, 6 * (size_t)(n_pairs + 1))) ||
            (rc = alloc(s, &s->d_prm_c, 6 * (size_t)(n_pairs + 1))) || (rc = alloc(s, &s->d_mode_c, n_pairs + 1)) ||
            (rc = alloc(s, &s->d_fm_c, 12 * (size_t)(n_pairs + 1))) ||
            (rc = alloc(s, &s->d_Km_c, 144 * (size_t)(n_pairs + 1))) ||
            (rc = alloc(s, &s->d_Dm_c, 144 * (size_t)(n_pairs + 1))) || (rc = alloc(s, &s->d_nact_c, n_pairs + 1)) ||
            (rc = alloc(s, &s->d_status_c, n_pairs + 1))) {
            free_sim(s);
            return rc;
        }
        cudaError_t e0 = cudaMemset(s->d_cnt, 0, sizeof(int) * 6);
        // the masked last slot of every bucket reads valid descriptors
        for (int p = 0; p < 2 && e0 == cudaSuccess; ++p) {
            std::vector<sdfc::InstanceDesc> fill(n_pairs + 1, s->batch->inst[0]);
            for (auto& d : fill) d.ntiles = 0;
            e0 = cudaMemcpy(s->d_inst_c[p], fill.data(), sizeof(sdfc::InstanceDesc) * fill.size(),
                            cudaMemcpyHostToDevice);
        }
        if (e0 != cudaSuccess) {
            free_sim(s);
            return fail(ctx, SDFC_ERR_CUDA, std::string("sim_create: ") + cudaGetErrorString(e0));
        }
    }
    s->movers = md;
    cudaError_t e = cudaMemcpy(s->d_mover, md.data(), sizeof(MoverDev) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n_pairs > 0) {
        e = cudaMemcpy(s->d_pair_inst, inst.data(), sizeof(int) * n_pairs, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(s->d_role, role.data(), sizeof(int) * n_pairs, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(s->d_Efixed, Ef.data(), sizeof(double) * Ef.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(s->d_prm, prm.data(), sizeof(double) * prm.size(), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemcpy(s->d_pair_begin, begin.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(s->d_q, 0, sizeof(double) * nd * n);
    if (e == cudaSuccess) e = cudaMemset(s->d_qd, 0, sizeof(double) * nd * n);
    if (e == cudaSuccess) e = cudaMemset(s->d_qzero, 0, sizeof(double) * nd * n);
    if (e == cudaSuccess) e = cudaMemset(s->d_fext, 0, sizeof(double) * 6 * n);
    if (e == cudaSuccess) e = cudaMemset(s->d_conv, 0, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMemset(s->d_evals, 0, sizeof(unsigned long long) * ((size_t)n + 1));
    if (e != cudaSuccess) {
        free_sim(s);
        return fail(ctx, SDFC_ERR_CUDA, std::string("sim_create: ") + cudaGetErrorString(e));
    }
    ctx->sims.push_back(s);
    *out = s;
    return SDFC_OK;
}

void sdfc_sim_destroy(sdfc_sim* s) {
    if (!s) return;
    sdfc_context* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    auto it = std::find(ctx->sims.begin(), ctx->sims.end(), s);
    if (it != ctx->sims.end()) ctx->sims.erase(it);
    free_sim(s);
}

// Drops the captured graphs (they launch the kernels of the configuration they were captured
// under); the next step or backward pass captures them again.
static void drop_graphs(sdfc_sim* s) {
    for (cudaGraphExec_t& g : s->round_exec)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    for (cudaGraphExec_t& g : s->compact_exec)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    if (s->back_exec) {
        cudaGraphExecDestroy(s->back_exec);
        s->back_exec = nullptr;
    }
}

int sdfc_sim_set_precision(sdfc_sim* s, int precision) {
    if (!s) return SDFC_ERR_INVALID_ARGUMENT;
    if (precision != SDFC_PRECISION_FP64 && precision != SDFC_PRECISION_MIXED)
        return fail(s->ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_set_precision: unknown precision");
    if (s->batch) s->batch->precision = precision;
    drop_graphs(s);
    return SDFC_OK;
}

int sdfc_sim_set_tuning(sdfc_sim* s, const sdfc_tuning* t) {
    if (!s) return SDFC_ERR_INVALID_ARGUMENT;
    if (!s->batch) return fail(s->ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_set_tuning: the sim has no contact pairs");
    int rc = sdfc_batch_set_tuning(s->batch, t);
    if (rc) return rc;
    drop_graphs(s);
    return SDFC_OK;
}

int sdfc_sim_get_tuning(sdfc_sim* s, sdfc_tuning* t) {
    if (!s || !s->batch) return SDFC_ERR_INVALID_ARGUMENT;
    return sdfc_batch_get_tuning(s->batch, t);
}

int sdfc_sim_autotune(sdfc_sim* s, sdfc_tuning* chosen) {
    if (!s) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    int rc = use_device(ctx);
    if (rc) return rc;
    if (s->n_pairs == 0) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_autotune: the sim has no contact pairs");
    cudaStream_t st = ctx->stream;
    const int n = s->n, np = s->n_pairs, tb = 128;
    // the opening evaluation of a step from the current state: every scene at its Newton point
    // (the state sim_begin_kernel writes is rewritten by the next step)
    sim_begin_kernel<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->nd, s->d_mover, s->d_q, s->d_qd, s->d_state,
                                                      s->d_remaining);
    sim_pose_kernel<<<(np + tb - 1) / tb, tb, 0, st>>>(np, s->d_pair_inst, s->d_role, s->d_Efixed, s->d_mover,
                                                      s->d_state, s->d_EA, s->d_phiA, s->d_EB, s->d_phiB, s->d_mode);
    SDFC_CUDA_TRY(ctx, cudaGetLastError());
    sdfc::BatchInputs in{s->d_EA, s->d_phiA, s->d_EB, s->d_phiB, s->d_prm};
    in.mode = s->d_mode;
    sdfc::BatchOutputs out{s->d_fm, s->d_Km, s->d_Dm, s->d_nact, s->d_status};
    if ((rc = sdfc_impl::autotune(s->batch, in, true, out, st, chosen))) return rc;
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    drop_graphs(s);
    return SDFC_OK;
}

int sdfc_sim_set_state(sdfc_sim* s, const double* q, const double* qdot) {
    if (!s || !q || !qdot) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    int rc = use_device(ctx);
    if (rc) return rc;
    const size_t bytes = sizeof(double) * s->nd * s->n;
    SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->d_q, q, bytes, cudaMemcpyHostToDevice, ctx->stream));
    SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->d_qd, qdot, bytes, cudaMemcpyHostToDevice, ctx->stream));
    if (s->record_cap > 0) {  // a new initial state restarts the recording
        s->recorded = 0;
        SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->d_qhis, s->d_q, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
        SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->d_qd0rec, s->d_qd, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return SDFC_OK;
}

int sdfc_sim_get_state(sdfc_sim* s, double* q, double* qdot) {
    if (!s || !q || !qdot) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    int rc = use_device(ctx);
    if (rc) return rc;
    SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(q, s->d_q, sizeof(double) * s->nd * s->n, cudaMemcpyDeviceToHost, ctx->stream));
    SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(qdot, s->d_qd, sizeof(double) * s->nd * s->n, cudaMemcpyDeviceToHost,
                                       ctx->stream));
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return SDFC_OK;
}

int sdfc_sim_set_external_force(sdfc_sim* s, const double* f) {
    if (!s || !f) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    int rc = use_device(ctx);
    if (rc) return rc;
    SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->d_fext, f, sizeof(double) * 6 * s->n, cudaMemcpyHostToDevice, ctx->stream));
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return SDFC_OK;
}

}  // extern "C"

namespace {

CompactLists lists_of(sdfc_sim* s, int parity) {
    if (!s->d_cnt) return CompactLists{nullptr, nullptr, nullptr, nullptr, nullptr};
    return CompactLists{s->d_cnt + 3 * parity, s->d_scene_list[parity], s->d_pair_list[parity], s->d_inst_c[parity],
                        s->d_tile_c[parity]};
}

void launch_newton(sdfc_sim* s, cudaStream_t st, int grid_scenes, const int* scene_list, const int* scene_cnt,
                   CompactLists nx) {
    const sdfc::InstanceDesc* inst_full = s->batch ? s->batch->d_inst : nullptr;
    if (s->nd == 6 && !s->free_thread) {
        sim_newton_free_warp_kernel<<<grid_scenes, 32, 0, st>>>(s->n, s->d_pair_begin, s->d_role, s->d_mover, s->d_fext,
                                                                 s->d_fm, s->d_Km, s->d_Dm, s->d_state, s->d_remaining,
                                                                 s->d_evals, scene_list, scene_cnt, inst_full, nx,
                                                                 s->d_ctl, s->d_q, s->d_qd, s->d_conv);
    } else {
        constexpr int ts = kSceneThreads;
        sim_newton_kernel<<<(grid_scenes + ts - 1) / ts, ts, 0, st>>>(
            s->n, s->d_pair_begin, s->d_role, s->d_mover, s->d_fext, s->d_fm, s->d_Km, s->d_Dm, s->d_state,
            s->d_remaining, s->d_evals, scene_list, scene_cnt, inst_full, nx, s->d_ctl, s->d_q, s->d_qd, s->d_conv);
    }
}

// Enqueues one Newton round over every scene on `st`; the still-active scenes are listed for
// the next round (parity 1 - parity).
int enqueue_round(sdfc_sim* s, cudaStream_t st, int parity) {
    const int n = s->n, np = s->n_pairs, tb = 128;
    sdfc::BatchInputs in{s->d_EA, s->d_phiA, s->d_EB, s->d_phiB, s->d_prm};
    in.mode = s->d_mode;
    sdfc::BatchOutputs out{s->d_fm, s->d_Km, s->d_Dm, s->d_nact, s->d_status};
    if (s->d_cnt) SDFC_CUDA_TRY(s->ctx, cudaMemsetAsync(s->d_cnt + 3 * (1 - parity), 0, 3 * sizeof(int), st));
    if (np > 0) {
        sim_pose_kernel<<<(np + tb - 1) / tb, tb, 0, st>>>(np, s->d_pair_inst, s->d_role, s->d_Efixed, s->d_mover,
                                                          s->d_state, s->d_EA, s->d_phiA, s->d_EB, s->d_phiB,
                                                          s->d_mode);
        int rc = sdfc_impl::run_batch(s->batch, in, true, out, st);
        if (rc) return rc;
    }
    launch_newton(s, st, n, nullptr, nullptr, lists_of(s, 1 - parity));
    return SDFC_OK;
}

// Enqueues one compacted round of capacity `cap` scenes reading the lists of `parity`.
int enqueue_compact(sdfc_sim* s, cudaStream_t st, int parity, int cap) {
    const int Bp = cap * s->max_pairs_scene + 1, Bt = cap * s->max_tiles_scene, tb = 128;
    const int* cnt = s->d_cnt + 3 * parity;
    SDFC_CUDA_TRY(s->ctx, cudaMemsetAsync(s->d_cnt + 3 * (1 - parity), 0, 3 * sizeof(int), st));
    sim_pose_compact_kernel<<<(Bp + Bt + tb - 1) / tb, tb, 0, st>>>(
        Bp, Bt, cnt, s->d_pair_list[parity], s->d_tile_c[parity], s->d_pair_inst, s->d_role, s->d_Efixed, s->d_prm,
        s->d_mover, s->d_state, s->d_EA_c, s->d_phiA_c, s->d_EB_c, s->d_phiB_c, s->d_prm_c, s->d_mode_c);
    sdfc_batch view = *s->batch;  // the batch's scratch, the compact instance and tile tables
    view.d_inst = s->d_inst_c[parity];
    view.d_tile_inst = s->d_tile_c[parity];
    view.n = Bp;
    view.total_tiles = Bt;
    view.timing = false;
    sdfc::BatchInputs in{s->d_EA_c, s->d_phiA_c, s->d_EB_c, s->d_phiB_c, s->d_prm_c};
    in.mode = s->d_mode_c;
    sdfc::BatchOutputs out{s->d_fm_c, s->d_Km_c, s->d_Dm_c, s->d_nact_c, s->d_status_c};
    int rc = sdfc_impl::run_batch(&view, in, true, out, st);
    if (rc) return rc;
    sim_scatter_kernel<<<Bp, 128, 0, st>>>(cnt, s->d_pair_list[parity], s->d_mode_c, s->d_fm_c, s->d_Km_c, s->d_Dm_c,
                                           s->d_nact_c, s->d_status_c, s->d_fm, s->d_Km, s->d_Dm, s->d_nact,
                                           s->d_status);
    launch_newton(s, st, cap, s->d_scene_list[parity], cnt, lists_of(s, 1 - parity));
    return SDFC_OK;
}

// Captures a round into a graph (replayed every round of its kind: its kernels skip the
// scenes that are done, so replaying it is always correct).  cap < 0: a full round.
int capture_round(sdfc_sim* s, int parity, int cap, cudaGraphExec_t* exec) {
    sdfc_context* ctx = s->ctx;
    if (!s->capture_stream)
        SDFC_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&s->capture_stream, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    SDFC_CUDA_TRY(ctx, cudaStreamBeginCapture(s->capture_stream, cudaStreamCaptureModeThreadLocal));
    int rc = cap < 0 ? enqueue_round(s, s->capture_stream, parity) : enqueue_compact(s, s->capture_stream, parity, cap);
    cudaError_t e = cudaStreamEndCapture(s->capture_stream, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return fail(ctx, SDFC_ERR_CUDA, std::string("sim capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(ctx, SDFC_ERR_CUDA, std::string("sim instantiate: ") + cudaGetErrorString(e));
    return SDFC_OK;
}

// The graph of the next round: compacted to the smallest bucket that holds `active` scenes.
int round_graph(sdfc_sim* s, int active, cudaGraphExec_t* out) {
    const int p = s->parity;
    int b = -1;
    for (int k = 0; k < (int)s->buckets.size(); ++k)
        if (s->buckets[k] >= active) b = k;
    cudaGraphExec_t* slot = b < 0 ? &s->round_exec[p] : &s->compact_exec[2 * b + p];
    if (!*slot) {
        int rc = capture_round(s, p, b < 0 ? -1 : s->buckets[b], slot);
        if (rc) return rc;
    }
    if (b >= 0) ++s->compact_rounds;
    *out = *slot;
    return SDFC_OK;
}

// Captures one reverse step of the adjoint (replayed T times; the step index lives
// in device memory and the last kernel decrements it).
int capture_backward(sdfc_sim* s) {
    sdfc_context* ctx = s->ctx;
    if (!s->capture_stream)
        SDFC_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&s->capture_stream, cudaStreamNonBlocking));
    const int n = s->n, np = s->n_pairs, tb = 128;
    cudaStream_t st = s->capture_stream;
    cudaGraph_t graph = nullptr;
    SDFC_CUDA_TRY(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = SDFC_OK;
    if (np > 0) {
        adj_pose_kernel<<<(np + tb - 1) / tb, tb, 0, st>>>(np, n, s->nd, s->d_pair_inst, s->d_role, s->d_Efixed,
                                                          s->d_mover, s->d_qhis, s->d_t, s->d_EA, s->d_phiA, s->d_EB,
                                                          s->d_phiB);
        sdfc::BatchInputs in{s->d_EA, s->d_phiA, s->d_EB, s->d_phiB, s->d_prm};
        sdfc::BatchOutputs out{s->d_fm, s->d_Km, s->d_Dm, s->d_nact, s->d_status};
        rc = sdfc_impl::run_batch(s->batch, in, true, out, st);
    }
    if (!rc) {
        constexpr int ts = kSceneThreads;
        adj_step_kernel<<<(n + ts - 1) / ts, ts, 0, st>>>(n, s->nd, s->d_pair_begin, s->d_role, s->d_mover, s->d_fext,
                                                         s->d_fm, s->d_Km, s->d_Dm, s->d_qhis, s->d_qd0rec, s->d_dfdq,
                                                         s->energy_on ? s->d_gEhis : nullptr, s->d_dfdE, s->d_t,
                                                         s->d_adj, s->d_gout);
        adj_advance_kernel<<<1, 1, 0, st>>>(s->d_t);
    }
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return fail(ctx, SDFC_ERR_CUDA, std::string("sim backward capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&s->back_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return fail(ctx, SDFC_ERR_CUDA, std::string("sim backward instantiate: ") + cudaGetErrorString(e));
    return SDFC_OK;
}

}  // namespace

// Penetration energy at the end state of recorded step t (0-based; its trajectory row t + 1) and
// its joint-space gradient.  The energy reads the bodies' poses alone, so the poses come from the
// recorded row with zero velocities.
int record_energy_step(sdfc_sim* s, cudaStream_t st, int t) {
    const int n = s->n, np = s->n_pairs, nd = s->nd, tb = 128;
    const double* q = s->d_qhis + (size_t)nd * n * (t + 1);
    double* E_out = s->d_Ehis + (size_t)n * t;
    double* g_out = s->d_gEhis + (size_t)nd * n * t;
    if (np > 0) {
        energy_pose_kernel<<<(np + tb - 1) / tb, tb, 0, st>>>(np, nd, s->d_pair_inst, s->d_role, s->d_Efixed,
                                                             s->d_mover, q, s->d_qzero, s->d_EA, s->d_phiA, s->d_EB,
                                                             s->d_phiB);
        sdfc::BatchInputs in{s->d_EA, s->d_phiA, s->d_EB, s->d_phiB, s->d_prm};
        int rc = sdfc_impl::run_energy(s->batch, in, s->d_epair, s->d_dEpair, st);
        if (rc) return rc;
    }
    energy_reduce_kernel<<<(n + tb - 1) / tb, tb, 0, st>>>(n, nd, s->d_pair_begin, s->d_role, s->d_mover, q,
                                                          s->d_epair, s->d_dEpair, E_out, g_out);
    return SDFC_OK;
}

extern "C" {

int sdfc_sim_record_energy(sdfc_sim* s, int on) {
    if (!s) return SDFC_ERR_INVALID_ARGUMENT;
    int rc = sdfc_sim_record(s, 0);  // a recording kept so far has no energies: stop it
    if (rc) return rc;
    s->energy_on = on ? 1 : 0;
    return SDFC_OK;
}

int sdfc_sim_energy(sdfc_sim* s, double* per_step, double* total) {
    if (!s) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    if (!s->energy_on || s->record_cap == 0)
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_energy: energy recording is off");
    int rc = use_device(ctx);
    if (rc) return rc;
    const int n = s->n, T = s->recorded;
    std::vector<double> h((size_t)n * std::max(T, 1), 0.0);
    if (T > 0) {
        SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), s->d_Ehis, sizeof(double) * n * T, cudaMemcpyDeviceToHost,
                                           ctx->stream));
        SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    for (int i = 0; i < n; ++i) {
        double acc = 0.0;
        for (int t = 0; t < T; ++t) {
            const double e = h[(size_t)t * n + i];
            if (per_step) per_step[(size_t)i * T + t] = e;
            acc += e;
        }
        if (total) total[i] = acc;
    }
    return SDFC_OK;
}

int sdfc_sim_set_tolerance(sdfc_sim* s, double tol) {
    if (!s) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    if (!(tol > 0.0)) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_set_tolerance: tolerance must be > 0");
    int rc = use_device(ctx);
    if (rc) return rc;
    for (auto& m : s->movers) m.tol = tol;
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    SDFC_CUDA_TRY(ctx, cudaMemcpy(s->d_mover, s->movers.data(), sizeof(MoverDev) * s->n, cudaMemcpyHostToDevice));
    return SDFC_OK;
}

int sdfc_sim_record(sdfc_sim* s, int max_steps) {
    if (!s) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    if (max_steps < 0) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_record: max_steps must be >= 0");
    int rc = use_device(ctx);
    if (rc) return rc;
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (s->back_exec) {  // its kernels hold the old history pointer
        cudaGraphExecDestroy(s->back_exec);
        s->back_exec = nullptr;
    }
    cudaFree(s->d_qhis);
    cudaFree(s->d_qd0rec);
    cudaFree(s->d_Ehis);
    cudaFree(s->d_gEhis);
    s->d_qhis = s->d_qd0rec = s->d_Ehis = s->d_gEhis = nullptr;
    s->record_cap = s->recorded = 0;
    if (max_steps == 0) return SDFC_OK;
    const size_t n3 = (size_t)s->nd * s->n;
    if ((rc = dev_alloc(ctx, (void**)&s->d_qhis, sizeof(double) * n3 * ((size_t)max_steps + 1))) ||
        (rc = dev_alloc(ctx, (void**)&s->d_qd0rec, sizeof(double) * n3)) ||
        (s->energy_on && ((rc = dev_alloc(ctx, (void**)&s->d_Ehis, sizeof(double) * s->n * (size_t)max_steps)) ||
                          (rc = dev_alloc(ctx, (void**)&s->d_gEhis, sizeof(double) * n3 * (size_t)max_steps))))) {
        cudaFree(s->d_qhis);
        cudaFree(s->d_qd0rec);
        cudaFree(s->d_Ehis);
        s->d_qhis = s->d_qd0rec = s->d_Ehis = nullptr;
        return rc;
    }
    SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->d_qhis, s->d_q, sizeof(double) * n3, cudaMemcpyDeviceToDevice, ctx->stream));
    SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->d_qd0rec, s->d_qd, sizeof(double) * n3, cudaMemcpyDeviceToDevice, ctx->stream));
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    s->record_cap = max_steps;
    return SDFC_OK;
}

int sdfc_sim_history(sdfc_sim* s, int* steps, double* q_his) {
    if (!s || !steps) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    int rc = use_device(ctx);
    if (rc) return rc;
    if (s->record_cap == 0) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_history: recording is off");
    *steps = s->recorded;
    if (!q_his) return SDFC_OK;
    const int n = s->n, T1 = s->recorded + 1, nd = s->nd;
    std::vector<double> h((size_t)nd * n * T1);
    SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), s->d_qhis, sizeof(double) * h.size(), cudaMemcpyDeviceToHost,
                                       ctx->stream));
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    for (int t = 0; t < T1; ++t)  // step-major on the device, scene-major for the caller
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < nd; ++c) q_his[(nd * ((size_t)i * T1 + t)) + c] = h[nd * ((size_t)t * n + i) + c];
    return SDFC_OK;
}

int sdfc_sim_backward(sdfc_sim* s, const double* df_dq, double* df_dq0, double* df_dqdot0, double* df_dfext) {
    return sdfc_sim_backward_energy(s, df_dq, nullptr, df_dq0, df_dqdot0, df_dfext);
}

int sdfc_sim_backward_energy(sdfc_sim* s, const double* df_dq, const double* df_dE, double* df_dq0,
                             double* df_dqdot0, double* df_dfext) {
    if (!s) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    if (!df_dq) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_backward: null df_dq");
    if (df_dE && !s->energy_on)
        return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_backward: energy recording is off (sdfc_sim_record_energy)");
    if (s->record_cap == 0) return fail(ctx, SDFC_ERR_INVALID_ARGUMENT, "sim_backward: recording is off");
    int rc = use_device(ctx);
    if (rc) return rc;
    const int n = s->n, T = s->recorded, tb = 128, nd = s->nd;
    cudaStream_t st = ctx->stream;
    std::vector<double> g(18 * (size_t)n, 0.0);
    if (T > 0) {
        const size_t need = (size_t)nd * n * T;
        if (need > s->dfdq_cap) {
            if (s->back_exec) {  // its kernels hold the old dL/dq pointer
                cudaGraphExecDestroy(s->back_exec);
                s->back_exec = nullptr;
            }
            cudaFree(s->d_dfdq);
            s->d_dfdq = nullptr;
            s->dfdq_cap = 0;
            if ((rc = dev_alloc(ctx, (void**)&s->d_dfdq, sizeof(double) * need))) return rc;
            s->dfdq_cap = need;
        }
        SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->d_dfdq, df_dq, sizeof(double) * need, cudaMemcpyHostToDevice, st));
        if (df_dE)
            SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->d_dfdE, df_dE, sizeof(double) * n, cudaMemcpyHostToDevice, st));
        else
            SDFC_CUDA_TRY(ctx, cudaMemsetAsync(s->d_dfdE, 0, sizeof(double) * n, st));
        adj_begin_kernel<<<(n + tb - 1) / tb, tb, 0, st>>>(n, T, s->d_adj, s->d_t);
        SDFC_CUDA_TRY(ctx, cudaGetLastError());
        if (!s->back_exec && (rc = capture_backward(s))) return rc;
        for (int t = T; t >= 1; --t) SDFC_CUDA_TRY(ctx, cudaGraphLaunch(s->back_exec, st));
        SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(g.data(), s->d_gout, sizeof(double) * g.size(), cudaMemcpyDeviceToHost, st));
        SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    }
    for (int i = 0; i < n; ++i) {
        const double* gi = &g[18 * (size_t)i];
        if (df_dq0) std::memcpy(df_dq0 + (size_t)nd * i, gi, sizeof(double) * nd);
        if (df_dqdot0) std::memcpy(df_dqdot0 + (size_t)nd * i, gi + 6, sizeof(double) * nd);
        if (df_dfext) std::memcpy(df_dfext + 6 * (size_t)i, gi + 12, sizeof(double) * 6);
    }
    return SDFC_OK;
}

int sdfc_sim_step(sdfc_sim* s, int num_steps, int* converged) {
    if (!s || num_steps < 0) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    int rc = use_device(ctx);
    if (rc) return rc;
    if (s->record_cap > 0 && s->recorded + num_steps > s->record_cap)
        return fail(ctx, SDFC_ERR_CAPACITY, "sim_step: more steps than sdfc_sim_record's max_steps");
    cudaStream_t st = ctx->stream;
    const int n = s->n;
    const int tb = 128;
    const int per_check = 2;  // rounds enqueued between completion checks
    // one round loop for the whole call (each scene takes its steps one after another, without
    // waiting for the others), or one per step (SDFC_SIM_LOCKSTEP)
    const int loops = num_steps == 0 ? 0 : (s->lockstep ? num_steps : 1);
    const int target = s->lockstep ? 1 : num_steps;
    for (int l = 0; l < loops; ++l) {
        *s->h_ctl = SimCtl{target, s->recorded, s->record_cap > 0 ? s->d_qhis : nullptr};
        SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->d_ctl, s->h_ctl, sizeof(SimCtl), cudaMemcpyHostToDevice, st));
        sim_begin_kernel<<<(n + tb - 1) / tb, tb, 0, st>>>(n, s->nd, s->d_mover, s->d_q, s->d_qd, s->d_state,
                                                          s->d_remaining);
        // every scene ends each step within kMaxEvalsPerStep evaluations, one per round
        const long long max_rounds = (long long)target * kMaxEvalsPerStep + per_check;
        int active = n;
        for (long long r = 0; r < max_rounds && active > 0; r += per_check) {
            for (int k = 0; k < per_check; ++k) {
                cudaGraphExec_t g = nullptr;
                if ((rc = round_graph(s, active, &g))) return rc;
                SDFC_CUDA_TRY(ctx, cudaGraphLaunch(g, st));
                s->parity ^= 1;
            }
            // (the staged control block has been read once this completes)
            SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_remaining, s->d_remaining, sizeof(int), cudaMemcpyDeviceToHost, st));
            SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(st));
            s->rounds += per_check;
            active = *s->h_remaining;
        }
        if (active > 0) return fail(ctx, SDFC_ERR_CUDA, "sim_step: scenes still iterating after the round bound");
        if (s->record_cap > 0) {
            if (s->energy_on)
                for (int t = 0; t < target; ++t)
                    if ((rc = record_energy_step(s, st, s->recorded + t))) return rc;
            s->recorded += target;
        }
    }
    SDFC_CUDA_TRY(ctx, cudaGetLastError());
    if (converged)
        SDFC_CUDA_TRY(ctx, cudaMemcpyAsync(converged, s->d_conv, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return SDFC_OK;
}

int sdfc_sim_stats(sdfc_sim* s, long long* rounds, long long* evaluations) {
    if (!s) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    int rc = use_device(ctx);
    if (rc) return rc;
    unsigned long long e = 0;
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    SDFC_CUDA_TRY(ctx, cudaMemcpy(&e, s->d_evals, sizeof e, cudaMemcpyDeviceToHost));
    if (rounds) *rounds = s->rounds;
    if (evaluations) *evaluations = (long long)e;
    return SDFC_OK;
}

int sdfc_sim_scene_evaluations(sdfc_sim* s, long long* evaluations) {
    if (!s || !evaluations) return SDFC_ERR_INVALID_ARGUMENT;
    sdfc_context* ctx = s->ctx;
    int rc = use_device(ctx);
    if (rc) return rc;
    SDFC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    SDFC_CUDA_TRY(ctx, cudaMemcpy(evaluations, s->d_evals + 1, sizeof(long long) * s->n, cudaMemcpyDeviceToHost));
    return SDFC_OK;
}

}  // extern "C"
