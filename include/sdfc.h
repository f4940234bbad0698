/*
 * sdfc.h — C ABI of the GB300 point-vs-SDF penalty contact library
 * (libsdfcontact.so).
 *
 * It replaces, for the redmax simulator of Assemble-Them-All, the contact
 * force between the surface points of one body and the signed-distance grid
 * of another:
 *
 *   ForceGeneralSDFContact::computeForce               simulation/redmax/Force/ForceGeneralSDFContact.cpp:46-67
 *   ForceGeneralSDFContact::computeForceWithDerivative simulation/redmax/Force/ForceGeneralSDFContact.cpp:69-105
 *     (the Force plugin interface, simulation/redmax/Force/Force.h:40-47)
 *   collision_detection_general_SDF                    simulation/redmax/CollisionDetection/CollisionDetection.cpp:124-147
 *   BodySDFObj::distance / collision                   simulation/redmax/Body/BodySDFObj.cpp:207-377
 *
 * Conventions (the reference's):
 *   - poses E are 4x4 row-major homogeneous matrices [R p; 0 1] (Body::_E_0i);
 *   - body twists phi = (w, v) are in the body frame (Body::_phi);
 *   - grids are indexed values[i + ni*(j + nj*k)] in the SDF body's frame
 *     (BodySDFObj::_SDF, simulation/externals/sdfgen/array3.h:70-79), with
 *     _min_box, _max_box, _dx/_dy/_dz and _col_th as in BodySDFObj.h:13-15;
 *   - contact points are the contact body's Body::_contact_points, body frame;
 *   - fm is the 12-vector [body A (6); body B (6)] and Km = dfm/dq, Dm =
 *     dfm/dphi the 12x12 row-major blocks that ForceGeneralSDFContact adds
 *     into the simulator's maximal-coordinate arrays (ForceGeneralSDFContact.cpp:88-99).
 *     The library writes (=) these sub-blocks; the caller adds them at the
 *     bodies' indices as the reference does.
 *
 * All entry points return SDFC_OK (0) or a negative status; no C++ exception
 * crosses this boundary.  Host arrays are caller-owned; device memory is owned
 * by the context.  A context is bound to one CUDA device and is not
 * thread-safe (the reference calls its forces from one thread).
 */
#ifndef SDFC_H
#define SDFC_H

#ifdef __cplusplus
extern "C" {
#endif

#define SDFC_OK 0
#define SDFC_ERR_INVALID_ARGUMENT (-1)
#define SDFC_ERR_CUDA (-2)
#define SDFC_ERR_NOT_FOUND (-3)
#define SDFC_ERR_CAPACITY (-4)

/* storage of grid values / contact points on the device */
#define SDFC_STORAGE_F64 0
#define SDFC_STORAGE_F32 1
/* Grid values as FP16 codes in bricks of 8x8x8 nodes, each brick with an FP32 scale and
 * offset: value = offset + scale * code (see sdfc_f16_brick_encode).  A quarter of the
 * FP64 grid's memory; its values keep about 11 significant bits (the brick's offset is 0
 * where the SDF changes sign, so the values near the surface keep FP16's relative
 * precision). */
#define SDFC_STORAGE_F16_BRICKS 2
/* Grid values as FP32 node values alone: 4 bytes per node, where SDFC_STORAGE_F32 also keeps an
 * FP64 copy and a per-cell array of the 8 FP32 corners (40 bytes per node in all, which speeds
 * detection on grids that many instances share).  Every evaluation sees the same values as
 * with SDFC_STORAGE_F32 (the FP32 values, widened where FP64 is read), so results are
 * identical; this storage is for batches of many distinct large grids (256^3 grids of hundreds
 * of parts), whose 40-byte layout would not fit in device memory. */
#define SDFC_STORAGE_F32_NODES 3

/* How the SDF gradient and Hessian of an active contact are evaluated.
 * The reference takes central differences of the trilinear interpolant with
 * step 1e-5 (BodySDFObj::query_dSDF / query_ddSDF, BodySDFObj.cpp:176-205).
 * SDFC_DERIV_ANALYTIC (default): the interpolant's analytic cell derivatives
 *   wherever that stencil stays inside one cell (equal to the differences up
 *   to their FP64 round-off, which the 1/eps^2 of the Hessian amplifies), and
 *   the reference's stencil elsewhere.
 * SDFC_DERIV_STENCIL: the reference's 26-query stencil for every contact, in
 *   the reference's operation order (bit-identical gradient and Hessian). */
#define SDFC_DERIV_ANALYTIC 0
#define SDFC_DERIV_STENCIL 1

/* Arithmetic of the per-contact force and Jacobian terms.  In both the
 * grid-frame point and the penetration depth are FP64 (bit-identical to the
 * reference's BodySDFObj::distance) and all sums over contacts are FP64.
 * SDFC_PRECISION_FP64 (default): every per-contact term in FP64.
 * SDFC_PRECISION_MIXED: the normal, tangential velocity, SDF derivatives and
 *   the 24 Jacobian columns in FP32 (warp partial sums of 32 contacts in FP32),
 *   for throughput; its error against the FP64 path is stated in the tests. */
#define SDFC_PRECISION_FP64 0
#define SDFC_PRECISION_MIXED 1

typedef struct sdfc_context sdfc_context;
typedef struct sdfc_batch sdfc_batch;
typedef struct sdfc_sim sdfc_sim;

/* Contact coefficients of one pair: ForceGeneralSDFContact::_kn, _kt, _mu,
 * _damping, _scale (ForceGeneralSDFContact.h:16-20) and the contact body's
 * Body::_contact_scale.  kn and kt are used scaled by scale*contact_scale
 * (ForceGeneralSDFContact.cpp:155-156). */
typedef struct {
    double kn, kt, mu, damping, scale, contact_scale;
} sdfc_params;

/* ---------------------------------------------------------------- context */

/* Creates a context on CUDA device `device`.  Replaces nothing in the
 * reference (it has no device state); owns all device buffers. */
int sdfc_create(sdfc_context** ctx, int device);
void sdfc_destroy(sdfc_context* ctx);
/* Message of the last failing call on this context (never NULL). */
const char* sdfc_last_error(const sdfc_context* ctx);
/* Derivative mode and precision of sdfc_evaluate and of batches created afterwards. */
int sdfc_set_derivative_mode(sdfc_context* ctx, int mode);
int sdfc_set_precision(sdfc_context* ctx, int precision);

/* Uploads an SDF body's grid (BodySDFObj::_SDF and its box/spacing/threshold,
 * BodySDFObj.h:13-16; filled by BodySDFObj::precompute_SDF / load_SDF,
 * BodySDFObj.cpp:38-116).  `values` holds ni*nj*nk doubles, i fastest.
 * storage = SDFC_STORAGE_F32 keeps FP32 values (exact for grids made by sdfgen,
 * which computes in FP32); SDFC_STORAGE_F64 keeps FP64 values;
 * SDFC_STORAGE_F16_BRICKS keeps FP16 bricks, and every evaluation then uses the decoded
 * values (sdfc_grid_values) as the grid.  Rejects
 * grids on which the reference's cell index could leave the array
 * ((max_box - min_box)/dx >= n on some axis), non-finite values, n < 2.
 * Writes a handle to *grid. */
int sdfc_upload_grid(sdfc_context* ctx, const double* values, int ni, int nj, int nk, const double min_box[3],
                     const double max_box[3], const double dxyz[3], double col_th, int storage, int* grid);

/* sdfc_upload_grid for node values already on the device: d_values holds ni*nj*nk FP32 values
 * (i fastest) in device memory of the context's device, e.g. a grid generated on the GPU.  storage
 * is SDFC_STORAGE_F32 or SDFC_STORAGE_F32_NODES.  The values are copied (the caller keeps its
 * array); the grid's bounds and cell-corner array are computed on the device.  The call reads
 * the values on the context's own stream, which does not wait for work on other streams: the
 * values must be complete when it is made.  It returns once the grid is ready.  Non-finite
 * values are rejected as by sdfc_upload_grid.  Same counterpart in the reference (BodySDFObj::_SDF). */
int sdfc_upload_grid_device(sdfc_context* ctx, const float* d_values, int ni, int nj, int nk,
                            const double min_box[3], const double max_box[3], const double dxyz[3], double col_th,
                            int storage, int* grid);

/* The grid as the evaluations see it (host, ni*nj*nk doubles, i fastest): the FP64
 * values, the FP32 values widened, or the decoded FP16 bricks. */
int sdfc_grid_values(sdfc_context* ctx, int grid, double* values);

/* Host-only FP16 brick codec of SDFC_STORAGE_F16_BRICKS (no device needed).  Bricks are
 * nb = ceil(n/8) per axis, brick b = bx + nbx*(by + nby*bz); node (i, j, k) is code
 * b*512 + (i&7) + 8*(j&7) + 64*(k&7) of brick (i>>3, j>>3, k>>3); nodes past the grid's
 * end repeat its last node.  so[2b], so[2b+1] = scale, offset.  Encoding: offset 0 if the
 * brick's values straddle 0, else the value nearest 0; scale = max|v - offset| / 32768;
 * code = FP16(FP32((v - offset) / scale)).  Decoding: value = fmaf(scale, code, offset), an
 * FP32 fused multiply-add (the FP32 paths use it as is, the FP64 paths widened).
 * codes holds nbx*nby*nbz*512 FP16 bit patterns, so 2*nbx*nby*nbz floats. */
int sdfc_f16_brick_encode(const double* values, int ni, int nj, int nk, unsigned short* codes, float* so);
int sdfc_f16_brick_decode(const unsigned short* codes, const float* so, int ni, int nj, int nk, double* values);

/* Uploads a contact body's contact points (Body::_contact_points, body frame;
 * BodyMeshObj::precompute_contact_points, simulation/redmax/Body/BodyMeshObj.cpp:184-238).
 * `xyz` holds n points as x,y,z doubles.  SDFC_STORAGE_F32 stores them as
 * FP32 (exact when they are FP32-representable).  Writes a handle to *points. */
int sdfc_upload_points(sdfc_context* ctx, const double* xyz, int n, int storage, int* points);

/* ---------------------------------------------------------------- one pair */

/* One Force call of one ForceGeneralSDFContact(contact body A, SDF body B):
 * detection (CollisionDetection.cpp:124-147) then the contact sums
 * (ForceGeneralSDFContact.cpp:147-219 for want_deriv == 0, :221-447 with
 * want_deriv != 0).  Host arrays: E_A, E_B [16]; phi_A, phi_B [6]; fm [12];
 * Km, Dm [144] (only written when want_deriv; may be NULL otherwise).
 * *n_active receives the size of the active contact set. */
int sdfc_evaluate(sdfc_context* ctx, int points, int grid, const double* E_A, const double* phi_A, const double* E_B,
                  const double* phi_B, const sdfc_params* params, int want_deriv, double* fm, double* Km, double* Dm,
                  int* n_active);

/* Active contact ids (indices into the contact body's points, ascending, as
 * collision_detection_general_SDF lists them) of the last sdfc_evaluate on
 * this context.  Writes min(cap, n) ids and *n = n. */
int sdfc_active_ids(sdfc_context* ctx, int* ids, int cap, int* n);

/* ---------------------------------------------------------------- batches */

/* A batch of n pair instances with fixed topology: instance k pits point set
 * points[k] against grid grids[k].  This is the planner's inner loop
 * (examples/run_joint_plan.py:511-589: many candidate pull directions and
 * assemblies) folded into one launch per evaluation; the reference runs these
 * as separate processes (utils/parallel.py:10). */
int sdfc_batch_create(sdfc_context* ctx, int n, const int* points, const int* grids, sdfc_batch** batch);
void sdfc_batch_destroy(sdfc_batch* batch);
/* Derivative mode (SDFC_DERIV_*) and precision (SDFC_PRECISION_*) of this batch. */
int sdfc_batch_set_derivative_mode(sdfc_batch* batch, int mode);
int sdfc_batch_set_precision(sdfc_batch* batch, int precision);

/* Evaluates every instance.  Arrays are per instance, row-major, HOST memory:
 * E_A, E_B [n*16]; phi_A, phi_B [n*6]; params [n]; fm [n*12]; Km, Dm [n*144]
 * (want_deriv only); n_active [n]; status [n] (bit 0: a non-finite output; bit 1: a
 * non-finite pose, twist or coefficient, whose instance then finds no contact, as the
 * reference's distance query puts non-finite points outside the grid; n_active and status may
 * be null).  Host<->device transfers are part of the
 * call, which returns when the results are in the caller's arrays.  Where the
 * device reads pageable host memory through the host's page tables (Grace's
 * C2C link) the kernels read the input arrays and write the result arrays
 * themselves; elsewhere (or with SDFC_STAGED_COPIES set in the environment when
 * the context is created) they are staged through pinned buffers. */
int sdfc_batch_evaluate(sdfc_batch* batch, const double* E_A, const double* phi_A, const double* E_B,
                        const double* phi_B, const sdfc_params* params, int want_deriv, double* fm, double* Km,
                        double* Dm, int* n_active, int* status);

/* Same with DEVICE arrays, enqueued on `stream` (a cudaStream_t; NULL is the
 * legacy default stream) without synchronising; capturable in a CUDA graph.
 * params is an n x 6 device array (kn, kt, mu, damping, scale, contact_scale). */
int sdfc_batch_evaluate_device(sdfc_batch* batch, const double* E_A, const double* phi_A, const double* E_B,
                               const double* phi_B, const double* params, int want_deriv, double* fm, double* Km,
                               double* Dm, int* n_active, int* status, void* stream);

/* Penetration energy of every instance: energy[i] = sum over its active contacts of
 * kn d^2 / 2 (d = SDF + col_th < 0 the contact's depth, kn scaled by scale * contact_scale as
 * in the force law) and dE[12 i ..] its gradient wrt the twist coordinates of body A then B
 * (w then v, body frames, like the rows of fm): kn d dd/dq.  No counterpart in the reference,
 * which has no energy; it serves losses on penetration (the rollout adjoint).  Host arrays
 * (E_A, E_B [n*16], params [n], energy [n], dE [n*12]); velocities play no part. */
int sdfc_batch_energy(sdfc_batch* batch, const double* E_A, const double* E_B, const sdfc_params* params,
                      double* energy, double* dE);
/* Same with DEVICE arrays (phi_A, phi_B [n*6] are read but do not change the result; params
 * n x 6) on `stream`. */
int sdfc_batch_energy_device(sdfc_batch* batch, const double* E_A, const double* phi_A, const double* E_B,
                             const double* phi_B, const double* params, double* energy, double* dE, void* stream);

/* sdfc_batch_evaluate_device with a per-instance request (DEVICE int[n]): 0 skips the
 * instance (its outputs are left as they are), 1 evaluates fm only
 * (ForceGeneralSDFContact::computeForce), 2 fm, Km and Dm (computeForceWithDerivative).
 * One launch set serves a batch whose instances need different things, e.g. the
 * Newton and line-search points of batched implicit steps.  Km and Dm must be given. */
int sdfc_batch_evaluate_masked_device(sdfc_batch* batch, const double* E_A, const double* phi_A, const double* E_B,
                                      const double* phi_B, const double* params, const int* request, double* fm,
                                      double* Km, double* Dm, int* n_active, int* status, void* stream);

/* Per-phase device time of the last evaluation of this batch, the GPU
 * counterpart of ForceGeneralSDFContact's "collision detection" and "compute
 * force" timers (Force::Timer, simulation/redmax/Force/Force.h:15-36;
 * ForceGeneralSDFContact.cpp:65-66).  Enable with sdfc_batch_set_timing(b, 1)
 * (CUDA events are then recorded between the launches); ms[0] = detection,
 * ms[1] = contact forces, ms[2] = reduction.  Synchronises on the events. */
int sdfc_batch_set_timing(sdfc_batch* batch, int enable);
int sdfc_batch_last_timing(sdfc_batch* batch, float* ms);

/* ---------------------------------------------------------------- launch tuning */

/* How a batch's force pass is launched.  No counterpart in the reference (its only
 * parallelism knob is the process count of utils/parallel.py:10).  Each instance's active
 * contacts (counted on the device by detection) are cut into chunks (128 contacts for
 * SDFC_FORCE_CTAS, 32 for SDFC_FORCE_WORKERS) and the chunks into S interleaved shares,
 * S = min(slots, ceil(chunks / chunks_per_slot)) (none without contacts): each share is summed
 * on its own and the shares in order at the end, so an instance with many contacts is spread
 * over many CTAs and one with few over one.
 *   slots            partial sums per instance, at most (1..128, a power of two; by default 128,
 *                    halved while instances x slots exceeds 2^18 partial rows);
 *   force_variant    SDFC_FORCE_CTAS: persistent CTAs of 128 threads, as many as the
 *                    multiprocessors hold, taking (instance, share) items from a queue;
 *                    SDFC_FORCE_WORKERS: persistent one-warp CTAs taking the same items;
 *                    SDFC_FORCE_GRID: one CTA of 128 threads per (instance, share) for every
 *                    share up to `slots` (those past an instance's S return at once);
 *   worker_ctas      one-warp CTAs launched by SDFC_FORCE_WORKERS (0: multiprocessors x resident);
 *   chunks_per_slot  chunks per share, at least (>= 1);
 *   ms               measured time of one evaluation with this configuration (0 if not measured).
 * Every configuration sums each share in a fixed order, so results are reproducible run to run
 * for a given configuration; different configurations group the sums differently and may
 * differ in the last bits. */
#define SDFC_FORCE_CTAS 0
#define SDFC_FORCE_WORKERS 1
#define SDFC_FORCE_GRID 2
typedef struct {
    int slots, force_variant, worker_ctas, chunks_per_slot;
    float ms;
} sdfc_tuning;

/* Times the candidate configurations (the queue forms x chunks_per_slot 1-32 with slots at the
 * batch's cap, the grid form x slots 1-16) on one evaluation of these DEVICE
 * inputs (as sdfc_batch_evaluate_device; want_deriv as there), keeps the fastest for the batch
 * and for later batches of the same shape in this context (instances, tiles, points, grid
 * storages, precision, derivative mode), and writes it to *chosen (may be NULL).  A batch whose
 * shape was tuned before takes that tuning without timing.  The outputs are overwritten.  Not
 * during a stream capture (it synchronises and may reallocate the batch's scratch). */
int sdfc_batch_autotune(sdfc_batch* batch, const double* E_A, const double* phi_A, const double* E_B,
                        const double* phi_B, const double* params, int want_deriv, double* fm, double* Km,
                        double* Dm, int* n_active, int* status, void* stream, sdfc_tuning* chosen);
/* The batch's launch configuration (set by sdfc_batch_autotune, or the default one). */
int sdfc_batch_get_tuning(sdfc_batch* batch, sdfc_tuning* tuning);
int sdfc_batch_set_tuning(sdfc_batch* batch, const sdfc_tuning* tuning);

/* Number of points the last evaluations of this batch re-checked in FP64
 * because their FP32 distance fell inside the guard band (diagnostic; the
 * counter accumulates until reset with reset != 0). */
int sdfc_batch_recheck_count(sdfc_batch* batch, unsigned long long* count, int reset);

/* ---------------------------------------------------------------- batched implicit-Euler steps */

/* A batch of planner scenes stepped together: in each scene one part moves on
 * a joint attached to the world and every other part is fixed, exactly the
 * scene of the planner (examples/run_joint_plan.py:140-178, 218).  Each step
 * is redmax's BDF1 step (Simulation::integration_BDF1 and Simulation::newton,
 * simulation/redmax/Simulation.cpp:999-1079, 1248-1270) with its reduced
 * system (Simulation::computeMatrices, :379-503): tolerance 1e-8 on |g|, at
 * most max(20 ndof, 100) Newton iterations, backtracking line search halving
 * the step up to 20 times, 3 consecutive line-search failures stop.  Every
 * force evaluation of every scene of one Newton round runs as one batched
 * evaluation on the GPU; the reduced systems and their solves run in FP64 on the GPU.
 * All movers of one sim share one joint type; q, qdot arrays are n x ndof. */
#define SDFC_JOINT_TRANSLATIONAL 3 /* JointTranslational: q = position (3 dof) */
#define SDFC_JOINT_FREE3D_EXP 6    /* JointFree3DExp: q = (position, exponential rotation
                                      coordinates) (6 dof); rotation vectors longer than 1.5 pi
                                      are reparameterised after each step like the reference */

/* The moving part: Body::_mass, Body::_Inertia (Ixx, Iyy, Izz, m, m, m),
 * Joint::_E_pj_0 (row-major 4x4), Body::_E_ji, the options gravity and
 * timestep (the reference reads timestep as FP32), Joint::_Kr / _Dr. */
typedef struct {
    int joint;
    double mass, inertia[6], E_pj0[16], E_ji[16];
    double gravity[3], h;
    double joint_stiffness, joint_damping;
} sdfc_mover;

/* One ForceGeneralSDFContact of scene `instance`: the mover against one fixed
 * part.  mover_is_contact = 1: the mover's points (handle `points`) against the
 * fixed part's grid (`grid`); 0: the fixed part's points against the mover's
 * grid.  E_fixed is the fixed part's pose. */
typedef struct {
    int instance, points, grid, mover_is_contact;
    double E_fixed[16];
    sdfc_params params;
} sdfc_scene_pair;

int sdfc_sim_create(sdfc_context* ctx, int n, const sdfc_mover* movers, int n_pairs, const sdfc_scene_pair* pairs,
                    sdfc_sim** sim);
void sdfc_sim_destroy(sdfc_sim* sim);
/* Precision of the force evaluations (SDFC_PRECISION_*); the solves are FP64. */
int sdfc_sim_set_precision(sdfc_sim* sim, int precision);
/* Joint state of every scene (host, n x ndof): Simulation::set_state / get_q / get_qdot. */
int sdfc_sim_set_state(sdfc_sim* sim, const double* q, const double* qdot);
int sdfc_sim_get_state(sdfc_sim* sim, double* q, double* qdot);
/* External force on each mover (host, n x 6, world frame, torque then force):
 * Simulation::set_body_external_force (Body::_f_external; the reference scales
 * it by the inertia diagonal, Body.cpp:267-268). */
int sdfc_sim_set_external_force(sdfc_sim* sim, const double* f);
/* num_steps BDF1 steps of every scene (Simulation::forward, :914-990).  Within one call each
 * scene takes its steps one after another without waiting for the other scenes (a scene whose
 * step has converged starts its next step in the next round), so the call's rounds follow the
 * scene with the most evaluations rather than each step's slowest scene; the trajectories are
 * those of steps taken one call at a time.
 * converged (host, n, may be NULL): 1 where the last step's Newton converged
 * (Simulation::is_converged). */
int sdfc_sim_step(sdfc_sim* sim, int num_steps, int* converged);
/* Totals since creation: Newton rounds (batched force evaluations) and scene
 * force evaluations (diagnostic). */
int sdfc_sim_stats(sdfc_sim* sim, long long* rounds, long long* evaluations);
/* sdfc_batch_autotune for the sim's batch of contact pairs, on the evaluation that opens the
 * next step at the current state (every scene's pairs with derivatives).  Call between steps;
 * the sim's captured rounds are rebuilt with the chosen configuration. */
int sdfc_sim_autotune(sdfc_sim* sim, sdfc_tuning* chosen);
/* The sim's launch configuration: read, or set directly (as sdfc_batch_set_tuning). */
int sdfc_sim_get_tuning(sdfc_sim* sim, sdfc_tuning* tuning);
int sdfc_sim_set_tuning(sdfc_sim* sim, const sdfc_tuning* tuning);
/* Force evaluations of each scene since creation (host, n): a scene's evaluation evaluates
 * every contact pair of the scene once (diagnostic, e.g. contact points per second of scenes
 * with uneven point counts). */
int sdfc_sim_scene_evaluations(sdfc_sim* sim, long long* evaluations);

/* Adjoint of the rollout (Simulation::reset(backward_flag = true) + Simulation::backward,
 * simulation/redmax/Simulation.cpp:1512-1634, integrator BDF1).
 * sdfc_sim_record starts recording at the current state (q_0, qdot_0) for at most
 * max_steps steps (sdfc_sim_step fails with SDFC_ERR_CAPACITY beyond it; 0 stops
 * recording).  Only the joint trajectory is kept (n x ndof doubles per step) where the
 * reference stores H_lu, M, D per step (BackwardData.h); the backward pass recomputes
 * each step's H and D from it.  sdfc_sim_set_state restarts the recording.  Like the
 * reference, the adjoint does not differentiate the free joint's reparameterisation. */
int sdfc_sim_record(sdfc_sim* sim, int max_steps);
/* Recorded steps T and, if q_his is not NULL, the trajectory (host, n x (T+1) x ndof,
 * q_0 first): Simulation::get_q_his. */
int sdfc_sim_history(sdfc_sim* sim, int* steps, double* q_his);
/* Simulation::backward_BDF1 for every scene over the T recorded steps.
 * df_dq (host, n x T x ndof): dL/dq_k for k = 1..T (BackwardInfo::_df_dq).
 * Outputs (host, may be NULL): df_dq0 (n x ndof) and df_dqdot0 (n x ndof), the reference's
 * BackwardResults::_df_dq0/_df_dqdot0 with zero direct terms, and df_dfext (n x 6,
 * world frame, torque then force like sdfc_sim_set_external_force), which the
 * reference does not compute: dL/d(external force), the force held constant over the
 * T steps. */
int sdfc_sim_backward(sdfc_sim* sim, const double* df_dq, double* df_dq0, double* df_dqdot0, double* df_dfext);

/* Penetration energy of the rollout (no counterpart in the reference).  With energy recording
 * on (call before sdfc_sim_record; switching it stops a recording), every recorded step also
 * has the penetration energy E_t of each scene at the step's end state (the sum over the
 * scene's pairs of sdfc_batch_energy, evaluated from the recorded trajectory when the
 * sdfc_sim_step call's rounds are done) and its gradient wrt the joint coordinates.
 * sdfc_sim_energy: per_step (host, n x T, may be NULL) and total (host, n, may be NULL) = sum_t E_t.
 * sdfc_sim_backward_energy: sdfc_sim_backward for L(q_1..q_T, sum_t E_t) given also
 * df_dE (host, n) = dL/d(sum_t E_t) per scene (NULL: 0). */
int sdfc_sim_record_energy(sdfc_sim* sim, int on);
int sdfc_sim_energy(sdfc_sim* sim, double* per_step, double* total);
int sdfc_sim_backward_energy(sdfc_sim* sim, const double* df_dq, const double* df_dE, double* df_dq0,
                             double* df_dqdot0, double* df_dfext);
/* Newton tolerance on |g| of every scene (the reference's 1e-8, Simulation.cpp:1008, by default).
 * A tighter tolerance lets finite differences of a rollout resolve its adjoint. */
int sdfc_sim_set_tolerance(sdfc_sim* sim, double tol);

/* ---------------------------------------------------------------- allocation-free evaluation */

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory when they need a contact force: inside a real-time or hard-latency
 * loop (cudaMalloc may synchronise the device), under a host application
 * that owns all device memory through its own pool, or while recording into a
 * CUDA stream capture.  One Force call of one (contact body A, SDF body B)
 * pair like sdfc_evaluate with want_deriv (FP64 arithmetic, analytic cell
 * derivatives), needing no context: every argument marked "device" is
 * caller-owned device memory on the current device; min_box, max_box and dxyz
 * are host arrays.  Grid: ni*nj*nk FP64 values, i fastest; points: n points as
 * x,y,z doubles; E_A, E_B [16], phi_A, phi_B [6], params [6] (kn, kt, mu,
 * damping, scale, contact_scale); outputs fm [12], Km, Dm [144] (want_deriv
 * only), n_active [1].  Enqueued on `stream` (a cudaStream_t; NULL is the
 * legacy default stream) without synchronising.
 *
 * Its working memory is a file-scope device array of about 2.6 MB that every
 * GPU loading the library holds until exit; n may not exceed
 * SDFC_NOALLOC_MAX_POINTS (larger n returns SDFC_ERR_CAPACITY, negative n
 * SDFC_ERR_INVALID_ARGUMENT).  A CUDA error already pending on the calling
 * thread when the call starts is left there and the call returns
 * SDFC_ERR_CUDA without launching anything.  The first
 * call on a device looks up that array's device address; make that first call
 * before any stream capture begins.  All calls share the array: calls whose
 * work may overlap on the GPU (other streams, other host threads) race and
 * must be serialised by the caller.  Nothing carries over between calls. */
#define SDFC_NOALLOC_MAX_POINTS 131072
int sdfc_evaluate_noalloc(const double* grid_values, int ni, int nj, int nk, const double* min_box,
                          const double* max_box, const double* dxyz, double col_th, const double* points, int n,
                          const double* E_A, const double* phi_A, const double* E_B, const double* phi_B,
                          const double* params, int want_deriv, double* fm, double* Km, double* Dm, int* n_active,
                          void* stream);

/* ---------------------------------------------------------------- distances */

/* Per instance of the batch, the reference's distance of each of body A's points (the
 * instance's point set, body frame, posed by E_A as Simulation::get_body_vertices poses mesh
 * vertices, rm/Simulation.cpp:252-264) to body B's grid (posed by E_B), BodySDFObj::distance
 * (rm/Body/BodySDFObj.cpp:207-213): the trilinear value at the point in B's frame plus B's
 * col_th, FLT_MAX + col_th outside B's box; FP64, bit-identical.
 * min_d (n doubles): each instance's minimum, +inf for an empty point set.  With A's mesh
 * vertices as the point set this is Simulation::get_body_distance (rm/Simulation.cpp:276-296);
 * two calls make body_in_contact (:298-303).  SDFMesh::distance / min_distance (rm/Mesh.cpp:
 * 18-20, 143-198) are the case of identity poses and a grid uploaded with col_th = 0.
 * d (may be NULL): every point's distance, instance after instance, each instance's points in
 * the caller's order.  E_A, E_B: n row-major 4x4 poses each. */
int sdfc_batch_distance(sdfc_batch* b, const double* E_A, const double* E_B, double* min_d, double* d);
/* The same on device arrays, queued on `stream` (null: the context's stream). */
int sdfc_batch_distance_device(sdfc_batch* b, const double* d_EA, const double* d_EB, double* d_min, double* d_d,
                               void* stream);

/* SDFMesh::distance (rm/Mesh.cpp:190-198) and min_distance (:18-20) on an uploaded grid: the
 * trilinear value of SDFMesh::query_SDF (:143-188; FLT_MAX outside the box) at each of the n
 * points X (n x 3 doubles, grid frame), FP64, bit-identical; the grid's col_th is not added.
 * d (may be NULL): n values; min_d (may be NULL): their minimum (+inf for n = 0). */
int sdfc_grid_distance(sdfc_context* ctx, int grid, const double* X, int n, double* d, double* min_d);

/* ---------------------------------------------------------------- disassembly check */

/* A convex hull for the planner's disassembly check: its vertices (nv x 3 doubles, the
 * part's frame) and facet planes (nf x 4: unit normal n and offset o, n . x + o <= 0 inside,
 * as qhull reports them; trimesh.convex.convex_hull in the reference).  Writes a handle. */
int sdfc_upload_hull(sdfc_context* ctx, const double* verts, int nv, const double* planes, int nf, int* hull);
/* PhysicsPlanner.is_disassembled (examples/run_joint_plan.py:291-302) for n poses E (n x 16,
 * row-major E_0i) of the moving part: out[q] = 1 when the moving hull, posed, and the still hull
 * (world frame) have no surface point in common (the reference's FCL mesh-mesh collision of
 * the two hulls; for convex hulls: the solids meet and neither lies inside the other) and
 * neither hull's axis-aligned box contains the other's.  FP64 GJK per pose; flags (may be
 * NULL): bit 0 solids meet, bit 1 moving hull inside the still hull, bit 2 the reverse, bit 3
 * box containment, bits 8.. GJK iterations. */
int sdfc_disassembled(sdfc_context* ctx, int hull_move, int hull_still, const double* E, int n, int* out, int* flags);
/* The same on device arrays, queued on `stream` (null: the context's stream). */
int sdfc_disassembled_device(sdfc_context* ctx, int hull_move, int hull_still, const double* d_E, int n, int* d_out,
                             int* d_flags, void* stream);

/* ---------------------------------------------------------------- grid files */

/* The reference's .sdf text cache (BodySDFObj::save_SDF / load_SDF, rm/Body/BodySDFObj.cpp:
 * 86-116; SDFMesh::save_SDF / load_SDF, rm/Mesh.cpp:103-135): the same text, byte for byte
 * (std::ostream's default 6-significant-digit doubles, so the cache is lossy), and the same
 * values on reading.  Host only.  load: with values NULL only the header (shape, boxes,
 * spacing); else also capacity >= ni*nj*nk values.  SDFC_ERR_NOT_FOUND when the file does not
 * open (the reference then builds the grid), SDFC_ERR_INVALID_ARGUMENT when it is malformed. */
int sdfc_sdf_save_text(const char* path, const double* values, int ni, int nj, int nk, const double min_box[3],
                       const double max_box[3], const double dxyz[3]);
int sdfc_sdf_load_text(const char* path, int shape[3], double min_box[3], double max_box[3], double dxyz[3],
                       double* values, long long capacity);
/* A binary cache of FP16-brick grids (no reference counterpart; for SDFC_STORAGE_F16_BRICKS):
 * save encodes the FP64 values with sdfc_f16_brick_encode; load returns the header and, if
 * codes and so are not NULL, the codes and per-brick (scale, offset) exactly as saved (sized as
 * for sdfc_f16_brick_encode), which sdfc_upload_grid_bricks uploads without re-encoding. */
int sdfc_sdf_save_bricks(const char* path, const double* values, int ni, int nj, int nk, const double min_box[3],
                         const double max_box[3], const double dxyz[3]);
int sdfc_sdf_load_bricks(const char* path, int shape[3], double min_box[3], double max_box[3], double dxyz[3],
                         unsigned short* codes, float* so);
/* sdfc_upload_grid with SDFC_STORAGE_F16_BRICKS from already encoded bricks. */
int sdfc_upload_grid_bricks(sdfc_context* ctx, const unsigned short* codes, const float* so, int ni, int nj, int nk,
                            const double min_box[3], const double max_box[3], const double dxyz[3], double col_th,
                            int* grid);

/* ---------------------------------------------------------------- SDF grids from meshes */

/* sdfgen::make_level_set3 (simulation/externals/sdfgen/makelevelset3.h:14-16,
 * makelevelset3.cpp:161-227) on the GPU: the signed distance phi of the closed triangle
 * mesh (verts: nv x 3 floats; tris: nt x 3 vertex indices) at the nodes origin + (i dx,
 * j dy, k dz), phi[i + ni*(j + nj*k)], exact distances within exact_band cells of the
 * mesh, fast sweeping elsewhere, negative inside (crossing parity along +i).
 * Bit-identical to the reference's FP32 result.  Host arrays in and out. */
int sdfc_make_level_set3(sdfc_context* ctx, const float* verts, int nv, const unsigned* tris, int nt,
                         const float origin[3], float dx, float dy, float dz, int ni, int nj, int nk, int exact_band,
                         float* phi);
/* The same from device arrays (d_tris entries must be < nv: not checked here), on
 * `stream` (null: the context's stream); returns after the work is queued. */
int sdfc_make_level_set3_device(sdfc_context* ctx, const float* d_verts, int nv, const unsigned* d_tris, int nt,
                                const float origin[3], float dx, float dy, float dz, int ni, int nj, int nk,
                                int exact_band, float* d_phi, void* stream);
/* The grid of BodySDFObj::precompute_SDF (simulation/redmax/Body/BodySDFObj.cpp:38-70) for the
 * body-frame mesh vertices V (nv x 3 doubles, the body's _V) with the body's dx and res:
 * node counts shape = (ni, nj, nk), _min_box, _max_box, the spacing (_dx, _dy, _dz), and
 * (if origin_f is not null) the FP32 origin and spacing handed to make_level_set3 are
 * origin_f and (float)spacing.  Host-only arithmetic in the reference's order. */
int sdfc_sdf_grid_layout(const double* V, int nv, double dx, int res, int shape[3], double min_box[3],
                         double max_box[3], double spacing[3], float origin_f[3]);

#ifdef __cplusplus
}
#endif
#endif /* SDFC_H */
