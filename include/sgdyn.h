/* sgdyn: batched articulated-body kinematics and dynamics on GB300 (sm_103a), C ABI.
 *
 * Drop-in boundary for SAPIEN's PinocchioModel path. Every batched entry point below is
 * the GPU counterpart of one method of the reference C++ class sapien::PinocchioModel
 * (pinocchio/pinocchio_model.h:27-130, pinocchio/pinocchio_model.cpp) and its pybind
 * binding (pinocchio/pinocchio_model.cpp:306-367). The citation beside each function
 * names the method it replaces.
 *
 * Conventions
 *  - All compute functions take DEVICE pointers (or managed memory) to FP64 arrays and
 *    enqueue work on `stream` (a cudaStream_t; NULL = legacy default stream). They return
 *    after the launch; results are ready when the stream reaches that point. Pinned host
 *    memory that is mapped at the same address on the device (cudaHostAlloc, or
 *    cudaHostRegister with mapping, under unified addressing) is accepted as well: the
 *    kernels then read inputs from and write results to host memory directly over the
 *    host link, with no staging copy (SGDYN_COL_MAJOR keeps those accesses coalesced).
 *    Pageable host memory is rejected with SGDYN_ERR_NULL.
 *  - Arrays are batched over n environments. layout SGDYN_ENV_MAJOR: [n][cols] row-major
 *    (a torch tensor of shape [n, cols]); SGDYN_COL_MAJOR: [cols][n] (structure of arrays).
 *  - q is in external (SAPIEN) joint order, one coordinate per revolute / continuous /
 *    prismatic joint (continuous joints take their angle, exactly like posS2P,
 *    pinocchio_model.cpp:49-72) and 7 per free-flyer joint (x y z qx qy qz qw; an
 *    extension: the reference's posS2P rejects nq > 2). Velocities, accelerations and
 *    torques have nv columns in external order.
 *  - Every function returns SGDYN_OK (0) or a negative status; sgdyn_last_error()
 *    returns a message for the calling thread's last failure.
 *  - A model is immutable while launches that use it are in flight. The first launch on
 *    a device uploads the model tables with cudaMalloc/cudaMemcpy; call
 *    sgdyn_model_upload() first when launches will be captured into a CUDA graph.
 */
#ifndef SGDYN_H
#define SGDYN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGDYN_OK 0
#define SGDYN_ERR_INVALID_ARGUMENT (-1) /* bad joint/link name: reference std::invalid_argument */
#define SGDYN_ERR_RUNTIME (-2)          /* reference std::runtime_error: bad index, bad sizes, unsupported joint */
#define SGDYN_ERR_CUDA (-3)             /* CUDA launch or memory error */
#define SGDYN_ERR_UNSUPPORTED (-4)      /* model outside the kernels' limits (joints, free flyers) */
#define SGDYN_ERR_NULL (-5)             /* null or non-device pointer */

#define SGDYN_ENV_MAJOR 0
#define SGDYN_COL_MAJOR 1

/* op bits for sgdyn_step */
#define SGDYN_OP_FK 1
#define SGDYN_OP_JACOBIAN 2
#define SGDYN_OP_MASS_MATRIX 4
#define SGDYN_OP_INVERSE_DYNAMICS 8
#define SGDYN_OP_FORWARD_DYNAMICS 16

typedef struct sgdyn_model sgdyn_model;

/* Message for the calling thread's most recent failure ("" if none). */
const char* sgdyn_last_error(void);

/* PinocchioModel::fromURDFXML (pinocchio_model.cpp:39-47): build from URDF text with
 * gravity g (model.gravity = (g, 0)). The default joint order is the tree order and the
 * default link order is the URDF tree order, until set_*_order is called. */
int sgdyn_model_from_urdf(const char* urdf_xml, const double gravity[3], sgdyn_model** out);
void sgdyn_model_free(sgdyn_model* m);

/* Native model source (addition): the articulation SAPIEN's create_pinocchio_model exports
 * (python/py_package/wrapper/pinocchio_model.py:317-326 with urdf_exporter.py:21-152), built
 * without the URDF text. Poses are (x y z qw qx qy qz). Joint types: 0 fixed, 1 revolute
 * (continuous when lower < -1e5 and upper > 1e5), 2 prismatic, 3 free (root only; becomes
 * fixed when force_fix_root). parent = -1 marks the root joint. Link i is named link_i,
 * the joint whose child is link i joint_i; the joint order is set to the non-fixed joints
 * in the given order and the link order to link_0 .. link_{nlinks-1}. */
typedef struct {
  double mass;
  double cmass_pose[7]; /* centre-of-mass frame in the link frame */
  double inertia[3];    /* principal moments in the centre-of-mass frame */
} sgdyn_link_desc;
typedef struct {
  int type;
  int parent;
  int child;
  double pose_in_parent[7];
  double pose_in_child[7];
  double lower, upper;
} sgdyn_joint_desc;
int sgdyn_model_from_articulation(const sgdyn_link_desc* links, int nlinks, const sgdyn_joint_desc* joints,
                                  int njoints, const double gravity[3], int force_fix_root, sgdyn_model** out);

/* PinocchioModel::setJointOrder (pinocchio_model.cpp:99-128). */
int sgdyn_model_set_joint_order(sgdyn_model* m, const char* const* names, int n);
/* PinocchioModel::setLinkOrder (pinocchio_model.cpp:130-140). */
int sgdyn_model_set_link_order(sgdyn_model* m, const char* const* names, int n);

/* Sizes: external q columns, velocity dimension, links in the link order, joints incl. universe. */
int sgdyn_model_info(const sgdyn_model* m, int* nq_ext, int* nv, int* nlinks, int* njoints);
/* PinocchioModel::getRandomConfiguration (pinocchio_model.cpp:142-144), for n rows at once
 * (HOST memory, env-major [n, nq_ext], external joint order): each revolute or prismatic
 * coordinate uniform in its URDF [lower, upper] (0, 0 without a <limit>), each continuous
 * angle uniform in [-pi, pi). Deterministic for a seed on every platform (std::mt19937_64,
 * 53-bit uniforms, joints in tree order within a row). Fails for a model with a free flyer,
 * whose position has no limits. */
int sgdyn_model_random_configuration(const sgdyn_model* m, int64_t n, uint64_t seed, double* qpos);
/* Kind of the k-th joint in external order: 1 revolute, 2 prismatic, 3 continuous, 4 free flyer. */
int sgdyn_model_joint_kind(const sgdyn_model* m, int k, int* kind);
/* Name of the moving joint with tree index j (1..njoints-1) or of BODY frame b. */
int sgdyn_model_joint_name(const sgdyn_model* m, int j, const char** name);
int sgdyn_model_body_count(const sgdyn_model* m, int* nbodies);
int sgdyn_model_body_name(const sgdyn_model* m, int b, const char** name);
/* Upload the model tables to the current device (done lazily by the first launch). */
int sgdyn_model_upload(sgdyn_model* m);
/* Host copy of the packed kernel tables (DModel header, DJoint[njoints], DLink[nlinks],
 * DFrame[njoints]; layout in sapien_gb300/csrc/device_model.h). Joint frames in the table
 * may be rotated so that the joint axis is +z (DFrame holds the rotation back to the
 * model's joint frame). Valid until the model changes. */
int sgdyn_model_table(const sgdyn_model* m, const void** data, int64_t* bytes);

/* PinocchioModel::computeForwardKinematics + getLinkPose for every link
 * (pinocchio_model.cpp:146-161), FP64: link_poses [n][nlinks*7] = (x y z qw qx qy qz)
 * per link, in the articulation base frame. */
int sgdyn_compute_forward_kinematics(const sgdyn_model* m, int64_t n, const double* q, double* link_poses, int layout,
                                     void* stream);

/* PinocchioModel::computeFullJacobian (pinocchio_model.cpp:163-165): the WORLD Jacobian
 * data.J, J [n][6*nv] = rows (vx vy vz wx wy wz) x external columns. */
int sgdyn_compute_full_jacobian(const sgdyn_model* m, int64_t n, const double* q, double* J, int layout,
                                void* stream);

/* PinocchioModel::computeFullJacobian followed by getLinkJacobian(link, local)
 * (pinocchio_model.cpp:167-186): J [n][6*nv]. local != 0 gives the link (body) frame. */
int sgdyn_compute_link_jacobian(const sgdyn_model* m, int64_t n, int link, int local, const double* q, double* J,
                                int layout, void* stream);

/* PinocchioModel::computeSingleLinkLocalJacobian (pinocchio_model.cpp:188-199). */
int sgdyn_compute_single_link_local_jacobian(const sgdyn_model* m, int64_t n, int link, const double* q, double* J,
                                             int layout, void* stream);

/* PinocchioModel::computeGeneralizedMassMatrix (pinocchio_model.cpp:201-206): M [n][nv*nv], symmetric. */
int sgdyn_compute_generalized_mass_matrix(const sgdyn_model* m, int64_t n, const double* q, double* M, int layout,
                                          void* stream);

/* PinocchioModel::computeCoriolisMatrix (pinocchio_model.cpp:208-212): C [n][nv*nv]. */
int sgdyn_compute_coriolis_matrix(const sgdyn_model* m, int64_t n, const double* q, const double* qd, double* C,
                                  int layout, void* stream);

/* PinocchioModel::computeInverseDynamics (RNEA, pinocchio_model.cpp:214-219): tau [n][nv]. */
int sgdyn_compute_inverse_dynamics(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                   const double* qdd, double* tau, int layout, void* stream);

/* PinocchioModel::computeForwardDynamics (ABA, pinocchio_model.cpp:221-226): qdd [n][nv]. */
int sgdyn_compute_forward_dynamics(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                   const double* tau, double* qdd, int layout, void* stream);

/* PhysxArticulation::computePassiveForce (src/physx/articulation.cpp:400-418) on SAPIEN's
 * batched GPU state buffers (src/physx/physx_system.cpp:1074-1081): qpos / qvel float32
 * [n][in_stride] (in_stride = maxDof), result float32 into qf [n][out_stride]. Computed in
 * FP64 as RNEA(q, qd, 0) with the gravity and / or velocity terms selected. */
int sgdyn_compute_passive_force_f32(const sgdyn_model* m, int64_t n, const float* qpos, const float* qvel,
                                    int64_t in_stride, int gravity, int coriolis_and_centrifugal, float* qf,
                                    int64_t out_stride, void* stream);

/* One fused sweep computing any subset (ops = SGDYN_OP_* bits) of the five calls above
 * on the same q / qd: outputs for unrequested ops may be NULL. No reference counterpart
 * as a single call: it replaces a sequence of the reference methods. */
int sgdyn_step(const sgdyn_model* m, int64_t n, int ops, const double* q, const double* qd, const double* qdd,
               const double* tau, double* link_poses, double* J, double* M, double* tau_out, double* qdd_out,
               int layout, void* stream);

/* How sgdyn_step runs a request for all five ops: 0 as one launch (each thread computes
 * all five ops for one environment), 1 as two concurrent launches over the same
 * environments (CRBA + RNEA + ABA on `stream`, FK + Jacobian on an internal second stream of
 * the device, ordered after the work already on `stream` and before what follows there; the
 * FK + Jacobian warps repeat the joint placements but fill FP64 schedulers the others leave
 * idle), 2 automatic (the default: two launches while the batch gives fewer than two warps
 * per FP64 scheduler and `stream` is not being captured), -1 only reads the mode. Results
 * agree to rounding. (Addition.) */
int sgdyn_step_split(int mode, int* mode_out);

/* Lanes per environment for the single-model fused sweep and single-op entry points
 * (addition): 0 = automatic (default), 1, 2, 4 or 8. With L > 1 a team of L lanes shares an
 * environment: the joints near the root run on every lane and the subtrees off them on one
 * lane each, which shortens a wide tree's sequential sweep; worth it when the batch leaves
 * the GPU's FP64 schedulers idle (automatic: only then, and only if the tree splits). */
int sgdyn_model_set_lanes(sgdyn_model* m, int lanes);
/* The team table the kernels use for `lanes` lanes per environment (ints: L, trunk count,
 * longest lane, attach count, trunk joints, per-lane joints padded with 0, attach joints,
 * owner per joint (-1 = trunk)); valid until the next call on this thread. */
int sgdyn_model_team_table(const sgdyn_model* m, int lanes, const int** data, int* count);

/* Run-time specialisation (addition). The fused sweep behind sgdyn_step and the five
 * single-op entry points, the forward rollout kernel and the RNEA / ABA vector-Jacobian
 * product kernels, are compiled per model with NVRTC on
 * first use (tables baked in as constants; same arithmetic) when enabled and n >= min_n;
 * otherwise, or if the run-time compiler or the driver library is unavailable, the generic
 * kernel runs. enable / min_n < 0 leave a setting unchanged; the current values are
 * returned. Defaults: enabled unless SGDYN_JIT=0, min_n = 2048 (SGDYN_JIT_MIN_N), trees of
 * at most 16 joints incl. the universe (SGDYN_JIT_MAX_JOINTS; larger unrolled sweeps ran
 * slower). Compile
 * ahead with sgdyn_jit_prepare (needed before capturing launches into a CUDA graph).
 * `ops`: an SGDYN_OP_* mask for the fused sweep, -1 for the forward rollout kernel, -2 / -3
 * for the RNEA / ABA vector-Jacobian product kernels, -4 / -5 for the forward rollout and the
 * reverse sweep with three lanes per environment, -6 for forward dynamics on three lanes, -7
 * for the CRBA + RNEA + ABA sweep of a model run with teams (sgdyn_model_set_lanes 2, 4 or 8)
 * as one warp per role of the team (the size limit then counts the trunk and the longest
 * role). */
int sgdyn_jit_config(int enable, int64_t min_n, int* enabled, int64_t* min_n_out);
/* Size limit of run-time specialisation (joints incl. the universe; < 0 leaves it). */
int sgdyn_jit_max_joints(int max_joints, int* max_joints_out);
/* How the run-time-specialised sweep computes forward dynamics (addition): 0 automatic (the
 * default: the route with fewer FP64 operations for the model and op set), 1 the
 * articulated-body passes (ABA), 2 from the mass matrix (CRBA, the bias forces by RNEA at
 * zero acceleration, M = L^T D L with the tree's sparsity, qdd = M^-1 (tau - b); inverse
 * dynamics in the same sweep then reads tau = b + M qdd); -1 only reads the setting.
 * Results agree to rounding. The generic kernels always run the articulated-body passes, and
 * the host path (sgdyn_host_*) unless the mode is 2. */
int sgdyn_fd_method(int mode, int* mode_out);
/* Whether the specialised sweep for (model, ops) takes the mass-matrix route (*yes = 1). */
int sgdyn_fd_by_mass_matrix(const sgdyn_model* m, int ops, int* yes);
int sgdyn_jit_prepare(const sgdyn_model* m, int ops);
/* The generated translation unit for (model, ops); valid until the next call on this thread. */
int sgdyn_jit_source(const sgdyn_model* m, int ops, const char** source);

/* PinocchioModel::computeInverseKinematics (CLIK, pinocchio_model.cpp:228-300), one solve per
 * environment. target [n][7] = link pose (x y z qw qx qy qz) in the base frame, FP64.
 * q0 [n][nq_ext] or NULL (neutral start), mask [nv] int (1 active, 0 frozen) or NULL (all
 * active). Outputs: q_out [n][nq_ext] (best iterate), success [n] int, err [n][6] (log6 error
 * of the best iterate, linear then angular). */
int sgdyn_compute_inverse_kinematics(const sgdyn_model* m, int64_t n, int link, const double* target,
                                     const double* q0, const int* mask, double eps, int max_iterations, double dt,
                                     double damp, double* q_out, int* success, double* err, int layout, void* stream);

/* ---- host path for single instances and small batches -------------------------------
 * The same sweeps as the entry points above, compiled for the CPU and run on HOST memory
 * (any host pointers; `layout` as above), environments split over `nthreads` host threads
 * (<= 1: the calling thread). They serve the reference's one-configuration-at-a-time
 * callers, for which a GPU launch plus synchronisation costs more than the sweep itself;
 * batches belong on the device entry points. Results agree with the device kernels to
 * rounding. Each replaces the reference method named beside it:
 *   sgdyn_host_step                          computeForwardKinematics + getLinkPose (:146-161),
 *                                            computeFullJacobian (:163-165),
 *                                            computeGeneralizedMassMatrix (:201-206),
 *                                            computeInverseDynamics (:214-219),
 *                                            computeForwardDynamics (:221-226), as sgdyn_step
 *   sgdyn_host_compute_link_jacobian         getLinkJacobian (:167-186) /
 *                                            computeSingleLinkLocalJacobian (:188-199)
 *   sgdyn_host_compute_coriolis_matrix       computeCoriolisMatrix (:208-212)
 *   sgdyn_host_compute_inverse_kinematics    computeInverseKinematics (:228-300)
 * (pinocchio/pinocchio_model.cpp line numbers). */
int sgdyn_host_step(const sgdyn_model* m, int64_t n, int ops, const double* q, const double* qd, const double* qdd,
                    const double* tau, double* link_poses, double* J, double* M, double* tau_out, double* qdd_out,
                    int layout, int nthreads);
int sgdyn_host_compute_link_jacobian(const sgdyn_model* m, int64_t n, int link, int local, const double* q,
                                     double* J, int layout, int nthreads);
int sgdyn_host_compute_coriolis_matrix(const sgdyn_model* m, int64_t n, const double* q, const double* qd, double* C,
                                       int layout, int nthreads);
int sgdyn_host_compute_inverse_kinematics(const sgdyn_model* m, int64_t n, int link, const double* target,
                                          const double* q0, const int* mask, double eps, int max_iterations,
                                          double dt, double damp, double* q_out, int* success, double* err,
                                          int layout, int nthreads);

/* ---- heterogeneous batches (addition: the reference evaluates one robot per call) ------
 * Robots of different size and topology in one persistent launch. A batch is planned once
 * (tables packed, environments grouped per model into tiles of up to 32, tiles ordered by
 * descending velocity dimension) and stepped many times; a step allocates nothing, so it
 * can be recorded into a CUDA graph. Arrays are row-major and padded to the batch maxima:
 * q [n][max_nq], qd / qdd / tau / tau_out / qdd_out [n][max_nv], M [n][max_nv*max_nv]
 * (environment e's nv x nv matrix packed at the start of its row), J [n][6*max_nv],
 * link_poses [n][max_nlinks*7]. Supported op sets: MASS_MATRIX|INVERSE_DYNAMICS|
 * FORWARD_DYNAMICS, INVERSE_DYNAMICS|FORWARD_DYNAMICS, all five, or one of the three. */
typedef struct sgdyn_batch sgdyn_batch;
/* model_of_env: host array [n] of indices into models[] (models must outlive the batch). */
int sgdyn_batch_create(const sgdyn_model* const* models, int nmodels, const int* model_of_env, int64_t n,
                       sgdyn_batch** out);
void sgdyn_batch_free(sgdyn_batch* b);
int sgdyn_batch_info(const sgdyn_batch* b, int64_t* n, int* max_nq, int* max_nv, int* max_nlinks);
/* Launch shape: persistent CTAs per SM, warps per CTA, tile order (0 = descending DoF, 1 =
 * input order). Chosen by sapien_gb300.autotune. */
int sgdyn_batch_set_launch(sgdyn_batch* b, int ctas_per_sm, int warps_per_cta, int order);
/* Threads per environment, per model (1, 2, 4 or 8; default 1). With L > 1 a team of L
 * lanes shares an environment: the joints near the root (trunk) run on every lane and the
 * subtrees hanging off them on one lane each, so a wide tree's sequential sweep gets
 * shorter at the price of more lanes. Chosen by sapien_gb300.autotune. Re-plans the batch
 * (allocates): not while a stream of the batch's device is being captured. */
int sgdyn_batch_set_lanes(sgdyn_batch* b, const int* lanes_per_model);
int sgdyn_batch_step(sgdyn_batch* b, int ops, const double* q, const double* qd, const double* qdd, const double* tau,
                     double* link_poses, double* J, double* M, double* tau_out, double* qdd_out, void* stream);
/* Semi-implicit Euler on the batch's padded rows, in place: qd += dt qdd, then q advanced
 * by dt qd with each environment's model (angles and slides add; a free flyer moves on
 * SE(3) by its body twist, like Pinocchio's integrate). With sgdyn_batch_step (ABA) this
 * makes one rollout step; both launches can be captured into one CUDA graph. */
int sgdyn_batch_integrate(sgdyn_batch* b, double dt, double* q, double* qd, const double* qdd, void* stream);
/* One rollout step in one launch: qdd_out = ABA(q, qd, tau), then the semi-implicit Euler
 * update of sgdyn_batch_integrate, each environment right after its own sweep, in place
 * on q / qd. Results equal sgdyn_batch_step (SGDYN_OP_ABA) followed by
 * sgdyn_batch_integrate, bit for bit. */
int sgdyn_batch_step_integrate(sgdyn_batch* b, double dt, double* q, double* qd, const double* tau, double* qdd_out,
                               void* stream);

/* ---- differentiation (additions; the reference has no derivative API, see
 * pinocchio/cmake/pinocchio.cmake:4 which builds Pinocchio without autodiff) ----------
 * Configuration adjoints / derivatives are tangent-space quantities with nv columns
 * (for a free-flyer root: with respect to its body twist, as Pinocchio's derivative
 * API defines them). Free flyers are supported only as the root joint. */

/* Vector-Jacobian product of computeInverseDynamics: given tau_bar [n][nv] returns
 * q_bar, qd_bar, qdd_bar [n][nv] (any output may be NULL). qdd_bar = M tau_bar. */
int sgdyn_compute_inverse_dynamics_vjp(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                       const double* qdd, const double* tau_bar, double* q_bar, double* qd_bar,
                                       double* qdd_bar, int layout, void* stream);

/* Vector-Jacobian product of computeForwardDynamics: given qdd_bar returns q_bar, qd_bar,
 * tau_bar (tau_bar = M^-1 qdd_bar). */
int sgdyn_compute_forward_dynamics_vjp(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                       const double* tau, const double* qdd_bar, double* q_bar, double* qd_bar,
                                       double* tau_bar, int layout, void* stream);

/* Vector-Jacobian product of the link poses: pos_bar [n][nlinks*3] (adjoint of link
 * positions), rot_bar [n][nlinks*9] (adjoint of row-major link rotations) or NULL ->
 * q_bar [n][nv]. */
int sgdyn_compute_forward_kinematics_vjp(const sgdyn_model* m, int64_t n, const double* q, const double* pos_bar,
                                         const double* rot_bar, double* q_bar, int layout, void* stream);

/* Dense derivatives of RNEA: dtau_dq, dtau_dqd, dtau_dqdd (= M; may be NULL), each
 * [n][nv*nv] row-major (row = torque, column = input). Analogue of Pinocchio's
 * computeRNEADerivatives, which the reference does not expose. This and
 * sgdyn_compute_aba_derivatives take stream-ordered scratch (cudaMallocAsync / cudaFreeAsync
 * on `stream`, about 8 (18 nv + 44 njoints) bytes per environment, plus the factor of M
 * for ABA) and enqueue two kernels. */
int sgdyn_compute_rnea_derivatives(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                   const double* qdd, double* dtau_dq, double* dtau_dqd, double* dtau_dqdd,
                                   int layout, void* stream);

/* Dense derivatives of ABA: dqdd_dq, dqdd_dqd, dqdd_dtau (= M^-1; may be NULL). */
int sgdyn_compute_aba_derivatives(const sgdyn_model* m, int64_t n, const double* q, const double* qd,
                                  const double* tau, double* dqdd_dq, double* dqdd_dqd, double* dqdd_dtau,
                                  int layout, void* stream);

/* Semi-implicit Euler rollout of T steps, qd += dt ABA(q, qd, tau_t); q <- q (+) dt qd
 * (angles and slides add; a free-flyer root moves on SE(3) by the body twist dt qd, as
 * Pinocchio's integrate). Contiguous env-major arrays: q0, qT [n][nq], qd0, qdT
 * [n][nv], tau [T][n][nv]. With q_ckpt [C][n][nq] and qd_ckpt [C][n][nv],
 * C = ceil(T / checkpoint_every), the state at steps 0, K, 2K, ... is recorded for the
 * backward pass (both NULL for a plain forward rollout). */
int sgdyn_rollout_forward(const sgdyn_model* m, int64_t n, int T, double dt, const double* q0, const double* qd0,
                          const double* tau, int checkpoint_every, double* q_ckpt, double* qd_ckpt, double* qT,
                          double* qdT, void* stream);

/* Lanes per environment of the ABA-based sweeps: sgdyn_rollout_forward, the reverse sweep
 * of sgdyn_rollout_backward / _noalloc, and forward dynamics requested alone
 * (sgdyn_compute_forward_dynamics, sgdyn_step with only SGDYN_OP_FORWARD_DYNAMICS)
 * (addition): 0 automatic (the default:
 * three lanes while one warp per ten environments leaves no FP64 scheduler with two warps),
 * 1, or 3 (one lane per Cartesian axis of every spatial quantity, warp shuffles between
 * them, so each lane issues about half the FP64 instructions of one lane per environment;
 * one-DoF joints and a free-flyer root); -1 only reads the
 * setting. Results agree to rounding. */
int sgdyn_rollout_lanes(int lanes, int* lanes_out);

/* Bytes of device scratch sgdyn_rollout_backward needs for n environments: the
 * intermediates of one checkpoint segment. */
int sgdyn_rollout_scratch_bytes(const sgdyn_model* m, int64_t n, int checkpoint_every, int64_t* bytes);

/* Reverse pass of sgdyn_rollout_forward: given the adjoints of the final state (either may
 * be NULL = zero) returns q0_bar, qd0_bar and tau_bar [T][n][nv]. A free flyer's block of
 * qT_bar / q0_bar ([n][nq]) holds its tangent adjoint (with respect to a right
 * perturbation q exp6(eps), eps a body twist) in its first six slots; the seventh is
 * ignored on input and zero on output. Checkpoint segments are
 * recomputed from their q / qd checkpoints, their spatial intermediates kept in `scratch`
 * (caller-owned device memory of at least sgdyn_rollout_scratch_bytes bytes), and then
 * reversed step by step. A scratch of k times the minimum lets k segments recompute at
 * once (one thread per segment and environment), which fills the GPU at small n;
 * ceil(T / checkpoint_every) times the minimum recomputes all segments in one launch.
 * With room for two groups of segments (and `stream` not being captured) the recompute of
 * the next group runs on an internal second stream of the device while the current group
 * is reversed on `stream`; every launch on it is ordered after the work already on
 * `stream` and before what follows there, so the call stays stream-ordered. */
int sgdyn_rollout_backward(const sgdyn_model* m, int64_t n, int T, double dt, int checkpoint_every,
                           const double* q_ckpt, const double* qd_ckpt, const double* tau, const double* qT_bar,
                           const double* qdT_bar, double* q0_bar, double* qd0_bar, double* tau_bar, double* scratch,
                           int64_t scratch_bytes, void* stream);

/* Same reverse pass as sgdyn_rollout_backward for callers that must not allocate device
 * memory while they run (real-time loops that reserve everything at start-up, plug-ins
 * whose host owns the memory budget). No counterpart in the reference. Its scratch is a
 * fixed SGDYN_NOALLOC_SCRATCH_BYTES device array that the library holds on every GPU that
 * loads it, until exit; calls needing more (sgdyn_rollout_scratch_bytes) fail with
 * SGDYN_ERR_RUNTIME. It calls no allocator: the model must already be on the device
 * (sgdyn_model_upload). Every call looks the array's address up on the current device; the
 * first lookup on a device may load the library's device code, so make one call on each
 * device (n = 0 does only the lookup) before any stream capture. All calls share the
 * array: calls that overlap on the GPU race. */
#define SGDYN_NOALLOC_SCRATCH_BYTES (64LL << 20)
int sgdyn_rollout_backward_noalloc(const sgdyn_model* m, int64_t n, int T, double dt, int checkpoint_every,
                                   const double* q_ckpt, const double* qd_ckpt, const double* tau,
                                   const double* qT_bar, const double* qdT_bar, double* q0_bar, double* qd0_bar,
                                   double* tau_bar, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SGDYN_H */
