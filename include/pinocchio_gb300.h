/*
 * pinocchio_gb300 -- C ABI of the GB300 batched rigid-body dynamics engine.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status (GB_OK == 0) and never throws.  On failure gb_last_error()
 * returns a message (thread-local).  Nothing here falls back to the CPU: a
 * call without a usable CUDA device returns GB_ERR_CUDA.
 *
 * Batch layouts (argument `layout`):
 *   GB_LAYOUT_INSTANCE -- the reference's layout: an Eigen column-major
 *       n x batch matrix, one column per instance (instance b of a vector of
 *       length n starts at p + b*n).  Matrix outputs are nv x nv row-major
 *       per instance (the reference's RowMatrixXs, multibody/data.hpp:401-416),
 *       instance b at p + b*nv*nv.
 *   GB_LAYOUT_SOA -- structure of arrays: element k of every instance is
 *       contiguous (element k of instance b at p + k*batch + b; matrix entry
 *       (r, c) of instance b at p + (r*nv + c)*batch + b).
 * All arrays passed to gb_rnea ... gb_integrate are device (or managed)
 * memory; the *_in_parallel entry points take host memory, as the reference's
 * rneaInParallel / abaInParallel do.
 */
#ifndef PINOCCHIO_GB300_H
#define PINOCCHIO_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes; mirror the reference's std::invalid_argument cases
 * (include/pinocchio/macros.hpp:162-223) plus device failures */
enum {
  GB_OK = 0,
  GB_ERR_INVALID_ARGUMENT = 1, /* null pointer, negative batch, bad enum    */
  GB_ERR_SIZE = 2,             /* size mismatch (PINOCCHIO_CHECK_ARGUMENT_SIZE) */
  GB_ERR_UNSUPPORTED = 3,      /* joint type / tree shape not supported      */
  GB_ERR_GRAVITY = 4,          /* derivatives need gravity.angular() == 0    */
  GB_ERR_POOL = 5,             /* pool empty or num_threads > pool size      */
  GB_ERR_CUDA = 6,             /* CUDA runtime error (message has details)   */
  GB_ERR_NUMERIC = 7           /* a kernel saw a non-positive pivot / NaN    */
};

enum { GB_FP64 = 0, GB_MIXED = 1 };               /* arithmetic of the kernels  */
enum { GB_LOCAL = 0, GB_WORLD = 1 };              /* reference multibody/fwd.hpp:73-81 */
enum { GB_LAYOUT_INSTANCE = 0, GB_LAYOUT_SOA = 1 };
/* joint types: revolute about x / y / z (JointModelRX/RY/RZ, multibody/joint/joint-revolute.hpp),
 * the free-flyer (JointModelFreeFlyer, joint-free-flyer.hpp; root joint only), prismatic along
 * x / y / z (JointModelPX/PY/PZ, joint-prismatic.hpp), revolute about / prismatic along a unit
 * axis of the joint frame (JointModelRevoluteUnaligned, joint-revolute-unaligned.hpp;
 * JointModelPrismaticUnaligned, joint-prismatic-unaligned.hpp) given by gb_model_desc.axis,
 * translation (JointModelTranslation, joint-translation.hpp: nq = nv = 3, anywhere in the tree;
 * the kernels run it as three prismatic joints along x, y, z with identity placements, which
 * is the same transform, joint velocity and configuration space).  Per-joint arrays (external
 * forces, forward-kinematics outputs) are indexed by the caller's joints. */
enum {
  GB_JOINT_NONE = 0,
  GB_JOINT_RX = 1,
  GB_JOINT_RY = 2,
  GB_JOINT_RZ = 3,
  GB_JOINT_FREEFLYER = 4,
  GB_JOINT_PX = 5,
  GB_JOINT_PY = 6,
  GB_JOINT_PZ = 7,
  GB_JOINT_REVOLUTE_UNALIGNED = 8,
  GB_JOINT_PRISMATIC_UNALIGNED = 9,
  GB_JOINT_TRANSLATION = 10, /* JointModelTranslation (joint-translation.hpp): q = v in R^3 */
  GB_JOINT_SPHERICAL = 11,   /* JointModelSpherical (joint-spherical.hpp): q = unit quaternion
                                (x, y, z, w), v = angular velocity in the joint frame */
  GB_JOINT_PLANAR = 12,      /* JointModelPlanar (joint-planar.hpp): q = (x, y, cos t, sin t),
                                v = (vx, vy, wz) in the joint frame.  Models with spherical or
                                planar joints run one configuration per thread (gb_model_set_layout
                                refuses the lane layouts), in gb_batch_multi too. */
  GB_JOINT_RUBX = 13,        /* JointModelRUBX/RUBY/RUBZ (joint-revolute-unbounded.hpp): revolute   */
  GB_JOINT_RUBY = 14,        /* about x / y / z with q = (cos t, sin t) taken as given (not        */
  GB_JOINT_RUBZ = 15,        /* renormalised), nq = 2, nv = 1; what the URDF "continuous" joint is */
  GB_JOINT_REVOLUTE_UNBOUNDED_UNALIGNED = 16, /* JointModelRevoluteUnboundedUnaligned
                                (joint-revolute-unbounded-unaligned.hpp): the same about
                                gb_model_desc.axis */
  GB_JOINT_SPHERICAL_ZYX = 17 /* JointModelSphericalZYX (joint-spherical-ZYX.hpp): q = the Euler
                                angles (z, y, x), R = Rz(q0) Ry(q1) Rx(q2), v = dq/dt, nq = nv = 3,
                                anywhere in the tree (a vector space: integrate adds v dt) */
};
enum { GB_MATRIX_UPPER = 0, GB_MATRIX_SYMMETRIC = 1 }; /* CRBA / RNEA-derivative M output */
/* functions of a heterogeneous batch task / of a launch setting */
enum { GB_FUNC_RNEA = 0, GB_FUNC_ABA = 1, GB_FUNC_CRBA = 2, GB_FUNC_RNEA_DERIVATIVES = 3, GB_FUNC_ABA_DERIVATIVES = 4 };

typedef struct gb_model gb_model;
typedef struct gb_pool gb_pool;

/* Flattened kinematic tree.  Joint 0 is the universe (jtype GB_JOINT_NONE).
 * parents[i] < i and joints are in depth-first order, as ModelTpl builds them
 * (reference multibody/model.hxx:61-170, algorithm/crba.hxx:573-595).
 * placement: njoints x 12 (rotation row-major, then translation) -- jointPlacements.
 * inertia:   njoints x 10 (mass, lever[3], inertia about the COM packed
 *            [xx, xy, yy, xz, yz, zz]) -- inertias (spatial/symmetric3.hpp:46-49).
 * armature:  nv values (may be NULL for zeros); gravity: 6 values [lin; ang]
 *            (may be NULL for (0, 0, -9.81, 0, 0, 0), multibody/model.hxx:40).
 * axis:      njoints x 3, the axis of each unaligned joint (normalised on creation; the
 *            entries of other joints are ignored); may be NULL when there is none.
 * mimic:     njoints entries (may be NULL: no mimic joint): mimic[i] = j > 0 makes joint i a
 *            mimic of joint j < i (JointModelMimic, multibody/joint/joint-mimic.hpp:557-760):
 *            joint i keeps its own type, placement and body, adds no entry to q or v (nq and
 *            nv count the other joints; nvExtended counts it too), and moves with
 *            q_i = mimic_scaling[i] q_j + mimic_offset[i] (for an unbounded revolute joint:
 *            its angle, atan2 of (sin, cos)), v_i = mimic_scaling[i] v_j; its torque adds to
 *            joint j's (LinearAffineTransform / UnboundedRevoluteAffineTransform,
 *            joint-common-operations.hpp:52-90).  Both joints are one-dof joints with the same
 *            nq, joint j is no mimic itself.  Mimic joints are supported by rnea,
 *            nonLinearEffects, computeGeneralizedGravity, crba (without the Cholesky factors),
 *            forwardKinematics, computeJointJacobians (6 x nvExtended, the mimic joints' own
 *            columns included, as the reference's data.J) and integrate; every other function
 *            returns GB_ERR_UNSUPPORTED, as the reference rejects mimic joints in ABA, the
 *            derivatives and the Cholesky (aba.hxx:250, rnea-derivatives.hxx:157,
 *            cholesky.hxx:37).  armature has nv entries. */
typedef struct {
  int njoints;
  const int* parents;
  const int* jtype;
  const double* placement;
  const double* inertia;
  const double* armature;
  int nv_armature;
  const double* gravity;
  const double* axis;
  const int* mimic;
  const double* mimic_scaling;
  const double* mimic_offset;
} gb_model_desc;

/* Replaces building a ModelTpl + DataTpl (multibody/model.hpp:98-220,
 * multibody/data.hxx:20-340): validates the tree, derives nvSubtree /
 * parents_fromRow, and uploads the level tables to the current device. */
int gb_model_create(const gb_model_desc* desc, gb_model** out);
int gb_model_destroy(gb_model* model);
int gb_model_dims(const gb_model* model, int* nq, int* nv, int* njoints);
/* nvExtended (multibody/model.hpp): nv plus one per mimic joint (= nv without mimic joints) */
int gb_model_nv_extended(const gb_model* model, int* nv_extended);
const char* gb_last_error(void);

/* Numeric status of a model's kernels (bits of *flags), replacing the checks the
 * reference makes with assertions and exceptions around its factorisations
 * (PINOCCHIO_CHECK_INPUT_ARGUMENT / assert, include/pinocchio/macros.hpp:162-223;
 * the LLT of PerformStYSInversion, multibody/joint/joint-common-operations.hpp:20-45):
 *   GB_NUMERIC_PIVOT     -- a pivot of a factorisation was not > 0 (or NaN): the
 *                           joint-space inertia StU + armature of an ABA step, a pivot of
 *                           the 6x6 LLT of a free-flyer, D of the tree Cholesky of the
 *                           CRBA, a pivot of the contact solves (singular or indefinite
 *                           inertia, or NaN inputs);
 *   GB_NUMERIC_NONFINITE -- an output (tau of RNEA, ddq of ABA / the ABA derivatives)
 *                           was NaN or infinite.
 * The kernels OR the bits into a word of the model's device memory; the affected
 * outputs are then NaN or infinite, as the reference's would be.  This call
 * synchronises the device, fills *flags (0: nothing seen since the model was
 * created or the last reset; reset != 0 clears the word after reading it) and
 * returns GB_ERR_NUMERIC with a message naming the failures when *flags != 0,
 * GB_OK otherwise. */
enum { GB_NUMERIC_PIVOT = 1, GB_NUMERIC_NONFINITE = 2 };
int gb_numeric_status(const gb_model* model, unsigned int* flags, int reset);

/* Diagnostic without a reference counterpart: how many warps of the pipelined
 * kernels (asynchronous bulk copies and producer / consumer barriers, each
 * wait limited to 2 s) gave up waiting since the library was loaded, or since
 * the last reset (reset != 0 clears the count after reading it).  Non-zero
 * means some outputs of those calls were not written.  Synchronises the
 * device. */
int gb_pipeline_timeouts(unsigned int* count, int reset);
/* Exercises that failure path without a fault: one warp waits limit_us
 * microseconds (1..100000) on a barrier nothing arrives on and records one
 * timeout in the count above; the context stays usable. */
int gb_pipeline_wait_selftest(unsigned int limit_us, void* stream);

/* Utility without a reference counterpart: a stream-ordered copy of `bytes` bytes between
 * host and device memory (any direction; page-locked host memory makes it asynchronous),
 * for moving a batch's inputs and outputs next to the calls that use them.  bytes == 0 is a
 * no-op; NULL pointers otherwise are rejected. */
int gb_memcpy_async(void* dst, const void* src, size_t bytes, void* stream);

/* tau = rnea(model, data, q, v, a) for every instance
 * (reference algorithm/rnea.hxx:117-161, public rnea.hxx:766). */
int gb_rnea(const gb_model* model, int precision, int layout, long batch, const double* q, const double* v,
            const double* a, double* tau, void* stream);

/* nle = nonLinearEffects(model, data, q, v) = C(q, v) v + g(q)
 * (reference algorithm/rnea.hxx:221-336, public rnea.hpp:105-109, rnea.hxx:801-808). */
int gb_nonlinear_effects(const gb_model* model, int precision, int layout, long batch, const double* q,
                         const double* v, double* nle, void* stream);

/* g = computeGeneralizedGravity(model, data, q)
 * (reference algorithm/rnea.hxx:346-446, public rnea.hpp:133-136, rnea.hxx:816-822). */
int gb_generalized_gravity(const gb_model* model, int precision, int layout, long batch, const double* q, double* g,
                           void* stream);

/* External forces.  fext holds, per instance, njoints x 6 values: the force
 * [linear; angular] applied to joint i, expressed in joint i's own frame, as
 * the reference's container::aligned_vector<Force> fext of size model.njoints
 * (joint 0's entries are not read); in `layout` like the other arrays (an
 * instance's 6 * njoints values contiguous, or value-major with stride batch).
 * These calls run one thread per configuration whatever layout the model has. */

/* tau = rnea(model, data, q, v, a, fext) (reference algorithm/rnea.hxx:164-218,
 * public rnea.hpp:74-79, rnea.hxx:784-793): f_i -= fext_i after the forward
 * step of joint i. */
int gb_rnea_fext(const gb_model* model, int precision, int layout, long batch, const double* q, const double* v,
                 const double* a, const double* fext, double* tau, void* stream);

/* tau = computeStaticTorque(model, data, q, fext) = the generalized gravity minus
 * the joint torques of fext (reference algorithm/rnea.hxx:448-489, public
 * rnea.hpp:159-167, rnea.hxx:828-837). */
int gb_static_torque(const gb_model* model, int precision, int layout, long batch, const double* q,
                     const double* fext, double* tau, void* stream);

/* ddq = aba(model, data, q, v, tau, convention) for every instance
 * (reference algorithm/aba.hxx:933-948; WORLD 242-293, LOCAL 486-540). */
int gb_aba(const gb_model* model, int precision, int convention, int layout, long batch, const double* q,
           const double* v, const double* tau, double* ddq, void* stream);

/* ddq = aba(model, data, q, v, tau, fext, convention) (reference
 * algorithm/aba.hxx:958-973; WORLD 296-357, LOCAL 543-605): the bias force of
 * joint i is v_i x* (I_i v_i) - fext_i. */
int gb_aba_fext(const gb_model* model, int precision, int convention, int layout, long batch, const double* q,
                const double* v, const double* tau, const double* fext, double* ddq, void* stream);

/* M = crba(model, data, q, convention) (reference algorithm/crba.hxx:602-617),
 * upper triangle (GB_MATRIX_UPPER, the lower part is written as zero) or full
 * symmetric.  When U and D are non-NULL the tree-sparse factorisation
 * M = U diag(D) U^T of cholesky::decompose (algorithm/cholesky.hxx:18-62) is
 * computed in FP64 in the same launch (U unit upper, row-major per instance). */
int gb_crba(const gb_model* model, int precision, int convention, int matrix_mode, int layout, long batch,
            const double* q, double* M, double* U, double* D, void* stream);

/* computeRNEADerivatives(model, data, q, v, a) -> (dtau_dq, dtau_dv, M)
 * (reference algorithm/rnea-derivatives.hxx:472-541, public 708-790).  M is
 * dtau/da (upper or symmetric, see matrix_mode).  tau may be NULL. */
int gb_rnea_derivatives(const gb_model* model, int precision, int matrix_mode, int layout, long batch,
                        const double* q, const double* v, const double* a, double* dtau_dq, double* dtau_dv,
                        double* M, double* tau, void* stream);

/* computeRNEADerivatives(model, data, q, v, a, fext) (reference
 * algorithm/rnea-derivatives.hxx:550-633, public 728-750, 772-790): the world
 * force of joint i is reduced by oMi.act(fext_i) before the backward sweep. */
int gb_rnea_derivatives_fext(const gb_model* model, int precision, int matrix_mode, int layout, long batch,
                             const double* q, const double* v, const double* a, const double* fext, double* dtau_dq,
                             double* dtau_dv, double* M, double* tau, void* stream);

/* computeABADerivatives(model, data, q, v, tau) -> (ddq_dq, ddq_dv, Minv)
 * (reference algorithm/aba-derivatives.hxx:380-453, public 910-1051).  Minv
 * is returned symmetric.  ddq may be NULL.  In GB_MIXED (nv <= 32) the
 * -Minv * dtau products run in a pipelined kernel whose barrier waits are
 * bounded (2 s each): a wait that gives up leaves those outputs unwritten and
 * is reported only by gb_pipeline_timeouts (the call itself has returned
 * GB_OK), so a caller that needs the guarantee polls it after the call. */
int gb_aba_derivatives(const gb_model* model, int precision, int layout, long batch, const double* q,
                       const double* v, const double* tau, double* ddq_dq, double* ddq_dv, double* Minv,
                       double* ddq, void* stream);

/* computeABADerivatives(model, data, q, v, tau, fext) (reference
 * algorithm/aba-derivatives.hxx:463-541, public 930-950, 978-990): oMi.act(fext_i)
 * is subtracted from the world force of joint i after the first and the
 * second forward sweep. */
int gb_aba_derivatives_fext(const gb_model* model, int precision, int layout, long batch, const double* q,
                            const double* v, const double* tau, const double* fext, double* ddq_dq,
                            double* ddq_dv, double* Minv, double* ddq, void* stream);

/* Minv = computeMinverse(model, data, q) (reference algorithm/aba.hxx:838-880,
 * public aba.hpp:101-109): the reference fills the upper triangle
 * (GB_MATRIX_UPPER, the lower part written as zero); GB_MATRIX_SYMMETRIC gives
 * the symmetric matrix its Python binding returns.  Passes 1-2 of the ABA
 * derivatives without velocity terms and the Minv recursion. */
int gb_compute_minverse(const gb_model* model, int precision, int matrix_mode, int layout, long batch,
                        const double* q, double* Minv, void* stream);

/* Vector-Jacobian products of the forward dynamics, for reverse-mode
 * differentiation (no counterpart in the reference, whose callers form the
 * full Jacobians of computeABADerivatives, aba-derivatives.hxx:380-453, and
 * multiply): for an incoming gradient g on ddq, tau_bar = Minv g,
 * q_bar = ddq_dq^T g and v_bar = ddq_dv^T g, from the same sweeps as
 * gb_aba_derivatives but O(nv^2) per instance instead of the O(nv^3) products.
 * g, q_bar, v_bar, tau_bar (and the optional ddq) are nv x batch in `layout`. */
int gb_aba_derivatives_vjp(const gb_model* model, int precision, int layout, long batch, const double* q,
                           const double* v, const double* tau, const double* g, double* q_bar, double* v_bar,
                           double* tau_bar, double* ddq, void* stream);

/* The batched ABA derivatives of gb_aba_derivatives, computed without any
 * device allocation: no counterpart in the reference (whose algorithms never
 * allocate on their own).  For callers that must not allocate -- real-time
 * control loops whose cycle must not wait on an allocator, plugins whose host
 * application owns every device allocation and its budget -- the workspace is
 * a fixed 64 MiB device array inside the library (held by every GPU that loads
 * it until exit) instead of a cudaMallocAsync block.  Batches whose workspace
 * exceeds it (~1000 FP64 / ~1400 mixed configurations of the 32-dof humanoid)
 * are rejected with GB_ERR_SIZE.  The first call on a device resolves the
 * array's address, so make it before any stream capture; the address is kept
 * for the process, so do not call this after a cudaDeviceReset.  All calls
 * share the array: calls that overlap on the GPU race and must be serialised
 * by the caller. */
int gb_aba_derivatives_noalloc(const gb_model* model, int precision, int layout, long batch, const double* q,
                               const double* v, const double* tau, double* ddq_dq, double* ddq_dv, double* Minv,
                               double* ddq, void* stream);

/* Contact dynamics with a given constraint Jacobian.  J holds, per instance, an
 * nc x nv row-major matrix (nc * nv values in `layout`); gamma, lambda_c and
 * impulse_c nc values (they, and J, may be NULL when nc == 0).  M = U D U^T comes
 * from the CRBA with the FP64 tree factorisation, the rest is FP64 in both
 * precisions except the bias forces (FP32 sweeps in GB_MIXED).  As in the
 * reference, J M^-1 J^T + inv_damping I must be positive definite (a rank-deficient
 * J needs inv_damping > 0); otherwise the outputs are NaN.  inv_damping < 0 is
 * rejected, nc is limited to 0..1024.
 *
 * forwardDynamics(model, data, q, v, tau, J, gamma, inv_damping) (reference
 * algorithm/contact-dynamics.hxx:81-165, contact-dynamics.hpp:60-74, deprecated there):
 * ddq and lambda_c with M ddq + nle = tau + J^T lambda_c and
 * J ddq + gamma = -inv_damping lambda_c. */
int gb_forward_dynamics(const gb_model* model, int precision, int layout, long batch, int nc, const double* q,
                        const double* v, const double* tau, const double* J, const double* gamma,
                        double inv_damping, double* ddq, double* lambda_c, void* stream);

/* impulseDynamics(model, data, q, v_before, J, r_coeff, inv_damping) (reference
 * algorithm/contact-dynamics.hxx:255-327, contact-dynamics.hpp:230-248, deprecated there):
 * dq_after and impulse_c with M (dq_after - v_before) = J^T impulse_c and
 * J dq_after = -r_coeff J v_before - inv_damping impulse_c. */
int gb_impulse_dynamics(const gb_model* model, int precision, int layout, long batch, int nc, const double* q,
                        const double* v_before, const double* J, double r_coeff, double inv_damping,
                        double* dq_after, double* impulse_c, void* stream);

/* computeKKTContactDynamicMatrixInverse(model, data, q, J, KKTMatrix_inv, inv_damping)
 * (reference algorithm/contact-dynamics.hxx:166-225, contact-dynamics.hpp:150-163):
 * K = [[M, J^T], [J, -inv_damping I]]^-1, (nv + nc) x (nv + nc) row-major per instance,
 * FP64 in both precisions. */
int gb_kkt_contact_inverse(const gb_model* model, int precision, int layout, long batch, int nc, const double* q,
                           const double* J, double inv_damping, double* K, void* stream);

/* ---- constraintDynamics with rigid constraint models (reference algorithm/constrained-dynamics.hpp:90-110,
 * constrained-dynamics.hxx:188-520; contact models algorithm/contact-info.hpp:140-230; proximal settings
 * algorithm/proximal.hpp:22-110) ---------------------------------------------------------------------- */
enum { GB_CONTACT_3D = 0, GB_CONTACT_6D = 1 };  /* ContactType, contact-info.hpp:19-24 */
enum { GB_FRAME_WORLD = 0, GB_FRAME_LOCAL = 1, GB_FRAME_LOCAL_WORLD_ALIGNED = 2 };  /* ReferenceFrame, multibody/fwd.hpp:46-56 */

/* RigidConstraintModel(type, model, joint1_id, joint1_placement, joint2_id, joint2_placement,
 * reference_frame): a point (3 rows) or frame (6 rows) constraint between a frame of joint 1 and a
 * frame of joint 2 (joint 0: the world), joints indexed as in gb_model_desc, placements R row-major
 * then t, relative to the joint frames; reference_frame GB_FRAME_LOCAL or
 * GB_FRAME_LOCAL_WORLD_ALIGNED; the desired contact acceleration and the Baumgarte gains Kp, Kd
 * (corrector) [linear; angular] (GB_CONTACT_3D reads the first three of each). */
typedef struct gb_constraint_desc {
  int type;
  int reference_frame;
  int joint1_id;
  int joint2_id;
  double joint1_placement[12];
  double joint2_placement[12];
  double desired_acceleration[6];
  double Kp[6];
  double Kd[6];
} gb_constraint_desc;

/* ProximalSettings(absolute_accuracy, relative_accuracy, mu, max_iter) (proximal.hpp:22-110). */
typedef struct gb_proximal_settings {
  double absolute_accuracy;
  double relative_accuracy;
  double mu;
  int max_iter;
} gb_proximal_settings;

/* The constraint models of initConstraintDynamics(model, data, contact_models)
 * (constrained-dynamics.hxx:21-60), uploaded once for all the calls of `model`.  n may be 0.
 * Rejected: a reference frame other than LOCAL / LOCAL_WORLD_ALIGNED, an unknown type, a joint
 * index out of range, n outside 0..64. */
typedef struct gb_constraint_set gb_constraint_set;
int gb_constraint_set_create(const gb_model* model, int n, const gb_constraint_desc* constraints,
                             gb_constraint_set** out);
int gb_constraint_set_destroy(gb_constraint_set* set);
/* the number of constraint models and the constraint dimension (the length of lambda_c) */
int gb_constraint_set_dims(const gb_constraint_set* set, int* n, int* constraint_dim);

/* ddq = constraintDynamics(model, data, q, v, tau, contact_models, contact_datas, settings) per
 * instance: the world-frame kinematics, M and the bias forces nle, the constraint Jacobian rows
 * and drifts of the set, then the proximal iterations
 *   lambda_k = (J M^-1 J^T + mu I)^-1 (rhs + mu lambda_{k-1} - J M^-1 (tau - nle)), lambda_0 = 0,
 * until the reference's absolute or relative residual falls below its accuracy or max_iter
 * iterations ran; ddq = M^-1 (tau - nle + J^T lambda).  lambda_c holds the constraint_dim
 * multipliers (data.lambda_c; each constraint's segment is its contact_force in its frame).
 * Optional outputs: iterations (one int per instance, settings.iter) and residuals (two doubles per
 * instance, instance-major: absolute_residual, relative_residual).  FP64 after the CRBA in both
 * precisions except the bias forces (FP32 sweeps in GB_MIXED).  mu = 0 needs full-rank
 * constraints (otherwise the outputs are NaN and the numeric status is set). */
int gb_constraint_dynamics(const gb_model* model, int precision, const gb_constraint_set* set,
                           const gb_proximal_settings* settings, int layout, long batch, const double* q,
                           const double* v, const double* tau, double* ddq, double* lambda_c, int* iterations,
                           double* residuals, void* stream);

/* computeConstraintDynamicsDerivatives(model, data, contact_models, contact_datas, settings, ddq_dq,
 * ddq_dv, ddq_dtau, dlambda_dq, dlambda_dv, dlambda_dtau) (reference
 * algorithm/constrained-dynamics-derivatives.hpp:27-100, hxx:344-1050) after constraintDynamics on the
 * same inputs, both in one call: ddq and lambda_c as gb_constraint_dynamics, the derivatives of ddq
 * (nv x nv, row-major per instance) and of lambda_c (constraint_dim x nv) with respect to q (in the
 * tangent space), v and tau, following the reference's proximal recursion over each instance's
 * iteration count; iterations may be NULL.  Constraints to the world (joint2_id = 0), with Baumgarte
 * gains on GB_FRAME_LOCAL constraints only (others: GB_ERR_UNSUPPORTED; the reference's corrector
 * terms in world-aligned axes disagree with central differences of its own constraintDynamics);
 * gravity without an angular part (GB_ERR_GRAVITY).
 * The inverse-dynamics derivatives at ddq use the precision's sweeps, the rest is FP64. */
int gb_constraint_dynamics_derivatives(const gb_model* model, int precision, const gb_constraint_set* set,
                                       const gb_proximal_settings* settings, int layout, long batch,
                                       const double* q, const double* v, const double* tau, double* ddq,
                                       double* lambda_c, double* ddq_dq, double* ddq_dv, double* ddq_dtau,
                                       double* dlambda_dq, double* dlambda_dv, double* dlambda_dtau,
                                       int* iterations, void* stream);

/* ContactCholeskyDecomposition(model, contact_models).compute(model, data, contact_models,
 * contact_datas, mu) at each configuration q and its accessors (algorithm/contact-cholesky.hpp:
 * 168-265, contact-cholesky.hxx:152-304, 617-759), n = constraint dim + nv, row-major per
 * configuration in `layout`; every output may be NULL:
 *   kkt           n x n   matrix():  [[-mu I, J], [J^T, M]], the constraint rows first;
 *   kkt_inverse   n x n   inverse(): [[-OSIM, OSIM J M^-1], [M^-1 J^T OSIM, M^-1 - M^-1 J^T OSIM J M^-1]];
 *   osim_inverse  nc x nc getInverseOperationalSpaceInertiaMatrix(): J M^-1 J^T + mu I;
 *   osim          nc x nc getOperationalSpaceInertiaMatrix(): its inverse;
 *   minv          nv x nv getInverseMassMatrix(): M^-1;
 *   jminv         nc x nv getJMinv(): J M^-1.
 * J is the constraint Jacobian of the set's models at q (as constraintDynamics builds it).  The
 * factorisation is FP64 in both precisions (the CRBA's Cholesky is). */
int gb_contact_cholesky(const gb_model* model, int precision, const gb_constraint_set* set, double mu, int layout,
                        long batch, const double* q, double* kkt, double* kkt_inverse, double* osim_inverse,
                        double* osim, double* minv, double* jminv, void* stream);

/* forwardKinematics(model, data, q[, v[, a]]) (reference algorithm/kinematics.hxx:42-272):
 * per instance, for every joint i = 0 .. njoints-1 (joint 0 the universe:
 * identity, zero), oMi[12 i ..] = the world placement (rotation row-major, then
 * translation); with v, vout[6 i ..] = data.v[i], the joint-frame spatial
 * velocity [linear; angular]; with v and a, aout[6 i ..] = data.a[i], the
 * joint-frame spatial acceleration (no gravity).  v, a, vout, aout may be NULL
 * (an output needs its input). */
int gb_forward_kinematics(const gb_model* model, int precision, int layout, long batch, const double* q,
                          const double* v, const double* a, double* oMi, double* vout, double* aout, void* stream);

/* J = computeJointJacobians(model, data, q) (reference algorithm/jacobian.hxx:17-95):
 * data.J, 6 x nv column-major per instance (column k = [linear; angular] of
 * the motion subspace of dof k, in the world frame about the world origin). */
int gb_compute_joint_jacobians(const gb_model* model, int precision, int layout, long batch, const double* q,
                               double* J, void* stream);

/* qout = integrate(model, q, v) (reference algorithm/joint-configuration.hpp:41-80;
 * free-flyer: multibody/liegroup/special-euclidean.hpp:660-699), always FP64. */
int gb_integrate(const gb_model* model, int layout, long batch, const double* q, const double* v, double* qout,
                 void* stream);

/* One task of a heterogeneous batch: `batch` configurations of `model`,
 * GB_LAYOUT_INSTANCE device arrays; function GB_FUNC_RNEA (x = a, out = tau)
 * or GB_FUNC_ABA (x = tau, out = ddq, LOCAL convention). */
typedef struct {
  const gb_model* model;
  int function;
  long batch;
  const double* q;
  const double* v;
  const double* x;
  double* out;
} gb_task;

/* Many configurations over several models in one persistent launch: the
 * batch of rneaInParallel / abaInParallel (algorithm/parallel/{rnea,aba}.hpp)
 * generalised to several models.  At most 16 tasks; threads_per_block 0
 * selects the default (128).  The launch allocates nothing, so it can be
 * captured in a CUDA graph. */
int gb_batch_multi(const gb_task* tasks, int ntasks, int precision, int threads_per_block, void* stream);

/* Launch setting chosen by the autotuner for one model and function:
 * configurations per CTA (32, 64, 96 or 128; default 128). */
int gb_model_set_launch(gb_model* model, int function, int threads_per_block);

/* Layout of one model's function chosen by the autotuner: one thread per
 * configuration (GB_INSTANCE_PER_THREAD, the default) or one warp per
 * configuration (GB_INSTANCE_PER_WARP), for batches too small to fill the GPU.
 * RNEA and ABA (including nonLinearEffects / generalized gravity and the
 * *_in_parallel entry points): the warp's lanes take the joints of one tree
 * level in parallel.  ABA derivatives (and computeMinverse, the VJP): a team of
 * 4, 8 or 32 lanes per configuration (GB_INSTANCE_PER_4_LANES, _8_LANES,
 * GB_INSTANCE_PER_WARP) splits the loops over matrix columns of every joint
 * (subtree, ancestor and Minv-row columns), for deep trees at small batches.
 * RNEA and ABA also: one lane per branch (GB_INSTANCE_PER_BRANCH: a team of 4-32
 * lanes per configuration, one lane per chain of joints, chains of one level
 * of the chain tree in parallel).
 * FP64 results are identical in every layout. */
enum {
  GB_INSTANCE_PER_THREAD = 0,
  GB_INSTANCE_PER_WARP = 1,
  GB_INSTANCE_PER_4_LANES = 2,
  GB_INSTANCE_PER_8_LANES = 3,
  GB_INSTANCE_PER_BRANCH = 4
};
int gb_model_set_layout(gb_model* model, int function, int layout);

/* ModelPool (reference multibody/pool/model.hpp:19-165): `size` nominal
 * per-thread slots; the GPU needs one model copy only, the size is kept for
 * the reference's num_threads <= pool.size() check. */
int gb_pool_create(const gb_model* model, long size, gb_pool** out);
int gb_pool_destroy(gb_pool* pool);
int gb_pool_size(const gb_pool* pool, long* size);
int gb_pool_set_precision(gb_pool* pool, int precision);

/* rneaInParallel(num_threads, pool, q, v, a, tau)
 * (reference algorithm/parallel/rnea.hpp:39-84).  q: nq x batch, v, a, tau:
 * nv x batch, column-major HOST arrays.  num_threads must be in
 * [1, pool size]; the GPU runs the whole batch in one launch. */
int gb_rnea_in_parallel(long num_threads, gb_pool* pool, long batch, const double* q, const double* v,
                        const double* a, double* tau);

/* abaInParallel(num_threads, pool, q, v, tau, a) (reference
 * algorithm/parallel/aba.hpp:40-84; WORLD convention as at line 82). */
int gb_aba_in_parallel(long num_threads, gb_pool* pool, long batch, const double* q, const double* v,
                       const double* tau, double* a);

#ifdef __cplusplus
}
#endif

#endif /* PINOCCHIO_GB300_H */
