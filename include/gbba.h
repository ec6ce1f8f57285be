/*
 * gbba.h - C ABI of the GB300 bundle-adjustment engine.
 *
 * This is the drop-in boundary that replaces the ceres::Problem / ceres::Solve
 * block of the reference's bundle-adjustment call sites:
 *   - IncrementalReconstructionEngine::BundleAdjustment
 *       libs/sfm/src/sfm_incremental_engine.cpp:1395-1473 (problem build,
 *       options, Solve) and :1476 (IsSolutionUsable + write-back);
 *   - GlobalReconstructionEngine::bundleAdjustment_t_Xi / _Rt_Xi
 *       libs/sfm/src/sfm_global_engine.cpp:1546-1594, 1756-1802;
 *   - the two-view refinement, libs/sfm/src/sfm_global_engine.cpp:1142-1174.
 * The flat parameter layout is the one of the reference containers
 * BA_Problem_data_camMotionAndIntrinsic<6,K> / BAProblemData<N>
 * (libs/sfm/include/mvg/sfm/problem_data_container.h:16-121): extrinsics as
 * [angle-axis(3), t(3)] per camera, intrinsics as one block per group, points
 * as [X,Y,Z], observations as (x,y) pairs with per-observation indices.
 *
 * Conventions (the reference's, libs/sfm + ceres 1.10):
 *   - the caller owns every array; refinement is in place;
 *   - no exceptions and no abort: every entry point returns a gbba_status and
 *     fills a summary that mirrors ceres::Solver::Summary;
 *   - cost = 1/2 * sum_i rho(|r_i|^2) (ceres residual_block.cc:160-166);
 *   - a handle is not thread safe: use one handle per host thread.
 * No C++ types cross this boundary.
 */
#ifndef GBBA_H_
#define GBBA_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBBA_ABI_VERSION 1

typedef enum gbba_status {
  GBBA_SUCCESS = 0,
  GBBA_ERROR_INVALID_ARGUMENT = 1, /* bad sizes, index out of range, NULL array */
  GBBA_ERROR_CUDA = 2,             /* a CUDA runtime call failed */
  GBBA_ERROR_OUT_OF_MEMORY = 3,    /* device allocation failed (nothing aborted) */
  GBBA_ERROR_NUMERICAL = 4,        /* non-finite cost at the initial point */
  GBBA_ERROR_NOT_SUPPORTED = 5,
  GBBA_ERROR_TOO_LARGE = 6,        /* problem exceeds a documented limit */
  GBBA_ERROR_NO_DEVICE = 7,
  GBBA_ERROR_TIMEOUT = 8           /* a bounded device-side wait gave up */
} gbba_status;

/* Camera models.  Residual r = predicted - observed, with
 *   p = R(w) X + t      (ceres::AngleAxisRotatePoint, rotation.h:566-625)
 *   x = p0/p2, y = p1/p2
 * PINHOLE_F : pred = f*(x,y)            k = 1 [f]; observations pre-centred by
 *             the principal point (pinhole_ceres_functor.h:24-54,
 *             sfm_bundle_adjustment_helper_tonly.h:11-76).
 * RADIAL_K3 : pred = pp + f*(x,y)*(1+k1 r2+k2 r4+k3 r6)      k = 6
 *             [f,ppx,ppy,k1,k2,k3] (pinhole_brown_rt_ceres_functor.h:60-107,
 *             brown_pinhole_camera.h:15-41).
 * BROWN_T2  : RADIAL_K3 plus the tangential terms the reference has only as a
 *             commented-out formula (brown_pinhole_camera.h:35-36):
 *             xd += 2 t1 x y + t2 (r2 + 2x^2), yd += 2 t2 x y + t1 (r2 + 2y^2)
 *             k = 8 [f,ppx,ppy,k1,k2,k3,t1,t2]. */
typedef enum gbba_camera_model {
  GBBA_PINHOLE_F = 0,
  GBBA_RADIAL_K3 = 1,
  GBBA_BROWN_T2 = 2
} gbba_camera_model;

typedef enum gbba_loss {
  GBBA_LOSS_SQUARED = 0, /* ceres TrivialLoss / NULL loss */
  GBBA_LOSS_HUBER = 1    /* ceres::HuberLoss(a): rho(s) = s if s <= a^2, else 2a sqrt(s) - a^2 */
} gbba_loss;

typedef enum gbba_linear_solver {
  GBBA_SOLVER_AUTO = 0,            /* dense Schur up to options.dense_schur_max_size, else iterative */
  GBBA_SOLVER_DENSE_SCHUR = 1,     /* dense Cholesky of the reduced camera system S */
  GBBA_SOLVER_ITERATIVE_SCHUR = 2  /* block-Jacobi PCG on S; every free intrinsic group must belong to one
                                      camera (else GBBA_ERROR_NOT_SUPPORTED); the dense solver takes any
                                      grouping (a free group shared by several cameras uses the point-major
                                      Schur build, whose FP atomics are not bit-repeatable) */
} gbba_linear_solver;

typedef enum gbba_precision {
  GBBA_PRECISION_FP64 = 0,  /* every kernel in FP64: the plain GPU path */
  GBBA_PRECISION_MIXED = 1  /* FP32 Jacobians / Schur build / factor, FP64 cost and refinement */
} gbba_precision;

/* How the dense path builds S.  AUTO takes the atomic-free camera-pair build
 * whenever every free intrinsic block belongs to one camera (S then splits
 * into camera-pair blocks) and the point-major build with atomic additions
 * otherwise; POINT_ATOMIC forces the latter (both give the same S up to the
 * order of the sums). */
typedef enum gbba_schur_build {
  GBBA_SCHUR_BUILD_AUTO = 0,
  GBBA_SCHUR_BUILD_POINT_ATOMIC = 1
} gbba_schur_build;

typedef enum gbba_memory {
  GBBA_MEMORY_HOST = 0,   /* arrays are host pointers; copies are done by the call */
  GBBA_MEMORY_DEVICE = 1  /* arrays are device pointers on the handle's device */
} gbba_memory;

/* Same values as ceres::TerminationType (include/ceres/types.h:324-344). */
typedef enum gbba_termination {
  GBBA_CONVERGENCE = 0,
  GBBA_NO_CONVERGENCE = 1,
  GBBA_FAILURE = 2
} gbba_termination;

typedef struct gbba_problem {
  int32_t camera_model;          /* gbba_camera_model */
  int32_t memory;                /* gbba_memory of every array below */
  int64_t num_cameras;           /* extrinsic blocks */
  int64_t num_intrinsics;        /* intrinsic groups */
  int64_t num_points;
  int64_t num_observations;
  double* extrinsics;            /* [num_cameras][6]  angle-axis, t   (in/out) */
  double* intrinsics;            /* [num_intrinsics][k]               (in/out) */
  double* points;                /* [num_points][3]                   (in/out) */
  const double* observations;    /* [num_observations][2] pixels */
  const uint32_t* camera_index;     /* [num_observations] */
  const uint32_t* intrinsic_index;  /* [num_observations] */
  const uint32_t* point_index;      /* [num_observations] */
  const uint8_t* camera_constant;    /* [num_cameras] 1 = SetParameterBlockConstant, or NULL */
  const uint8_t* intrinsic_constant; /* [num_intrinsics] or NULL */
  uint32_t extrinsic_fixed_mask; /* bit j: coordinate j of every extrinsic block held
                                    (rotation-only-fixed translation refinement, :1438) */
  uint32_t intrinsic_fixed_mask; /* bit j: coordinate j of every intrinsic block held
                                    (ceres::SubsetParameterization, :1396-1409) */
} gbba_problem;

/* Extra precision safeguards of the mixed path (options.mixed_flags). */
typedef enum gbba_mixed_flags {
  /* Kahan-compensated FP32 sums of the camera-pair blocks of S (the Schur
   * complement's cancellation: U - W V^-1 W^T) */
  GBBA_MIXED_KAHAN_SCHUR = 1,
  /* point blocks V whose FP32 Cholesky pivots span more than 1e4 (condition
   * above ~1e4: near-parallel rays, short baselines) are summed and inverted
   * again in FP64 from an FP64 Jacobian */
  GBBA_MIXED_FP64_POINT_INVERSE = 2
} gbba_mixed_flags;

typedef struct gbba_options {
  /* ceres::Solver::Options names and defaults (include/ceres/solver.h:81-129) */
  int32_t max_num_iterations;             /* 50 */
  int32_t max_num_consecutive_invalid_steps; /* 5 */
  double function_tolerance;              /* 1e-6 */
  double gradient_tolerance;              /* 1e-10 */
  double parameter_tolerance;             /* 1e-8 */
  double initial_trust_region_radius;     /* 1e4 */
  double max_trust_region_radius;         /* 1e16 */
  double min_trust_region_radius;         /* 1e-32 */
  double min_relative_decrease;           /* 1e-3 */
  double min_lm_diagonal;                 /* 1e-6 */
  double max_lm_diagonal;                 /* 1e32 */
  int32_t jacobi_scaling;                 /* 1 */
  int32_t loss_type;                      /* gbba_loss */
  double loss_scale;                      /* Huber a (pixels) */
  int32_t linear_solver;                  /* gbba_linear_solver */
  int32_t precision;                      /* gbba_precision */
  int32_t max_linear_solver_iterations;   /* 500 (PCG) */
  int32_t dense_schur_max_size;           /* AUTO switches to PCG above this S size: 16384 */
  double eta;                             /* 0.1: PCG forcing sequence (ceres q-tolerance) */
  int32_t refinement_interval;            /* PCG: every this many iterations the residual is recomputed
                                             as b - S x (FP64 accumulation) instead of updated (ceres's
                                             residual_reset_period): 10 */
  int32_t use_cuda_graphs;                /* 1: capture the per-iteration launch sequence */
  void* stream;                           /* cudaStream_t, or NULL for the handle's stream */
  int32_t fp64_polish_iterations;         /* mixed path: after it stops, at most this many plain-FP64
                                             LM iterations continue from its solution with function and
                                             parameter tolerances 1000x tighter (0 = off): 10 */
  int32_t schur_build;                    /* gbba_schur_build: GBBA_SCHUR_BUILD_AUTO */
  /* Optional per-iteration trace, host memory (NULL = off): entry i holds the
   * cost at the accepted parameters after LM iteration i (entry 0: the
   * initial cost; ceres's IterationSummary::cost) and the wall time in
   * seconds since the call began, setup included.  At most trace_capacity
   * entries are written (summary.num_iterations + 1 when they fit); the
   * iterations of the optional FP64 polish are not traced. */
  double* trace_cost;
  double* trace_time_s;
  int32_t trace_capacity;
  uint32_t mixed_flags;                   /* gbba_mixed_flags of the mixed path: 0 */
} gbba_options;

typedef struct gbba_summary {
  double initial_cost;
  double final_cost;
  int32_t num_iterations;          /* LM iterations run (successful + unsuccessful) */
  int32_t num_successful_steps;
  int32_t num_unsuccessful_steps;
  int32_t termination_type;        /* gbba_termination */
  int32_t usable;                  /* ceres Summary::IsSolutionUsable() */
  int32_t linear_solver_iterations;/* total PCG iterations (0 for dense) */
  int64_t reduced_system_size;     /* rows of S */
  double total_time_s;
  double jacobian_time_s;          /* Schur build (residual + Jacobian + elimination) */
  double linear_solver_time_s;     /* factorisation / PCG + back-substitution */
  double residual_time_s;          /* cost evaluations of candidate steps */
  /* Device time of individual kernels, from CUDA events recorded around their
   * launches on the solve's stream (used for roofline accounting). */
  double schur_kernel_time_s;      /* point-major Schur elimination kernel(s) */
  int32_t schur_kernel_launches;
  int32_t factor_launches;         /* kernels in the dense factorisation + solves */
  double factor_time_s;            /* dense Cholesky + triangular solves */
} gbba_summary;

typedef struct gbba_handle gbba_handle;

/* Create a handle bound to CUDA device `device`.  It owns a stream and a
 * workspace that is grown on demand and reused across solves. */
gbba_status gbba_create(int device, gbba_handle** out);
void gbba_destroy(gbba_handle* handle);
void gbba_default_options(gbba_options* options);
const char* gbba_status_string(gbba_status status);
int gbba_abi_version(void);
/* Number of CUDA kernel launches issued through this handle so far. */
int64_t gbba_launch_count(const gbba_handle* handle);
/* Device time (CUDA events on the call's stream) of the main kernel(s) of the
 * handle's last triangulation call (gbtri_*) or problem pack / write-back
 * (gbsfm_pack_ba, gbsfm_unpack_ba), without input checks and host copies;
 * GBBA_ERROR_NOT_SUPPORTED before any such call.  No counterpart in
 * the reference, which has no device kernels: it serves roofline accounting. */
gbba_status gbba_last_kernel_time(gbba_handle* handle, double* seconds);

/* Refine extrinsics, intrinsics and points in place: the replacement of
 * ceres::Solve with SPARSE_SCHUR/DENSE_SCHUR on the reference problems.
 * Parameters are written back only when the solution is usable. */
gbba_status gbba_solve(gbba_handle* handle, const gbba_problem* problem,
                       const gbba_options* options, gbba_summary* summary);

/* Solve `num_problems` independent problems (local-BA windows) in one call.
 * Each problem is solved with the same options; summaries[i] belongs to
 * problems[i].  All problems must use the same camera model and memory. */
gbba_status gbba_solve_batched(gbba_handle* handle, const gbba_problem* problems,
                               int32_t num_problems, const gbba_options* options,
                               gbba_summary* summaries);

/* Autotuner (no counterpart in the reference, whose ceres solve has no
 * tunable kernels).  It times `iterations` LM iterations of `problem` with
 * `options` on the device for each candidate of three choices, one after the
 * other, and keeps the fastest of each in the handle for its later solves:
 *   - the work-item size of the camera-pair products of the Schur build (one
 *     warp per item of at most `pair_chunk` observation pairs of one
 *     camera-pair block: smaller items spread the long diagonal blocks over
 *     more warps, larger ones read fewer partial sums), by the Schur phase's
 *     time (skipped on the iterative path, which forms no pair products);
 *   - for the dense FP32 factorisation, the engine of its trailing update:
 *     the tensor cores (tcgen05, 3xTF32) or the FP32 pipes, by the
 *     factorisation's time;
 *   - for the iterative (PCG) path, the warps per camera of its camera-side
 *     kernels (preconditioner blocks, implicit Schur products), by the time of
 *     the linear solver and the Schur phase together.
 * The problem's parameters are restored after each trial, so the call leaves
 * them unchanged. */
#define GBBA_TUNE_MAX_CANDIDATES 4
typedef struct gbba_tuning {
  int32_t pair_chunk;                                    /* chosen work-item size (pairs) */
  int32_t num_candidates;
  int32_t candidates[GBBA_TUNE_MAX_CANDIDATES];          /* 32, 64, 128 */
  double schur_time_s[GBBA_TUNE_MAX_CANDIDATES];         /* Schur-phase device time per LM iteration */
  int32_t factor_tensor;                                 /* chosen: 1 tensor cores, 0 FP32 pipes (-1: not tuned) */
  int32_t camera_warps;                                  /* chosen: 2, 4 or 8 (0: not tuned) */
  double factor_time_s[2];                               /* dense factorisation per LM iteration: FP32 pipes, tensor */
  double pcg_time_s[3];                                  /* linear solver + Schur phase per LM iteration: 2, 4, 8 warps */
} gbba_tuning;
gbba_status gbba_autotune(gbba_handle* handle, const gbba_problem* problem, const gbba_options* options,
                          int32_t iterations, gbba_tuning* tuning);

/* Differentiation contract, forward half: residuals r = pred - obs (not
 * robustified, [num_observations][2], may be NULL) and the robustified cost
 * 1/2 sum rho(|r|^2) (may be NULL).  Replaces ceres::Problem::Evaluate's
 * residual output (include/ceres/problem.h:392-468). */
gbba_status gbba_project_forward(gbba_handle* handle, const gbba_problem* problem,
                                 int32_t loss_type, double loss_scale,
                                 double* residuals, double* cost);

/* Differentiation contract, backward half: per-observation Jacobian blocks of
 * the robustified residual (ceres Corrector applied, corrector.cc:118-155),
 * row-major per block: jac_extrinsic [N_o][2][6], jac_intrinsic [N_o][2][k],
 * jac_point [N_o][2][3]; and the gradient J^T r of the robustified problem
 * laid out as [extrinsics | intrinsics | points] (same layout as the
 * parameters).  Any output may be NULL.  The projection is recomputed, no
 * intermediate of the forward call is stored. */
gbba_status gbba_project_backward(gbba_handle* handle, const gbba_problem* problem,
                                  int32_t loss_type, double loss_scale,
                                  double* jac_extrinsic, double* jac_intrinsic,
                                  double* jac_point, double* gradient);

/* The same contract for the Jacobian of the mixed-precision path
 * (GBBA_PRECISION_MIXED): the FP32 instantiation of the hand-written adjoint
 * that the mixed solve's Schur build evaluates, at FP32 copies of the
 * parameters and observations, with the residual and the Corrector scale in
 * FP64.  Outputs as for gbba_project_backward, widened to double.  Replaces
 * the same ceres::Problem::Evaluate Jacobian (problem.h:392-468), at FP32
 * accuracy. */
gbba_status gbba_project_backward_mixed(gbba_handle* handle, const gbba_problem* problem,
                                        int32_t loss_type, double loss_scale,
                                        double* jac_extrinsic, double* jac_intrinsic,
                                        double* jac_point, double* gradient);

/* Forward projection that allocates nothing.  It has no counterpart in the
 * reference; it exists for callers that cannot call cudaMalloc -- a host
 * application whose device memory is already owned by its own pool
 * allocator, or a real-time loop that may not pay an allocation's implicit
 * synchronisation.  Same outputs as gbba_project_forward (residuals r = pred -
 * obs, [num_observations][2], and the robustified cost 1/2 sum rho(|r|^2)),
 * but every array of `problem` and both outputs must be DEVICE memory on the
 * current device (problem->memory == GBBA_MEMORY_DEVICE; `cost` points to one
 * double, either output may be NULL), no handle is needed, and the call is
 * asynchronous on `stream` (a cudaStream_t; NULL is the default stream).
 * Its scratch is a fixed array inside the library (GBBA_NOALLOC_MAX_BLOCKS
 * partial sums, ~128 KB held by every GPU that loads the library until exit):
 * problems above GBBA_NOALLOC_MAX_BLOCKS * GBBA_NOALLOC_OBS_PER_BLOCK
 * observations (33,554,432) are rejected with GBBA_ERROR_TOO_LARGE.  The first
 * call on each device looks up the scratch's device address (a failed lookup
 * is retried by the next call); make that first call before any stream
 * capture.  All calls share the scratch: calls that overlap on the GPU race.
 * An out-of-range index yields NaN residuals for its observation and a NaN
 * cost instead of a fault; the next valid call is unaffected.  If a CUDA error
 * from the caller's earlier work is already pending on the calling thread, the
 * call does nothing and returns GBBA_ERROR_CUDA, leaving that error pending
 * (cudaPeekAtLastError / cudaGetLastError still report it to the caller). */
#define GBBA_NOALLOC_MAX_BLOCKS 16384
#define GBBA_NOALLOC_OBS_PER_BLOCK 2048
gbba_status gbba_project_forward_noalloc(const gbba_problem* problem, int32_t loss_type, double loss_scale,
                                         double* residuals, double* cost, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GBBA_H_ */
