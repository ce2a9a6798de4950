/*
 * pb_gpu.h -- C ABI of the GB300 reduced-Schur bundle-adjustment backend.
 *
 * The backend replaces plabundle's device Schur path behind
 *   plabundle::Solver::solve(const Problem&, const SolveOptions&, SolverWorkspace&)
 *   (include/plabundle/solver.h:40 in the reference), selected through
 *   SolveOptions.backend.requested (include/plabundle/options.h:151).
 * Inside the reference the seam is runConcreteBackend (src/solver.cpp:275-302), which calls
 *   internal::optimizePointsWithPlaMatrix(cameras, tracks, BAOptions, workspace)
 *   (src/internal/BundleAdjustPlaMatrix.h:27-30, src/internal/BundleAdjustPlaMatrix.cpp:162-631).
 * A context here plays the role of SolverWorkspace::Impl (src/solver.cpp:22-25): it owns the
 * device buffers, the reduced-matrix pattern and the launch shapes, and is reused by sequential
 * solves of problems with the same structure.
 *
 * Conventions
 *   - Every entry point returns a pb_status; no C++ exception crosses the boundary.
 *   - Host buffers are owned by the caller and only read or written during the call.
 *   - A context is used by one host thread at a time (SolverWorkspace rule,
 *     include/plabundle/solver.h:13-14); all its work runs on the context's own stream.
 *   - Cameras are records of PB_CAMERA_STRIDE doubles:
 *       0-8 camera-to-world rotation (row-major), 9-11 centre, 12 fx, 13 fy, 14 cx, 15 cy,
 *       16 k1, 17 k2, 18 k3, 19 p1, 20 p2, 21 u sign, 22 v sign, 23 depth flip, 24 width,
 *       25 height, 26-31 zero.
 *   - Observations are grouped by track: track_offsets[t]..track_offsets[t+1].
 *   - Reduced-system layout (pb_gpu_get_reduced): pose blocks of 6 columns
 *     [rotation(3), centre(3)] (the gauge scale camera uses [rotation(3), tangent(2), 0]) in
 *     camera-block order, followed by one column per refined intrinsic parameter of each
 *     calibration group.  The reference pads every primary block to 13 columns
 *     (src/internal/BundleAdjustPlaMatrixProblem.h:41); the padding carries no information.
 */
#ifndef PB_GPU_H
#define PB_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PB_CAMERA_STRIDE 32
#define PB_INTRINSIC_COUNT 13

typedef enum pb_status {
    PB_OK = 0,
    PB_ERR_INVALID_ARGUMENT = 1,
    PB_ERR_CUDA = 2,
    PB_ERR_NO_CONVERGENCE = 3,
    PB_ERR_SINGULAR_BLOCK = 4,
    PB_ERR_CANCELLED = 5,
    PB_ERR_BOUNDS = 6,
    PB_ERR_TIMEOUT = 7,
    PB_ERR_UNSUPPORTED = 8,
    PB_ERR_INVALID_PROJECTION = 9,
    PB_ERR_STATE = 10
} pb_status;

/* plabundle::SolveStatus numbering (include/plabundle/backend.h:17-27). */
typedef enum pb_solve_status {
    PB_SOLVE_NOT_RUN = 0,
    PB_SOLVE_SUCCESS = 1,
    PB_SOLVE_NO_CONVERGENCE = 2,
    PB_SOLVE_CANCELLED = 3,
    PB_SOLVE_INVALID_INPUT = 4,
    PB_SOLVE_UNSUPPORTED = 5,
    PB_SOLVE_BACKEND_UNAVAILABLE = 6,
    PB_SOLVE_NUMERICAL_FAILURE = 7
} pb_solve_status;

typedef enum pb_precision { PB_PRECISION_FP64 = 0, PB_PRECISION_MIXED = 1 } pb_precision;

typedef struct pb_gpu_ctx pb_gpu_ctx;

/* Problem in track-CSR form: plabundle::Problem (include/plabundle/problem.h:37-54) for frame
 * cameras (Track::initialPoint, Observation{cameraIndex,u,v,weight,measurementScale}). */
typedef struct pb_problem_desc {
    int32_t n_cameras;
    const double* cameras;                     /* n_cameras * PB_CAMERA_STRIDE */
    int32_t n_tracks;
    const int64_t* track_offsets;              /* n_tracks + 1 */
    const double* points;                      /* n_tracks * 3 */
    int64_t n_obs;
    const int32_t* obs_camera;
    const double* obs_u;
    const double* obs_v;
    const double* obs_weight;
    const double* obs_scale;
    int32_t n_fixed_cameras;
    const int32_t* fixed_cameras;
    int32_t n_fixed_tracks;
    const int32_t* fixed_tracks;
    const int32_t* calibration_group_ids;      /* n_cameras or NULL: Problem::cameraCalibrationGroupIds */
    const double* intrinsic_reference_cameras; /* n_cameras * 32 or NULL */
    /* Control-point constraints of the tracks (Track::controlPointConstraints,
     * ControlPointConstraint, include/plabundle/constraints.h:73-87, :127-133): n_control_points
     * entries; control_point_track[i] the track index; control_point_data[15 * i]: target point (3),
     * sigmaMeters, weight, uncertainty (0 isotropic sigma, 1 covariance, 2 square-root
     * information), uncertaintyMatrix (9, row-major).  May be 0 / NULL. */
    int32_t n_control_points;
    const int32_t* control_point_track;
    const double* control_point_data;
    /* Scale-bar constraints (Problem::scaleBarConstraints, ScaleBarConstraint,
     * include/plabundle/constraints.h:93-101): n_scale_bars entries; scale_bar_tracks[2 * i] and
     * [2 * i + 1] the two track indices; scale_bar_data[3 * i]: measuredDistanceMeters,
     * sigmaMeters, weight.  Their tracks become primary point blocks (prepareActiveProblem,
     * BundleAdjustPlaMatrixProblem.cpp:235-266) and the problem is solved on the general path.
     * May be 0 / NULL. */
    int32_t n_scale_bars;
    const int32_t* scale_bar_tracks;
    const double* scale_bar_data;
    /* Rig topology (Problem::rig, placamera::RigTopology, include/plabundle/problem.h:52; the
     * reference's README "Rig BA"): captures hold a rig-to-world rotation and the rig centre in
     * world coordinates, sensors a camera-to-rig rotation and the camera centre in rig
     * coordinates, and every camera is bound to one capture and one sensor of the same rig
     * (RigCameraBinding, resolved to indices by the caller).
     *   rig_captures[12 * k]: rigToWorldRotation (9, row-major), rigCenterInWorld (3);
     *   rig_capture_info[2 * k]: rigId, fixedPose (0/1);
     *   rig_sensors[12 * s]: cameraToRigRotation (9, row-major), cameraCenterInRig (3);
     *   rig_sensor_info[2 * s]: rigId, fixedExtrinsic (0/1);
     *   rig_camera_capture / rig_camera_sensor: n_cameras indices.
     * The composed camera is R = R_rig R_sensor, C = C_rig + R_rig c_sensor; the poses passed in
     * `cameras` are replaced by the composition (runConcreteBackend, src/solver.cpp:282).  Every
     * rig needs at least one fixed sensor.  The pose blocks are then one per non-fixed capture
     * followed by one per non-fixed sensor (prepareActiveProblem,
     * BundleAdjustPlaMatrixProblem.cpp:156-199) and the problem uses the plain parameterisation
     * (useReferencePointParameterization, BundleAdjustPlaMatrixAssembly.cpp:24-30).
     * n_rig_captures == 0: no rig. */
    int32_t n_rig_captures;
    const double* rig_captures;
    const int32_t* rig_capture_info;
    int32_t n_rig_sensors;
    const double* rig_sensors;
    const int32_t* rig_sensor_info;
    const int32_t* rig_camera_capture;
    const int32_t* rig_camera_sensor;
} pb_problem_desc;

/* SolveOptions (include/plabundle/options.h:58-187) as flat fields. */
typedef struct pb_solve_options {
    int32_t max_iterations;            /* SolverControlOptions::maxIterations */
    int32_t robust_loss;               /* ImageRobustLoss: 0 LS, 1 Huber, 2 Cauchy */
    double robust_loss_scale;          /* imageRobustLossScalePixels */
    double armijo_coefficient;         /* referenceArmijoCoefficient */
    int32_t line_search_steps;         /* referenceLineSearchSteps */
    int32_t enable_point_filter;
    double filter_max_reproj_error;
    double filter_sigma_factor;
    double max_initial_track_rms;
    int32_t refine_camera_pose;        /* CalibrationOptions::refineCameraPose */
    int32_t gauge_policy;              /* GaugePolicy: 0 AutoAnchor, 1 RequireExplicit, 2 CallerManaged */
    int32_t gauge_anchor_camera;       /* Gauge::referenceAnchorCameraIndex */
    int32_t gauge_scale_camera;        /* Gauge::referenceScaleCameraIndex */
    double gauge_baseline;             /* Gauge::referenceBaseline */
    uint32_t intrinsic_mask;           /* bit p: sharedIntrinsicParameterEnabled(options, p) */
    int32_t precision;                 /* pb_precision */
    int32_t max_linear_iterations;     /* 0: max(200, 30 * primary blocks) */
    double linear_relative_tolerance;  /* 0: 2e-10 (online Schur path) */
    double linear_absolute_tolerance;  /* 0: 1e-12 */
    int32_t refinement_sweeps;         /* block-Jacobi mixed path: 1..3 refinement sweeps (unused by dense CG) */
    int32_t preconditioner_cluster_size; /* BackendOptions::plaMatrixPreconditionerClusterSize (1..16;
                                          * accepted, the solution does not depend on it) */
    int32_t linear_solver;             /* 0 auto, 1 dense-Cholesky-preconditioned CG, 2 block-Jacobi PCG */
    double calibration[32];            /* CalibrationOptions numeric fields (27 used) */
    double control_point_weight;       /* ConstraintOptions::controlPointWeight (1) */
    double control_point_huber_delta;  /* ConstraintOptions::controlPointHuberDeltaMeters (0.2) */
    int32_t factor_reuse;              /* dense-factor reuse across LM iterations: 0 default (the mixed
                                        * path keeps its FP32 factor while it preconditions well, the
                                        * FP64 path refactors every iteration), 1 keep on both paths,
                                        * 2 refactor every iteration on both paths */
    int32_t general_path;              /* 1: the general path (SolverControlOptions::useReferenceOnlineSchur
                                        * = false): undamped equations per linearisation, damped Schur
                                        * solve to 1e-12, finite-difference directional decrease, retry
                                        * with ten times the damping at the same state; 0: the online
                                        * reference path (a problem with scale bars always takes the
                                        * general path, as canUseReferenceOnlineSchur decides,
                                        * BundleAdjustPlaMatrixReferenceSchur.cpp:667-673) */
    double scale_bar_weight;           /* ConstraintOptions::scaleBarWeight (1) */
    double scale_bar_huber_delta;      /* ConstraintOptions::scaleBarHuberDeltaMeters (0.2) */
} pb_solve_options;

/* PlaMatrixDiagnostics (include/plabundle/result.h:91-128) + QualitySummary fields. */
typedef struct pb_solve_report {
    int32_t status;                    /* pb_solve_status */
    int32_t solution_usable;
    int32_t iterations;
    int32_t accepted_steps;
    int32_t rejected_steps;
    int32_t linearizations;
    int32_t objective_evaluations;
    int32_t linear_iterations;
    int32_t refinement_sweeps;
    int32_t active_tracks;
    int32_t observation_count;
    int32_t rejected_initial_tracks;
    int32_t optimized_tracks;
    int32_t camera_blocks;
    int32_t intrinsic_blocks;
    int32_t pattern_builds;
    int32_t pattern_reuses;
    int32_t gpu_kernel_launches;
    double initial_cost;
    double final_cost;
    double mean_rms_before;
    double mean_rms_after;
    double valid_track_ratio;
    double filter_threshold;
    double assembly_ms;
    double linear_ms;
    double back_substitution_ms;
    double objective_ms;
    double total_ms;
    int32_t promoted_point_blocks;     /* tracks of scale bars solved as primary point blocks */
    int32_t general_path_used;         /* 1 when the solve ran on the general path */
    int32_t rig_capture_blocks;        /* ActiveProblem::rigCaptureBlockCount (0 without a rig) */
    int32_t rig_sensor_blocks;         /* ActiveProblem::rigSensorBlockCount */
} pb_solve_report;

/* Context lifetime (SolverWorkspace construction / clear()). */
pb_status pb_gpu_create(int32_t device, pb_gpu_ctx** out);
pb_status pb_gpu_destroy(pb_gpu_ctx* ctx);
const char* pb_gpu_last_error(const pb_gpu_ctx* ctx);
const char* pb_status_name(int32_t status);

/* Uploads a problem: validation, AutoAnchor gauge (BundleAdjustValidation.cpp:814-893),
 * active-track gate and block numbering (BundleAdjustPlaMatrixProblem.cpp:29-278), intrinsic
 * groups (BundleAdjustPlaMatrixModel.cpp:84-231), reduced pattern and launch shapes
 * (prepareOffDiagonalTopology, BundleAdjustPlaMatrixReferenceSchur.cpp:568-659).  The pattern is
 * reused when a later upload has the identical structure. */
pb_status pb_gpu_upload(pb_gpu_ctx* ctx, const pb_problem_desc* problem, const pb_solve_options* options);

/* Reset the state to the uploaded initial cameras/points (device-side copy, no host traffic). */
pb_status pb_gpu_reset_state(pb_gpu_ctx* ctx);

/* Sizes: [n_cameras, n_tracks, n_obs, primary blocks, camera blocks, intrinsic blocks,
 *         track blocks, active tracks, observation count, rejected initial tracks,
 *         n_pairs (upper off-diagonal pairs, reference numbering), reduced dimension,
 *         intrinsic columns per group, gauge anchor, gauge scale, chunks]. */
pb_status pb_gpu_get_sizes(pb_gpu_ctx* ctx, int64_t* sizes, double* gauge_baseline);
pb_status pb_gpu_get_active(pb_gpu_ctx* ctx, int8_t* active_track, int32_t* camera_block,
                            int32_t* intrinsic_block, int32_t* track_block);
/* Upper-triangular primary block pairs (row < col) in the reference's slot order. */
pb_status pb_gpu_get_pairs(pb_gpu_ctx* ctx, int32_t* pairs);

/* Kernel (a): per-observation residual, point Jacobian (2x3, scaled), pose Jacobian (2x6 as
 * scattered for the camera block), intrinsic Jacobian (2x13), normal weight, robust cost and a
 * validity flag, at the current state, in the original observation order.  For a rig problem the
 * pose Jacobian is the composed camera's own (before the chain to its capture and sensor). */
pb_status pb_gpu_linearize_observations(pb_gpu_ctx* ctx, int32_t precision, double* residual,
                                        double* point_jacobian, double* pose_jacobian,
                                        double* intrinsic_jacobian, double* normal_weight, double* cost,
                                        int8_t* valid);

/* Kernel (b): online point Schur (buildReferenceReducedNormalEquations,
 * BundleAdjustPlaMatrixReferenceSchur.cpp:675-980) with damping lambda. */
pb_status pb_gpu_linearize_schur(pb_gpu_ctx* ctx, double lambda, int32_t precision, double* cost,
                                 int32_t* point_system_singular);
/* Dense copy of the reduced system (dimension from pb_gpu_get_sizes) and its right-hand sides:
 * rhs = -gradient, direct_rhs = the image terms before point elimination (directPrimaryRhs). */
pb_status pb_gpu_get_reduced(pb_gpu_ctx* ctx, double* dense_matrix, double* rhs, double* direct_rhs);

/* Kernel (c): solve of the damped reduced system (solveDampedSchurComplement, call site
 * BundleAdjustPlaMatrix.cpp:311-357).  Up to 32768 unknowns on the mixed path (16384 on the
 * FP64 path): conjugate gradients on the FP64 matrix preconditioned by a dense Cholesky factor
 * of the Jacobi-scaled matrix (FP32 factor on the mixed path, FP64 on the FP64 path); larger
 * systems: block-Jacobi PCG.  One cooperative kernel per solve. */
pb_status pb_gpu_solve_reduced(pb_gpu_ctx* ctx, double* step, int32_t* converged, int32_t* iterations,
                               double* relative_residual);
/* (For a rig problem, `step` is the solution over the rig blocks, captures then sensors, 6 columns
 * each, followed by the intrinsic columns: the system pb_gpu_get_reduced copies, of the dimension
 * pb_gpu_get_sizes reports.) */

/* Kernel (d1): back-substitution (recoverReferencePointSteps, ...ReferenceSchur.cpp:982-1082);
 * eliminated_step is in track-block order. */
pb_status pb_gpu_back_substitute(pb_gpu_ctx* ctx, double* eliminated_step, double* directional_decrease,
                                 int32_t* success);

/* Kernel (d2): objective at the current state and at trial states state (+) alpha_k * step. */
pb_status pb_gpu_eval_cost(pb_gpu_ctx* ctx, double* cost);
pb_status pb_gpu_eval_cost_batch(pb_gpu_ctx* ctx, const double* alphas, int32_t n_alphas, double* costs);
pb_status pb_gpu_apply_step(pb_gpu_ctx* ctx, double alpha);

/* Whole LM solve (the online branch of optimizePointsWithPlaMatrix and
 * finalizeBundleAdjustResult, src/internal/BundleAdjustQuality.cpp:403-502). */
pb_status pb_gpu_solve(pb_gpu_ctx* ctx, const pb_solve_options* options, pb_solve_report* report);

/* Results: refined cameras (published intrinsics applied), points, per-track valid mask and
 * strict RMS before/after, intrinsic group parameters (n_groups * 13). Any pointer may be NULL. */
pb_status pb_gpu_download_state(pb_gpu_ctx* ctx, double* cameras, double* points, int8_t* valid,
                                double* rms_before, double* rms_after, double* intrinsics);

/* Cost history of the last pb_gpu_solve (no counterpart in the reference, whose diagnostics keep
 * only the initial and final costs, include/plabundle/result.h:91-128): the initial cost, then the
 * cost after every accepted LM step, with the LM iteration (0 for the initial cost) and the host
 * time in ms since the solve started.  *count receives the number of entries; at most `capacity`
 * are written; any array may be NULL. */
pb_status pb_gpu_get_history(pb_gpu_ctx* ctx, int32_t capacity, int32_t* iterations, double* costs, double* ms,
                             int32_t* count);

/* Rig problems: the current capture and sensor parameters (Result::refinedRig,
 * include/plabundle/result.h:149), 12 doubles each in the layout of pb_problem_desc's
 * rig_captures / rig_sensors, and the pose block of every capture and sensor (-1: fixed or without
 * residuals; ActiveProblem::rigCaptureBlockByCamera / rigSensorBlockByCamera,
 * BundleAdjustPlaMatrixProblem.h:13-39, per capture / sensor instead of per camera).  Any pointer
 * may be NULL.  PB_ERR_STATE when the uploaded problem has no rig. */
pb_status pb_gpu_get_rig(pb_gpu_ctx* ctx, double* captures, double* sensors, int32_t* capture_block,
                         int32_t* sensor_block);

/* One call: upload + solve + download (the path a caller of Solver::solve takes). */
pb_status pb_gpu_solve_problem(pb_gpu_ctx* ctx, const pb_problem_desc* problem, const pb_solve_options* options,
                               pb_solve_report* report, double* cameras_out, double* points_out, int8_t* valid_out,
                               double* rms_before, double* rms_after);

/* Cooperative cancellation (SolverControlOptions::cancelFlag): checked between LM iterations. */
pb_status pb_gpu_request_cancel(pb_gpu_ctx* ctx, int32_t cancel);

/* The context's CUDA stream (cudaStream_t), so that callers can order their own work and CUDA
 * events with the backend's kernels. */
pb_status pb_gpu_get_stream(pb_gpu_ctx* ctx, void** stream);

/* Enables per-phase CUDA-event timing of the following solves (adds one synchronisation per
 * timed phase; off by default). */
pb_status pb_gpu_set_timing(pb_gpu_ctx* ctx, int32_t enable);

/* Device time of the last solve's dominant kernels: [assembly kernel ms, assembly launches,
 * pcg kernel ms, pcg launches, cost kernel ms, cost launches, reduce kernel ms, reduce launches],
 * filled when timing is enabled. */
pb_status pb_gpu_kernel_times(pb_gpu_ctx* ctx, double* out8);

/* Batched solves of independent problems, e.g. local bundle-adjustment windows (no counterpart
 * in the reference, which solves one problem per Solver::solve call).  Each problem is solved
 * exactly as pb_gpu_solve_problem solves it, with the same options; n_workers host threads each
 * own a context and its stream and take problems from a shared queue, so the kernels of
 * different problems overlap on the device.  Per problem i: reports[i], and, when the pointer
 * arrays and their entries are non-NULL, refined cameras / points / valid mask into
 * cameras_out[i], points_out[i], valid_out[i], and the wall-clock time of its solve in
 * latency_ms[i] (may be NULL).  Returns PB_OK, or the first failing status of any problem
 * (all reports are still filled). */
pb_status pb_gpu_solve_batch(int32_t device, int32_t n_problems, const pb_problem_desc* problems,
                             const pb_solve_options* options, int32_t n_workers, pb_solve_report* reports,
                             double* const* cameras_out, double* const* points_out, int8_t* const* valid_out,
                             double* latency_ms);

/* Device-side snapshot of the current state (poses, points, group intrinsics) and its restore
 * (no counterpart in the reference).  Together with pb_gpu_set_observations they re-solve a
 * problem after a measurement update from a known state without a new upload, e.g. the
 * warm-started re-solves of a finite-difference check of pb_gpu_backward.  A new upload drops
 * the snapshot. */
pb_status pb_gpu_save_state(pb_gpu_ctx* ctx);
pb_status pb_gpu_restore_state(pb_gpu_ctx* ctx);
/* Replaces the measurements (u, v) of n observations, given by their original index, in the
 * uploaded problem (no counterpart in the reference).  The gauge, the active-track gate and the
 * intrinsic groups decided at upload are kept. */
pb_status pb_gpu_set_observations(pb_gpu_ctx* ctx, int64_t n, const int64_t* index, const double* u, const double* v);

/* Backward pass: implicit differentiation of the converged solve (no counterpart in the
 * reference, which has no adjoint).  At the fixed point of the current state, for a scalar loss
 * L of the refined state with partial derivatives
 *   grad_cameras     n_cameras * 6: dL/d(final pose) as (rotation increment of the solver's pose
 *                    retraction C2W' = D E(w)^T D C2W, E = Rx Ry Rz, D = diag(1,-1,-1); world
 *                    centre), or NULL;
 *   grad_points      n_tracks * 3: dL/d(final point), world, or NULL;
 *   grad_intrinsics  n_groups * 13: dL/d(group parameter), or NULL;
 * it solves H mu = dL/dz with H the exact Hessian of the robust objective (robust-loss second
 * derivatives and residual curvature included) reduced over the points and solved by the same
 * dense-Cholesky-preconditioned CG / block-Jacobi PCG as the forward solve, and returns
 *   grad_observations     n_obs * 2: dL/d(u, v) (original order; 0 for unused observations);
 *   grad_initial_cameras  n_cameras * 6: dL/d(initial pose) as (rotation increment, centre).
 *                         Non-zero only through the gauge: fixed cameras (their final pose is
 *                         the initial one) and the AutoAnchor baseline, which is taken from the
 *                         initial centres of the anchor and scale cameras;
 *   grad_initial_points   n_tracks * 3: dL/d(initial point), non-zero for fixed tracks only.
 * Any output may be NULL.  The state must be a converged fixed point of the uploaded problem
 * (after pb_gpu_solve); clamped intrinsics are treated as free.  The reduced-system buffers are
 * reused, so a pb_gpu_linearize_schur is needed before the next pb_gpu_solve_reduced.  The
 * reduced system is summed in a fixed order without atomics; only the few gauge and fixed-
 * camera cross terms of the gradients use FP64 atomics, so those entries of
 * grad_initial_cameras / grad_initial_points may vary in the last bits from run to run. */
typedef struct pb_adjoint_report {
    int32_t status;                /* pb_status of the call */
    int32_t linear_iterations;     /* CG / PCG iterations of the adjoint solve */
    int32_t gpu_kernel_launches;
    int32_t point_blocks_singular; /* 1 when a point block of the exact Hessian was singular */
    double relative_residual;      /* |H mu - dL/dz| / |dL/dz| of the reduced solve */
    double hessian_ms;             /* exact-Hessian records and the reduced system */
    double solve_ms;
    double gradient_ms;            /* back-substitution and the gradients */
    double total_ms;
} pb_adjoint_report;
pb_status pb_gpu_backward(pb_gpu_ctx* ctx, const double* grad_cameras, const double* grad_points,
                          const double* grad_intrinsics, double* grad_observations, double* grad_initial_cameras,
                          double* grad_initial_points, pb_adjoint_report* report);

/* One Newton step of the robust objective from the current state with the exact Hessian of the
 * backward pass, applied without a line search (no counterpart in the reference).  For polishing
 * a converged state to its fixed point well past the LM stopping rule, e.g. the re-converged
 * solves of a finite-difference check; from a state far from a minimum the exact Hessian can be
 * indefinite and the call fails with PB_ERR_SINGULAR_BLOCK.  step_max: largest |primary step
 * component|; gradient_norm: |reduced gradient| at the state before the step (may be NULL). */
pb_status pb_gpu_newton_step(pb_gpu_ctx* ctx, double* step_max, double* gradient_norm);

/* ---- Internal block-Schur interface: the general (non-online) path's linear solve ----------
 *
 * pb_bne is plamatrix::internal::BlockNormalEquations<double> (PlaMatrix is absent from the
 * reference tree; its interface is restated from the reference's use sites): block normal
 * equations H x = -g with primary blocks of primary_block_size columns (13 in the reference,
 * src/internal/BundleAdjustPlaMatrixProblem.h:41) and eliminated blocks of 3 (points).  A
 * residual block r (rows) with Jacobians J_b and weight w adds H_bc += w J_b^T J_c and
 * g_b += w J_b^T r for every pair of its blocks.  A container is filled by one thread at a time;
 * per-thread shards are merged, as the reference's OpenMP assembly does
 * (src/internal/BundleAdjustPlaMatrixAssembly.cpp:843-912).  Jacobians are row-major,
 * rows x block size.  Host-side only: no call below touches the GPU. */
#define PB_BNE_MAX_PRIMARY_BLOCK_SIZE 16
typedef struct pb_bne pb_bne;
/* BlockNormalEquations<double>(primaryBlocks, eliminatedBlocks, primaryBlockSize, eliminatedBlockSize)
 * (BundleAdjustPlaMatrixAssembly.cpp:856-857); eliminated_block_size must be 3. */
pb_status pb_bne_create(int32_t primary_blocks, int32_t eliminated_blocks, int32_t primary_block_size,
                        int32_t eliminated_block_size, pb_bne** out);
pb_status pb_bne_destroy(pb_bne* eq);
/* clearValues (BundleAdjustPlaMatrixAssembly.cpp:861): zeroes every value, keeps the pattern. */
pb_status pb_bne_clear_values(pb_bne* eq);
/* [primaryBlockCount, eliminatedBlockCount, primaryBlockSize, eliminatedBlockSize, stored upper
 * primary pairs, stored primary-eliminated couplings] (BundleAdjustPlaMatrixAssembly.cpp:851-854). */
pb_status pb_bne_sizes(const pb_bne* eq, int32_t* sizes6);
/* addResidualBlocks(primary, primaryJacobians, n, eliminated, eliminatedJacobian, residual, rows,
 * weight) (BundleAdjustPlaMatrixAssembly.cpp:413-421); eliminated < 0: no eliminated block. */
pb_status pb_bne_add_residual_blocks(pb_bne* eq, const int32_t* primary, const double* const* primary_jacobians,
                                     int32_t n_primary, int32_t eliminated, const double* eliminated_jacobian,
                                     const double* residual, int32_t rows, double weight);
/* addPrimaryResidualBlocks (BundleAdjustPlaMatrixAssembly.cpp:431-437, AssemblySurvey.cpp:35-40). */
pb_status pb_bne_add_primary_residual_blocks(pb_bne* eq, const int32_t* primary, const double* const* primary_jacobians,
                                             int32_t n_primary, const double* residual, int32_t rows, double weight);
/* addPrimaryResidualBlock(block, J, r, rows[, w]) (BundleAdjustPlaMatrixAssembly.cpp:373,
 * AssemblySurvey.cpp:80-84: the priors, weight 1). */
pb_status pb_bne_add_primary_residual_block(pb_bne* eq, int32_t block, const double* jacobian, const double* residual,
                                            int32_t rows, double weight);
/* addEliminatedResidualBlock (BundleAdjustPlaMatrixAssembly.cpp:376-377, :423-428). */
pb_status pb_bne_add_eliminated_residual_block(pb_bne* eq, int32_t block, const double* jacobian,
                                               const double* residual, int32_t rows, double weight);
/* addResidualBlock: one primary and one eliminated block. */
pb_status pb_bne_add_residual_block(pb_bne* eq, int32_t primary, const double* primary_jacobian, int32_t eliminated,
                                    const double* eliminated_jacobian, const double* residual, int32_t rows,
                                    double weight);
/* addPrimaryGradientBlock / addPrimaryHessianBlock(row, col, block)
 * (BundleAdjustPlaMatrixReferenceSchur.cpp:911-926); a block below the diagonal (row > col) is
 * stored as the transpose of its upper mirror. */
pb_status pb_bne_add_primary_gradient_block(pb_bne* eq, int32_t block, const double* gradient);
pb_status pb_bne_add_primary_hessian_block(pb_bne* eq, int32_t row_block, int32_t col_block, const double* block);
/* finalizePrimaryDiagonal(scale, add) (BundleAdjustPlaMatrixReferenceSchur.cpp:930): non-zero
 * primary diagonal entries are multiplied by scale, zero ones are set to add. */
pb_status pb_bne_finalize_primary_diagonal(pb_bne* eq, double scale, double add);
/* mergeFrom / mergeEliminatedShardFrom(shard, offset) (BundleAdjustPlaMatrixAssembly.cpp:899-912):
 * adds every value of the other container; a shard's eliminated block k is block offset + k. */
pb_status pb_bne_merge_from(pb_bne* eq, const pb_bne* other);
pb_status pb_bne_merge_eliminated_shard_from(pb_bne* eq, const pb_bne* shard, int32_t eliminated_offset);
/* Dense copy (any pointer may be NULL): primary matrix (P*pb)^2 with both triangles, primary
 * gradient, eliminated blocks (E*9), eliminated gradient (E*3), couplings: (eliminated, primary)
 * index pairs and pb x 3 blocks in storage order (sizes[5] of them). */
pb_status pb_bne_export(const pb_bne* eq, double* primary_matrix, double* primary_gradient, double* eliminated_blocks,
                        double* eliminated_gradient, int32_t* coupling_index, double* couplings);

/* SchurComplementSolverOptions (BundleAdjustPlaMatrix.cpp:317-340). */
typedef struct pb_schur_options {
    int32_t max_iterations;              /* maxIterations; 0: max(200, 30 * primary blocks) */
    double relative_tolerance;           /* relativeTolerance; 0: 1e-12 (the general path's) */
    double absolute_tolerance;           /* absoluteTolerance; 0: 1e-12 */
    int32_t preconditioner_cluster_size; /* accepted (1..16); the dense-factor preconditioner subsumes any grouping */
    int32_t use_initial_guess;           /* useInitialGuess: primary_step holds the start vector on entry */
    int32_t use_mixed_precision;         /* useMixedPrecision: FP32 factor preconditioning the FP64 CG */
} pb_schur_options;

/* SchurComplementSolverReport (BundleAdjustPlaMatrix.cpp:372-399). */
typedef struct pb_schur_report {
    int32_t converged;
    int32_t iterations;
    int32_t schur_pattern_reused;
    int32_t schur_assembly_on_device;
    int32_t mixed_precision_used;
    int32_t symbolic_analysis_reused;
    int32_t eliminated_singular;         /* an eliminated block was singular after damping */
    double relative_residual;            /* |b - S x| / |b| of the damped reduced system (residual check) */
    double small_block_inverse_ms;
    double schur_accumulation_ms;
    double schur_assembly_ms;
    double cholesky_factorization_ms;
    double triangular_solve_ms;          /* the preconditioned CG */
    double linear_solve_ms;
    double back_substitution_ms;
    double total_ms;
    char preconditioner_name[64];
    char device_name[64];
} pb_schur_report;

/* solveDampedSchurComplement(equations, damping, options, workspace, &primary, &eliminated)
 * (call sites src/internal/BundleAdjustPlaMatrix.cpp:349-357, src/linescan_plamatrix.cpp:147-158)
 * on the context's device and stream: damping scales the diagonals of the primary and eliminated
 * blocks by (1 + damping) (a zero primary diagonal entry becomes 1); the eliminated blocks are
 * Schur-eliminated, the reduced system is solved by CG preconditioned with a dense Cholesky factor
 * (FP64, or FP32 with use_mixed_precision) to the tolerances, and the eliminated steps are
 * back-substituted.  primary_step: P * primary_block_size, eliminated_step: E * 3 (host).  A
 * singular eliminated block or a reduced system that is not positive definite returns
 * PB_ERR_SINGULAR_BLOCK with a "numerically SPD (positive definite)" message, which the reference
 * driver treats as a retryable breakdown (BundleAdjustPlaMatrix.cpp:34-40); a system that did not
 * reach the tolerance returns PB_OK with report->converged = 0.  The pattern is reused while the
 * container's structure is unchanged (report->schur_pattern_reused).  Reduced dimension up to
 * 16384 (32768 with use_mixed_precision), else PB_ERR_UNSUPPORTED. */
pb_status pb_gpu_solve_damped_schur(pb_gpu_ctx* ctx, const pb_bne* equations, double damping,
                                    const pb_schur_options* options, double* primary_step, double* eliminated_step,
                                    pb_schur_report* report);

/* Allocation-free robust objective of caller-owned device arrays.  No counterpart in the
 * reference: it serves callers that keep their own cameras, points and observations in device
 * memory and may not allocate (a real-time loop whose device memory is reserved up front, where
 * a cudaMalloc or cudaFree would synchronise the device and stall its other streams), and that
 * cannot create a context (pb_gpu_create / pb_gpu_upload allocate).  It is the line-search cost
 * kernel with its per-block partials in one fixed file-scope device array:
 *   - cameras: n_cameras * PB_CAMERA_STRIDE records (effective intrinsics), points: n_points * 3,
 *     observations: camera index, point index, u, v and w = weight / measurementScale^2; all
 *     device pointers, read only;
 *   - cost (host): sum of the robust costs of the observations that project validly;
 *     invalid_projections (host, may be NULL): how many did not (behind the camera, non-finite);
 *   - at most PB_NOALLOC_MAX_OBS observations, else PB_ERR_BOUNDS before any launch; a camera or
 *     point index out of range is skipped on the device and reported as PB_ERR_BOUNDS;
 *   - the scratch array is shared by all calls on a device: calls that overlap in time on one
 *     device race, so callers serialise them; nothing in it has to start at zero (every element
 *     read is written earlier in the same call);
 *   - the first call on a device resolves the array's address (cudaGetSymbolAddress, which may
 *     load the module), so that first call should come before any stream capture; the address
 *     is kept for the life of the process, so the call must not be used across a
 *     cudaDeviceReset of that device;
 *   - work is enqueued on `stream` (a cudaStream_t, NULL for the legacy default stream); the call
 *     copies its three totals back and synchronises `stream` before it returns;
 *   - an error already pending on the calling thread (cudaPeekAtLastError) is left in place and
 *     the call returns PB_ERR_CUDA without launching. */
#define PB_NOALLOC_MAX_OBS 4194304
pb_status pb_gpu_objective_noalloc(const double* cameras, int32_t n_cameras, const double* points, int32_t n_points,
                                   const int32_t* obs_camera, const int32_t* obs_point, const double* obs_u,
                                   const double* obs_v, const double* obs_w, int64_t n_obs, int32_t robust_loss,
                                   double robust_loss_scale, void* stream, double* cost, int64_t* invalid_projections);

#ifdef __cplusplus
}
#endif

#endif /* PB_GPU_H */
