/*
 * ba_oracle.h -- CPU FP64 restatement of plabundle's reduced-Schur bundle adjustment: the online
 * reduced-Schur path and the general path (block normal equations + damped Schur solve).
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg (and `bench.py --impl reference`) may load this library; the
 * product path never does.
 *
 * Parity status: UNPINNED.  The reference cannot be built here (its linear solver
 * PlaMatrix and camera model PlaCamera are not vendored and not installed) and its
 * tests carry no golden vectors for this path.  This file restates the reference's
 * own in-tree algorithm; the external pieces are restated from the reference's call
 * sites and in-tree templates:
 *   - projection: src/internal/BundleAdjustProjection.h:58-91 (Brown-Conrady, OpenCV
 *     tangential convention, depth test 1e-9);
 *   - intrinsic Jacobian column mapping: src/internal/CameraState.cpp:427-474;
 *   - damping form of the online Schur path: V and reduced diagonals x (1 + lambda)
 *     (src/internal/BundleAdjustPlaMatrixReferenceSchur.cpp:362-365, :930);
 *   - finalizePrimaryDiagonal(scale, add): positive diagonal entries are scaled,
 *     structurally empty (zero) diagonal entries are set to `add`;
 *   - finiteMedian: median of the finite values, mean of the two middle values for
 *     an even count;
 *   - 3x3 inverse: adjugate / determinant, singular when |det| <= 1e-15.
 * Same layout conventions as include/pb_gpu.h (camera records of 32 doubles).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_CAMERA_STRIDE = 32 };

typedef struct orc_problem {
    int32_t n_cameras;
    const double* cameras;               /* n_cameras * 32 */
    int32_t n_tracks;
    const int64_t* track_offsets;        /* n_tracks + 1, observations grouped by track */
    const double* points;                /* n_tracks * 3 (initial points) */
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
    const int32_t* calibration_group_ids; /* n_cameras or NULL */
    const double* intrinsic_reference_cameras; /* n_cameras * 32 or NULL */
    /* control points (Track::controlPointConstraints): track index and 15 doubles each --
     * target (3), sigmaMeters, weight, uncertainty kind (0 sigma, 1 covariance, 2 sqrt
     * information), matrix (9, row-major) */
    int32_t n_control_points;
    const int32_t* control_point_track;
    const double* control_point_data;
    /* scale bars (Problem::scaleBarConstraints): two track indices and (measuredDistanceMeters,
     * sigmaMeters, weight) each; their active, non-fixed tracks become primary point blocks and
     * the problem is solved on the general path */
    int32_t n_scale_bars;
    const int32_t* scale_bar_tracks;
    const double* scale_bar_data;
    /* rig topology (Problem::rig): captures (rigToWorldRotation 9, rigCenterInWorld 3) with
     * (rigId, fixedPose), sensors (cameraToRigRotation 9, cameraCenterInRig 3) with (rigId,
     * fixedExtrinsic), and the capture and sensor index of every camera; n_rig_captures == 0: none */
    int32_t n_rig_captures;
    const double* rig_captures;
    const int32_t* rig_capture_info;
    int32_t n_rig_sensors;
    const double* rig_sensors;
    const int32_t* rig_sensor_info;
    const int32_t* rig_camera_capture;
    const int32_t* rig_camera_sensor;
} orc_problem;

typedef struct orc_options {
    int32_t max_iterations;
    int32_t robust_loss;            /* 0 least squares, 1 Huber, 2 Cauchy */
    double robust_loss_scale;
    double armijo_coefficient;
    int32_t line_search_steps;
    int32_t enable_point_filter;
    double filter_max_reproj_error;
    double filter_sigma_factor;
    double max_initial_track_rms;
    int32_t refine_camera_pose;
    int32_t gauge_policy;           /* 0 AutoAnchor, 1 RequireExplicitGauge, 2 CallerManaged */
    int32_t gauge_anchor_camera;
    int32_t gauge_scale_camera;
    double gauge_baseline;
    uint32_t intrinsic_mask;        /* bit p set: shared intrinsic parameter p refined */
    int32_t num_threads;            /* 0: all OpenMP threads */
    int32_t linear_solver;          /* 0 auto, 1 dense Cholesky, 2 block-Jacobi PCG */
    int32_t max_linear_iterations;  /* 0: max(50, 12 * primary blocks) */
    double linear_relative_tolerance;
    double linear_absolute_tolerance;
    double calibration[32];         /* CalibrationOptions numeric fields, see ORC_CAL_* */
    double control_point_weight;    /* ConstraintOptions::controlPointWeight */
    double control_point_huber_delta; /* ConstraintOptions::controlPointHuberDeltaMeters */
    int32_t general_path;           /* 1: the general path (useReferenceOnlineSchur = false) */
    /* 1: a linear solve counts as converged only when its true residual |b - S x| passes the
     * tolerance (the reference's post-solve check of its direct CPU path); 0: the refined direct
     * solution (or the PCG on its recursive residual) is accepted, as a CG solver that stops on
     * its recursive residual does.  Near a fixed point of an ill-conditioned problem the true
     * residual sits at the FP64 floor, where 1 rejects the step and ends the solve on a damped
     * step. */
    int32_t residual_gate;
    double scale_bar_weight;        /* ConstraintOptions::scaleBarWeight */
    double scale_bar_huber_delta;   /* ConstraintOptions::scaleBarHuberDeltaMeters */
} orc_options;

typedef struct orc_report {
    int32_t status;                 /* plabundle::SolveStatus numbering */
    int32_t solution_usable;
    int32_t iterations;
    int32_t accepted_steps;
    int32_t rejected_steps;
    int32_t linearizations;
    int32_t objective_evaluations;
    int32_t linear_iterations;
    double initial_cost;
    double final_cost;
    int32_t active_tracks;
    int32_t observation_count;
    int32_t rejected_initial_tracks;
    int32_t optimized_tracks;
    double mean_rms_before;
    double mean_rms_after;
    double valid_track_ratio;
    double filter_threshold;
    double solve_seconds;
    double assembly_seconds;
    double linear_seconds;
} orc_report;

void* orc_create(const orc_problem* problem, const orc_options* options, int32_t* status);
void orc_destroy(void* handle);
/* validateControlPointConstraint + makeControlPointWhitening of one 15-double control-point
 * record: 1 and the whitening W (row-major 3x3) when valid, else 0. */
int32_t orc_control_point_whitening(const double* record, double* W);
/* counts: [primary, camera_blocks, intrinsic_blocks, track_blocks, active_tracks,
 *          observation_count, rejected_initial_tracks, n_pairs(after first build),
 *          gauge_anchor, gauge_scale, fixed_cameras, first fixed camera (-1: none),
 *          reference point parameterisation (1) or plain (0)] */
int32_t orc_info(void* handle, int32_t* counts, double* gauge_baseline);
int32_t orc_active(void* handle, int8_t* active_track, int32_t* camera_block, int32_t* intrinsic_block,
                   int32_t* track_block);
/* Per-observation linearisation at the initial state (all observations; invalid ones flagged).
 * residual[2], point_jacobian[6], pose_jacobian[2*13] (the camera primary term as
 * scattered by observationPrimaryTerms, zero when the camera has no block),
 * intrinsic_jacobian[2*13], normal_weight, cost, valid. */
int32_t orc_linearize_observations(void* handle, double* residual, double* point_jacobian, double* pose_jacobian,
                                   double* intrinsic_jacobian, double* normal_weight, double* cost, int8_t* valid);
/* Builds the damped reduced system at the current state. */
int32_t orc_build(void* handle, double damping, double* cost, int32_t* singular);
int32_t orc_pairs(void* handle, int32_t* pairs);
int32_t orc_reduced(void* handle, double* diagonal, double* off_diagonal, double* gradient, double* direct_rhs);
int32_t orc_solve_linear(void* handle, double* primary_step, int32_t* converged, int32_t* iterations);
int32_t orc_back_substitute(void* handle, const double* primary_step, double* eliminated_step,
                            double* directional_decrease, int32_t* success);
double orc_cost(void* handle);
/* General path: buildNormalEquations at the current state into the handle's block normal
 * equations; counts: [primary blocks, eliminated blocks, couplings]. */
int32_t orc_general_build(void* handle, double* cost, int32_t* counts);
/* Dense primary matrix ((13 P)^2, both triangles), primary gradient (13 P), eliminated blocks (9 E),
 * eliminated gradient (3 E), couplings (eliminated, primary) and 13x3 blocks in (eliminated,
 * primary) order. */
int32_t orc_general_export(void* handle, double* primary_matrix, double* primary_gradient, double* eliminated_blocks,
                           double* eliminated_gradient, int32_t* coupling_index, double* couplings);
/* solveDampedSchurComplement restated on the built equations (dense FP64). */
int32_t orc_general_solve(void* handle, double damping, double tolerance, double* primary_step,
                          double* eliminated_step, int32_t* converged);
/* Rig problems: the current captures and sensors (12 doubles each) and the rig block of every
 * capture and sensor (-1: none); returns InvalidInput without a rig. */
int32_t orc_rig(void* handle, double* captures, double* sensors, int32_t* capture_block, int32_t* sensor_block);
/* Full solve from the initial state. */
int32_t orc_solve(void* handle, orc_report* report, double* cameras_out, double* points_out, int8_t* valid_out,
                  double* rms_before, double* rms_after, double* intrinsics_out);

#ifdef __cplusplus
}
#endif
