"""Problem, option and result containers mirroring plabundle's public API.

The reference's public types live in ``include/plabundle/problem.h``,
``include/plabundle/options.h`` and ``include/plabundle/result.h``.  The field
names below follow those headers so that a caller of ``plabundle::Solver::solve``
finds the same knobs.  The camera model is the frame-pinhole Brown-Conrady camera
of ``src/internal/BundleAdjustProjection.h:31-91`` (camera-to-world rotation,
world centre, fx/fy/cx/cy, k1..k3, p1/p2 in the OpenCV tangential convention,
u/v axis signs and a depth-axis flip), stored as one record of 32 float64 values:

    0-8   camera-to-world rotation, row-major      21 u axis sign (+1/-1)
    9-11  camera centre in world                   22 v axis sign (+1/-1)
    12 fx 13 fy 14 cx 15 cy                        23 depth axis flipped (0/1)
    16 k1 17 k2 18 k3 19 p1 20 p2                  24 image width 25 image height

Observations are stored grouped by track (track-CSR): ``track_offsets[t]`` ..
``track_offsets[t+1]`` index the observation arrays of track ``t``.
"""
from __future__ import annotations

import dataclasses
import enum
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

CAMERA_STRIDE = 32
INTRINSIC_COUNT = 13


class Backend(enum.IntEnum):
    """plabundle::Backend (include/plabundle/backend.h:8-15) plus the GB300 backend."""

    Auto = 0
    PlaMatrixCpu = 1
    PlaMatrixCuda = 2
    PlaMatrixVulkan = 3
    PlaMatrixOpenCl = 4
    Gb300 = 5


def backend_name(backend: Backend) -> str:
    """backendName (src/backend.cpp:50-66) extended with ``gb300_cuda``."""
    return {
        Backend.Auto: "auto",
        Backend.PlaMatrixCpu: "plamatrix_cpu",
        Backend.PlaMatrixCuda: "plamatrix_cuda",
        Backend.PlaMatrixVulkan: "plamatrix_vulkan",
        Backend.PlaMatrixOpenCl: "plamatrix_opencl",
        Backend.Gb300: "gb300_cuda",
    }.get(backend, "unknown")


class SolveStatus(enum.IntEnum):
    """plabundle::SolveStatus (include/plabundle/backend.h:17-27)."""

    NotRun = 0
    Success = 1
    NoConvergence = 2
    Cancelled = 3
    InvalidInput = 4
    UnsupportedConfiguration = 5
    BackendUnavailable = 6
    NumericalFailure = 7


class ImageRobustLoss(enum.IntEnum):
    """include/plabundle/options.h:18-23."""

    LeastSquares = 0
    Huber = 1
    Cauchy = 2


class GaugePolicy(enum.IntEnum):
    """include/plabundle/problem.h:15-20."""

    AutoAnchor = 0
    RequireExplicitGauge = 1
    CallerManaged = 2


class IntrinsicParameter(enum.IntEnum):
    """include/plabundle/options.h:25-45."""

    FocalLength = 0
    FocalAspectRatio = 1
    PrincipalPointX = 2
    PrincipalPointY = 3
    RadialK1 = 4
    RadialK2 = 5
    RadialK3 = 6
    TangentialP1 = 7
    TangentialP2 = 8
    SkewB2 = 9
    RadialK4 = 10
    TangentialP3 = 11
    TangentialP4 = 12


@dataclass
class Gauge:
    """include/plabundle/problem.h:22-28."""

    policy: GaugePolicy = GaugePolicy.AutoAnchor
    referenceAnchorCameraIndex: int = -1
    referenceScaleCameraIndex: int = -1
    referenceBaseline: float = 0.0


class ControlPointUncertainty(enum.IntEnum):
    """ControlPointConstraint::Uncertainty (include/plabundle/constraints.h:79-84)."""

    IsotropicSigma = 0
    Covariance = 1
    SqrtInformation = 2


@dataclass
class ControlPointConstraint:
    """ControlPointConstraint (include/plabundle/constraints.h:73-87): the target of a track's
    point in the solver frame with its uncertainty."""

    point: Sequence[float] = (0.0, 0.0, 0.0)
    sigmaMeters: float = 1.0
    weight: float = 1.0
    uncertainty: ControlPointUncertainty = ControlPointUncertainty.IsotropicSigma
    uncertaintyMatrix: Sequence[float] = (0.0,) * 9   # row-major covariance (m^2) or sqrt information (1/m)

    def record(self) -> np.ndarray:
        return np.array(list(self.point) + [self.sigmaMeters, self.weight, float(int(self.uncertainty))] +
                        list(self.uncertaintyMatrix), np.float64)


@dataclass
class ScaleBarConstraint:
    """ScaleBarConstraint (include/plabundle/constraints.h:93-101): the measured distance between
    the points of two tracks."""

    trackIndexA: int = -1
    trackIndexB: int = -1
    measuredDistanceMeters: float = 0.0
    sigmaMeters: float = 1.0
    weight: float = 1.0
    sourceIndex: int = -1


@dataclass
class RigCapture:
    """placamera::RigCapture: one capture of a rig (rig-to-world rotation, rig centre in world
    coordinates)."""

    rigId: int = 0
    captureId: int = 0
    rigToWorldRotation: Sequence[float] = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)  # row-major
    rigCenterInWorld: Sequence[float] = (0.0, 0.0, 0.0)
    fixedPose: bool = False


@dataclass
class RigSensor:
    """placamera::RigSensor: the extrinsic of one sensor of a rig (camera-to-rig rotation, camera
    centre in rig coordinates), shared by all captures of the rig."""

    rigId: int = 0
    sensorId: int = 0
    cameraToRigRotation: Sequence[float] = (1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0)  # row-major
    cameraCenterInRig: Sequence[float] = (0.0, 0.0, 0.0)
    fixedExtrinsic: bool = False


@dataclass
class RigCameraBinding:
    """placamera::RigCameraBinding: the capture and sensor a camera model is composed from."""

    cameraIndex: int = 0
    rigId: int = 0
    captureId: int = 0
    sensorId: int = 0


@dataclass
class RigTopology:
    """placamera::RigTopology (Problem::rig, include/plabundle/problem.h:52).  The composed camera
    is R_camera_world = R_rig_world R_camera_rig, C_camera_world = C_rig_world + R_rig_world
    C_camera_rig (the reference's README, "Rig BA")."""

    captures: List[RigCapture] = field(default_factory=list)
    sensors: List[RigSensor] = field(default_factory=list)
    cameraBindings: List[RigCameraBinding] = field(default_factory=list)

    def empty(self) -> bool:
        return not self.captures and not self.sensors and not self.cameraBindings

    def arrays(self, n_cameras: int):
        """The C-ABI arrays: capture records [n, 12] and (rigId, fixedPose) [n, 2], sensor records
        [n, 12] and (rigId, fixedExtrinsic) [n, 2], and each camera's capture and sensor index
        (-1 for a camera without a binding; the library rejects it).  Bindings name captures and
        sensors by (rigId, captureId) and (rigId, sensorId), as the reference looks them up
        (prepareActiveProblem, BundleAdjustPlaMatrixProblem.cpp:47-66)."""
        cap = np.array([list(c.rigToWorldRotation) + list(c.rigCenterInWorld) for c in self.captures],
                       np.float64).reshape(-1, 12)
        cap_info = np.array([(c.rigId, int(bool(c.fixedPose))) for c in self.captures], np.int32).reshape(-1, 2)
        sen = np.array([list(s.cameraToRigRotation) + list(s.cameraCenterInRig) for s in self.sensors],
                       np.float64).reshape(-1, 12)
        sen_info = np.array([(s.rigId, int(bool(s.fixedExtrinsic))) for s in self.sensors], np.int32).reshape(-1, 2)
        ck = {(c.rigId, c.captureId): i for i, c in reversed(list(enumerate(self.captures)))}
        sk = {(s.rigId, s.sensorId): i for i, s in reversed(list(enumerate(self.sensors)))}
        cam_cap = np.full(n_cameras, -1, np.int32)
        cam_sen = np.full(n_cameras, -1, np.int32)
        for b in self.cameraBindings:
            if 0 <= b.cameraIndex < n_cameras:
                cam_cap[b.cameraIndex] = ck.get((b.rigId, b.captureId), -1)
                cam_sen[b.cameraIndex] = sk.get((b.rigId, b.sensorId), -1)
        return (np.ascontiguousarray(cap), np.ascontiguousarray(cap_info), np.ascontiguousarray(sen),
                np.ascontiguousarray(sen_info), cam_cap, cam_sen)


@dataclass
class Problem:
    """plabundle::Problem (include/plabundle/problem.h:37-54) for frame cameras.

    Control points are the (track, ControlPointConstraint) pairs of Track::controlPointConstraints;
    scale bars are Problem::scaleBarConstraints (their tracks become primary point blocks and the
    problem is solved on the general path, canUseReferenceOnlineSchur,
    BundleAdjustPlaMatrixReferenceSchur.cpp:667-673).  `rig` is Problem::rig: captures, sensors and
    the binding of every camera.  Laser planes and ranges, pose priors and the camera-plane
    constraint are not carried.
    """

    cameras: np.ndarray                 # [n_cameras, 32] float64
    points: np.ndarray                  # [n_tracks, 3] float64, Track::initialPoint
    track_offsets: np.ndarray           # [n_tracks + 1] int64
    obs_camera: np.ndarray              # [n_obs] int32, Observation::cameraIndex
    obs_u: np.ndarray                   # [n_obs] float64
    obs_v: np.ndarray                   # [n_obs] float64
    obs_weight: np.ndarray              # [n_obs] float64
    obs_scale: np.ndarray               # [n_obs] float64, Observation::measurementScale
    fixedCameraIndices: List[int] = field(default_factory=list)
    fixedTrackIndices: List[int] = field(default_factory=list)
    cameraCalibrationGroupIds: Optional[np.ndarray] = None   # [n_cameras] int32
    sharedIntrinsicReferenceCameras: Optional[np.ndarray] = None  # [n_cameras, 32]
    gauge: Gauge = field(default_factory=Gauge)
    controlPoints: List[Tuple[int, ControlPointConstraint]] = field(default_factory=list)
    scaleBarConstraints: List[ScaleBarConstraint] = field(default_factory=list)
    rig: RigTopology = field(default_factory=RigTopology)

    @property
    def n_cameras(self) -> int:
        return int(self.cameras.shape[0])

    @property
    def n_tracks(self) -> int:
        return int(self.points.shape[0])

    @property
    def n_obs(self) -> int:
        return int(self.obs_camera.shape[0])

    def normalized(self) -> "Problem":
        """Contiguous arrays of the dtypes the C-ABI expects."""
        def c(a, dt):
            return np.ascontiguousarray(a, dtype=dt)
        return dataclasses.replace(
            self,
            cameras=c(self.cameras, np.float64).reshape(-1, CAMERA_STRIDE),
            points=c(self.points, np.float64).reshape(-1, 3),
            track_offsets=c(self.track_offsets, np.int64),
            obs_camera=c(self.obs_camera, np.int32),
            obs_u=c(self.obs_u, np.float64),
            obs_v=c(self.obs_v, np.float64),
            obs_weight=c(self.obs_weight, np.float64),
            obs_scale=c(self.obs_scale, np.float64),
            cameraCalibrationGroupIds=None if self.cameraCalibrationGroupIds is None
            else c(self.cameraCalibrationGroupIds, np.int32),
            sharedIntrinsicReferenceCameras=None if self.sharedIntrinsicReferenceCameras is None
            else c(self.sharedIntrinsicReferenceCameras, np.float64).reshape(-1, CAMERA_STRIDE),
        )


def summarize_problem(problem: Problem) -> dict:
    """summarizeProblem (src/problem.cpp:113-140): camera, track and observation counts."""
    return {"cameraCount": problem.n_cameras, "trackCount": problem.n_tracks,
            "observationCount": problem.n_obs}


@dataclass
class SolverControlOptions:
    """include/plabundle/options.h:58-76."""

    maxIterations: int = 20
    imageRobustLoss: ImageRobustLoss = ImageRobustLoss.LeastSquares
    imageRobustLossScalePixels: float = 1.0
    referenceArmijoCoefficient: float = 1.0e-3
    referenceLineSearchSteps: int = 34
    # True: the online reduced-Schur path; False: the general path (the reference's default is
    # False; this backend defaults to the online path, its headline path)
    useReferenceOnlineSchur: bool = True
    enablePointFilter: bool = True
    filterMaxReprojError: float = 2.5
    filterSigmaFactor: float = 3.0
    maxInitialTrackRms: float = 100.0
    numThreads: int = 0
    logIterationProgress: bool = False


@dataclass
class CalibrationOptions:
    """include/plabundle/options.h:78-125 (numeric bounds and prior sigmas)."""

    refineCameraPose: bool = True
    refineSharedFocalLength: bool = False
    refineSharedFocalAspectRatio: bool = False
    refineSharedPrincipalPoint: bool = False
    refineSharedModelCoefficients: bool = False
    refineSharedRadialDistortion: bool = False
    refineSharedHighOrderDistortion: bool = True
    refineSharedMetashapeParameters: bool = False
    useSharedIntrinsicParameterMask: bool = False
    sharedIntrinsicParameterMask: List[bool] = field(default_factory=lambda: [True] * INTRINSIC_COUNT)
    minSharedFocalScale: float = 0.5
    maxSharedFocalScale: float = 4.0
    minSharedFocalAspectScale: float = 0.85
    maxSharedFocalAspectScale: float = 1.18
    maxSharedPrincipalPointOffsetFraction: float = 0.08
    sharedFocalPriorSigma: float = 0.35
    sharedPrincipalPointPriorSigmaFraction: float = 0.04
    sharedFocalAspectPriorSigma: float = 0.08
    maxSharedRadialK1Abs: float = 0.35
    maxSharedRadialK2Abs: float = 0.35
    maxSharedRadialK3Abs: float = 0.35
    maxSharedTangentialP1Abs: float = 0.02
    maxSharedTangentialP2Abs: float = 0.02
    maxSharedSkewFraction: float = 0.10
    maxSharedRadialK4Abs: float = 0.35
    maxSharedTangentialP3Abs: float = 0.35
    maxSharedTangentialP4Abs: float = 0.35
    sharedRadialK1PriorSigma: float = 0.15
    sharedRadialK2PriorSigma: float = 0.15
    sharedRadialK3PriorSigma: float = 0.15
    sharedTangentialP1PriorSigma: float = 0.01
    sharedTangentialP2PriorSigma: float = 0.01
    sharedSkewPriorSigmaFraction: float = 0.02
    sharedRadialK4PriorSigma: float = 0.15
    sharedTangentialP3PriorSigma: float = 0.15
    sharedTangentialP4PriorSigma: float = 0.15
    sharedLowOrderDistortionScale: float = 1.0

    def numeric_block(self) -> List[float]:
        """The 27 numeric calibration fields in the order the C-ABI reads them."""
        return [self.minSharedFocalScale, self.maxSharedFocalScale, self.minSharedFocalAspectScale,
                self.maxSharedFocalAspectScale, self.maxSharedPrincipalPointOffsetFraction,
                self.sharedFocalPriorSigma, self.sharedPrincipalPointPriorSigmaFraction,
                self.sharedFocalAspectPriorSigma, self.maxSharedRadialK1Abs, self.maxSharedRadialK2Abs,
                self.maxSharedRadialK3Abs, self.maxSharedTangentialP1Abs, self.maxSharedTangentialP2Abs,
                self.maxSharedSkewFraction, self.maxSharedRadialK4Abs, self.maxSharedTangentialP3Abs,
                self.maxSharedTangentialP4Abs, self.sharedRadialK1PriorSigma, self.sharedRadialK2PriorSigma,
                self.sharedRadialK3PriorSigma, self.sharedTangentialP1PriorSigma,
                self.sharedTangentialP2PriorSigma, self.sharedSkewPriorSigmaFraction,
                self.sharedRadialK4PriorSigma, self.sharedTangentialP3PriorSigma,
                self.sharedTangentialP4PriorSigma, self.sharedLowOrderDistortionScale]


def shared_intrinsic_parameter_enabled(cal: CalibrationOptions, parameter: IntrinsicParameter) -> bool:
    """sharedIntrinsicParameterEnabled / parameterEnabled (src/backend.cpp:8-47)."""
    p = IntrinsicParameter(parameter)
    if p == IntrinsicParameter.FocalLength:
        enabled = cal.refineSharedFocalLength
    elif p == IntrinsicParameter.FocalAspectRatio:
        enabled = cal.refineSharedFocalAspectRatio
    elif p in (IntrinsicParameter.PrincipalPointX, IntrinsicParameter.PrincipalPointY):
        enabled = cal.refineSharedPrincipalPoint
    elif p == IntrinsicParameter.RadialK1:
        enabled = cal.refineSharedModelCoefficients or cal.refineSharedRadialDistortion
    elif p in (IntrinsicParameter.RadialK2, IntrinsicParameter.RadialK3, IntrinsicParameter.TangentialP1,
               IntrinsicParameter.TangentialP2):
        enabled = ((cal.refineSharedModelCoefficients or cal.refineSharedRadialDistortion)
                   and cal.refineSharedHighOrderDistortion)
    else:
        enabled = cal.refineSharedMetashapeParameters
    return bool(enabled and (not cal.useSharedIntrinsicParameterMask
                             or cal.sharedIntrinsicParameterMask[int(p)]))


def intrinsic_mask(cal: CalibrationOptions) -> int:
    return sum(1 << p for p in range(INTRINSIC_COUNT)
               if shared_intrinsic_parameter_enabled(cal, IntrinsicParameter(p)))


class Precision(enum.IntEnum):
    """Arithmetic of the GB300 kernels."""

    Fp64 = 0     # every kernel in double precision
    Mixed = 1    # FP32 Jacobians/Schur/PCG, compensated sums, FP64 cost and refinement


@dataclass
class BackendOptions:
    """include/plabundle/options.h:127-168, plus the GB300 precision switches."""

    requested: Backend = Backend.Gb300
    plaMatrixDevice: int = 0
    enablePlaMatrixMixedPrecision: bool = True
    plaMatrixPreconditionerClusterSize: int = 1
    allowFallback: bool = False
    minPlaMatrixCudaCameras: int = 128
    minPlaMatrixCudaObservations: int = 30000
    minPlaMatrixDenseCameras: int = 120
    minPlaMatrixCudaDenseObservations: int = 150000
    refinementSweeps: int = 3
    maxLinearIterations: int = 0
    linearSolver: int = 0   # 0 auto, 1 dense-Cholesky-preconditioned CG, 2 block-Jacobi PCG
    # dense-factor reuse across LM iterations: 0 default (mixed path keeps its FP32 factor, FP64
    # path refactors every iteration), 1 keep on both paths, 2 refactor on both paths
    factorReuse: int = 0
    # relative tolerance of the reduced solve; 0: the reference's tolerance of the path (2e-10 on
    # the online path, 1e-12 on the general path, BundleAdjustPlaMatrix.cpp:321-330)
    linearRelativeTolerance: float = 0.0


@dataclass
class QualityGateOptions:
    """include/plabundle/options.h:170-178."""

    enabled: bool = True
    maxAcceptedRmsGrowth: float = 1.25
    minAcceptedValidTrackRatio: float = 0.60
    maxAcceptedConstraintRmsGrowth: float = 1.25


@dataclass
class ConstraintOptions:
    """ConstraintOptions (include/plabundle/options.h:122-135): the control-point and scale-bar
    fields."""

    controlPointWeight: float = 1.0
    controlPointHuberDeltaMeters: float = 0.2
    scaleBarWeight: float = 1.0
    scaleBarHuberDeltaMeters: float = 0.2


@dataclass
class SolveOptions:
    """include/plabundle/options.h:180-187."""

    solver: SolverControlOptions = field(default_factory=SolverControlOptions)
    constraints: ConstraintOptions = field(default_factory=ConstraintOptions)
    calibration: CalibrationOptions = field(default_factory=CalibrationOptions)
    backend: BackendOptions = field(default_factory=BackendOptions)
    quality: QualityGateOptions = field(default_factory=QualityGateOptions)


@dataclass
class RefinedPoint:
    """include/plabundle/result.h:15-23 (arrays over all tracks)."""

    valid: np.ndarray
    converged: bool
    point: np.ndarray
    rmsBefore: np.ndarray
    rmsAfter: np.ndarray
    iterations: int


@dataclass
class PlaMatrixDiagnostics:
    """include/plabundle/result.h:91-128 (the fields the GB300 backend fills)."""

    initialCost: float = 0.0
    finalCost: float = 0.0
    acceptedSteps: int = 0
    rejectedSteps: int = 0
    linearizations: int = 0
    objectiveEvaluations: int = 0
    rejectedInitialTracks: int = 0
    referenceOnlineSchurUsed: bool = True
    linearSolverName: str = "block_jacobi_pcg_gb300"
    preconditionerName: str = "block_jacobi"
    deviceName: str = ""
    linearIterations: int = 0
    assemblySeconds: float = 0.0
    objectiveSeconds: float = 0.0
    linearSolveSeconds: float = 0.0
    backSubstitutionSeconds: float = 0.0
    schurPatternBuilds: int = 0
    schurPatternReuses: int = 0
    schurAssemblyOnDevice: bool = True
    mixedPrecisionUsed: bool = False
    refinementSweeps: int = 0


@dataclass
class QualitySummary:
    """include/plabundle/result.h:50-89 (image and control-point fields)."""

    totalTracks: int = 0
    optimizedTracks: int = 0
    validTrackRatio: float = 0.0
    meanRmsBefore: float = 0.0
    meanRmsAfter: float = 0.0
    refinedCameraCount: int = 0
    refinedCalibrationGroupCount: int = 0
    filterThreshold: float = 0.0
    controlPointConstraintCount: int = 0
    controlPointRmsBeforeMeters: float = 0.0
    controlPointRmsAfterMeters: float = 0.0
    scaleBarConstraintCount: int = 0
    scaleBarRmsBeforeMeters: float = 0.0
    scaleBarRmsAfterMeters: float = 0.0


@dataclass
class Result:
    """plabundle::Result (include/plabundle/result.h:130-155)."""

    requestedBackend: Backend = Backend.Gb300
    usedBackend: Backend = Backend.Gb300
    status: SolveStatus = SolveStatus.NotRun
    solutionUsable: bool = False
    usedGpu: bool = True
    backendFallback: bool = False
    backendMessage: str = ""
    backendSelectionReason: str = ""
    qualityGateRejected: bool = False
    qualityGateMessage: str = ""
    observationCount: int = 0
    totalSeconds: float = 0.0
    quality: QualitySummary = field(default_factory=QualitySummary)
    plaMatrix: PlaMatrixDiagnostics = field(default_factory=PlaMatrixDiagnostics)
    points: Optional[RefinedPoint] = None
    refinedCameras: Optional[np.ndarray] = None
    intrinsicGroups: Optional[np.ndarray] = None
    refinedRig: Optional[RigTopology] = None    # Result::refinedRig (include/plabundle/result.h:149)

    def usable(self) -> bool:
        return self.solutionUsable and self.status in (SolveStatus.Success, SolveStatus.NoConvergence)
