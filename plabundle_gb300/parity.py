"""Solver-neutral parity reports: ID-keyed comparison of two solve outcomes.

Mirrors the reference's photo-alignment outcome comparison (`makePhotoAlignmentOutcome`,
`comparePhotoAlignmentOutcomes`, src/photo_alignment.cpp:190-319, include/plabundle/
photo_alignment.h:40-113): cameras and tracks are matched by id, and the report holds per-camera
centre distance and rotation angle, per-track point distance for tracks valid in both, the ids
whose valid flag differs, the mean-RMS differences, and whether the termination status and the
backends match.  `equivalent` applies the tolerances the same way.  The comparison is
vectorised over the arrays of `Result` (numpy) rather than per-id maps.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from .problem import Backend, Result, SolveStatus

_RAD_TO_DEG = 180.0 / np.pi


@dataclass
class PhotoAlignmentComparisonTolerance:
    """photo_alignment.h:62-72."""

    rms: float = 1.0e-8
    cameraCenterMeters: float = 1.0e-8
    cameraRotationDegrees: float = 1.0e-8
    pointMeters: float = 1.0e-8
    requireTerminationStatusMatch: bool = True
    requireTerminationReasonMatch: bool = True
    requireRequestedBackendMatch: bool = True
    requireUsedBackendMatch: bool = True


@dataclass
class PhotoAlignmentCameraDifference:
    id: str
    centerDistanceMeters: float
    rotationAngleDegrees: float


@dataclass
class PhotoAlignmentTrackDifference:
    id: str
    referenceValid: bool
    candidateValid: bool
    pointDistanceMeters: float


@dataclass
class PhotoAlignmentComparison:
    comparable: bool = False
    equivalent: bool = False
    terminationStatusMatches: bool = False
    terminationReasonMatches: bool = False
    requestedBackendMatches: bool = False
    usedBackendMatches: bool = False
    rmsBeforeDifference: float = 0.0
    rmsAfterDifference: float = 0.0
    maximumCameraCenterDifferenceMeters: float = 0.0
    maximumCameraRotationDifferenceDegrees: float = 0.0
    maximumPointDifferenceMeters: float = 0.0
    validTrackMaskMismatchIds: List[str] = field(default_factory=list)
    cameraDifferences: List[PhotoAlignmentCameraDifference] = field(default_factory=list)
    trackDifferences: List[PhotoAlignmentTrackDifference] = field(default_factory=list)
    message: str = ""


@dataclass
class PhotoAlignmentOutcome:
    """photo_alignment.h:40-54 with the camera and track states as arrays (rows in id order)."""

    cameraIds: Sequence[str]
    trackIds: Sequence[str]
    cameras: np.ndarray            # n_cameras x 32 refined camera records
    points: np.ndarray             # n_tracks x 3
    valid: np.ndarray              # n_tracks bool
    terminationStatus: SolveStatus = SolveStatus.NotRun
    terminationReason: str = ""
    requestedBackend: Backend = Backend.Gb300
    usedBackend: Backend = Backend.Gb300
    solutionUsable: bool = False
    meanRmsBefore: float = 0.0
    meanRmsAfter: float = 0.0


def make_outcome(result: Result, camera_ids: Optional[Sequence[str]] = None,
                 track_ids: Optional[Sequence[str]] = None) -> PhotoAlignmentOutcome:
    """makePhotoAlignmentOutcome (photo_alignment.cpp:190-240): ids default to the indices."""
    cams = np.asarray(result.refinedCameras, np.float64)
    pts = np.asarray(result.points.point, np.float64)
    nc, nt = cams.shape[0], pts.shape[0]
    cid = [str(i) for i in range(nc)] if camera_ids is None else list(camera_ids)
    tid = [str(i) for i in range(nt)] if track_ids is None else list(track_ids)
    if len(cid) != nc or len(tid) != nt:
        raise ValueError("solver result camera/track counts do not match the ids")
    return PhotoAlignmentOutcome(cameraIds=cid, trackIds=tid, cameras=cams, points=pts,
                                 valid=np.asarray(result.points.valid, bool), terminationStatus=result.status,
                                 terminationReason=result.backendMessage, requestedBackend=result.requestedBackend,
                                 usedBackend=result.usedBackend, solutionUsable=result.solutionUsable,
                                 meanRmsBefore=result.quality.meanRmsBefore, meanRmsAfter=result.quality.meanRmsAfter)


def _validate(o: PhotoAlignmentOutcome):
    if len(set(o.cameraIds)) != len(o.cameraIds) or len(set(o.trackIds)) != len(o.trackIds):
        raise ValueError("photo-alignment outcome ids must be unique")
    if o.cameras.shape != (len(o.cameraIds), 32) or o.points.shape != (len(o.trackIds), 3):
        raise ValueError("photo-alignment outcome arrays do not match its ids")


def _validate_tolerance(t: PhotoAlignmentComparisonTolerance):
    for v in (t.rms, t.cameraCenterMeters, t.cameraRotationDegrees, t.pointMeters):
        if not np.isfinite(v) or v < 0.0:
            raise ValueError("photo-alignment comparison tolerances must be finite and non-negative")


def rotation_difference_degrees(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Angle of a^T b for stacks of row-major 3x3 rotations (photo_alignment.cpp:64-77)."""
    tr = np.einsum("ij,ij->i", a.reshape(-1, 9), b.reshape(-1, 9))
    return np.arccos(np.clip(0.5 * (tr - 1.0), -1.0, 1.0)) * _RAD_TO_DEG


def compare_outcomes(reference: PhotoAlignmentOutcome, candidate: PhotoAlignmentOutcome,
                     tolerance: Optional[PhotoAlignmentComparisonTolerance] = None) -> PhotoAlignmentComparison:
    """comparePhotoAlignmentOutcomes (photo_alignment.cpp:241-319)."""
    tol = tolerance or PhotoAlignmentComparisonTolerance()
    _validate_tolerance(tol)
    _validate(reference)
    _validate(candidate)
    out = PhotoAlignmentComparison()
    if set(reference.cameraIds) != set(candidate.cameraIds) or set(reference.trackIds) != set(candidate.trackIds):
        out.message = "camera or track id sets differ"
        raise ValueError("photo-alignment outcomes must contain the same camera and track ids")
    out.comparable = True
    out.terminationStatusMatches = reference.terminationStatus == candidate.terminationStatus
    out.terminationReasonMatches = reference.terminationReason == candidate.terminationReason
    out.requestedBackendMatches = reference.requestedBackend == candidate.requestedBackend
    out.usedBackendMatches = reference.usedBackend == candidate.usedBackend
    out.rmsBeforeDifference = abs(reference.meanRmsBefore - candidate.meanRmsBefore)
    out.rmsAfterDifference = abs(reference.meanRmsAfter - candidate.meanRmsAfter)
    # rows of the candidate in the reference's id order (ids sorted, as the reference's maps are)
    corder = np.array(sorted(range(len(reference.cameraIds)), key=lambda i: reference.cameraIds[i]), np.int64)
    cpos = {k: i for i, k in enumerate(candidate.cameraIds)}
    cmap = np.array([cpos[reference.cameraIds[i]] for i in corder], np.int64)
    torder = np.array(sorted(range(len(reference.trackIds)), key=lambda i: reference.trackIds[i]), np.int64)
    tpos = {k: i for i, k in enumerate(candidate.trackIds)}
    tmap = np.array([tpos[reference.trackIds[i]] for i in torder], np.int64)
    rc, cc = reference.cameras[corder], candidate.cameras[cmap]
    centre = np.sqrt(((rc[:, 9:12] - cc[:, 9:12]) ** 2).sum(1))
    angle = rotation_difference_degrees(rc[:, :9], cc[:, :9])
    if centre.size:
        out.maximumCameraCenterDifferenceMeters = float(centre.max())
        out.maximumCameraRotationDifferenceDegrees = float(angle.max())
    out.cameraDifferences = [PhotoAlignmentCameraDifference(reference.cameraIds[i], float(d), float(a))
                             for i, d, a in zip(corder, centre, angle)]
    rv, cv = reference.valid[torder], candidate.valid[tmap]
    both = rv & cv
    dist = np.where(both, np.sqrt(((reference.points[torder] - candidate.points[tmap]) ** 2).sum(1)), 0.0)
    if both.any():
        out.maximumPointDifferenceMeters = float(dist[both].max())
    out.validTrackMaskMismatchIds = [reference.trackIds[i] for i in torder[rv != cv]]
    out.trackDifferences = [PhotoAlignmentTrackDifference(reference.trackIds[i], bool(a), bool(b), float(d))
                            for i, a, b, d in zip(torder, rv, cv, dist)]
    ok = ((not tol.requireTerminationStatusMatch or out.terminationStatusMatches) and
          (not tol.requireTerminationReasonMatch or out.terminationReasonMatches) and
          (not tol.requireRequestedBackendMatch or out.requestedBackendMatches) and
          (not tol.requireUsedBackendMatch or out.usedBackendMatches))
    out.equivalent = bool(ok and out.rmsBeforeDifference <= tol.rms and out.rmsAfterDifference <= tol.rms and
                          out.maximumCameraCenterDifferenceMeters <= tol.cameraCenterMeters and
                          out.maximumCameraRotationDifferenceDegrees <= tol.cameraRotationDegrees and
                          out.maximumPointDifferenceMeters <= tol.pointMeters and
                          not out.validTrackMaskMismatchIds)
    out.message = "photo-alignment outcomes are equivalent" if out.equivalent else "photo-alignment outcomes differ"
    return out


def summary(c: PhotoAlignmentComparison) -> dict:
    """The scalar part of a comparison, for logs and benchmark lines."""
    return {"equivalent": c.equivalent, "termination_status_matches": c.terminationStatusMatches,
            "rms_before_difference": c.rmsBeforeDifference, "rms_after_difference": c.rmsAfterDifference,
            "max_camera_centre_difference_m": c.maximumCameraCenterDifferenceMeters,
            "max_camera_rotation_difference_deg": c.maximumCameraRotationDifferenceDegrees,
            "max_point_difference_m": c.maximumPointDifferenceMeters,
            "valid_mask_mismatches": len(c.validTrackMaskMismatchIds)}
