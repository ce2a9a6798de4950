"""The parity reporter (plabundle_gb300/parity.py) on constructed outcomes: the reference's
comparison semantics (photo_alignment.cpp:241-319) - id-keyed matching, per-camera centre
distance and rotation angle, point distances of tracks valid in both, valid-mask mismatch ids,
and `equivalent` under the tolerances."""
import numpy as np
import pytest

from plabundle_gb300.parity import (PhotoAlignmentComparisonTolerance, PhotoAlignmentOutcome, compare_outcomes,
                                    rotation_difference_degrees, summary)
from plabundle_gb300.problem import SolveStatus
from plabundle_gb300.synth import rotation_from_axis_angle


def _outcome(seed=0, nc=5, nt=40):
    rng = np.random.default_rng(seed)
    cams = np.zeros((nc, 32))
    for c in range(nc):
        cams[c, :9] = rotation_from_axis_angle(rng.normal(0, 0.3, 3)).ravel()
        cams[c, 9:12] = rng.normal(0, 10, 3)
    pts = rng.normal(0, 5, (nt, 3))
    return PhotoAlignmentOutcome(cameraIds=[f"cam{c}" for c in range(nc)], trackIds=[f"t{t}" for t in range(nt)],
                                 cameras=cams, points=pts, valid=np.ones(nt, bool), terminationStatus=SolveStatus.Success,
                                 meanRmsBefore=2.0, meanRmsAfter=0.5)


def _copy(o, perm_c=None, perm_t=None):
    pc = np.arange(len(o.cameraIds)) if perm_c is None else perm_c
    pt = np.arange(len(o.trackIds)) if perm_t is None else perm_t
    return PhotoAlignmentOutcome(cameraIds=[o.cameraIds[i] for i in pc], trackIds=[o.trackIds[i] for i in pt],
                                 cameras=o.cameras[pc].copy(), points=o.points[pt].copy(), valid=o.valid[pt].copy(),
                                 terminationStatus=o.terminationStatus, meanRmsBefore=o.meanRmsBefore,
                                 meanRmsAfter=o.meanRmsAfter)


def test_identical_outcomes_in_any_order_are_equivalent():
    a = _outcome()
    rng = np.random.default_rng(1)
    b = _copy(a, rng.permutation(5), rng.permutation(40))
    c = compare_outcomes(a, b)
    assert c.comparable and c.equivalent
    assert c.maximumCameraCenterDifferenceMeters == 0.0 and c.maximumPointDifferenceMeters == 0.0
    assert c.maximumCameraRotationDifferenceDegrees < 1e-5  # acos resolution near 0
    assert [d.id for d in c.cameraDifferences] == sorted(a.cameraIds)


def test_differences_are_measured_and_keyed_by_id():
    a = _outcome()
    b = _copy(a)
    b.cameras[2, 9:12] += np.array([3e-6, 4e-6, 0.0])          # 5e-6 m
    R = b.cameras[3, :9].reshape(3, 3)
    b.cameras[3, :9] = (R @ rotation_from_axis_angle(np.array([0.0, 0.0, np.deg2rad(0.01)]))).ravel()
    b.points[7] += np.array([0.0, 0.0, 2e-3])
    b.valid[11] = False
    b.points[11] += 100.0                                          # not compared: valid in one only
    c = compare_outcomes(a, b, PhotoAlignmentComparisonTolerance(cameraCenterMeters=1e-5,
                                                                 cameraRotationDegrees=0.02, pointMeters=1e-2))
    assert not c.equivalent                                        # the mask mismatch alone breaks it
    assert c.validTrackMaskMismatchIds == ["t11"]
    d = {x.id: x for x in c.cameraDifferences}
    assert d["cam2"].centerDistanceMeters == pytest.approx(5e-6, rel=1e-9)
    assert d["cam3"].rotationAngleDegrees == pytest.approx(0.01, rel=1e-6)
    assert c.maximumPointDifferenceMeters == pytest.approx(2e-3, rel=1e-9)
    s = summary(c)
    assert s["valid_mask_mismatches"] == 1
    b.valid[11] = True
    b.points[11] -= 100.0
    assert compare_outcomes(a, b, PhotoAlignmentComparisonTolerance(cameraCenterMeters=1e-5,
                                                                    cameraRotationDegrees=0.02,
                                                                    pointMeters=1e-2)).equivalent


def test_status_and_id_set_rules():
    a = _outcome()
    b = _copy(a)
    b.terminationStatus = SolveStatus.NoConvergence
    assert not compare_outcomes(a, b).equivalent
    assert compare_outcomes(a, b, PhotoAlignmentComparisonTolerance(requireTerminationStatusMatch=False)).equivalent
    b = _copy(a)
    b.cameraIds = list(b.cameraIds)
    b.cameraIds[0] = "other"
    with pytest.raises(ValueError):
        compare_outcomes(a, b)
    with pytest.raises(ValueError):
        compare_outcomes(a, a, PhotoAlignmentComparisonTolerance(rms=-1.0))


def test_rotation_difference_is_the_relative_angle():
    R1 = rotation_from_axis_angle(np.array([0.1, -0.2, 0.3]))
    R2 = R1 @ rotation_from_axis_angle(np.array([0.0, np.deg2rad(7.0), 0.0]))
    assert rotation_difference_degrees(R1[None], R2[None])[0] == pytest.approx(7.0, rel=1e-12)
