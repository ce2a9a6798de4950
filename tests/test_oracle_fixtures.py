"""The committed converged-oracle fixtures of the 500-camera block and the rig block, on CPU:
their records are complete and consistent, and the comparison the GPU tests and the bench apply
to a GPU result reads zero error on the oracle's own solution and sees a planted difference."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_c1_fixture as C1  # noqa: E402
import make_rig_fixture as RIG  # noqa: E402


def _fixture(mod):
    fx = mod.load_fixture()
    if fx is None:
        pytest.skip("fixture absent")
    return fx


def _own_solution(meta, arrays):
    """The oracle's solution as a GPU result would hand it to compare(): full-size point, valid
    and after-RMS arrays rebuilt from the stored sample, mask and near-threshold records."""
    n = meta["n_tracks"]
    points = np.zeros((n, 3))
    points[arrays["point_sample_tracks"]] = arrays["point_sample"]
    valid = np.unpackbits(arrays["out_valid_bits"])[:n].astype(bool)
    rms = np.zeros(n)
    rms[arrays["near_threshold_tracks"]] = arrays["near_threshold_rms_after"]
    return points, valid, rms


@pytest.mark.parametrize("which", ["c1", "rig"])
def test_fixture_records_are_complete(which):
    mod = C1 if which == "c1" else RIG
    meta, arrays = _fixture(mod)
    rep = meta["report"]
    assert rep["status"] == 1 and rep["iterations"] > 0 and np.isfinite(rep["final_cost"])
    assert rep["final_cost"] < rep["initial_cost"]
    n = meta["n_tracks"]
    assert arrays["out_valid_bits"].size == (n + 7) // 8
    assert arrays["point_sample_tracks"].max() < n and arrays["point_sample"].shape == (arrays["point_sample_tracks"].size, 3)
    assert meta["wall_seconds"] > 0 and meta["threads"] >= 1
    for k, size in meta["float_sizes"].items():
        idx = arrays["sample_idx_" + k]
        assert idx.size > 0 and idx.max() < size and np.all(np.diff(idx) > 0)
    if which == "rig":
        assert arrays["out_cameras"].shape == (3000, 32)
        assert arrays["out_captures"].shape == (600, 12) and arrays["out_sensors"].shape == (5, 12)
        assert arrays["in_rig_camera_capture"].shape == (3000,) and arrays["in_rig_camera_sensor"].max() == 4
    else:
        assert arrays["out_cameras"].shape == (500, 32)


def test_c1_comparison_is_zero_on_the_oracle_solution_and_sees_a_planted_shift():
    meta, arrays = _fixture(C1)
    points, valid, rms = _own_solution(meta, arrays)
    cams = arrays["out_cameras"].copy()
    thr = meta["report"]["filter_threshold"]
    cmp = C1.compare(meta, arrays, cams, arrays["out_intrinsics"], valid, rms, points, meta["report"]["final_cost"], thr)
    assert cmp["final_cost_rel_err"] == 0 and cmp["camera_centre_rel_err"] == 0 and cmp["point_sample_rel_err"] == 0
    assert cmp["intrinsics_rel_err"] == 0 and cmp["inlier_mask_flips"] == 0
    # planted in the oracle's solution: one centre moved by 1e-4 of the extent, one track flipped
    C0 = cams[:, 9:12]
    extent = float(np.linalg.norm(C0 - C0.mean(0), axis=1).max())
    cams[7, 10] += 1e-4 * extent
    t = int(arrays["near_threshold_tracks"][0]) if arrays["near_threshold_tracks"].size else 0
    valid2 = valid.copy()
    valid2[t] = not valid2[t]
    cmp = C1.compare(meta, arrays, cams, arrays["out_intrinsics"], valid2, rms, points, meta["report"]["final_cost"], thr)
    assert abs(cmp["camera_centre_rel_err"] - 1e-4) < 1e-9
    assert cmp["inlier_mask_flips"] == 1 and len(cmp["flip_margins_px"]) == 1


def test_rig_comparison_is_zero_on_the_oracle_solution_and_sees_a_planted_shift():
    meta, arrays = _fixture(RIG)
    points, valid, rms = _own_solution(meta, arrays)
    thr = meta["report"]["filter_threshold"]
    caps = arrays["out_captures"].copy()
    sens = arrays["out_sensors"].copy()
    cmp = RIG.compare(meta, arrays, arrays["out_cameras"], caps, sens, valid, rms, points,
                      meta["report"]["final_cost"], thr)
    assert cmp["final_cost_rel_err"] == 0 and cmp["camera_centre_rel_err"] == 0
    assert cmp["capture_centre_rel_err"] == 0 and cmp["sensor_max_abs_err"] == 0 and cmp["inlier_mask_flips"] == 0
    sens[2, 9] += 2e-6  # a lever-arm component moved by 2 micrometres
    cmp = RIG.compare(meta, arrays, arrays["out_cameras"], caps, sens, valid, rms, points,
                      meta["report"]["final_cost"], thr)
    assert abs(cmp["sensor_max_abs_err"] - 2e-6) < 1e-12
