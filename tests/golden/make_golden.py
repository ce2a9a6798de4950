"""Generates the golden fixtures of the online reduced-Schur path.

Each fixture holds a seeded synthetic problem (stored in full, so the tests do not depend on the
random streams of the numpy that runs them), the options it is solved with, and the converged
solution of the CPU FP64 oracle: report fields, final cameras and points, per-track strict RMS
and the inlier mask.  `SHA256SUMS` pins every array of every fixture.

    python tests/golden/make_golden.py          # rewrites the fixtures and SHA256SUMS

The reference has no golden vectors for this path (its native-problem test only checks that
the cost decreases), so these fixtures pin the restatement against itself across changes and
give the GPU tests a target that needs no oracle run.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from plabundle_gb300 import synth  # noqa: E402
from plabundle_gb300.problem import ImageRobustLoss, SolveOptions  # noqa: E402

PROBLEM_KEYS = ("cameras", "points", "track_offsets", "obs_camera", "obs_u", "obs_v", "obs_weight", "obs_scale")


def ring_case():
    p = synth.ring_problem(seed=21, n_cameras=10, n_points=400)
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    o.solver.maxIterations = 20
    return p, o, {"loss": "huber", "scale": 1.5, "max_iterations": 20, "intrinsics": []}


def aerial_case():
    p = synth.aerial_grid_problem(seed=23, n_along=5, n_lines=4, n_points=1500)
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Cauchy
    o.solver.imageRobustLossScalePixels = 1.5
    o.calibration.refineSharedFocalLength = True
    o.calibration.refineSharedPrincipalPoint = True
    o.calibration.refineSharedRadialDistortion = True
    o.solver.maxIterations = 80
    return p, o, {"loss": "cauchy", "scale": 1.5, "max_iterations": 80,
                  "intrinsics": ["focal", "principal_point", "radial"]}


CASES = {"ring_10cam_400pt": ring_case, "aerial_20cam_1500pt": aerial_case}


def options_from_meta(meta):
    """SolveOptions of a fixture's metadata."""
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber if meta["loss"] == "huber" else ImageRobustLoss.Cauchy
    o.solver.imageRobustLossScalePixels = meta["scale"]
    o.solver.maxIterations = meta["max_iterations"]
    o.calibration.refineSharedFocalLength = "focal" in meta["intrinsics"]
    o.calibration.refineSharedPrincipalPoint = "principal_point" in meta["intrinsics"]
    o.calibration.refineSharedRadialDistortion = "radial" in meta["intrinsics"]
    return o


def problem_from_fixture(z):
    """Problem of a fixture (all arrays stored, calibration groups included)."""
    from plabundle_gb300.problem import Problem
    groups = z["cameraCalibrationGroupIds"] if "cameraCalibrationGroupIds" in z else None
    if groups is not None and groups.size == 0:
        groups = None
    return Problem(cameras=z["cameras"], points=z["points"], track_offsets=z["track_offsets"],
                   obs_camera=z["obs_camera"], obs_u=z["obs_u"], obs_v=z["obs_v"], obs_weight=z["obs_weight"],
                   obs_scale=z["obs_scale"], cameraCalibrationGroupIds=groups)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    import oracle as O
    sums = {}
    for name, make in CASES.items():
        p, o, meta = make()
        p = p.normalized()
        ref = O.Oracle(p, o, num_threads=1).solve()
        rep = ref["report"]
        arrays = {k: getattr(p, k) for k in PROBLEM_KEYS}
        arrays["cameraCalibrationGroupIds"] = (p.cameraCalibrationGroupIds if p.cameraCalibrationGroupIds is not None
                                               else np.zeros(0, np.int32))
        arrays.update({"out_cameras": ref["cameras"], "out_points": ref["points"],
                       "out_valid": ref["valid"].astype(np.int8), "out_rms_before": ref["rms_before"],
                       "out_rms_after": ref["rms_after"], "out_intrinsics": ref["intrinsics"]})
        report = {k: (float(v) if isinstance(v, (float, np.floating)) else int(v)) for k, v in rep.items()
                  if isinstance(v, (int, float, np.integer, np.floating))}
        arrays["meta"] = np.frombuffer(json.dumps({"options": meta, "report": report}).encode(), np.uint8)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **arrays)
        for k, v in arrays.items():
            sums[f"{name}:{k}"] = digest(v)
        print(name, "status", report.get("status"), "iterations", report.get("iterations"),
              "final cost", report.get("final_cost"))
    with open(os.path.join(HERE, "SHA256SUMS"), "w") as f:
        for k in sorted(sums):
            f.write(f"{sums[k]}  {k}\n")


if __name__ == "__main__":
    main()
