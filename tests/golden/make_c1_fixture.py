"""Generates the fixture of the 500-camera aerial solve: the CPU FP64 oracle run to convergence.

The workload is the one the time-to-converge metric is quoted on: the 25x20 nadir grid
(`synth.aerial_grid_problem(seed=11)`: 500 cameras, 200 k points, ~1.36 M observations), two
calibration groups refining f, cx, cy, k1..k3, p1, p2, Cauchy loss at 1.5 px, up to 200 LM
iterations with the reference's stopping rule.  The problem is too large to store, so the
fixture pins the generator instead: the SHA-256 of every integer array of the generated problem
(track structure, cameras of the observations, calibration groups) and a seeded sample of 2 048
entries of every floating-point array.  A machine whose generator reproduces the structure
exactly and the sampled values to 1e-10 relative (the elementary functions of numpy may round
differently on another CPU) solves the same problem; otherwise the tests skip rather than
compare against another problem.

The linear solves of the oracle are direct (dense FP64 Cholesky of the live unknowns with
iterative refinement) and are accepted as solved (no post-solve gate on the true residual): near
the fixed point of this ill-conditioned problem (focal length against altitude) the true residual
of any FP64 solve sits above the 2e-10 relative tolerance, where a gate rejects the step and ends
the solve on a damped step short of the fixed point.  A CG solver that stops on its recursive
residual - the GPU paths - does not see that floor; with the gate off the oracle follows the
same exact Gauss-Newton trajectory to the fixed point.

Stored: the oracle's report (status, iterations, initial / final cost, filter threshold, ...),
the refined cameras (500 x 32), the group intrinsics, the inlier mask (bit-packed), the strict
after-RMS of the tracks within 10 % of the filter threshold (for the margin of any track whose
inlier flag differs), a seeded sample of 4 096 refined points, and the wall time of the whole
CPU solve with its thread count and CPU model (a measured, converged solve beside the bench's
sampled CPU baseline).

    python tests/golden/make_c1_fixture.py [--threads N]    # ~10-20 min on 8 cores
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

PROBLEM_KEYS = ("cameras", "points", "track_offsets", "obs_camera", "obs_u", "obs_v", "obs_weight", "obs_scale",
                "cameraCalibrationGroupIds")
INTEGER_KEYS = ("track_offsets", "obs_camera", "cameraCalibrationGroupIds")
FLOAT_KEYS = ("cameras", "points", "obs_u", "obs_v", "obs_weight", "obs_scale")
FLOAT_SAMPLE = 2048
FLOAT_SAMPLE_SEED = 5
FLOAT_RTOL = 1e-10
FIXTURE = os.path.join(HERE, "aerial_500cam_200kpt_oracle.npz")
POINT_SAMPLE = 4096
POINT_SAMPLE_SEED = 97


def c1_workload():
    """(problem, options) of the 500-camera aerial solve, exactly as the benchmark builds them."""
    from plabundle_gb300 import synth
    from plabundle_gb300.problem import ImageRobustLoss, SolveOptions
    prob = synth.aerial_grid_problem(seed=11)
    opts = SolveOptions()
    opts.solver.imageRobustLoss = ImageRobustLoss.Cauchy
    opts.solver.imageRobustLossScalePixels = 1.5
    opts.calibration.refineSharedFocalLength = True
    opts.calibration.refineSharedPrincipalPoint = True
    opts.calibration.refineSharedRadialDistortion = True
    opts.solver.maxIterations = 200
    return prob, opts


def problem_digests(prob):
    p = prob.normalized()
    out = {}
    for k in PROBLEM_KEYS:
        a = getattr(p, k)
        out[k] = None if a is None else hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    return out


def float_samples(prob):
    """{key: (flat indices, values)} of a seeded sample of every floating-point problem array."""
    p = prob.normalized()
    rng = np.random.default_rng(FLOAT_SAMPLE_SEED)
    out = {}
    for k in FLOAT_KEYS:
        a = np.ascontiguousarray(getattr(p, k)).ravel()
        idx = np.sort(rng.choice(a.size, size=min(FLOAT_SAMPLE, a.size), replace=False)).astype(np.int64)
        out[k] = (idx, a[idx].copy())
    return out


def point_sample(n_tracks):
    rng = np.random.default_rng(POINT_SAMPLE_SEED)
    return np.sort(rng.choice(n_tracks, size=min(POINT_SAMPLE, n_tracks), replace=False)).astype(np.int64)


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def load_fixture(path=FIXTURE):
    """(meta dict, arrays dict) of the fixture, or None when it is absent."""
    if not os.path.exists(path):
        return None
    z = np.load(path)
    meta = json.loads(bytes(z["meta"]).decode())
    return meta, {k: z[k] for k in z.files if k != "meta"}


def problem_mismatch(meta, arrays, prob):
    """None when the generator reproduces the fixture's problem (integer arrays bit for bit, the
    sampled floating-point entries to FLOAT_RTOL), else a description of the first difference."""
    d = problem_digests(prob)
    for k in INTEGER_KEYS:
        if d[k] != meta["problem_sha256"][k]:
            return f"{k} differs (structure)"
    p = prob.normalized()
    for k in FLOAT_KEYS:
        a = np.ascontiguousarray(getattr(p, k)).ravel()
        idx, ref = arrays["sample_idx_" + k], arrays["sample_val_" + k]
        if a.size != meta["float_sizes"][k]:
            return f"{k} has {a.size} entries, the fixture {meta['float_sizes'][k]}"
        err = np.abs(a[idx] - ref) / np.maximum(1.0, np.abs(ref))
        if err.max() > FLOAT_RTOL:
            return f"{k} differs by {err.max():.3e} relative"
    return None


def compare(meta, arrays, cameras, intrinsics, valid, rms_after, points, final_cost, filter_threshold):
    """Parity of a solution of the 500-camera problem against the oracle's converged solution:
    relative final cost, camera-centre error relative to the scene extent (largest distance of
    an oracle centre from their mean), rotation error (largest entry), relative intrinsic error
    of the refined groups, point error on the seeded sample relative to the scene extent, and
    the inlier mask: the number of tracks whose flag differs, with the margin of each flipped
    track's after-RMS to the filter threshold (BundleAdjustQuality.cpp:381-401)."""
    ref_cost = meta["report"]["final_cost"]
    C0 = arrays["out_cameras"][:, 9:12]
    extent = float(np.linalg.norm(C0 - C0.mean(0), axis=1).max())
    cam_err = float(np.abs(cameras[:, 9:12] - C0).max() / extent)
    rot_err = float(np.abs(cameras[:, 0:9] - arrays["out_cameras"][:, 0:9]).max())
    ri = arrays["out_intrinsics"]
    intr = np.asarray(intrinsics)[:ri.shape[0]]
    denom = np.maximum(np.abs(ri), 1e-12)
    used = np.abs(intr - ri) > 0
    intr_err = float((np.abs(intr - ri) / denom)[used].max()) if used.any() else 0.0
    idx = arrays["point_sample_tracks"]
    pt_err = float(np.abs(points[idx] - arrays["point_sample"]).max() / extent)
    ref_valid = np.unpackbits(arrays["out_valid_bits"])[:meta["n_tracks"]].astype(bool)
    flips = np.nonzero(np.asarray(valid, bool) != ref_valid)[0]
    margins = [float(rms_after[t] - filter_threshold) for t in flips[:32]]
    return {"final_cost_rel_err": abs(final_cost - ref_cost) / abs(ref_cost),
            "camera_centre_rel_err": cam_err, "rotation_max_abs_err": rot_err,
            "intrinsics_rel_err": intr_err, "point_sample_rel_err": pt_err,
            "inlier_mask_flips": int(flips.size), "flip_margins_px": margins,
            "oracle_final_cost": ref_cost, "oracle_iterations": meta["report"]["iterations"],
            "oracle_status": meta["report"]["status"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    import oracle as O
    prob, opts = c1_workload()
    digests = problem_digests(prob)
    t0 = time.perf_counter()
    orc = O.Oracle(prob, opts, num_threads=args.threads, residual_gate=False)
    ref = orc.solve()
    wall = time.perf_counter() - t0
    rep = ref["report"]
    report = {k: (float(v) if isinstance(v, (float, np.floating)) else int(v)) for k, v in rep.items()
              if isinstance(v, (int, float, np.integer, np.floating))}
    thr = report["filter_threshold"]
    near = np.nonzero(np.abs(ref["rms_after"] - thr) <= 0.1 * thr)[0].astype(np.int64)
    idx = point_sample(prob.n_tracks)
    meta = {"workload": "aerial_grid_500cam_200kpt, seed 11, Cauchy 1.5 px, 2 groups (f, cx, cy, k1-k3, p1, p2), "
                        "max 200 LM iterations",
            "problem_sha256": digests, "n_tracks": int(prob.n_tracks), "n_obs": int(prob.n_obs),
            "report": report, "wall_seconds": wall, "threads": args.threads, "cpu": cpu_model(),
            "machine": platform.machine(), "point_sample_seed": POINT_SAMPLE_SEED,
            "oracle_linear_solve": "dense FP64 Cholesky of the live unknowns, iterative refinement, no post-solve gate",
            "float_sizes": {k: int(np.asarray(getattr(prob.normalized(), k)).size) for k in FLOAT_KEYS}}
    samples = float_samples(prob)
    extra = {}
    for k, (s_idx, s_val) in samples.items():
        extra["sample_idx_" + k] = s_idx
        extra["sample_val_" + k] = s_val
    np.savez_compressed(FIXTURE, meta=np.frombuffer(json.dumps(meta).encode(), np.uint8), **extra,
                        out_cameras=ref["cameras"], out_intrinsics=ref["intrinsics"],
                        out_valid_bits=np.packbits(ref["valid"].astype(np.uint8)),
                        near_threshold_tracks=near, near_threshold_rms_after=ref["rms_after"][near],
                        point_sample_tracks=idx, point_sample=ref["points"][idx])
    print(json.dumps({"status": report["status"], "iterations": report["iterations"],
                      "final_cost": report["final_cost"], "wall_seconds": wall, "threads": args.threads}))


if __name__ == "__main__":
    main()
