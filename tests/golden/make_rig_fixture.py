"""Generates the fixture of the 3 000-camera rig block: the CPU FP64 oracle run to convergence.

The workload is the large oblique survey configuration as `bench.py --workload rig3000` builds it:
`synth.rig_grid_problem(seed=21)` (600 captures of 5-camera rigs: a fixed nadir sensor and four
45-degree obliques whose extrinsics are refined, 1.5 M points, ~8.2 M observations, 0.7 px noise,
5 % outliers), 40 control points (2 cm, seed 3), 10 scale bars (5 mm, seed 5), Cauchy loss at
1.5 px, no intrinsics refined, up to 200 LM iterations with the reference's stopping rule; the
scale bars put the solve on the general path.  As for the 500-camera fixture
(`make_c1_fixture.py`), the problem is pinned by the SHA-256 of its integer arrays and a seeded
sample of every floating-point array (the rig records included); the oracle's linear solves are
direct, without a post-solve gate on the true residual.

Stored: the oracle's report, the refined cameras (3 000 x 32), captures and sensors (12 doubles
each), the inlier mask (bit-packed), a seeded sample of 4 096 refined points, and the wall time
of the whole CPU solve with its thread count and CPU model.

    python tests/golden/make_rig_fixture.py [--threads N]    # ~80 min on 8 x86 cores (the oracle's
                                                             # dense damped solve runs on one thread)
"""
from __future__ import annotations

import argparse
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
sys.path.insert(0, HERE)

import make_c1_fixture as C1  # noqa: E402  (digests, samples and the comparison helpers)

FIXTURE = os.path.join(HERE, "rig_block_600cap_oracle.npz")
RIG_SAMPLE = 256


def rig_workload():
    """(problem, options) of the rig block, exactly as the benchmark builds them."""
    from plabundle_gb300 import synth
    from plabundle_gb300.problem import ImageRobustLoss, SolveOptions
    prob = synth.rig_grid_problem(seed=21)
    synth.with_control_points(prob, n=40, sigma=0.02, seed=3)
    synth.with_scale_bars(prob, n=10, sigma=0.005, seed=5)
    opts = SolveOptions()
    opts.solver.imageRobustLoss = ImageRobustLoss.Cauchy
    opts.solver.imageRobustLossScalePixels = 1.5
    opts.solver.maxIterations = 200
    opts.backend.linearRelativeTolerance = 1e-6
    return prob, opts


def rig_arrays(prob):
    cap, cap_info, sen, sen_info, cam_cap, cam_sen = prob.rig.arrays(prob.n_cameras)
    return {"rig_captures": cap, "rig_sensors": sen, "rig_capture_info": cap_info, "rig_sensor_info": sen_info,
            "rig_camera_capture": cam_cap, "rig_camera_sensor": cam_sen}


def problem_mismatch(meta, arrays, prob):
    """None when the generator reproduces the fixture's problem (as `make_c1_fixture` checks it,
    plus the rig records: integer arrays exactly, the sampled capture and sensor entries to its
    tolerance), else a description of the first difference."""
    m = C1.problem_mismatch(meta, arrays, prob)
    if m:
        return m
    ra = rig_arrays(prob)
    for k in ("rig_capture_info", "rig_sensor_info", "rig_camera_capture", "rig_camera_sensor"):
        if not np.array_equal(ra[k], arrays["in_" + k]):
            return f"{k} differs (rig structure)"
    for k in ("rig_captures", "rig_sensors"):
        idx = arrays["sample_idx_" + k]
        a = ra[k].ravel()
        if a.size != meta["float_sizes"][k]:
            return f"{k} has {a.size} entries, the fixture {meta['float_sizes'][k]}"
        err = np.abs(a[idx] - arrays["sample_val_" + k]) / np.maximum(1.0, np.abs(arrays["sample_val_" + k]))
        if err.max() > C1.FLOAT_RTOL:
            return f"{k} differs by {err.max():.3e} relative"
    return None


def compare(meta, arrays, cameras, captures, sensors, valid, rms_after, points, final_cost, filter_threshold):
    """Parity of a solution of the rig block against the oracle's converged solution: the
    500-camera comparison's quantities (no intrinsics are refined here) plus the capture-centre
    error relative to the scene extent and the largest sensor-parameter difference."""
    out = C1.compare(meta, arrays, cameras, np.zeros((0, 13)), valid, rms_after, points, final_cost,
                     filter_threshold)
    out.pop("intrinsics_rel_err", None)
    C0 = arrays["out_cameras"][:, 9:12]
    extent = float(np.linalg.norm(C0 - C0.mean(0), axis=1).max())
    out["capture_centre_rel_err"] = float(np.abs(captures[:, 9:12] - arrays["out_captures"][:, 9:12]).max() / extent)
    out["sensor_max_abs_err"] = float(np.abs(sensors - arrays["out_sensors"]).max())
    return out


def load_fixture(path=FIXTURE):
    return C1.load_fixture(path)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    import oracle as O
    prob, opts = rig_workload()
    digests = C1.problem_digests(prob)
    t0 = time.perf_counter()
    orc = O.Oracle(prob, opts, num_threads=args.threads, residual_gate=False)
    ref = orc.solve()
    wall = time.perf_counter() - t0
    rep = ref["report"]
    report = {k: (float(v) if isinstance(v, (float, np.floating)) else int(v)) for k, v in rep.items()
              if isinstance(v, (int, float, np.integer, np.floating))}
    thr = report["filter_threshold"]
    near = np.nonzero(np.abs(ref["rms_after"] - thr) <= 0.1 * thr)[0].astype(np.int64)
    idx = C1.point_sample(prob.n_tracks)
    ra = rig_arrays(prob)
    meta = {"workload": "rig_block_600cap_5cam_1500kpt_40gcp_10bars, seed 21 (control points seed 3, scale bars "
                        "seed 5), Cauchy 1.5 px, no intrinsics refined, max 200 LM iterations, general path",
            "problem_sha256": digests, "n_tracks": int(prob.n_tracks), "n_obs": int(prob.n_obs),
            "report": report, "wall_seconds": wall, "threads": args.threads, "cpu": C1.cpu_model(),
            "machine": platform.machine(), "point_sample_seed": C1.POINT_SAMPLE_SEED,
            "oracle_linear_solve": "dense FP64 Cholesky of the live unknowns, iterative refinement, no post-solve gate",
            "float_sizes": dict({k: int(np.asarray(getattr(prob.normalized(), k)).size) for k in C1.FLOAT_KEYS},
                                rig_captures=int(ra["rig_captures"].size), rig_sensors=int(ra["rig_sensors"].size))}
    extra = {}
    for k, (s_idx, s_val) in C1.float_samples(prob).items():
        extra["sample_idx_" + k] = s_idx
        extra["sample_val_" + k] = s_val
    rng = np.random.default_rng(C1.FLOAT_SAMPLE_SEED)
    for k in ("rig_captures", "rig_sensors"):
        a = ra[k].ravel()
        s_idx = np.sort(rng.choice(a.size, size=min(RIG_SAMPLE, a.size), replace=False)).astype(np.int64)
        extra["sample_idx_" + k] = s_idx
        extra["sample_val_" + k] = a[s_idx].copy()
    for k in ("rig_capture_info", "rig_sensor_info", "rig_camera_capture", "rig_camera_sensor"):
        extra["in_" + k] = ra[k]
    np.savez_compressed(FIXTURE, meta=np.frombuffer(json.dumps(meta).encode(), np.uint8), **extra,
                        out_cameras=ref["cameras"], out_captures=ref["captures"], out_sensors=ref["sensors"],
                        out_intrinsics=np.zeros((0, 13)),
                        out_valid_bits=np.packbits(ref["valid"].astype(np.uint8)),
                        near_threshold_tracks=near, near_threshold_rms_after=ref["rms_after"][near],
                        point_sample_tracks=idx, point_sample=ref["points"][idx])
    print(json.dumps({"status": report["status"], "iterations": report["iterations"],
                      "final_cost": report["final_cost"], "wall_seconds": wall, "fixture": FIXTURE}))


if __name__ == "__main__":
    main()
