#!/usr/bin/env python
"""Time-to-converge of the GB300 reduced-Schur bundle adjustment.

Workload (one "step" = one complete bundle adjustment from the initial state to convergence):
the 500-camera / 200k-point aerial grid (25x20 nadir cameras at 100 m, 80/60 % overlap,
6000x4000 px, f=4000 px, sum-of-8-sinusoids terrain with 20 m amplitude, 3..12 observations per
track, two calibration groups refining f, cx, cy, k1..k3, p1, p2, 0.5 px noise, 3 % outliers,
Cauchy loss at 1.5 px), seeded synthetic data.  The headline arm runs FP32 Jacobians / Schur /
PCG with compensated sums, FP64 cost and gain ratio and FP64-residual refinement; the FP64 GPU
path runs the same kernels instantiated in double precision.

`python bench.py [--gpus N --steps K --warmup W] [--impl reference]`
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "BA time-to-converge at 1e-6 rel cost, mixed vs FP64 on GB300; Schur/PCG HBM GB/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="aerial",
                    choices=["aerial", "aerial_gcp", "aerial3000_gcp", "rig3000", "ring", "windows", "adjoint"])
    ap.add_argument("--windows", type=int, default=256, help="local-BA windows of the windows workload")
    ap.add_argument("--workers", type=int, default=0,
                    help="worker contexts of the windows workload (0: chosen by the batch autotuner)")
    ap.add_argument("--cpu-iterations", type=int, default=2,
                    help="LM iterations of the bounded CPU sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fd-obs", type=int, default=64,
                    help="observations of the finite-difference check of the adjoint workload")
    ap.add_argument("--no-secondary", action="store_true",
                    help="leave out the windows and backward-pass records of the default 1-GPU run")
    return ap.parse_args()


# LM iterations of a converged CPU solve of the large workloads, which a bounded CPU sample is
# scaled to.  The 500-camera grid uses the oracle's own converged solve, measured when its fixture
# was generated (tests/golden/aerial_500cam_200kpt_oracle.npz: 36 iterations); the control-point
# workloads have no CPU fixture and use the iteration counts of the FP64 GPU path on them.  The
# 20-camera ring is solved in full on the CPU (a fraction of a second), with no scaling.
FP64_GPU_ITERATIONS = {"aerial_gcp": 21, "aerial3000_gcp": 27, "rig3000": 40}


def converged_iterations(workload_name):
    """(LM iterations of a converged CPU solve, where the count comes from), or (None, ...) for a
    workload that the CPU solves in full."""
    if workload_name == "ring":
        return None, "full solve"
    if workload_name == "aerial":
        m = measured_converged_cpu_solve(workload_name)
        if m is not None:
            return m["iterations"], "the oracle's converged solve of the committed fixture"
    return FP64_GPU_ITERATIONS.get(workload_name, 36), "the FP64 GPU path's converged solve"

# DRAM traffic of one k_assemble<float> launch per observation: dram__bytes_read.sum +
# dram__bytes_write.sum of an ncu capture on the 250-camera / 100k-point aerial grid
# (663 659 observations; profiles/k_assemble_aerial250.md).  The chunk plan is the same at 500
# cameras, so the traffic scales with the observations.
ASSEMBLY_DRAM_BYTES_PER_OBS = (38.440192e6 + 253.206528e6) / 663659
# Warp instructions of one k_assemble<float> launch per observation (smsp__inst_executed.sum of the
# same capture).
ASSEMBLY_INST_PER_OBS = 681889338 / 663659
SMS = 152  # streaming multiprocessors of a GB300

# What the mixed path keeps in FP64 (everything else of the assembly and the CG preconditioner is
# FP32 or float-float on the FP32 pipe).
MIXED_FP64_SPLIT = ("projection and residual; 3x3 point blocks, their factor and the per-observation "
                    "projector (phases B and C of the assembly); point back-substitution; the reduced matrix "
                    "and vectors of the CG (FP64 SpMV), the cost, gain ratio and line search; FP32: Jacobians, "
                    "the dense preconditioner factor; float-float: robust weight, gradient chain, all Schur "
                    "products and sums")


def workload(name, problem=None):
    """(problem, options, config) of a named workload; `problem`: the 500-camera grid when the
    caller has generated it already (the generator is seeded, so it is the same problem)."""
    from plabundle_gb300 import synth
    from plabundle_gb300.problem import ImageRobustLoss, SolveOptions
    opts = SolveOptions()
    if name in ("aerial", "aerial_gcp", "aerial3000_gcp"):
        if name == "aerial" and problem is not None:
            prob = problem
        elif name == "aerial3000_gcp":
            # the 3 000-camera block of the large survey configuration (60 x 50 nadir grid,
            # 1.5 M points, ~10 M observations) without rigs or scale bars
            prob = synth.aerial_grid_problem(seed=21, n_along=60, n_lines=50, n_points=1_500_000)
        else:
            prob = synth.aerial_grid_problem(seed=11)
        opts.solver.imageRobustLoss = ImageRobustLoss.Cauchy
        opts.solver.imageRobustLossScalePixels = 1.5
        opts.calibration.refineSharedFocalLength = True
        opts.calibration.refineSharedPrincipalPoint = True
        opts.calibration.refineSharedRadialDistortion = True
        # time to converge: the solve runs until the reference's stopping rule (step RMS <= 1e-6)
        opts.solver.maxIterations = 200
        cfg = {"workload": "aerial_grid_%dcam_%dkpt" % (prob.n_cameras, round(prob.n_tracks / 1000)),
               "cameras": prob.n_cameras, "tracks": prob.n_tracks,
               "observations": prob.n_obs, "calibration_groups": 2, "loss": "cauchy_1.5px",
               "refined_intrinsics": "f, cx, cy, k1, k2, k3, p1, p2",
               "max_lm_iterations": opts.solver.maxIterations, "stopping": "step RMS <= 1e-6 (converged)"}
        if name in ("aerial_gcp", "aerial3000_gcp"):
            # 40 ground control points on tracks seen by two cameras (2 cm, three uncertainty forms):
            # complete control-point gauge, plain parameterisation
            synth.with_control_points(prob, n=40, sigma=0.02, seed=3)
            cfg.update(workload=cfg["workload"] + "_40gcp", control_points=len(prob.controlPoints))
    elif name == "rig3000":
        # the large oblique survey block: 600 captures of 5-camera rigs (nadir plus four obliques at
        # 45 degrees; the nadir sensor fixed, the four oblique extrinsics refined jointly), 1.5 M
        # points, ~8 M observations, 40 control points (2 cm), 10 scale bars (5 mm), 0.7 px noise,
        # 5 % outliers; the scale bars put the solve on the general path, the reduced solve runs to
        # 1e-6 relative residual
        prob = synth.rig_grid_problem(seed=21)
        synth.with_control_points(prob, n=40, sigma=0.02, seed=3)
        synth.with_scale_bars(prob, n=10, sigma=0.005, seed=5)
        opts.solver.imageRobustLoss = ImageRobustLoss.Cauchy
        opts.solver.imageRobustLossScalePixels = 1.5
        opts.solver.maxIterations = 200
        opts.backend.linearRelativeTolerance = 1e-6
        cfg = {"workload": "rig_block_%dcap_5cam_%dkpt_40gcp_10bars" % (len(prob.rig.captures),
                                                                       round(prob.n_tracks / 1000)),
               "cameras": prob.n_cameras, "captures": len(prob.rig.captures), "sensors": len(prob.rig.sensors),
               "tracks": prob.n_tracks, "observations": prob.n_obs, "control_points": len(prob.controlPoints),
               "scale_bars": len(prob.scaleBarConstraints), "loss": "cauchy_1.5px", "refined_intrinsics": "none",
               "linear_relative_tolerance": 1e-6, "max_lm_iterations": opts.solver.maxIterations,
               "stopping": "step RMS <= 1e-6 (converged)"}
    else:
        prob = synth.ring_problem(seed=7)
        opts.solver.imageRobustLoss = ImageRobustLoss.Huber
        opts.solver.imageRobustLossScalePixels = 1.5
        cfg = {"workload": "ring_20cam_2kpt", "cameras": prob.n_cameras, "tracks": prob.n_tracks,
               "observations": prob.n_obs, "loss": "huber_1.5px", "max_lm_iterations": opts.solver.maxIterations}
    return prob, opts, cfg


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def cpu_cores():
    return os.cpu_count() or 1


def max_over_ranks(value: float, world: int) -> float:
    """The largest value over the ranks of the job (a job's time is its slowest rank's); the
    process group's own device (NCCL: the current GPU, gloo: the host)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def window_seed(rank: int) -> int:
    """Seed of a rank's set of local-BA windows: every rank solves its own windows (weak scaling)."""
    return 1234 + rank


def cpu_sample(prob, opts, iterations, full_iterations):
    """Oracle (CPU FP64 restatement, all host threads) on `iterations` LM iterations of the
    workload, scaled to `full_iterations` iterations (ms per full solve); with
    `full_iterations` None, the whole solve under the workload's own budget, unscaled.  The
    scaling takes the LM loop's time per iteration (the oracle's own clock around the loop) and
    adds the rest of the call (quality finalisation and output copies) once."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    import copy
    o2 = copy.deepcopy(opts)
    if full_iterations is not None:
        o2.solver.maxIterations = iterations
    orc = O.Oracle(prob, o2, num_threads=cpu_cores())
    t = time.perf_counter()
    r = orc.solve()
    dt = time.perf_counter() - t
    it = max(1, r["report"]["iterations"])
    loop = min(dt, float(r["report"]["solve_seconds"]))
    per_it = loop / it
    info = {"sample_iterations": it, "sample_seconds": dt, "per_iteration_ms": per_it * 1e3,
            "fixed_ms": (dt - loop) * 1e3}
    if full_iterations is None:
        return dt * 1e3, info
    return (dt - loop + per_it * full_iterations) * 1e3, info


def cpu_sample_text(info, full_it, source):
    if full_it is None:
        return (f"the complete converged solve ({info['sample_iterations']} LM iterations, "
                f"{info['sample_seconds']:.2f} s); CPU FP64 restatement of the reference with OpenMP")
    return (f"{info['sample_iterations']} LM iterations of the workload ({info['sample_seconds']:.1f} s: "
            f"{info['per_iteration_ms']:.0f} ms per LM iteration, {info['fixed_ms']:.0f} ms of finalisation), "
            f"scaled to the {full_it} iterations of {source}; CPU FP64 restatement of the reference with OpenMP")


def problem_bytes(prob):
    p = prob.normalized()
    h2d = sum(a.nbytes for a in (p.cameras, p.points, p.track_offsets, p.obs_camera, p.obs_u, p.obs_v,
                                 p.obs_weight, p.obs_scale))
    if p.cameraCalibrationGroupIds is not None:
        h2d += p.cameraCalibrationGroupIds.nbytes
    d2h = p.cameras.nbytes + p.points.nbytes + p.n_tracks * (1 + 8 + 8)
    return h2d, d2h


def measured_converged_cpu_solve(workload_name):
    """Wall time of one complete converged CPU FP64 solve of the 500-camera workload, measured when
    its committed fixture was generated (a cross-check of the sampled CPU baseline), or None."""
    if workload_name != "aerial":
        return None
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_c1_fixture as FX
    fx = FX.load_fixture()
    if fx is None:
        return None
    m = fx[0]
    return {"seconds": m["wall_seconds"], "threads": m["threads"], "cpu": m["cpu"], "machine": m["machine"],
            "iterations": m["report"]["iterations"], "status": m["report"]["status"],
            "source": "tests/golden/aerial_500cam_200kpt_oracle.npz (make_c1_fixture.py)"}


def bench_config(cfg):
    """`config` of the headline line, the same on the GB300 arm and the reference arm."""
    return dict(cfg, l2="flushed between steps (256 MB write)", parallelism="replicas")


def run_reference(args, rank):
    if rank != 0:
        return
    prob, opts, cfg = workload(args.workload)
    full_it, source = converged_iterations(args.workload)
    vals = []
    for i in range(args.warmup + args.steps):
        ms, info = cpu_sample(prob, opts, args.cpu_iterations, full_it)
        if i >= args.warmup:
            vals.append(ms)
    v = statistics.mean(vals)
    line = {"metric": METRIC, "value": v, "unit": "ms", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": bench_config(cfg),
            "cpu_baseline": {"value": v, "unit": "ms", "cores": cpu_cores(), "kind": "port",
                             "sample": "per step: " + cpu_sample_text(info, full_it, source),
                             "converged_solve_measured": measured_converged_cpu_solve(args.workload)},
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_windows(args, rank, world, local_rank):
    line = measure_windows(args.windows, args.workers, args.steps, rank, world, local_rank)
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_windows(n_windows, workers, steps, rank, world, local_rank):
    """Batched local BA: independent ring windows (10-60 cameras, 1k-20k points, each generated
    like the 20-camera ring with its own seed), mixed precision, 20 LM iterations, solved through
    pb_gpu_solve_batch with `workers` contexts (0: chosen by the batch autotuner), against the same
    windows one at a time.  Host wall clock (the batch spans several streams); inputs start in host
    memory.  Returns the bench line (rank 0; None on the other ranks)."""
    import numpy as np
    import torch
    from plabundle_gb300 import synth
    from plabundle_gb300.batch import solve_batch, tune_workers
    from plabundle_gb300.problem import ImageRobustLoss, SolveOptions

    wins = synth.window_problems(n_windows=n_windows, seed=window_seed(rank))
    torch.cuda.set_device(local_rank)
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    o.solver.maxIterations = 20
    o.backend.enablePlaMatrixMixedPrecision = True
    # worker count: the batch's autotuner on a sample of this rank's windows (--workers 0), or as given
    tuned = None
    if workers <= 0:
        workers, tuned = tune_workers(wins, o, device=local_rank)
    solve_batch(wins[:2 * workers], o, n_workers=workers, device=local_rank)  # warm-up
    rates, lats = [], None
    for _ in range(max(1, steps)):
        # whole-job rate: every rank's windows over the slowest rank's time
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res, lat = solve_batch(wins, o, n_workers=workers, device=local_rank)
        torch.cuda.synchronize()
        dt = max_over_ranks(time.perf_counter() - t0, world)
        rates.append(world * len(wins) / dt)
        lats = lat
    t0 = time.perf_counter()
    res1, lat1 = solve_batch(wins, o, n_workers=1, device=local_rank)
    seq_rate = len(wins) / (time.perf_counter() - t0)
    ok = sum(1 for r in res if r["status"] in (1, 2))
    same = sum(1 for a, b in zip(res, res1) if a["final_cost"] == b["final_cost"])
    if rank != 0:
        return None
    return {"metric": "local-BA windows per second (batched)", "value": statistics.mean(rates), "unit": "windows/s",
            "impl": "gb300", "n_gpus": world, "steps": steps, "warmup": 1, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)", "data": "synthetic (seeded)",
            "config": {"workload": f"{len(wins)} ring windows per GPU, 10-60 cameras, 1k-20k points",
                       "observations": int(sum(p.n_obs for p in wins)), "workers": workers,
                       "workers_tuned": tuned,
                       "max_lm_iterations": 20, "loss": "huber_1.5px"},
            "latency_ms": {"p50": float(np.percentile(lats, 50)), "p99": float(np.percentile(lats, 99))},
            "one_at_a_time": {"windows_per_s": seq_rate, "latency_p50_ms": float(np.percentile(lat1, 50)),
                              "latency_p99_ms": float(np.percentile(lat1, 99))},
            "speedup_vs_one_at_a_time": statistics.mean(rates) / seq_rate,
            "solved": ok, "identical_to_one_at_a_time": same}


def run_adjoint(args, rank, world, local_rank):
    line = measure_adjoint(args.steps, args.warmup, args.fd_obs, rank, world, local_rank)
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_adjoint(steps, warmup, fd_obs, rank, world, local_rank, problem=None):
    """Backward pass of the converged 500-camera aerial solve (mixed precision): implicit
    differentiation with the exact Hessian of L = sum_i |C_i - (C_i_true + N(0, 0.1 m))|^2 with
    respect to every observation and initial pose.  value: device time of one pb_gpu_backward
    (Hessian records, reduced system, solve, gradients; CUDA events on the context's stream);
    e2e: the same call through the Python API with its host buffers (the loss gradient in,
    dL/d(u, v) and dL/d(initial pose) out).  Then the central finite-difference check (h = 1e-3
    px) on --fd-obs random observations: every perturbed solve restarts from the saved fixed
    point and is re-converged with full Gauss-Newton steps.  `problem`: the 500-camera grid when
    the caller has generated it already.  Returns the bench line (rank 0; None on the others)."""
    import numpy as np
    import torch
    from plabundle_gb300.adjoint import camera_centre_loss, newton_polish
    from plabundle_gb300.device import Gb300Context

    torch.cuda.set_device(local_rank)
    prob, opts, cfg = workload("aerial", problem)
    opts.backend.enablePlaMatrixMixedPrecision = True
    ctx = Gb300Context(local_rank)
    assert ctx.upload(prob, opts) == 0
    rep = ctx.solve()
    trace = newton_polish(ctx, iterations=4)
    d = ctx.download()
    rng = np.random.default_rng(2024)
    targets = prob.truth_cameras[:, 9:12] + rng.normal(0.0, 0.1, (prob.n_cameras, 3))
    L, g = camera_centre_loss(d["cameras"], targets)
    stream = torch.cuda.ExternalStream(ctx.stream_handle())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(warmup):
        out = ctx.backward(grad_cameras=g)
    sampler = ClockSampler(local_rank)
    sampler.start()
    dev_ms, e2e_ms, reports = [], [], []
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record(stream)
        out = ctx.backward(grad_cameras=g)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
        dev_ms.append(e0.elapsed_time(e1))
        reports.append(out["report"])
    clocks = sampler.stop()
    go = out["observations"]
    # finite differences
    ctx.save_state()
    pick = rng.choice(np.nonzero(np.abs(go).sum(1) > 0)[0], fd_obs, replace=False)
    h = 1e-3
    fd = np.zeros((pick.size, 2))
    t_fd = time.perf_counter()
    for i, k in enumerate(pick):
        for a in range(2):
            vals = []
            for sgn in (1.0, -1.0):
                u, v = prob.obs_u[k], prob.obs_v[k]
                ctx.set_observations([k], [u + sgn * h * (a == 0)], [v + sgn * h * (a == 1)])
                ctx.restore_state()
                newton_polish(ctx, iterations=3)
                vals.append(camera_centre_loss(ctx.download()["cameras"], targets)[0])
                ctx.set_observations([k], [u], [v])
            fd[i, a] = (vals[0] - vals[1]) / (2.0 * h)
    t_fd = time.perf_counter() - t_fd
    ctx.restore_state()
    err = np.linalg.norm(go[pick] - fd) / np.linalg.norm(fd)
    per_obs = np.linalg.norm(go[pick] - fd, axis=1) / np.maximum(np.linalg.norm(fd, axis=1), 1e-300)
    last = reports[-1]
    ctx.close()
    if rank != 0:
        return None
    nobs = prob.n_obs
    return {"metric": "adjoint backward time (exact-Hessian implicit differentiation)",
            "value": statistics.mean(dev_ms), "unit": "ms", "impl": "gb300", "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": statistics.mean(dev_ms),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 Hessian records, f32 factor + f64 CG", "data": "synthetic (seeded)",
            "config": dict(cfg, loss_of_solution="sum |C_i - (C_true + N(0, 0.1 m))|^2",
                           l2="flushed between steps (256 MB write)", parallelism="replicas"),
            "phases_ms": {k: last[k] for k in ("hessian_ms", "solve_ms", "gradient_ms", "total_ms")},
            "adjoint_linear_iterations": last["linear_iterations"],
            "adjoint_relative_residual": last["relative_residual"],
            "forward_solve": {"status": rep["status"], "iterations": rep["iterations"],
                              "newton_polish_gradient_norms": [gn for _, gn in trace]},
            "loss": L,
            "fd_check": {"observations": int(pick.size), "h_px": h, "relative_error": float(err),
                         "per_observation_relative_error_median": float(np.median(per_obs)),
                         "per_observation_relative_error_max": float(per_obs.max()),
                         "seconds": t_fd},
            "e2e": {"value": statistics.mean(e2e_ms), "unit": "ms", "h2d_bytes_per_step": int(g.nbytes),
                    "d2h_bytes_per_step": int(16 * nobs + 48 * prob.n_cameras + 24 * prob.n_tracks)},
            "gpu_launches": int(last["gpu_kernel_launches"]),
            "clocks": clocks}


def run_gb300(args, rank, world, local_rank):
    import ctypes as C
    import numpy as np
    import torch
    from plabundle_gb300 import native
    from plabundle_gb300.device import Gb300Context

    torch.cuda.set_device(local_rank)
    prob, opts, cfg = workload(args.workload)
    opts.backend.enablePlaMatrixMixedPrecision = True
    ctx = Gb300Context(local_rank)
    assert ctx.upload(prob, opts) == 0, ctx.L.pb_gpu_last_error(ctx.ctx)
    stream = torch.cuda.ExternalStream(ctx.stream_handle())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed_solves(k, warm):
        for _ in range(warm):
            ctx.solve()
        times, reps = [], []
        for _ in range(k):
            flush.fill_(1.0)  # L2 flush (256 MB > 129 MB L2) outside the timed events
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            reps.append(ctx.solve())
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        return times, reps

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    t_mixed, reps_mixed = timed_solves(args.steps, args.warmup)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    ms_mixed = max_over_ranks(statistics.mean(t_mixed), world)
    out_mixed = ctx.download()
    rig_mixed = ctx.rig()
    hist_mixed = ctx.history()
    launches = sum(r["gpu_kernel_launches"] for r in reps_mixed)

    # FP64 GPU paths (same kernels in double precision): the trajectory-parity arm refactors the
    # FP64 dense preconditioner every LM iteration; the like-for-like arm keeps it across LM
    # iterations under the mixed path's reuse policy (pb_solve_options.factor_reuse = 1)
    ctx.copts.precision = 0
    t_64, reps_64 = timed_solves(max(1, args.steps // 2), 1)
    out_64 = ctx.download()
    rig_64 = ctx.rig()
    hist_64 = ctx.history()
    ms_64 = statistics.mean(t_64)
    ctx.copts.factor_reuse = 1
    t_64r, reps_64r = timed_solves(max(1, args.steps // 2), 1)
    out_64r = ctx.download()
    hist_64r = ctx.history()
    ms_64r = statistics.mean(t_64r)
    ctx.copts.factor_reuse = 0
    ctx.copts.precision = 1

    # per-kernel device times of one mixed solve (CUDA events on the context stream)
    ctx.set_timing(True)
    rep_t = ctx.solve()
    kt = ctx.kernel_times()
    ctx.set_timing(False)
    out_t = ctx.download()

    s = ctx.sizes()
    p = ctx.problem
    nop, ntp = s["observation_count"], s["active_tracks"]
    # algorithmic bytes of one assembly launch: observation records (camera index, u, v, weight,
    # track index, local camera: 33 B) + robust weight written (4 B); per track the point (24 B),
    # block id and observation offset (8 B) and the factor / rhs written (12 x 4 B); the reduced
    # system written (pose blocks both triangles, border, rhs and direct rhs in FP32).
    nnzb = 2 * s["n_pairs"] + s["camera_blocks"]
    red_bytes = 4 * (36 * nnzb + 6 * s["camera_blocks"] * (s["dim"] - 6 * s["camera_blocks"]) + 2 * s["dim"])
    ni = s["ni"]
    asm_bytes = (37 + 4 * (2 * (6 + ni) + 6)) * nop + (24 + 8 + 96) * ntp + red_bytes
    asm_ms = kt["assemble_ms"] / max(1, kt["assemble_launches"])
    peak, peak_kind = measured_peaks()
    achieved = asm_bytes / (asm_ms * 1e-3) / 1e9 if asm_ms > 0 else None
    # issue roofline: warp instructions of one launch (per observation, from the committed ncu
    # capture) over the CUDA-event time, against 4 issue slots per SM per cycle at the sampled clock
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    issue_peak = 4 * SMS * sm_mhz * 1e-3  # G warp instructions / s
    issue_achieved = ASSEMBLY_INST_PER_OBS * nop / (asm_ms * 1e-3) / 1e9 if asm_ms > 0 else None
    # CG (k_dense_cg): bytes one iteration reads -- the FP64 reduced matrix (pose blocks, both
    # border orientations, intrinsic block), the FP32 triangular factor X and X^T (lower triangles
    # of the padded dimension), and eight FP64 vectors; served from L2 after the first iteration
    n = s["dim"]
    npad = 64 * ((n + 63) // 64)
    cg_iter_bytes = (8 * (36 * nnzb + 2 * 6 * s["camera_blocks"] * (n - 6 * s["camera_blocks"])
                          + (n - 6 * s["camera_blocks"]) ** 2)
                     + 2 * 4 * npad * (npad + 64) // 2 + 8 * 8 * n)
    cg_ms = kt["pcg_ms"]
    cg_iters = rep_t["linear_iterations"]
    cg_gbs = cg_iter_bytes * cg_iters / (cg_ms * 1e-3) / 1e9 if cg_ms > 0 else None

    # first call of a fresh context (host planning, chunk plan and device pattern built, device
    # memory allocated) beside the warm end-to-end calls below
    desc, keep = native.problem_desc(prob)
    copts = native.solve_options(opts, prob)
    copts.precision = 1
    pp = keep[0]
    cams = np.zeros_like(pp.cameras)
    pts = np.zeros_like(pp.points)
    valid = np.zeros(pp.n_tracks, np.int8)
    rb = np.zeros(pp.n_tracks)
    ra = np.zeros(pp.n_tracks)
    rep = native.SolveReportC()
    cold_ctx = Gb300Context(local_rank)
    flush.fill_(1.0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = cold_ctx.L.pb_gpu_solve_problem(cold_ctx.ctx, C.byref(desc), C.byref(copts), C.byref(rep), cams.ctypes.data,
                                         pts.ctypes.data, valid.ctypes.data, rb.ctypes.data, ra.ctypes.data)
    cold_ms = (time.perf_counter() - t0) * 1e3
    assert st == 0
    cold_ctx.close()
    e2e = []
    for i in range(args.warmup + args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = ctx.L.pb_gpu_solve_problem(ctx.ctx, C.byref(desc), C.byref(copts), C.byref(rep), cams.ctypes.data,
                                        pts.ctypes.data, valid.ctypes.data, rb.ctypes.data, ra.ctypes.data)
        dt = (time.perf_counter() - t0) * 1e3
        assert st == 0
        if i >= args.warmup:
            e2e.append(dt)
    h2d, d2h = problem_bytes(prob)
    e2e_ms = statistics.mean(e2e)

    # accuracy of the mixed path against the FP64 GPU path
    f_m, f_d = reps_mixed[-1]["final_cost"], reps_64[-1]["final_cost"]
    C64 = out_64["cameras"][:, 9:12]
    scale = np.linalg.norm(C64 - C64.mean(0), axis=1).max()
    cam_err = float(np.abs(out_mixed["cameras"][:, 9:12] - C64).max() / scale)
    f_r = reps_64r[-1]["final_cost"]
    cam_err_r = float(np.abs(out_64r["cameras"][:, 9:12] - C64).max() / scale)

    # accuracy of the mixed path against the CPU FP64 oracle's converged solve of the same problem
    # (committed fixture; compared only when the generator reproduces the fixture's problem)
    vs_oracle = None
    if args.workload == "aerial":
        sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
        import make_c1_fixture as FX
        fx = FX.load_fixture()
        if fx is None:
            vs_oracle = {"unavailable": "fixture absent"}
        elif FX.problem_mismatch(fx[0], fx[1], prob):
            vs_oracle = {"unavailable": "generator does not reproduce the fixture's problem: "
                                        + FX.problem_mismatch(fx[0], fx[1], prob)}
        else:
            vs_oracle = FX.compare(fx[0], fx[1], out_t["cameras"], out_t["intrinsics"], out_t["valid"],
                                   out_t["rms_after"], out_t["points"], rep_t["final_cost"], rep_t["filter_threshold"])
            vs_oracle["oracle_cpu_solve_seconds"] = fx[0]["wall_seconds"]
            vs_oracle["oracle_cpu"] = f"{fx[0]['threads']} threads, {fx[0]['cpu']} ({fx[0]['machine']})"
    elif args.workload == "rig3000":
        sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
        import make_rig_fixture as RFX
        fx = RFX.load_fixture()
        if fx is None:
            vs_oracle = {"unavailable": "fixture absent"}
        elif RFX.problem_mismatch(fx[0], fx[1], prob):
            vs_oracle = {"unavailable": "generator does not reproduce the fixture's problem: "
                                        + RFX.problem_mismatch(fx[0], fx[1], prob)}
        else:
            rig_t = ctx.rig()
            vs_oracle = RFX.compare(fx[0], fx[1], out_t["cameras"], rig_t["captures"], rig_t["sensors"], out_t["valid"],
                                    out_t["rms_after"], out_t["points"], rep_t["final_cost"], rep_t["filter_threshold"])
            vs_oracle["oracle_cpu_solve_seconds"] = fx[0]["wall_seconds"]
            vs_oracle["oracle_cpu"] = f"{fx[0]['threads']} threads, {fx[0]['cpu']} ({fx[0]['machine']})"

    # the metric as its name states it: the time until the cost first comes within 1e-6 relative
    # of the converged FP64 cost (the oracle's CPU solve where its fixture matches, else the
    # lowest final cost of the GPU arms), from each solve's cost history (host ms since the solve
    # started, taken when the accepted cost is known)
    ref_cost = None
    if vs_oracle and "oracle_final_cost" in vs_oracle:
        ref_cost = vs_oracle["oracle_final_cost"]
    if ref_cost is None:
        ref_cost = min(reps_mixed[-1]["final_cost"], reps_64[-1]["final_cost"], reps_64r[-1]["final_cost"])

    def reach(h):
        hit = np.nonzero(h["cost"] <= ref_cost * (1.0 + 1e-6))[0]
        if hit.size == 0:
            return None
        k = int(hit[0])
        return {"ms": float(h["ms"][k]), "iteration": int(h["iterations"][k])}

    ttc = {"reference_cost": ref_cost, "mixed": reach(hist_mixed), "fp64_refactor": reach(hist_64),
           "fp64_reuse": reach(hist_64r)}
    if ttc["mixed"] and ttc["fp64_reuse"] and ttc["fp64_refactor"]:
        ttc["speedup_vs_fp64_path"] = min(ttc["fp64_reuse"]["ms"], ttc["fp64_refactor"]["ms"]) / ttc["mixed"]["ms"]

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        full_it, source = converged_iterations(args.workload)
        cpu_ms, info = cpu_sample(prob, opts, args.cpu_iterations, full_it)
        cpu = {"value": cpu_ms, "unit": "ms", "cores": cpu_cores(), "kind": "port",
               "sample": cpu_sample_text(info, full_it, source),
               "converged_solve_measured": measured_converged_cpu_solve(args.workload)}
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": ms_mixed, "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64 (mixed)", "data": "synthetic (seeded)",
        "config": bench_config(cfg),
        "fp64_path_ms_per_step": ms_64, "fp64_reuse_path_ms_per_step": ms_64r,
        "speedup_vs_fp64_path": min(ms_64, ms_64r) / ms_mixed,
        "speedup_vs_fp64_refactor_path": ms_64 / ms_mixed,
        "mixed_vs_fp64": {"final_cost_rel_diff": abs(f_m - f_d) / f_d, "camera_centre_rel_err": cam_err,
                          "mixed_iterations": reps_mixed[-1]["iterations"], "fp64_iterations": reps_64[-1]["iterations"],
                          "mixed_status": reps_mixed[-1]["status"], "fp64_status": reps_64[-1]["status"],
                          "fp64_reuse_vs_fp64": {"final_cost_rel_diff": abs(f_r - f_d) / f_d,
                                                 "camera_centre_rel_err": cam_err_r,
                                                 "iterations": reps_64r[-1]["iterations"],
                                                 "status": reps_64r[-1]["status"]}},
        "mixed_vs_oracle": vs_oracle,
        "time_to_1e-6_rel_cost": ttc,
        "fp64_on_mixed_path": MIXED_FP64_SPLIT,
        "roofline": {"kernel": "k_assemble<float> (linearise + online point Schur)", "bound": "issue",
                     "achieved": issue_achieved, "peak": issue_peak, "unit": "G warp-instructions/s",
                     "frac": (issue_achieved / issue_peak) if issue_achieved else None,
                     "traffic": ASSEMBLY_DRAM_BYTES_PER_OBS * nop,
                     "avg_launch_ms": asm_ms,
                     "peak_kind": f"4 issue slots per SM per cycle x {SMS} SMs at the sampled {sm_mhz:.0f} MHz",
                     "instructions_per_launch": ASSEMBLY_INST_PER_OBS * nop,
                     "hbm": {"achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": (achieved / peak) if achieved else None,
                             "algorithmic_bytes_per_launch": asm_bytes, "peak_kind": f"{peak_kind} copy bandwidth"},
                     "note": "issue-bound, not HBM-bound: float-float products on the FP32 pipe; warp instructions "
                             "per observation and traffic per observation from the ncu capture of the 250-camera "
                             "case (profiles/k_assemble_aerial250.md), scaled by the observations of a launch"},
        "pcg": {"kernel": "k_dense_cg<float> (FP64 matrix, FP32 dense-factor preconditioner)",
                "iterations_per_solve": cg_iters, "device_ms_per_solve": cg_ms,
                "us_per_iteration": 1e3 * cg_ms / cg_iters if cg_iters else None,
                "bytes_per_iteration": cg_iter_bytes, "achieved": cg_gbs, "peak": peak, "unit": "GB/s",
                "frac": (cg_gbs / peak) if cg_gbs else None, "served_from": "L2 (129 MB) after the first iteration",
                "note": "latency-bound: four grid barriers per iteration"},
        "kernel_ms_per_solve": {k: v for k, v in kt.items()},
        "solve_breakdown_ms": {k: rep_t[k] for k in ("assembly_ms", "linear_ms", "back_substitution_ms",
                                                     "objective_ms", "total_ms")},
        "linear_iterations": reps_mixed[-1]["linear_iterations"],
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "cold_first_call_ms": cold_ms},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rig_mixed is not None:
        # rig block: capture centres and sensor extrinsics of the mixed path against the FP64 path,
        # and the refined oblique lever arms and rotations against the generator's truth
        ts = getattr(prob, "truth_sensors", None)
        line["rig"] = {
            "capture_blocks": rep_t["rig_capture_blocks"], "sensor_blocks": rep_t["rig_sensor_blocks"],
            "mixed_vs_fp64_capture_centre_rel_err": float(np.abs(rig_mixed["captures"][:, 9:12] -
                                                                 rig_64["captures"][:, 9:12]).max() / scale),
            "mixed_vs_fp64_sensor_max_abs_diff": float(np.abs(rig_mixed["sensors"] - rig_64["sensors"]).max()),
            "sensor_lever_err_vs_truth_m": None if ts is None else
            float(np.abs(rig_mixed["sensors"][:, 9:12] - ts[:, 9:12]).max()),
            "sensor_rotation_err_vs_truth": None if ts is None else
            float(np.abs(rig_mixed["sensors"][:, :9] - ts[:, :9]).max()),
            "general_path": bool(rep_t["general_path_used"]), "promoted_point_blocks": rep_t["promoted_point_blocks"]}
    if cpu:
        line["cpu_baseline"] = cpu
    if args.workload == "aerial" and world == 1 and not args.no_secondary:
        # the two other workloads of the path, measured after the headline's timed region in the
        # same run: 256 batched local-BA windows and the backward pass of this converged solve
        ctx.close()
        line["secondary"] = secondary_records(prob, local_rank)
    print(json.dumps(line), flush=True)


def secondary_records(prob, local_rank):
    """Compact records of the windows, backward-pass and rig-block workloads (their own bench lines,
    with fewer timed repetitions: 2 timed batches of the 256 windows; 3 backward passes after 3
    warm-up passes and a 16-observation finite-difference check; 2 timed mixed solves and one of
    each FP64 arm of the 3 000-camera rig block)."""
    out = {}
    t0 = time.perf_counter()
    out["windows"] = measure_windows(256, 0, 2, 0, 1, local_rank)
    out["windows"]["wall_seconds"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    out["adjoint"] = measure_adjoint(3, 3, 16, 0, 1, local_rank, problem=prob)
    out["adjoint"]["wall_seconds"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    out["rig_block"] = measure_rig_block(local_rank)
    out["rig_block"]["wall_seconds"] = time.perf_counter() - t0
    return out


def measure_rig_block(local_rank, steps=2):
    """The large oblique survey block (workload rig3000: 600 five-camera rig captures, 1.5 M points,
    ~8 M observations, 40 control points, 10 scale bars): time to converge of the mixed path (CUDA
    events, L2 flushed, `steps` timed solves after one warm-up) against the FP64 path with the
    mixed path's factor reuse and the FP64 path refactoring every iteration (one timed solve each
    after one warm-up), with the errors between the arms and of the refined sensor extrinsics
    against the generator's truth."""
    import numpy as np
    import torch
    from plabundle_gb300.device import Gb300Context
    torch.cuda.set_device(local_rank)
    t_gen = time.perf_counter()
    prob, opts, cfg = workload("rig3000")
    t_gen = time.perf_counter() - t_gen
    opts.backend.enablePlaMatrixMixedPrecision = True
    ctx = Gb300Context(local_rank)
    assert ctx.upload(prob, opts) == 0, ctx.L.pb_gpu_last_error(ctx.ctx)
    stream = torch.cuda.ExternalStream(ctx.stream_handle())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(k):
        ctx.solve()
        ts, reps = [], []
        for _ in range(k):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            reps.append(ctx.solve())
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.mean(ts), reps[-1], ctx.download(), ctx.rig()

    ms_m, rep_m, out_m, rig_m = timed(steps)
    hist_m = ctx.history()
    # the mixed result against the oracle's converged CPU FP64 solve of the same problem (committed
    # fixture, compared only when the generator reproduces its problem)
    vs_oracle, ttc = None, None
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_rig_fixture as RFX
    fx = RFX.load_fixture()
    if fx is None:
        vs_oracle = {"unavailable": "fixture absent"}
    elif RFX.problem_mismatch(fx[0], fx[1], prob):
        vs_oracle = {"unavailable": "generator does not reproduce the fixture's problem: "
                                    + RFX.problem_mismatch(fx[0], fx[1], prob)}
    else:
        vs_oracle = RFX.compare(fx[0], fx[1], out_m["cameras"], rig_m["captures"], rig_m["sensors"], out_m["valid"],
                                out_m["rms_after"], out_m["points"], rep_m["final_cost"], rep_m["filter_threshold"])
        vs_oracle["oracle_cpu_solve_seconds"] = fx[0]["wall_seconds"]
        vs_oracle["oracle_cpu"] = f"{fx[0]['threads']} threads, {fx[0]['cpu']} ({fx[0]['machine']})"
        ref_cost = vs_oracle["oracle_final_cost"]
        hit = np.nonzero(hist_m["cost"] <= ref_cost * (1.0 + 1e-6))[0]
        ttc = {"reference_cost": ref_cost,
               "mixed": None if hit.size == 0 else {"ms": float(hist_m["ms"][hit[0]]),
                                                    "iteration": int(hist_m["iterations"][hit[0]])}}
    # end to end through the C ABI from host buffers (upload with the plan reused, solve, download)
    import ctypes as C
    from plabundle_gb300 import native
    desc, keep = native.problem_desc(prob)
    copts = native.solve_options(opts, prob)
    copts.precision = 1
    pp = keep[0]
    bufs = [np.zeros_like(pp.cameras), np.zeros_like(pp.points), np.zeros(pp.n_tracks, np.int8),
            np.zeros(pp.n_tracks), np.zeros(pp.n_tracks)]
    rep_e = native.SolveReportC()
    e2e = []
    for _ in range(2):
        t0 = time.perf_counter()
        st = ctx.L.pb_gpu_solve_problem(ctx.ctx, C.byref(desc), C.byref(copts), C.byref(rep_e),
                                        *[b.ctypes.data for b in bufs])
        e2e.append((time.perf_counter() - t0) * 1e3)
        assert st == 0
    h2d, d2h = problem_bytes(prob)
    ctx.copts.precision = 0
    ctx.copts.factor_reuse = 1
    ms_r, rep_r, out_r, rig_r = timed(1)
    hist_r = ctx.history()
    ctx.copts.factor_reuse = 2
    ms_f, rep_f, _, _ = timed(1)
    hist_f = ctx.history()
    if ttc is not None:
        for key, h in (("fp64_reuse", hist_r), ("fp64_refactor", hist_f)):
            hit = np.nonzero(h["cost"] <= ttc["reference_cost"] * (1.0 + 1e-6))[0]
            ttc[key] = None if hit.size == 0 else {"ms": float(h["ms"][hit[0]]), "iteration": int(h["iterations"][hit[0]])}
        if ttc["mixed"] and ttc.get("fp64_reuse") and ttc.get("fp64_refactor"):
            ttc["speedup_vs_fp64_path"] = min(ttc["fp64_reuse"]["ms"], ttc["fp64_refactor"]["ms"]) / ttc["mixed"]["ms"]
    ctx.close()
    C = out_r["cameras"][:, 9:12]
    scale = float(np.linalg.norm(C - C.mean(0), axis=1).max())
    ts = prob.truth_sensors
    return {"metric": "BA time-to-converge, mixed vs FP64 on GB300 (rig block)", "value": ms_m, "unit": "ms",
            "impl": "gb300", "n_gpus": 1, "steps": steps, "warmup": 1, "higher_is_better": False,
            "dtype": "f32+f64 (mixed)", "data": "synthetic (seeded)",
            "config": dict(cfg, l2="flushed between steps (256 MB write)"),
            "fp64_reuse_path_ms": ms_r, "fp64_refactor_path_ms": ms_f,
            "speedup_vs_fp64_path": min(ms_r, ms_f) / ms_m, "speedup_vs_fp64_refactor_path": ms_f / ms_m,
            "iterations": {"mixed": rep_m["iterations"], "fp64_reuse": rep_r["iterations"],
                           "fp64_refactor": rep_f["iterations"]},
            "status": {"mixed": rep_m["status"], "fp64_reuse": rep_r["status"], "fp64_refactor": rep_f["status"]},
            "solve_breakdown_ms": {k: rep_m[k] for k in ("assembly_ms", "linear_ms", "back_substitution_ms",
                                                         "objective_ms", "total_ms")},
            "mixed_vs_fp64": {"final_cost_rel_diff": abs(rep_m["final_cost"] - rep_r["final_cost"]) / rep_r["final_cost"],
                              "camera_centre_rel_err": float(np.abs(out_m["cameras"][:, 9:12] - C).max() / scale),
                              "capture_centre_rel_err": float(np.abs(rig_m["captures"][:, 9:12] -
                                                                     rig_r["captures"][:, 9:12]).max() / scale),
                              "sensor_max_abs_diff": float(np.abs(rig_m["sensors"] - rig_r["sensors"]).max()),
                              "inlier_mask_identical": bool(np.array_equal(out_m["valid"], out_r["valid"]))},
            "mixed_vs_oracle": vs_oracle, "time_to_1e-6_rel_cost": ttc,
            "sensor_lever_err_vs_truth_m": float(np.abs(rig_m["sensors"][:, 9:12] - ts[:, 9:12]).max()),
            "sensor_rotation_err_vs_truth": float(np.abs(rig_m["sensors"][:, :9] - ts[:, :9]).max()),
            "rig_blocks": {"captures": rep_m["rig_capture_blocks"], "sensors": rep_m["rig_sensor_blocks"],
                           "promoted_point_blocks": rep_m["promoted_point_blocks"]},
            "e2e": {"value": statistics.mean(e2e), "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "generator_seconds": t_gen}


def main():
    args = parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    if args.workload == "adjoint":
        run_adjoint(args, rank, world, local_rank)
        return
    if args.workload == "windows":
        run_windows(args, rank, world, local_rank)
    else:
        run_gb300(args, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
