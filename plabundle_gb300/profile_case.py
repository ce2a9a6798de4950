"""Fixed workloads for profiling the backend under ncu.

    python -m plabundle_gb300.profile_case --workload aerial500 --precision mixed --iterations 3
    python -m plabundle_gb300.profile_case --workload aerial250 --precision mixed --iterations 3
    python -m plabundle_gb300.profile_case --workload aerial250 --precision mixed --iterations 3 --linear-solver 2
    python -m plabundle_gb300.profile_case --workload rig3000 --precision mixed --iterations 2

`aerial500` is the 500-camera / 200k-point aerial grid of the benchmark (Cauchy 1.5 px, two
calibration groups refining f, cx, cy, k1-k3, p1, p2); `aerial250` the same generator at half
size (250 cameras, 100k points), small enough for `ncu --set full` captures; `rig3000` the oblique
rig block of the large survey configuration (600 five-camera rig captures, 1.5 M points, ~8 M
observations, 40 control points, 10 scale bars; general path).  One LM iteration is
solved first on a separate context (module loading, pattern build), then the profiled solve of
`--iterations` iterations.
"""
from __future__ import annotations

import argparse

from . import synth
from .device import Gb300Context
from .problem import ImageRobustLoss, SolveOptions


def workload(name: str, mixed: bool, iterations: int):
    if name == "rig3000":
        p = synth.rig_grid_problem(seed=21)
        synth.with_control_points(p, n=40, sigma=0.02, seed=3)
        synth.with_scale_bars(p, n=10, sigma=0.005, seed=5)
        o = SolveOptions()
        o.solver.imageRobustLoss = ImageRobustLoss.Cauchy
        o.solver.imageRobustLossScalePixels = 1.5
        o.backend.linearRelativeTolerance = 1e-6
        o.backend.enablePlaMatrixMixedPrecision = mixed
        o.solver.maxIterations = iterations
        return p, o
    if name == "aerial500":
        p = synth.aerial_grid_problem(seed=11)
    elif name == "aerial250":
        p = synth.aerial_grid_problem(seed=11, n_along=25, n_lines=10, n_points=100_000)
    else:
        raise ValueError(name)
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Cauchy
    o.solver.imageRobustLossScalePixels = 1.5
    o.calibration.refineSharedFocalLength = True
    o.calibration.refineSharedPrincipalPoint = True
    o.calibration.refineSharedRadialDistortion = True
    o.backend.enablePlaMatrixMixedPrecision = mixed
    o.solver.maxIterations = iterations
    return p, o


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="aerial250", choices=["aerial250", "aerial500", "rig3000"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--iterations", type=int, default=3)
    ap.add_argument("--linear-solver", type=int, default=0, choices=[0, 1, 2],
                    help="0 automatic, 1 dense-factor-preconditioned CG, 2 block-Jacobi PCG")
    a = ap.parse_args()
    mixed = a.precision == "mixed"
    p, o = workload(a.workload, mixed, 1)
    o.backend.linearSolver = a.linear_solver
    warm = Gb300Context(0)
    assert warm.upload(p, o) == 0
    warm.solve()
    warm.close()
    o.solver.maxIterations = a.iterations
    ctx = Gb300Context(0)
    assert ctx.upload(p, o) == 0
    rep = ctx.solve()
    print(a.workload, a.precision, "status", rep["status"], "iterations", rep["iterations"],
          "observations", p.n_obs, "final_cost", rep["final_cost"])


if __name__ == "__main__":
    main()
