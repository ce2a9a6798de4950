"""Batched solves of independent problems (local bundle-adjustment windows) through
pb_gpu_solve_batch: every problem is solved as `Solver.solve` would solve it, with worker
contexts on their own streams so that the windows overlap on the device.

`tune_workers` is the batch's autotuner: the number of worker contexts sets how the host
planning of the windows and their kernels overlap, and the best count depends on the host's
cores, the device and the window sizes, so it is chosen by measured throughput on a sample of
the caller's own windows.  Results do not depend on the count (every window is solved exactly as
alone)."""
from __future__ import annotations

import ctypes as C
import time
from typing import Dict, List, Sequence, Tuple

import numpy as np

from . import native
from .problem import Problem, SolveOptions


def solve_batch(problems: Sequence[Problem], options: SolveOptions, n_workers: int = 8, device: int = 0):
    """Returns (results, latency_ms): per problem a dict with the report fields and the refined
    cameras, points and valid mask; latency_ms[i] is the wall time of problem i's solve.  All
    problems share `options` and use the default (AutoAnchor) gauge."""
    L = native.load()
    n = len(problems)
    descs = (native.ProblemDesc * n)()
    keep: List[object] = []
    outs = []
    for i, p in enumerate(problems):
        d, k = native.problem_desc(p)
        descs[i] = d
        keep.append(k)
        pp = k[0]
        outs.append((np.zeros_like(pp.cameras), np.zeros_like(pp.points), np.zeros(pp.n_tracks, np.int8)))
    opts = native.solve_options(options, problems[0] if n else None)
    reports = (native.SolveReportC * n)()
    cam_ptrs = (C.c_void_p * n)(*[o[0].ctypes.data for o in outs])
    pt_ptrs = (C.c_void_p * n)(*[o[1].ctypes.data for o in outs])
    val_ptrs = (C.c_void_p * n)(*[o[2].ctypes.data for o in outs])
    latency = np.zeros(n)
    st = L.pb_gpu_solve_batch(device, n, C.cast(descs, C.c_void_p), C.byref(opts), n_workers,
                              C.cast(reports, C.c_void_p), C.cast(cam_ptrs, C.c_void_p), C.cast(pt_ptrs, C.c_void_p),
                              C.cast(val_ptrs, C.c_void_p), latency.ctypes.data)
    native.check(L, None, st, "solve_batch")
    results = []
    for i in range(n):
        r = reports[i].as_dict()
        r.update({"cameras": outs[i][0], "points": outs[i][1], "valid": outs[i][2].astype(bool)})
        results.append(r)
    del keep
    return results, latency


def tune_workers(problems: Sequence[Problem], options: SolveOptions, device: int = 0,
                 candidates: Sequence[int] = (4, 6, 8, 12, 16), sample: int = 48,
                 repeats: int = 2) -> Tuple[int, Dict[int, float]]:
    """Worker count with the highest measured throughput (problems per second) on the first
    `sample` problems, best of `repeats` timed batches per candidate after one untimed batch
    (device memory, module loading).  Returns (best count, {count: problems per second})."""
    sub = list(problems[:max(1, min(sample, len(problems)))])
    solve_batch(sub[:max(candidates)], options, n_workers=max(candidates), device=device)
    rates: Dict[int, float] = {}
    for w in candidates:
        best = 0.0
        for _ in range(max(1, repeats)):
            t0 = time.perf_counter()
            solve_batch(sub, options, n_workers=w, device=device)
            best = max(best, len(sub) / (time.perf_counter() - t0))
        rates[int(w)] = best
    return max(rates, key=rates.get), rates
