"""Batched solves of independent problems (local bundle-adjustment windows) through
pb_gpu_solve_batch: every problem is solved as `Solver.solve` would solve it, with worker
contexts on their own streams so that the windows overlap on the device."""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence

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
