"""CPU tests of the host-side planning of the assembly (no GPU).

``pb_host.cpp`` (active problem, block numbering, reduced pattern, processing order and the
assembly chunks with their item lists) is plain C++.  The test compiles it with g++ together with
``host_probe.cpp``, which re-derives every list the assembly kernel reads by brute force and
checks them against the planner's output, for both arithmetic paths.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from plabundle_gb300 import native, synth
from plabundle_gb300.problem import ImageRobustLoss, Precision, SolveOptions

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SMEM_BUDGET = 227 * 1024 - 1024


@pytest.fixture(scope="module")
def probe(host_probe):
    return host_probe


def run_probe(L, problem, options, precision):
    desc, keep = native.problem_desc(problem)
    o = native.solve_options(options, problem)
    o.precision = int(precision)
    stats = (C.c_longlong * 7)()
    rc = L.probe_chunks(C.byref(desc), C.byref(o), int(precision), SMEM_BUDGET, stats)
    assert rc == 0, L.probe_message().decode()
    del keep
    return list(stats)


def aerial_options():
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Cauchy
    o.calibration.refineSharedFocalLength = True
    o.calibration.refineSharedPrincipalPoint = True
    o.calibration.refineSharedRadialDistortion = True
    return o


def duplicate_camera_problem():
    """A ring problem in which some tracks observe the same camera twice."""
    p = synth.ring_problem(seed=3, n_cameras=8, n_points=200)
    offs = p.track_offsets
    cams, us, vs, ws, ss, new_offs = [], [], [], [], [], [0]
    for t in range(p.n_tracks):
        a, b = int(offs[t]), int(offs[t + 1])
        idx = list(range(a, b))
        if t % 5 == 0:
            idx.append(a)  # second observation of the track's first camera
        for k in idx:
            cams.append(p.obs_camera[k])
            us.append(p.obs_u[k] + (0.3 if k == a and len(idx) > b - a else 0.0))
            vs.append(p.obs_v[k])
            ws.append(p.obs_weight[k])
            ss.append(p.obs_scale[k])
        new_offs.append(len(cams))
    p.obs_camera = np.array(cams, np.int32)
    p.obs_u, p.obs_v = np.array(us), np.array(vs)
    p.obs_weight, p.obs_scale = np.array(ws), np.array(ss)
    p.track_offsets = np.array(new_offs, np.int64)
    return p


CASES = [
    ("ring", lambda: synth.ring_problem(seed=5, n_cameras=8, n_points=300), SolveOptions),
    ("ring20", lambda: synth.ring_problem(seed=7), SolveOptions),
    ("aerial", lambda: synth.aerial_grid_problem(seed=3, n_along=5, n_lines=4, n_points=3000), aerial_options),
    ("aerial_fixed", lambda: _fixed(synth.aerial_grid_problem(seed=4, n_along=6, n_lines=3, n_points=2000)),
     aerial_options),
    ("duplicate_camera", duplicate_camera_problem, SolveOptions),
]


def _fixed(p):
    p.fixedCameraIndices = [1, 4]
    p.fixedTrackIndices = list(range(0, p.n_tracks, 7))
    return p


@pytest.mark.parametrize("name,make,opts", CASES)
@pytest.mark.parametrize("precision", [Precision.Fp64, Precision.Mixed])
def test_chunk_item_lists_match_brute_force(probe, name, make, opts, precision):
    stats = run_probe(probe, make(), opts(), precision)
    nch, max_obs, slots, items, cams, nobs, smem = stats
    assert nch >= 1 and nobs > 0
    # two assembly CTAs per SM: at most 113 KB of shared memory each
    assert smem <= 113 * 1024
    assert 32 <= max_obs <= 256 and max_obs % 32 == 0
    # every observation with a pose block contributes at least its own term
    assert items >= nobs - 2 * 300


def test_chunks_of_the_500_camera_workload_are_consistent(probe):
    """The 500-camera aerial grid: the chunk lists the bench workload uses."""
    p = synth.aerial_grid_problem(seed=11, n_along=25, n_lines=20, n_points=40_000)
    nch, max_obs, slots, items, cams, nobs, smem = run_probe(probe, p, aerial_options(), Precision.Mixed)
    assert nch * max_obs >= nobs
    # chunks are filled: on average at least 3/4 of max_obs observations
    assert nobs / nch > 0.75 * max_obs


def test_preconditioner_cluster_sizes_are_accepted(probe):
    """BackendOptions::plaMatrixPreconditionerClusterSize 1..16 is valid (validateOptions) and
    leaves the solution unchanged: the host accepts it; 0 and 17 are invalid input."""
    import numpy as np
    p = synth.ring_problem(seed=3, n_cameras=8, n_points=200)
    for size, status in ((1, 0), (4, 0), (16, 0), (0, 4), (17, 4)):
        o = SolveOptions()
        o.backend.plaMatrixPreconditionerClusterSize = size
        desc, keep = native.problem_desc(p)
        copts = native.solve_options(o, p)
        out_i = np.zeros(12, np.int32)
        fixed = np.zeros(p.n_cameras + 2, np.int32)
        out_d = np.zeros(2)
        probe.probe_model(C.byref(desc), C.byref(copts), out_i.ctypes.data, fixed.ctypes.data, out_d.ctypes.data)
        assert out_i[0] == status, (size, out_i[0])
