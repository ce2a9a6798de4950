"""The allocation-free objective entry point, pb_gpu_objective_noalloc (no counterpart in the
reference; see include/pb_gpu.h).

It evaluates the robust image objective of caller-owned device arrays with the line-search cost
kernel, its per-block partials in one fixed file-scope device array.  The test compares it with
the context's objective (pb_gpu_eval_cost) on the same problem, on two consecutive calls (the
scratch array is reused, nothing in it is cleared between calls), and checks its size and index
limits.  The file sorts last so that it also runs after every other test in one session.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_inputs(problem, active):
    import torch
    p = problem.normalized()
    trk = np.repeat(np.arange(p.n_tracks, dtype=np.int32), np.diff(p.track_offsets))
    keep = active[trk] == 1
    w = p.obs_weight / (p.obs_scale * p.obs_scale)
    host = {
        "cameras": p.cameras, "points": p.points,
        "obs_camera": p.obs_camera[keep].astype(np.int32), "obs_point": trk[keep],
        "obs_u": p.obs_u[keep], "obs_v": p.obs_v[keep], "obs_w": w[keep],
    }
    return {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in host.items()}


def _call(L, d, n_obs, loss, scale, stream=None):
    cost = C.c_double(0.0)
    bad = C.c_int64(-1)
    st = L.pb_gpu_objective_noalloc(d["cameras"].data_ptr(), d["cameras"].shape[0], d["points"].data_ptr(),
                                    d["points"].shape[0], d["obs_camera"].data_ptr(), d["obs_point"].data_ptr(),
                                    d["obs_u"].data_ptr(), d["obs_v"].data_ptr(), d["obs_w"].data_ptr(), n_obs,
                                    loss, scale, stream, C.byref(cost), C.byref(bad))
    return st, cost.value, bad.value


def test_noalloc_objective_matches_the_context_objective_on_consecutive_calls():
    import torch
    from plabundle_gb300 import synth
    from plabundle_gb300.device import Gb300Context
    from plabundle_gb300.problem import ImageRobustLoss, SolveOptions
    # no calibration groups: the context's effective cameras are the input cameras
    p = synth.ring_problem(seed=5, n_cameras=8, n_points=300)
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    ctx = Gb300Context(0)
    assert ctx.upload(p, o) == 0
    ref = ctx.cost()
    d = _device_inputs(p, ctx.active()["active_track"])
    n = d["obs_u"].shape[0]
    stream = torch.cuda.current_stream().cuda_stream
    first = _call(ctx.L, d, n, int(ImageRobustLoss.Huber), 1.5, stream)
    second = _call(ctx.L, d, n, int(ImageRobustLoss.Huber), 1.5, stream)
    for st, cost, bad in (first, second):
        assert st == 0
        assert bad == 0
        # same terms summed in another order: FP64 rounding only
        np.testing.assert_allclose(cost, ref, rtol=1e-11)
    assert first[1] == second[1]


def test_noalloc_objective_rejects_sizes_and_indices_out_of_range():
    import torch
    from plabundle_gb300 import native
    L = native.load()
    cams = torch.zeros((2, 32), dtype=torch.float64, device="cuda")
    cams[:, 0] = cams[:, 4] = cams[:, 8] = 1.0
    cams[:, 12] = cams[:, 13] = 1000.0
    cams[:, 21] = cams[:, 22] = 1.0
    pts = torch.tensor([[0.0, 0.0, 10.0]], dtype=torch.float64, device="cuda")
    d = {"cameras": cams, "points": pts,
         "obs_camera": torch.tensor([0, 5], dtype=torch.int32, device="cuda"),
         "obs_point": torch.tensor([0, 0], dtype=torch.int32, device="cuda"),
         "obs_u": torch.zeros(2, dtype=torch.float64, device="cuda"),
         "obs_v": torch.zeros(2, dtype=torch.float64, device="cuda"),
         "obs_w": torch.ones(2, dtype=torch.float64, device="cuda")}
    # above the documented maximum: rejected before any launch
    st, _, _ = _call(L, d, (1 << 22) + 1, 0, 1.0)
    assert st == 6  # PB_ERR_BOUNDS
    # camera index 5 of 2 cameras: the access is skipped and reported
    st, _, _ = _call(L, d, 2, 0, 1.0)
    assert st == 6
    # the valid observation alone
    st, cost, bad = _call(L, d, 1, 0, 1.0)
    assert st == 0 and bad == 0 and cost == 0.0
