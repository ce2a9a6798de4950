"""Batched solves of independent windows (pb_gpu_solve_batch): each window's result equals its
own single solve on a fresh context bit for bit (same kernels, fixed-order reductions), for any
number of worker contexts."""
import numpy as np
import pytest

from plabundle_gb300 import synth
from plabundle_gb300.problem import ImageRobustLoss, SolveOptions

pytestmark = pytest.mark.gpu


def _options(mixed):
    o = SolveOptions()
    o.solver.imageRobustLoss = ImageRobustLoss.Huber
    o.solver.imageRobustLossScalePixels = 1.5
    o.backend.enablePlaMatrixMixedPrecision = mixed
    return o


@pytest.mark.parametrize("mixed", [False, True])
@pytest.mark.parametrize("workers", [1, 3])
def test_batch_matches_single_solves(mixed, workers):
    from plabundle_gb300.batch import solve_batch
    from plabundle_gb300.device import Gb300Context
    windows = synth.window_problems(n_windows=6, seed=77, cameras=(10, 24), points=(300, 1500))
    o = _options(mixed)
    results, latency = solve_batch(windows, o, n_workers=workers)
    assert len(results) == len(windows) and np.all(latency > 0)
    for p, r in zip(windows, results):
        ctx = Gb300Context(0)
        assert ctx.upload(p, o) == 0
        rep = ctx.solve()
        out = ctx.download()
        assert r["status"] == rep["status"] and r["iterations"] == rep["iterations"]
        assert r["final_cost"] == rep["final_cost"]
        assert np.array_equal(r["cameras"], out["cameras"])
        assert np.array_equal(r["valid"], out["valid"])
        ctx.close()
