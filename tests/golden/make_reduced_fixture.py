"""Records the reduced system that the GPU path assembles for the stored 20-camera aerial problem
(tests/golden/aerial_20cam_1500pt.npz: shared intrinsics in two groups, so every kind of chunk
partial -- pose pair blocks, camera rows, intrinsic entries -- feeds the fused reduce kernel).

For both precisions and dampings 0 and 1e-3 it stores the dense reduced matrix, its right-hand
side and the direct right-hand side exactly as pb_gpu_get_reduced returns them.  The assembly
and the reduce sum every output in a fixed order (no atomics, a chunk plan that depends only on
the problem), so the same build reproduces these arrays bit for bit on any GB300;
tests/test_gpu_reduce_order.py compares them with ==, which pins the summation order of the
reduce against any change.  Run on a GPU:

    python tests/golden/make_reduced_fixture.py OUT.npz
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

CASE = "aerial_20cam_1500pt"
DAMPINGS = (0.0, 1e-3)


def reduced_systems():
    from make_golden import options_from_meta, problem_from_fixture
    from plabundle_gb300.device import Gb300Context
    from plabundle_gb300.problem import Precision
    z = dict(np.load(os.path.join(HERE, CASE + ".npz")))
    meta = json.loads(z["meta"].tobytes().decode())
    p = problem_from_fixture(z)
    out = {}
    for prec in (Precision.Fp64, Precision.Mixed):
        o = options_from_meta(meta["options"])
        o.backend.enablePlaMatrixMixedPrecision = prec == Precision.Mixed
        ctx = Gb300Context(0)
        assert ctx.upload(p, o) == 0
        for i, damping in enumerate(DAMPINGS):
            ctx.linearize_schur(damping, prec)
            S, rhs, direct = ctx.reduced()
            tag = f"{prec.name.lower()}_{i}"
            out["S_" + tag], out["rhs_" + tag], out["direct_" + tag] = S, rhs, direct
        ctx.close()
    return out


def main():
    np.savez_compressed(sys.argv[1], **reduced_systems())


if __name__ == "__main__":
    main()
