"""Golden fixtures of the online reduced-Schur path (tests/golden, made by make_golden.py).

CPU: every stored array matches its SHA-256 in SHA256SUMS, and the oracle reproduces the stored
solution (same status and iteration count, cost to 1e-10, parameters to 1e-9; the oracle is
compiled with -ffp-contract=off, so only libm last-ulp differences between hosts remain).
GPU: the FP64 path reproduces the stored oracle trajectory (status, iterations, cost 1e-9,
camera centres 1e-8 of the scene extent) and the mixed path converges to the stored fixed point
within the targets (cost 1e-6, camera centres 1e-5), with the same inlier mask on both.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from golden.make_golden import CASES, options_from_meta, problem_from_fixture

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    z = dict(np.load(os.path.join(HERE, name + ".npz")))
    meta = json.loads(z["meta"].tobytes().decode())
    return z, meta


def scene_error(cams, ref):
    C = ref[:, 9:12]
    scale = np.linalg.norm(C - C.mean(0), axis=1).max()
    return float(np.abs(cams[:, 9:12] - C).max() / scale)


def test_fixture_arrays_match_their_hashes():
    sums = {}
    with open(os.path.join(HERE, "SHA256SUMS")) as f:
        for line in f:
            h, key = line.split()
            sums[key] = h
    assert len(sums) > 0
    for name in CASES:
        z, _ = load(name)
        for k, v in z.items():
            assert hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest() == sums[f"{name}:{k}"], (name, k)


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("threads", [1, 4])
def test_oracle_reproduces_the_fixture(name, threads):
    import oracle as O
    z, meta = load(name)
    p = problem_from_fixture(z)
    ref = O.Oracle(p, options_from_meta(meta["options"]), num_threads=threads).solve()
    rep, gold = ref["report"], meta["report"]
    assert rep["status"] == gold["status"] and rep["iterations"] == gold["iterations"]
    assert abs(rep["final_cost"] - gold["final_cost"]) <= 1e-10 * gold["final_cost"]
    assert scene_error(ref["cameras"], z["out_cameras"]) < 1e-9
    assert np.array_equal(ref["valid"].astype(np.int8), z["out_valid"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("mixed", [False, True])
def test_gpu_path_matches_the_fixture(name, mixed):
    from plabundle_gb300.device import Gb300Context
    z, meta = load(name)
    p = problem_from_fixture(z)
    o = options_from_meta(meta["options"])
    o.backend.enablePlaMatrixMixedPrecision = mixed
    if mixed:
        o.solver.maxIterations = max(o.solver.maxIterations, 80)
    ctx = Gb300Context(0)
    assert ctx.upload(p, o) == 0
    rep = ctx.solve()
    out = ctx.download()
    gold = meta["report"]
    rel = abs(rep["final_cost"] - gold["final_cost"]) / gold["final_cost"]
    err = scene_error(out["cameras"], z["out_cameras"])
    if mixed:
        if gold["status"] == 1:
            assert rep["status"] == 1
        assert rel < 1e-6, rel
        assert err < 1e-5, err
    else:
        assert rep["status"] == gold["status"] and rep["iterations"] == gold["iterations"]
        assert rel < 1e-9, rel
        assert err < 1e-8, err
    assert np.array_equal(out["valid"].astype(np.int8), z["out_valid"])
