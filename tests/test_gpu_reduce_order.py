"""The fused reduce kernel keeps its summation order (k_reduce_sums: the pose-pair, camera-row and
chunk-record sums of the chunk partials, each in its own fixed order, side by side in one launch).

The reduced system of the stored 20-camera aerial problem (both precisions, dampings 0 and 1e-3)
must equal, bit for bit, the arrays recorded in tests/golden/aerial_20cam_1500pt_reduced.npz by
tests/golden/make_reduced_fixture.py.  Every output of the assembly and the reduce is summed by
one thread in an order fixed by the problem's chunk plan, so any change to that order -- or to the
arithmetic of the sums -- shows up here as a difference in the last bits, which the oracle tests'
tolerances would not see.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_reduced_system_equals_the_recorded_bits():
    from golden.make_reduced_fixture import reduced_systems
    path = os.path.join(HERE, "aerial_20cam_1500pt_reduced.npz")
    if not os.path.exists(path):
        pytest.skip("recorded reduced systems absent")
    ref = np.load(path)
    got = reduced_systems()
    assert set(got) == set(ref.files)
    for k, v in got.items():
        assert np.array_equal(v, ref[k]), (k, np.abs(v - ref[k]).max())
