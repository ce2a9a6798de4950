"""The host planner's active problem on edge-case inputs against the oracle (CPU only): the
observation filter, fixed tracks and cameras, the initial-RMS gate, and a problem with no usable
observation."""
import pytest

import oracle as O
from edge_problems import CASES, no_usable_observation, options, ring
from plabundle_gb300.problem import SolveStatus
from test_control_points import host_model

KEYS = ("active_tracks", "observation_count", "rejected_initial_tracks", "camera_blocks", "track_blocks",
        "gauge_anchor", "gauge_scale")


@pytest.mark.parametrize("name,make,opts", CASES, ids=[c[0] for c in CASES])
def test_host_active_problem_matches_oracle(host_probe, name, make, opts):
    p, o = make(), opts()
    h = host_model(host_probe, p, o)
    assert h["status"] == 0, host_probe.probe_message()
    i = O.Oracle(p, o).info()
    for k in KEYS:
        assert h[k] == i[k], k
    if name == "initial_rms_gate":
        assert 0 < h["rejected_initial_tracks"] < p.n_tracks
    if name == "unusable_observations":
        assert h["observation_count"] < O.Oracle(ring(), opts()).info()["observation_count"]


def test_no_usable_observation_is_invalid_input(host_probe):
    p, o = no_usable_observation(), options()
    h = host_model(host_probe, p, o)
    assert h["status"] == 0 and h["active_tracks"] == 0 and h["observation_count"] == 0
    assert O.Oracle(p, o).solve()["report"]["status"] == SolveStatus.InvalidInput
