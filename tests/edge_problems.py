"""Edge-case problems shared by the host (CPU) and the GPU edge-case tests: unusable observations
of every kind the reference's observation filter drops, fixed tracks and cameras under an explicit
gauge, the initial-RMS track gate, and a problem with no usable observation."""
import numpy as np

from plabundle_gb300 import synth
from plabundle_gb300.problem import GaugePolicy, ImageRobustLoss, SolveOptions


def ring(seed=5):
    return synth.ring_problem(seed=seed, n_cameras=8, n_points=300)


def options(loss=ImageRobustLoss.Huber, max_initial_rms=None):
    o = SolveOptions()
    o.solver.imageRobustLoss = loss
    o.solver.imageRobustLossScalePixels = 1.5
    o.backend.enablePlaMatrixMixedPrecision = False
    if max_initial_rms is not None:
        o.solver.maxInitialTrackRms = max_initial_rms
    return o


def damaged():
    """60 observations made unusable or rescaled: non-finite pixels, camera indices out of range,
    zero and infinite weights (dropped), negative measurement scales (taken as 1)."""
    p = ring()
    k = np.random.default_rng(3).choice(p.n_obs, size=75, replace=False)
    p.obs_u = np.array(p.obs_u, float)
    p.obs_v = np.array(p.obs_v, float)
    p.obs_weight = np.array(p.obs_weight, float)
    p.obs_scale = np.array(p.obs_scale, float)
    p.obs_camera = np.array(p.obs_camera, np.int32)
    p.obs_u[k[:15]] = np.nan
    p.obs_v[k[15:20]] = np.inf
    p.obs_camera[k[20:25]] = p.n_cameras + 3
    p.obs_camera[k[25:30]] = -1
    p.obs_weight[k[30:40]] = 0.0
    p.obs_weight[k[40:50]] = np.inf
    p.obs_weight[k[50:55]] = -2.0
    p.obs_scale[k[55:65]] = -1.0
    p.obs_scale[k[65:75]] = 0.5
    return p


def fixed_gauge():
    """Two fixed cameras (the explicit gauge) and every fifteenth track fixed at its initial point."""
    p = ring(seed=7)
    p.fixedCameraIndices = [0, 4]
    p.fixedTrackIndices = list(range(0, p.n_tracks, 15))
    p.gauge.policy = GaugePolicy.RequireExplicitGauge
    return p


def ragged():
    """Ragged tracks: five empty tracks (repeated offsets), twenty tracks cut to one observation
    (inactive) and twenty cut to two (the minimum of an active track)."""
    p = ring(seed=11)
    off = np.asarray(p.track_offsets, np.int64)
    keep, offsets, points = [], [0], []
    for t in range(p.n_tracks):
        obs = list(range(off[t], off[t + 1]))
        if t < 20:
            obs = obs[:1]
        elif t < 40:
            obs = obs[:2]
        if t % 60 == 0:
            offsets.append(offsets[-1])
            points.append(p.points[t])
        keep += obs
        offsets.append(offsets[-1] + len(obs))
        points.append(p.points[t])
    k = np.array(keep)
    p.track_offsets = np.array(offsets, np.int64)
    p.points = np.array(points, float)
    p.obs_camera = np.asarray(p.obs_camera, np.int32)[k]
    for name in ("obs_u", "obs_v", "obs_weight", "obs_scale"):
        setattr(p, name, np.asarray(getattr(p, name), float)[k])
    return p


def no_usable_observation():
    p = ring()
    p.obs_weight = np.zeros(p.n_obs)
    return p


# name, problem, options; the options of the initial-RMS gate reject about a quarter of the tracks
CASES = [
    ("unusable_observations", damaged, lambda: options()),
    ("fixed_tracks_and_cameras", fixed_gauge, lambda: options()),
    ("least_squares", ring, lambda: options(ImageRobustLoss.LeastSquares)),
    ("cauchy", ring, lambda: options(ImageRobustLoss.Cauchy)),
    ("initial_rms_gate", lambda: ring(seed=9), lambda: options(max_initial_rms=40.0)),
    ("ragged_tracks", ragged, lambda: options()),
]
