"""Host side of the learned warm start: the phantom generator's bounding-box
evaluation equals the whole-grid evaluation bit for bit, and the training-pair
and time-reversal problems have the shapes the device runs expect."""
import numpy as np
import pytest


def whole_grid_phantom(n, rng, pml=20):
    """The vessel phantom evaluated on the whole grid for every feature."""
    gx, gy = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    p0 = np.zeros((n, n))
    lo, hi = pml + 0.25 * (n - 2 * pml), n - pml - 0.25 * (n - 2 * pml)
    for _ in range(15):
        x0, y0, x1, y1 = rng.uniform(lo, hi, 4)
        w = rng.uniform(1, 4) / 2
        vx, vy = x1 - x0, y1 - y0
        t = np.clip(((gx - x0) * vx + (gy - y0) * vy) / max(vx * vx + vy * vy, 1e-9), 0, 1)
        dist = np.hypot(gx - (x0 + t * vx), gy - (y0 + t * vy))
        p0 = np.maximum(p0, rng.uniform(0.5, 2) * np.clip(w + 0.5 - dist, 0, 1))
    for _ in range(5):
        cx, cy, r = rng.uniform(lo, hi), rng.uniform(lo, hi), rng.uniform(2, 6)
        p0 = np.maximum(p0, rng.uniform(0.5, 2) * np.clip(r + 0.5 - np.hypot(gx - cx, gy - cy), 0, 1))
    return p0


@pytest.mark.parametrize("n", [64, 256, 512])
def test_phantom_bounding_boxes_change_nothing(n):
    from kwave_gb300.phantoms import vessel_phantom

    for seed in range(12):
        assert np.array_equal(vessel_phantom(n, np.random.default_rng(seed)),
                              whole_grid_phantom(n, np.random.default_rng(seed)))


def test_pair_and_time_reversal_problems():
    from kwave_gb300.warmstart import pair_problem, tr_problem

    prob = pair_problem(3)
    mask = prob["sensor_mask"]
    assert mask.shape == (256, 256) and mask.dtype == bool and 100 <= mask.sum() <= 128
    assert prob["p0"].shape == (256, 256) and prob["p0"].max() > 0 and not prob["smooth_p0"]
    data = np.arange(int(mask.sum()) * prob["Nt"], dtype=float).reshape(-1, prob["Nt"])
    q = tr_problem(prob, data)
    assert q["p_mode"] == "dirichlet" and q["sensor_mask"] is mask and "p0" not in q
    # the reference's time reversal records p_final alone on the sensor mask
    assert tuple(q["record"]) == ("p_final",)
    assert np.array_equal(q["p"], data[:, ::-1]) and q["p_mask"] is mask
