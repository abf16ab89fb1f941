"""GPU adjoint of the lossless time loop (kw_plan_adjoint_p0) against the FP64
adjoint oracle (itself checked by dot-product test, finite differences and
torch autograd in test_adjoint_cpu.py).  FP32 against FP64 over tens of
steps: 1e-4 relative L2."""
import numpy as np
import pytest

from test_adjoint_cpu import problem, rel

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib

    _lib.require_device()


def box3d():
    rng = np.random.default_rng(9)
    shape = (16, 20, 24)
    g = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    p0 = np.exp(-sum((gi - n / 2) ** 2 for gi, n in zip(g, shape)) / 8.0)
    c = 1500.0 * (1 + 0.02 * np.tanh(rng.standard_normal(shape)))
    mask = np.zeros(shape, bool)
    mask[:, :, 5] = True
    return dict(shape=shape, spacing=(1e-4,) * 3, dt=0.3 * 1e-4 / c.max(), Nt=24, sound_speed=c, density=1000.0,
                p0=p0, smooth_p0=False, sensor_mask=mask, record=("p",), pml_size=(4, 4, 4), pml_alpha=(2.0,) * 3)


CASES = {
    "2d-40x48": lambda: problem(cartesian=False),
    "2d-64x64-record-start": lambda: problem(shape=(64, 64), cartesian=False, record_start=4),
    "3d-16x20x24": box3d,
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_adjoint_matches_oracle(name):
    from kwave_gb300.adjoint import adjoint_p0
    from oracle.adjoint_oracle import AdjointOracle

    prob = CASES[name]()
    A = AdjointOracle(prob)
    r = np.random.default_rng(4).standard_normal((A.S.shape[0], A.Nt - A.rs))
    g = adjoint_p0(prob, r)
    e = rel(g, A.adjoint(r))
    print(f"{name}: adjoint vs FP64 oracle {e:.2e}")
    assert e <= TOL, e


def test_dot_product_and_autograd():
    import torch
    from kwave_gb300.adjoint import SensorData, adjoint_p0, forward_p0, p0_gradient
    from oracle.adjoint_oracle import AdjointOracle

    prob = problem(cartesian=False)
    rng = np.random.default_rng(6)
    x = rng.standard_normal(prob["shape"])
    d = forward_p0(prob, x)
    y = rng.standard_normal(d.shape)
    lhs = float(np.sum(d.astype(np.float64) * y))
    rhs = float(np.sum(x * adjoint_p0(prob, y).astype(np.float64)))
    assert abs(lhs - rhs) <= 1e-4 * abs(lhs), (lhs, rhs)
    d_obs = forward_p0(prob, prob["p0"])
    p0 = 0.6 * prob["p0"]
    L, g = p0_gradient(prob, p0, d_obs)
    L_ref, g_ref, _ = AdjointOracle(prob).misfit_gradient(p0, d_obs.astype(np.float64))
    assert abs(L - L_ref) <= 1e-4 * L_ref and rel(g, g_ref) <= TOL
    t = torch.tensor(p0, dtype=torch.float64, requires_grad=True)
    loss = 0.5 * ((SensorData.apply(t, prob) - torch.as_tensor(d_obs, dtype=torch.float64)) ** 2).sum()
    loss.backward()
    assert rel(t.grad.numpy(), g) <= 1e-6


def test_cartesian_circle_adjoint_128():
    """The route of the reconstruction workload: a Cartesian circle of sensor
    points, whose residual goes back to the recorded grid corners through the
    transposed interpolation weights (adjoint.slot_residual) and then through
    the device adjoint, at 128^2 over 300 steps, against the FP64 adjoint
    oracle (which takes the residual back through the interpolation itself)."""
    from kwave_gb300.adjoint import adjoint_p0, forward_p0
    from oracle.adjoint_oracle import AdjointOracle
    from test_adjoint_cpu import circle

    prob = problem(shape=(128, 128), nt=300, cartesian=True)
    prob["sensor_mask"] = circle(64, 4.5e-3)
    A = AdjointOracle(prob)
    d = forward_p0(prob, prob["p0"])
    d64 = A.forward(prob["p0"])
    ef = rel(d, d64)
    r = np.random.default_rng(8).standard_normal((64, A.Nt - A.rs))
    g = adjoint_p0(prob, r)
    e = rel(g, A.adjoint(r))
    print(f"128^2 x 300 Cartesian circle: forward vs FP64 {ef:.2e}, adjoint vs FP64 {e:.2e}")
    assert ef <= TOL, ef
    assert e <= TOL, e


C_CASES = {
    "2d-40x48": lambda: problem(cartesian=False),
    "2d-40x48-cartesian": lambda: problem(cartesian=True),
    "3d-16x20x24": box3d,
}


@pytest.mark.parametrize("name", sorted(C_CASES))
def test_sound_speed_gradient_matches_oracle(name):
    """Both gradients of the misfit through the checkpointed GPU adjoint
    against the FP64 adjoint oracle (c_ref held at the base problem's)."""
    from kwave_gb300.adjoint import forward_p0, misfit_gradients
    from oracle.adjoint_oracle import AdjointOracle

    prob = C_CASES[name]()
    d_obs = forward_p0(prob, prob["p0"])
    p0 = 0.7 * prob["p0"]
    c = np.asarray(prob["sound_speed"], np.float64) * (1 - 0.01 * np.cos(np.arange(prob["p0"].size)).reshape(
        prob["shape"]))
    L, g_p0, g_c = misfit_gradients(prob, p0, d_obs, c=c, checkpoint_interval=5)
    L_ref, gr_p0, gr_c = AdjointOracle(prob).misfit_gradient(p0, d_obs.astype(np.float64), c=c)
    e0, ec = rel(g_p0, gr_p0), rel(g_c, gr_c)
    print(f"{name}: misfit {L:.4e} vs {L_ref:.4e}; grad p0 {e0:.2e}, grad c {ec:.2e} vs FP64")
    assert abs(L - L_ref) <= 1e-4 * L_ref
    assert e0 <= TOL and ec <= TOL, (e0, ec)


def test_checkpoint_interval_does_not_change_the_gradient():
    """K = 1 (every step kept, nothing recomputed), K = 7 and K = Nt (one
    checkpoint, the whole run recomputed) give bit-identical gradients: the
    regenerated steps are the forward's own steps."""
    from kwave_gb300.adjoint import forward_p0, misfit_gradients

    prob = problem(cartesian=False)
    d_obs = forward_p0(prob, prob["p0"])
    c = np.asarray(prob["sound_speed"]) * 1.005
    outs = [misfit_gradients(prob, 0.8 * prob["p0"], d_obs, c=c, checkpoint_interval=k) for k in (1, 7, prob["Nt"])]
    for L, g_p0, g_c in outs[1:]:
        assert L == outs[0][0]
        assert np.array_equal(g_p0, outs[0][1]) and np.array_equal(g_c, outs[0][2])


def test_sound_speed_gradient_finite_differences_on_a_crop():
    """Central differences of the GPU misfit along a smooth perturbation of c0
    confined to a 64 x 64 crop, at 256^2 over 600 steps with a 64-point
    Cartesian circle, against <grad c, v> from the checkpointed adjoint."""
    from kwave_gb300.adjoint import forward_p0, misfit_gradients
    from test_adjoint_cpu import circle

    prob = problem(shape=(256, 256), nt=600, cartesian=True, seed=12)
    prob["sensor_mask"] = circle(64, 1.0e-2)
    c_true = np.asarray(prob["sound_speed"], np.float64)
    d_obs = forward_p0(prob, prob["p0"])
    gx, gy = np.meshgrid(np.arange(256), np.arange(256), indexing="ij")
    v = np.zeros((256, 256))
    crop = (slice(96, 160), slice(80, 144))
    v[crop] = np.sin(np.pi * (gx[crop] - 96) / 64) * np.sin(np.pi * (gy[crop] - 80) / 64)
    c = c_true + 3.0 * v  # evaluate away from the data-generating medium
    L, _, g_c = misfit_gradients(prob, prob["p0"], d_obs, c=c)
    h = 0.5
    Lp, _, _ = misfit_gradients(prob, prob["p0"], d_obs, c=c + h * v)
    Lm, _, _ = misfit_gradients(prob, prob["p0"], d_obs, c=c - h * v)
    fd = (Lp - Lm) / (2 * h)
    an = float(np.sum(g_c.astype(np.float64) * v))
    print(f"FD {fd:.6e} adjoint {an:.6e} rel {abs(fd - an) / abs(fd):.2e}")
    assert abs(fd - an) <= 2e-2 * abs(fd)


def test_linear_operator_reuses_one_plan():
    """LinearP0 (one plan, p0 replaced with kw_plan_update_p0 for every
    forward) gives what a fresh plan per pass gives, bit for bit, over
    alternating forward and adjoint passes."""
    from kwave_gb300.adjoint import LinearP0, adjoint_p0, forward_p0

    prob = problem(cartesian=True)
    rng = np.random.default_rng(21)
    op = LinearP0(prob)
    try:
        for _ in range(2):
            x = rng.standard_normal(prob["shape"])
            d = op.forward(x)
            assert np.array_equal(d, forward_p0(prob, x))
            r = rng.standard_normal(d.shape)
            assert np.array_equal(op.adjoint(r), adjoint_p0(prob, r))
    finally:
        op.close()
