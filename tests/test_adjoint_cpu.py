"""The FP64 adjoint oracle of the lossless time loop.

The oracle is checked in four ways:

* its forward map against the FP64 solver oracle (itself pinned to the
  reference);
* the dot-product test <F x, y> = <x, F^T y>;
* central finite differences for the misfit gradients with respect to p0
  and c;
* PyTorch FP64 autograd through the same forward steps.

It is what a GPU adjoint of the time loop will be checked against.
"""
import numpy as np
import pytest

from oracle.adjoint_oracle import AdjointOracle
from oracle.kspace_oracle import OracleSimulation


def circle(n, radius):
    th = 2 * np.pi * np.arange(n) / n
    return np.stack([radius * np.cos(th), radius * np.sin(th)])


def problem(shape=(40, 48), nt=48, cartesian=True, record_start=1, seed=5):
    rng = np.random.default_rng(seed)
    gx, gy = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    p0 = np.zeros(shape)
    for _ in range(3):
        cx, cy = rng.uniform(14, shape[0] - 14), rng.uniform(14, shape[1] - 14)
        p0 += rng.uniform(0.5, 2) * np.exp(-((gx - cx) ** 2 + (gy - cy) ** 2) / (2 * rng.uniform(1.5, 3) ** 2))
    c = 1500.0 * (1 + 0.03 * np.tanh(rng.standard_normal(shape)))
    rho = 1000.0 * (1 + 0.02 * np.tanh(rng.standard_normal(shape)))
    if cartesian:
        mask = circle(24, 1.3e-3)
    else:
        mask = np.zeros(shape, bool)
        mask[10, 8:-8] = True
        mask[-11, 8:-8] = True
    return dict(shape=shape, spacing=(1e-4, 1e-4), dt=0.3 * 1e-4 / c.max(), Nt=nt, sound_speed=c, density=rho,
                p0=p0, smooth_p0=False, sensor_mask=mask, record=("p",), record_start_index=record_start,
                pml_size=(8, 8), pml_alpha=(2.0, 2.0), use_sg=True, use_kspace=True)


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / max(np.linalg.norm(np.ravel(b)), 1e-300))


@pytest.mark.parametrize("cartesian", [True, False])
def test_forward_matches_solver_oracle(cartesian):
    prob = problem(cartesian=cartesian)
    A = AdjointOracle(prob)
    ref = OracleSimulation(prob, np.float64).run()["p"]
    assert rel(A.forward(prob["p0"]), ref) < 1e-12


@pytest.mark.parametrize("cartesian,record_start", [(True, 1), (False, 6)])
def test_dot_product(cartesian, record_start):
    prob = problem(cartesian=cartesian, record_start=record_start)
    A = AdjointOracle(prob)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(prob["shape"])
    y = rng.standard_normal((A.S.shape[0], A.Nt - A.rs))
    lhs = float(np.sum(A.forward(x) * y))
    rhs = float(np.sum(x * A.adjoint(y)))
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), 1e-300), (lhs, rhs)


def test_gradients_against_finite_differences():
    prob = problem()
    A = AdjointOracle(prob)
    rng = np.random.default_rng(2)
    p_true = prob["p0"]
    d_obs = A.forward(p_true) + 0.01 * rng.standard_normal((A.S.shape[0], A.Nt - A.rs))
    p0 = 0.7 * p_true
    c = A.c
    L, g_p0, g_c = A.misfit_gradient(p0, d_obs, c)
    # p0: the misfit is quadratic in p0, so central differences are exact to rounding
    v = rng.standard_normal(p0.shape)
    h = 1e-3
    fd = (A.misfit_gradient(p0 + h * v, d_obs, c)[0] - A.misfit_gradient(p0 - h * v, d_obs, c)[0]) / (2 * h)
    assert abs(fd - np.sum(g_p0 * v)) <= 1e-7 * abs(fd), (fd, np.sum(g_p0 * v))
    # c: smooth perturbation, second-order differences
    w = np.exp(-(((np.arange(p0.shape[0])[:, None] - 20) ** 2 + (np.arange(p0.shape[1])[None, :] - 22) ** 2) / 40.0))
    h = 0.05
    fd = (A.misfit_gradient(p0, d_obs, c + h * w)[0] - A.misfit_gradient(p0, d_obs, c - h * w)[0]) / (2 * h)
    assert abs(fd - np.sum(g_c * w)) <= 1e-6 * abs(fd), (fd, np.sum(g_c * w))


@pytest.mark.parametrize("shape,nt,record_start", [((36, 40), 40, 1), ((30, 32), 30, 5)])
def test_gradients_against_torch_autograd(shape, nt, record_start):
    pytest.importorskip("torch")
    from oracle.torch_reference import misfit_and_grads

    prob = problem(shape=shape, nt=nt, record_start=record_start)
    A = AdjointOracle(prob)
    rng = np.random.default_rng(3)
    d_obs = A.forward(prob["p0"]) + 0.01 * rng.standard_normal((A.S.shape[0], A.Nt - A.rs))
    p0_np = 0.5 * prob["p0"]
    L, g_p0, g_c = A.misfit_gradient(p0_np, d_obs)
    Lt, gt_p0, gt_c = misfit_and_grads(prob, p0_np, d_obs)
    assert abs(Lt - L) <= 1e-12 * L
    assert rel(g_p0, gt_p0) < 1e-10
    assert rel(g_c, gt_c) < 1e-10


def test_rejects_what_it_does_not_cover():
    prob = problem()
    with pytest.raises(ValueError):
        AdjointOracle(dict(prob, alpha_coeff=0.5, alpha_power=1.5))
    with pytest.raises(ValueError):
        AdjointOracle(dict(prob, smooth_p0=True))


def test_gpu_wrapper_host_checks():
    """The GPU wrapper refuses, before any device call, what the transposed
    loop does not cover."""
    from kwave_gb300.adjoint import p0_gradient

    prob = problem(cartesian=False)
    with pytest.raises(ValueError):
        p0_gradient(dict(prob, smooth_p0=True), prob["p0"], np.zeros((1, 1)))


def test_gpu_wrapper_rejects_smoothing_everywhere():
    """Every entry of the GPU adjoint refuses a problem whose p0 would be
    smoothed -- smooth_p0 True or left unset, which means True in the
    reference -- before any device call: the forward would smooth, the
    transposed loop would not."""
    torch = pytest.importorskip("torch")
    from kwave_gb300.adjoint import SensorData, adjoint_p0

    prob = problem(cartesian=False)
    unset = {k: v for k, v in prob.items() if k != "smooth_p0"}
    for bad in (unset, dict(prob, smooth_p0=True)):
        with pytest.raises(ValueError, match="smooth_p0"):
            SensorData.apply(torch.zeros(prob["shape"], dtype=torch.float64), bad)
        with pytest.raises(ValueError, match="smooth_p0"):
            adjoint_p0(bad, np.zeros((1, 1)))


def test_cartesian_residual_to_slots():
    """A Cartesian sensor's residual taken back to its recorded grid points
    (the device adjoint's input) gives the same p0 gradient as the adjoint
    through the interpolation itself."""
    from kwave_gb300.adjoint import slot_residual
    from kwave_gb300.precompute import build_setup

    prob = problem(cartesian=True)
    S = build_setup(prob)
    assert S.sensor_kind == "cartesian"
    A = AdjointOracle(prob)
    binary = np.zeros(prob["shape"], bool)
    binary.ravel()[S.slots] = True
    B = AdjointOracle(dict(prob, sensor_mask=binary))
    r = np.random.default_rng(8).standard_normal((A.S.shape[0], A.Nt - A.rs))
    assert rel(B.adjoint(slot_residual(S, r)), A.adjoint(r)) < 1e-12


def test_steepest_descent_driver():
    """The reconstruction loop on the FP64 oracle's forward and adjoint: the
    misfit falls every iteration and the p0 error shrinks."""
    from kwave_gb300.adjoint import steepest_descent_p0

    prob = problem(cartesian=True)
    A = AdjointOracle(prob)
    d_obs = A.forward(prob["p0"])
    p, hist = steepest_descent_p0(A.forward, A.adjoint, d_obs, np.zeros(prob["shape"]), 8, p_true=prob["p0"])
    misfits = [h[0] for h in hist]
    assert all(b < a for a, b in zip(misfits, misfits[1:])), misfits
    assert hist[-1][1] < 0.9 * hist[0][1], hist


def test_vessel_problem_runs_on_the_oracle():
    """The reconstruction workload's generator, at a reduced size, gives a
    problem the adjoint oracle accepts (lossless, smoothing off, Cartesian
    circle inside the grid)."""
    import bench

    prob = bench.vessel_problem(n=64, nt=20, pml=8, n_sensor=32, radius=1.2e-3)
    A = AdjointOracle(prob)
    d = A.forward(prob["p0"])
    assert d.shape == (32, 20) and np.all(np.isfinite(d)) and np.abs(d).max() > 0


def test_adjoint_oracle_against_autograd_at_128():
    """The 128 x 128 check of the reconstruction workload's gradients: the
    adjoint oracle against FP64 torch autograd (p0 and c)."""
    pytest.importorskip("torch")
    from oracle.torch_reference import misfit_and_grads

    prob = problem(shape=(128, 128), nt=60, cartesian=False)
    A = AdjointOracle(prob)
    d_obs = A.forward(prob["p0"]) * 1.01
    p0 = 0.5 * prob["p0"]
    L, g_p0, g_c = A.misfit_gradient(p0, d_obs)
    Lt, gt_p0, gt_c = misfit_and_grads(prob, p0, d_obs)
    assert abs(Lt - L) <= 1e-12 * L
    assert rel(g_p0, gt_p0) < 1e-10 and rel(g_c, gt_c) < 1e-10


def test_cgls_driver_beats_steepest_descent():
    """CGLS on the FP64 oracle's forward and adjoint: the misfit falls every
    iteration, and after the same number of passes it is below steepest
    descent's (conjugate directions)."""
    from kwave_gb300.adjoint import cgls_p0, steepest_descent_p0

    prob = problem(cartesian=True)
    A = AdjointOracle(prob)
    d_obs = A.forward(prob["p0"])
    _, h_cg = cgls_p0(A.forward, A.adjoint, d_obs, np.zeros(prob["shape"]), 8, p_true=prob["p0"])
    _, h_sd = steepest_descent_p0(A.forward, A.adjoint, d_obs, np.zeros(prob["shape"]), 8, p_true=prob["p0"])
    m = [h[0] for h in h_cg]
    assert all(b < a for a, b in zip(m, m[1:])), m
    assert h_cg[-1][0] < h_sd[-1][0] and h_cg[-1][1] < h_sd[-1][1], (h_cg[-1], h_sd[-1])


@pytest.mark.parametrize("record_start", [1, 5])
def test_autograd_reference_with_independent_operators(record_start):
    """FP64 torch autograd through operators built from the reference's
    formulas in torch (k-vectors, kappa, shifts, PML, staggered density,
    sensor indices), not taken from the adjoint oracle, agrees with the
    oracle's adjoint gradients: the oracle's operator construction is checked
    too, not only its transposes."""
    pytest.importorskip("torch")
    from oracle.torch_reference import misfit_and_grads

    prob = problem(shape=(36, 40), nt=40, cartesian=False, record_start=record_start)
    A = AdjointOracle(prob)
    d_obs = A.forward(prob["p0"]) * 1.02
    p0 = 0.6 * prob["p0"]
    L, g_p0, g_c = A.misfit_gradient(p0, d_obs)
    Lt, gt_p0, gt_c = misfit_and_grads(prob, p0, d_obs, operators="independent")
    assert abs(Lt - L) <= 1e-10 * L
    assert rel(g_p0, gt_p0) < 1e-9 and rel(g_c, gt_c) < 1e-9
