"""Host logic of the unified ``kspaceFirstOrder`` entry point and of
``TimeReversal`` (no GPU).

The pre-processing (``pml_size="auto"``, normalisation, validation, PML
expansion, output cropping) is pinned against the reference's own results in
tests/golden/api/: the prepared problem run by the CPU oracle must reproduce
the reference's ``kspaceFirstOrder`` output, and ``TimeReversal`` driven by
the oracle must reproduce the reference's reconstruction.
"""
import warnings
from types import SimpleNamespace as NS

import numpy as np
import pytest

import api_cases
from kwave_gb300 import unified
from kwave_gb300.precompute import problem_from_kwave
from kwave_gb300.reconstruction import TimeReversal
from oracle.kspace_oracle import run_oracle


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# ---------------------------------------------------------------------------
# argument handling
# ---------------------------------------------------------------------------

def test_normalize_pml():
    assert unified.normalize_pml(20, 3) == (20, 20, 20)
    assert unified.normalize_pml((6, 9), 2) == (6, 9)
    assert unified.normalize_pml((6,), 3) == (6, 6, 6)
    assert unified.normalize_pml((1.5,), 2, "pml_alpha") == (1.5, 1.5)
    with pytest.raises(ValueError, match="pml_size must be"):
        unified.normalize_pml("big", 2)
    with pytest.raises(ValueError, match="1-to-2-element"):
        unified.normalize_pml((1, 2, 3), 2)
    with pytest.raises(ValueError, match="1-to-2-element"):
        unified.normalize_pml((), 2)


def test_resolve_dtype():
    assert unified.resolve_dtype(None) is np.float64
    assert unified.resolve_dtype("off") is np.float64
    assert unified.resolve_dtype("single") is np.float32
    assert unified.resolve_dtype(np.float32) is np.float32
    assert unified.resolve_dtype(float) is np.float64
    with pytest.raises(ValueError, match="float32 or float64"):
        unified.resolve_dtype(np.float16)
    with pytest.raises(ValueError, match="numpy dtype"):
        unified.resolve_dtype(object())


def test_optimal_pml_size_values():
    # N + 2 p with the smallest largest prime factor, first such p in 10..40
    assert list(unified.get_optimal_pml_size((44, 40, 36))) == [10, 12, 14]
    assert list(unified.get_optimal_pml_size((128, 128))) == [17, 17]
    assert list(unified.get_optimal_pml_size((100,))) == [14]
    assert unified.largest_prime_factor(97) == 97
    assert unified.largest_prime_factor(64) == 2
    with pytest.raises(ValueError):
        unified.get_optimal_pml_size((64, 64), pml_range=(20, 10))


def test_optimal_pml_size_matches_reference():
    import kwave_shim

    if not kwave_shim.reference_available():
        pytest.skip("reference checkout not present")
    kwave_shim.install()
    from kwave.utils.pml import get_optimal_pml_size as ref

    rng = np.random.default_rng(5)
    for _ in range(40):
        dim = int(rng.integers(1, 4))
        shape = tuple(int(n) for n in rng.integers(16, 300, size=dim))
        assert list(unified.get_optimal_pml_size(shape)) == list(ref(shape)), shape


def _small_problem(**kw):
    shape = (32, 30)
    prob = dict(shape=shape, spacing=(1e-4, 1e-4), Nt=10, dt=1e-8, sound_speed=1500.0, density=1000.0)
    prob.update(kw)
    return prob


@pytest.mark.parametrize("change,match", [
    (dict(Nt=0), "Nt must be >= 1"),
    (dict(dt=-1.0), "dt must be > 0"),
    (dict(sound_speed=np.full((3, 3), 1500.0)), "sound_speed has 9 elements"),
    (dict(sound_speed=-1.0), "must be positive"),
    (dict(density=0.0), "density must be positive"),
    (dict(alpha_coeff=-0.1), "non-negative"),
    (dict(p0=np.ones((4, 4))), "p0 has 16 elements"),
    (dict(p=np.ones(10)), "requires source.p_mask"),
    (dict(ux=np.ones(10)), "requires source.u_mask"),
    (dict(p_mask=np.ones((4, 4), bool)), "p_mask has 16 elements"),
    (dict(sensor_mask=np.ones((5, 5), bool)), "sensor.mask has 25 elements"),
    (dict(u_mask=np.ones((32, 30), bool), ux=np.ones(10), uy=np.ones((3, 10))), "single \\(1D\\) or many"),
])
def test_validation_errors(change, match):
    with pytest.raises(ValueError, match=match):
        unified.validate_problem(_small_problem(**change), (4, 4))


def test_validation_pml_and_warnings():
    with pytest.raises(ValueError, match="too large"):
        unified.validate_problem(_small_problem(), (16, 4))
    with pytest.raises(ValueError, match="non-negative"):
        unified.validate_problem(_small_problem(), (-1, 4))
    with pytest.warns(UserWarning, match="CFL"):
        unified.validate_problem(_small_problem(dt=1e-6), (4, 4))
    with pytest.warns(UserWarning, match="outside typical range"):
        unified.validate_problem(_small_problem(alpha_coeff=0.5, alpha_power=3.5), (4, 4))
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        unified.validate_problem(_small_problem(sensor_mask=np.ones((2, 5))), (4, 4))  # Cartesian


def test_expand_and_strip():
    rng = np.random.default_rng(0)
    c = 1500 + rng.random((6, 5))
    p0 = rng.random((6, 5))
    mask = rng.random((6, 5)) > 0.5
    cart = rng.random((2, 7))
    prob = dict(shape=(6, 5), sound_speed=c, density=1000.0, p0=p0.ravel(), sensor_mask=mask, u_mask=mask)
    out = unified.expand_problem(prob, (2, 1))
    assert out["shape"] == (10, 7)
    assert out["density"] == 1000.0                     # homogeneous values pass through
    assert np.array_equal(out["sound_speed"][2:-2, 1:-1], c)
    assert np.array_equal(out["sound_speed"][0, 1:-1], c[0])   # edge-extended
    assert np.array_equal(out["sound_speed"][:, 0], out["sound_speed"][:, 1])
    assert out["p0"].shape == (10, 7) and out["p0"][0].sum() == 0 and np.allclose(out["p0"][2:-2, 1:-1], p0)
    assert out["sensor_mask"].sum() == mask.sum() and not out["sensor_mask"][:2].any()
    assert out["u_mask"].sum() == mask.sum()
    # order of the mask points is kept (C order), so source/sensor rows line up
    assert np.array_equal(np.flatnonzero(out["sensor_mask"]).size, np.flatnonzero(mask).size)
    out = unified.expand_problem(dict(prob, sensor_mask=cart), (2, 1))
    assert out["sensor_mask"] is cart
    res = {"p_max_all": np.zeros((10, 7)), "p_max": np.zeros(7), "p": np.zeros((7, 3)), "p_final": np.zeros((6, 5))}
    st = unified.strip_pml(res, (2, 1), 2)
    assert st["p_max_all"].shape == (6, 5) and st["p_max"].shape == (7,) and st["p"].shape == (7, 3)
    assert st["p_final"].shape == (6, 5)


def test_reshape_to_grid():
    d = np.arange(24.0).reshape(6, 4)
    assert unified.reshape_to_grid(d, (2, 3)).shape == (2, 3, 4)
    assert unified.reshape_to_grid(d[:, 0], (2, 3)).shape == (2, 3)


def test_entry_point_rejections():
    kgrid, medium, source, sensor = api_cases.objects(_small_problem())
    with pytest.raises(ValueError, match="Unknown backend"):
        unified.kspaceFirstOrder(kgrid, medium, source, sensor, backend="python")
    with pytest.raises(ValueError, match="device must be 'gpu'"):
        unified.kspaceFirstOrder(kgrid, medium, source, sensor, device="cpu")
    with pytest.raises(ValueError, match="data_path must be provided"):
        unified.kspaceFirstOrder(kgrid, medium, source, sensor, save_only=True, pml_size=4)
    with pytest.raises(ValueError, match="must be set before"):
        unified.kspaceFirstOrder(NS(N=(32, 30), spacing=(1e-4, 1e-4), Nt="auto", dt="auto"), medium, source, sensor)
    k1 = NS(N=np.array([64]), spacing=np.array([1e-4]), Nt=10, dt=1e-8)
    with pytest.raises(NotImplementedError, match="2-D and 3-D"):
        unified.kspaceFirstOrder(k1, medium, source, None)


# ---------------------------------------------------------------------------
# pinned against the reference (tests/golden/api)
# ---------------------------------------------------------------------------

UNIFIED = api_cases.names("unified")


@pytest.mark.parametrize("name", UNIFIED)
def test_prepared_problem_reproduces_reference(name):
    """prepare_problem + the solver (here the CPU oracle) + strip_pml gives the
    reference kspaceFirstOrder result."""
    prob, opts, r32, _ = api_cases.load(name)
    kgrid, medium, source, sensor = api_cases.objects(prob)
    call = {k: v for k, v in opts.items() if k in ("pml_size", "pml_alpha", "pml_inside", "smooth_p0")}
    prepared, pml = unified.prepare_problem(kgrid, medium, source, sensor, **call)
    out = run_oracle(prepared, dtype=np.float32)
    if not opts.get("pml_inside", False):
        out = unified.strip_pml(out, pml, len(prob["shape"]))
    assert set(out) == set(r32)
    for k, v in r32.items():
        assert out[k].shape == v.shape, (k, out[k].shape, v.shape)
        assert rel_l2(out[k], v) <= 2e-6, (k, rel_l2(out[k], v))


def _oracle_legacy(kgrid, source, sensor, medium, simulation_options, execution_options):
    prob = problem_from_kwave(kgrid, medium, source, sensor, pml_size=tuple(simulation_options.pml_size),
                              pml_alpha=tuple(simulation_options.pml_alpha),
                              smooth_p0=simulation_options.smooth_p0)
    return run_oracle(prob, dtype=np.float32)


def test_time_reversal_reproduces_reference():
    prob, opts, r32, _ = api_cases.load("tr2d")
    kgrid, medium, _, _ = api_cases.objects(prob)
    sensor = NS(mask=prob["sensor_mask"], record=["p"], recorded_pressure=prob["recorded_pressure"])
    tr = TimeReversal(kgrid, medium, sensor, compensation_factor=opts["compensation_factor"])
    so = NS(pml_size=opts["pml_size"], pml_alpha=opts["pml_alpha"], smooth_p0=True)
    got = tr(_oracle_legacy, so, None)
    assert sensor.record == ["p"]                       # caller's list is not extended
    assert got.shape == r32["p0_recon"].shape
    assert np.all(got >= 0)
    assert rel_l2(got, r32["p0_recon"]) <= 2e-6


def test_time_reversal_rejections():
    prob, _, _, _ = api_cases.load("tr2d")
    kgrid, medium, _, _ = api_cases.objects(prob)
    mask = prob["sensor_mask"]
    with pytest.raises(ValueError, match="Sensor mask must be set"):
        TimeReversal(kgrid, medium, NS(mask=None))
    with pytest.raises(ValueError, match="t_array must be explicitly set"):
        TimeReversal(NS(N=kgrid.N, spacing=kgrid.spacing, Nt=kgrid.Nt, dt=kgrid.dt, t_array="auto"), medium,
                     NS(mask=mask, record=None))
    with pytest.raises(ValueError, match="compensation_factor must be positive"):
        TimeReversal(kgrid, medium, NS(mask=mask, record=None), compensation_factor=0)
    with pytest.raises(ValueError, match="at least one active point"):
        TimeReversal(kgrid, medium, NS(mask=np.zeros_like(mask), record=None))
    with pytest.raises(ValueError, match="does not match grid"):
        TimeReversal(kgrid, medium, NS(mask=mask[:20], record=None))
    tr = TimeReversal(kgrid, medium, NS(mask=mask, record=None))
    with pytest.raises(ValueError, match="recorded pressure"):
        tr(_oracle_legacy, NS(), None)


# ---------------------------------------------------------------------------
# cart2grid (kwave/utils/conversion.py:164-325)
# ---------------------------------------------------------------------------

def _circle(n, r):
    th = np.linspace(0, 2 * np.pi, n, endpoint=False)
    return np.stack([r * np.cos(th), r * np.sin(th)])


def test_cart2grid_values():
    from kwave_gb300 import cart2grid

    kg = NS(N=np.array([32, 40]), spacing=np.array([1e-4, 1e-4]))
    pts = _circle(24, 1.2e-3)
    grid, order_index, reorder = cart2grid(kg, pts, order="C")
    assert grid.shape == (32, 40) and grid.dtype.kind == "i"
    # every point lands where rounding puts it, and the reorder index lists the
    # points in C order of their grid positions
    ix = np.round(pts[0] / 1e-4).astype(int) + 16
    iy = np.round(pts[1] / 1e-4).astype(int) + 20
    assert grid[ix, iy].all() and grid.sum() == len(set(zip(ix, iy)))
    flat = np.ravel_multi_index((ix, iy), (32, 40))
    assert np.array_equal(np.sort(flat[reorder[:, 0].astype(int) - 1]), flat[reorder[:, 0].astype(int) - 1])
    assert sorted(order_index[:, 0]) == list(range(1, reorder.size + 1))
    with pytest.warns(FutureWarning, match="cart2grid"):
        cart2grid(kg, pts)
    with pytest.raises(AssertionError, match="within the grid"):
        cart2grid(kg, pts * 100, order="C")


def test_cart2grid_matches_reference():
    import kwave_shim

    if not kwave_shim.reference_available():
        pytest.skip("reference checkout not present")
    kwave_shim.install()
    from kwave.kgrid import kWaveGrid
    from kwave.utils.conversion import cart2grid as ref

    from kwave_gb300 import cart2grid

    rng = np.random.default_rng(3)
    cases = [([48, 40], _circle(60, 1.5e-3)), ([20, 24, 18], rng.uniform(-7e-4, 7e-4, size=(3, 30))),
             ([50], rng.uniform(-2e-3, 2e-3, size=(1, 12)))]
    for N, pts in cases:
        kg = kWaveGrid(N, [1e-4] * len(N))
        for order in ("C", "F"):
            mine = cart2grid(kg, pts, order=order)
            theirs = ref(kg, pts, order=order)
            for a, b in zip(mine, theirs):
                assert np.asarray(a).shape == np.asarray(b).shape
                assert np.array_equal(np.asarray(a), np.asarray(b)), (N, order)


def test_batch_host_checks():
    """Host-side checks of the batch API that need no GPU: an empty batch is
    refused before any device call, and the transmit-event generator gives
    the shapes the batched workload is quoted on."""
    import bench
    from kwave_gb300.solver import SimulationBatch

    with pytest.raises(ValueError):
        SimulationBatch([])
    sizes = bench._five_smooth(192, 512)
    assert sizes[0] == 192 and sizes[-1] == 512 and 243 in sizes and 250 in sizes and 7 * 32 not in sizes
    probs = bench.transmit_problems(3, nt=50, seed=4)
    for p in probs:
        assert all(n in sizes for n in p["shape"])
        n_src = int(p["p_mask"].sum())
        assert n_src == 32 * 3 and p["p"].shape[0] == n_src
        assert p["dt"] <= 0.3 * 5e-5 / p["sound_speed"].max() * (1 + 1e-12)
        assert np.array_equal(p["sensor_mask"], p["p_mask"])


def test_drop_in_switch_through_the_reference_call(monkeypatch):
    """The reference's own legacy call, kwave.kspaceFirstOrder2D.kspaceFirstOrder2D
    (kwave/kspaceFirstOrder2D.py:215-218), reaches the GB300 time loop after
    ``install()`` when the execution options select ``backend="gb300"``, with
    the options the reference bridge derives (kwave/solvers/native.py:6-30);
    ``backend="python"`` still reaches the reference's own solver, and
    ``uninstall()`` restores the original bridge.  The two solver classes are
    replaced by recorders, so no GPU is needed."""
    import kwave_shim

    if not kwave_shim.reference_available():
        pytest.skip("reference checkout not available")
    kwave_shim.install()
    import kwave.kspaceFirstOrder2D as K2
    import kwave.solvers.native as native
    from kwave.data import Vector
    from kwave.kgrid import kWaveGrid
    from kwave.kmedium import kWaveMedium
    from kwave.ksensor import kSensor
    from kwave.ksource import kSource
    from kwave.options.simulation_execution_options import SimulationExecutionOptions
    from kwave.options.simulation_options import SimulationOptions

    from kwave_gb300 import backend

    calls = []

    def recorder(tag):
        class Rec:
            def __init__(self, kgrid, medium, source, sensor, **kw):
                calls.append((tag, (kgrid, medium, source, sensor), kw))

            def run(self):
                return {"p": np.array([tag])}

            def close(self):
                pass

        return Rec

    monkeypatch.setattr(backend, "Simulation", recorder("gb300"))
    monkeypatch.setattr(native, "Simulation", recorder("python"))
    original = native.run_python_backend
    kg = kWaveGrid(Vector([32, 32]), Vector([1e-4, 1e-4]))
    kg.makeTime(1500.0, 0.3)
    med = kWaveMedium(sound_speed=1500.0, density=1000.0)
    src = kSource()
    src.p0 = np.zeros((32, 32))
    src.p0[16, 16] = 1.0
    mask = np.zeros((32, 32), bool)
    mask[8, :] = True
    sen = kSensor(mask)
    backend.install()
    try:
        assert native.run_python_backend is not original
        with pytest.warns(FutureWarning):
            out = K2.kspaceFirstOrder2D(kg, src, sen, med, SimulationOptions(), backend.execution_options())
        assert out["p"][0] == "gb300"
        with pytest.warns(FutureWarning):
            out = K2.kspaceFirstOrder2D(kg, src, sen, med, SimulationOptions(),
                                        SimulationExecutionOptions(backend="python", is_gpu_simulation=False))
        assert out["p"][0] == "python"
    finally:
        backend.uninstall()
    assert native.run_python_backend is original
    (t1, a1, kw1), (t2, a2, kw2) = calls
    assert (t1, t2) == ("gb300", "python")
    assert all(x is y for x, y in zip(a1, (kg, med, src, sen))) and all(x is y for x, y in zip(a2, a1))
    keys = ("use_sg", "use_kspace", "smooth_p0", "pml_size", "pml_alpha")
    assert {k: kw1[k] for k in keys} == {k: kw2[k] for k in keys}
    assert kw1["pml_size"] == (20, 20) and kw1["pml_alpha"] == (2.0, 2.0)
    assert kw1["use_sg"] and kw1["use_kspace"] and kw1["smooth_p0"]
    assert kw1["device"] == "gpu"
