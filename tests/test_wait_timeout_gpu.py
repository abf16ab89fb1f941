"""Failure detection of the bounded device waits, made to run out on purpose
without any fault: with kw_plan_set_wait_test the velocity stage's bulk-fed
row kernel withholds one copy in its first CTA and its waits give up after
20 ms.  The consumers leave together, the host reads the device error word,
and the next call reports the timeout; the context stays usable, and a fresh
plan on the same device then reproduces a golden case."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib

    _lib.require_device()


def test_wait_timeout_is_reported_and_the_device_stays_usable():
    from fixtures import load_case

    from kwave_gb300 import _lib
    from kwave_gb300.solver import Simulation, run_problem

    n0, n1 = 64, 128
    g = np.meshgrid(np.arange(n0), np.arange(n1), indexing="ij")
    p0 = np.exp(-((g[0] - 30) ** 2 + (g[1] - 60) ** 2) / 20.0)
    mask = np.zeros((n0, n1), bool)
    mask[20, :] = True
    prob = dict(shape=(n0, n1), spacing=(1e-4, 1e-4), dt=2e-8, Nt=6, sound_speed=1500.0, density=1000.0, p0=p0,
                smooth_p0=False, sensor_mask=mask, record=("p",), pml_size=(8, 8), pml_alpha=(2.0, 2.0))
    sim = Simulation.from_problem(prob).setup()
    try:
        _lib.check(_lib.lib().kw_plan_set_wait_test(sim._plan.handle, 1))
        sim._plan.run(3)
        with pytest.raises(_lib.KwaveGB300Error, match="timed out"):
            sim._plan.sync()
        # switched off and reset, the same plan runs clean again
        _lib.check(_lib.lib().kw_plan_set_wait_test(sim._plan.handle, 0))
        _lib.check(_lib.lib().kw_plan_reset(sim._plan.handle))
        sim._plan.run(6)
        sim._plan.sync()
    finally:
        sim.close()
    golden, r32, _, _ = load_case("pow2_2d_src")
    got = run_problem(golden)
    for k in r32:
        err = float(np.linalg.norm(got[k] - r32[k]) / np.linalg.norm(r32[k]))
        assert err <= 1e-5, (k, err)


def test_wait_test_needs_the_bulk_fed_stages():
    from kwave_gb300 import _lib
    from kwave_gb300.solver import Simulation

    prob = dict(shape=(30, 36), spacing=(1e-4, 1e-4), dt=2e-8, Nt=4, sound_speed=1500.0, density=1000.0,
                p0=np.ones((30, 36)), smooth_p0=False, sensor_mask=None, record=None, pml_size=(4, 4),
                pml_alpha=(2.0, 2.0))
    sim = Simulation.from_problem(prob).setup()
    try:
        assert _lib.lib().kw_plan_set_wait_test(sim._plan.handle, 1) == _lib.KW_ERR_UNSUPPORTED
    finally:
        sim.close()
