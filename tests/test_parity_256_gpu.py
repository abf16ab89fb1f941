"""Parity of the headline workload itself -- the 256^3 heterogeneous absorbing
IVP (power law y = 1.5, B/A 6, 8 ellipsoids, 20 p0 blobs, z = 20 plane
recording p and p_max) -- with the unmodified reference.

The golden (tests/golden/ivp3d_256/, made by make_golden_256.py) holds the
reference's float32 and float64 results after T steps, reduced to p_max on
the whole plane, the p series of 256 plane points and every 8th cell of the
final interior field.  The test regenerates the seeded inputs, checks them
against the sums stored with the golden, runs the same T steps on the GPU
through the device plan and requires every reduction within 1e-5 relative L2
of the float32 reference; the error against float64 is printed beside it.
The largest T for which both goldens exist is used.
"""
import numpy as np
import pytest

import ivp3d_256

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib

    _lib.require_device()


def test_headline_256_matches_reference():
    cps = ivp3d_256.checkpoints()
    if not cps:
        pytest.skip("no 256^3 golden in tests/golden/ivp3d_256")
    t = cps[-1]
    from bench import ivp3d_problem
    from kwave_gb300.solver import run_problem

    prob = ivp3d_problem(n=256, nt=t, seed=0)
    g = ivp3d_256.load(t)
    ivp3d_256.check_inputs(prob, g["ref32"])
    prob["record"] = ("p", "p_max", "p_final")
    got = run_problem(prob)
    assert got["p"].shape == (256 * 256, t)
    res = ivp3d_256.parity(got, t)
    for k, e in res.items():
        print(f"256^3 x {t} steps {k}: vs ref32 {e['vs_f32']:.2e} vs ref64 {e['vs_f64']:.2e} "
              f"(ref32 vs ref64 {e['f32_vs_f64']:.2e})")
    for k, e in res.items():
        assert np.isfinite(e["vs_f32"]), k
        assert e["vs_f32"] <= TOL, (k, e)
