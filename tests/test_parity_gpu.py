"""Parity of the GB300 time loop with the reference, on the GPU.

Each golden case (tests/golden/*.npz) holds outputs of the unmodified
reference solver in float32 and float64.  The GPU result must agree with the
float32 reference within 1e-5 relative L2 for every recorded key; its error
against the float64 reference is printed next to it.

One exception is allowed, and only where float32 itself cannot resolve the
quantity: when the reference's own float32 result is further than 5e-6 from
its float64 result (e.g. the small residual p_final of the 128x128 IVP after
604 steps, 2.6e-5), the GPU result must instead be at most 1.5x as far from
the float64 reference as the reference's float32 result is.
"""
import numpy as np
import pytest

from fixtures import case_names, load_case

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative L2 against the float32 reference

# features the device path does not provide yet
PENDING = {}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib

    _lib.require_device()


@pytest.mark.parametrize("name", case_names())
def test_gpu_matches_reference(name):
    if name in PENDING:
        pytest.skip(PENDING[name])
    from kwave_gb300.solver import run_problem

    prob, r32, r64, _ = load_case(name)
    got = run_problem(prob)
    assert set(got) == set(r32), (sorted(got), sorted(r32))
    for k in sorted(r32):
        assert got[k].shape == r32[k].shape, (k, got[k].shape, r32[k].shape)
        e32 = rel_l2(got[k], r32[k])
        e64 = rel_l2(got[k], r64[k])
        gap = rel_l2(r32[k], r64[k])
        print(f"{name}:{k} vs ref32 {e32:.2e} vs ref64 {e64:.2e} (ref32 vs ref64 {gap:.2e})")
        assert np.all(np.isfinite(got[k])), k
        if gap > 0.5 * TOL:
            assert e32 <= TOL or e64 <= 1.5 * gap + 1e-6, (k, e32, e64, gap)
        else:
            assert e32 <= TOL, (k, e32, e64)
