"""Pin the CPU oracle (oracle/kspace_oracle.py) against outputs of the unmodified
reference solver stored in tests/golden/*.npz (generated by make_golden.py)."""
import numpy as np
import pytest

from fixtures import case_names, load_case
from oracle.kspace_oracle import run_oracle

CASES = case_names()


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("prec", ["32", "64"])
def test_oracle_matches_reference(name, prec):
    prob, r32, r64, _ = load_case(name)
    ref = r32 if prec == "32" else r64
    out = run_oracle(prob, dtype=np.float32 if prec == "32" else np.float64)
    assert set(out) == set(ref), (sorted(out), sorted(ref))
    for k, v in ref.items():
        assert out[k].shape == v.shape, k
        assert out[k].dtype == v.dtype, (k, out[k].dtype, v.dtype)
        # identical NumPy operations: agreement to rounding of the Cartesian
        # interpolation only
        tol = 1e-12 if prec == "64" else 1e-6
        assert rel_l2(out[k], v) <= tol, (k, rel_l2(out[k], v))


def test_golden_cases_present():
    for required in ("ivp2d_128_circle", "het3d_abs_nl", "ivp3d_48_absorbing", "src2d_additive", "src2d_dirichlet"):
        assert required in CASES
