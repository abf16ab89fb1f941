"""The device's operator tables against the reference's legacy (C++-path)
precompute forms, run from the unmodified reference in this container:

* ``ddx_k_shift_pos/neg`` of kwave/kspaceFirstOrder2D.py:286-299 (kgrid.k_vec,
  ifftshift'ed, without kappa) against the KW_T_OPGRAD / KW_T_OPDIV tables,
  which are their Hermitian parts (equal away from an even length's Nyquist
  bin, real there);
* the absorption and dispersion operators and coefficients of
  kwave/kWaveSimulation_helper/create_absorption_variables.py:43-101
  (nabla1 = |k|^(y-2), nabla2 = |k|^(y-1), 0 at k = 0; tau, eta from
  db2neper) against |k|^a built from the KW_T_K tables and the host
  precompute's tau / eta;
* the PML profiles of kwave/utils/pml.py (get_pml, as the legacy function
  calls it at kspaceFirstOrder2D.py:277-280) against KW_T_PML / KW_T_PMLSG.

The legacy path's kappa (kspaceFirstOrder2D.py:303, numpy's normalised sinc
of c_ref k dt / 2) differs from the native solver's sinc(x / pi)
(kspace_solver.py:430), which is the form this backend follows; it is not
compared."""
import copy

import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref():
    import kwave_shim

    if not kwave_shim.reference_available():
        pytest.skip("reference checkout not available")
    kwave_shim.install()
    from kwave.data import Vector
    from kwave.kgrid import kWaveGrid
    from kwave.kmedium import kWaveMedium

    return Vector, kWaveGrid, kWaveMedium


def setup_of(shape, spacing, dt, c, alpha, y, pml):
    from kwave_gb300.precompute import build_setup

    prob = dict(shape=shape, spacing=spacing, dt=dt, Nt=2, sound_speed=c, density=1000.0, alpha_coeff=alpha,
                alpha_power=y, p0=np.ones(shape), smooth_p0=False, sensor_mask=None, record=None,
                pml_size=(pml,) * len(shape), pml_alpha=(2.0,) * len(shape), use_sg=True, use_kspace=True)
    return build_setup(prob, derive_on_device=False)


def table_c(S, name, a):
    t = S.tables[(name, a)].astype(np.float64)
    return t[0::2] + 1j * t[1::2]


@pytest.mark.parametrize("shape", [(48, 40), (45, 64)])
def test_shift_operators_are_the_hermitian_parts(ref, shape):
    Vector, kWaveGrid, _ = ref
    spacing = (1e-4, 1.2e-4)
    kg = kWaveGrid(Vector(list(shape)), Vector(list(spacing)))
    S = setup_of(shape, spacing, 2e-8, 1500.0, 0.0, 1.5, 8)
    for a, (n, d) in enumerate(zip(shape, spacing)):
        kv = np.asarray(kg.k_vec[a], dtype=np.float64).ravel()
        pos = np.fft.ifftshift(1j * kv * np.exp(1j * kv * d / 2))
        neg = np.fft.ifftshift(1j * kv * np.exp(-1j * kv * d / 2))
        for legacy, name in ((pos, "op_grad"), (neg, "op_div")):
            mine = table_c(S, name, a)
            keep = np.ones(n, bool)
            if n % 2 == 0:
                keep[n // 2] = False  # Nyquist: the Hermitian part keeps the real part only
                assert abs(mine[n // 2].imag) < 1e-6 * abs(legacy).max()
                assert abs(mine[n // 2].real - legacy[n // 2].real) <= 1e-6 * abs(legacy).max()
            err = np.abs(mine[keep] - legacy[keep]).max() / np.abs(legacy).max()
            assert err < 1e-6, (a, name, err)


@pytest.mark.parametrize("shape,y", [((40, 36), 1.5), ((24, 20, 18), 1.1)])
def test_absorption_operators_and_coefficients(ref, shape, y):
    Vector, kWaveGrid, kWaveMedium = ref
    from kwave.kWaveSimulation_helper.create_absorption_variables import create_absorption_variables

    spacing = (1e-4,) * len(shape)
    rng = np.random.default_rng(3)
    c = 1500.0 * (1 + 0.03 * rng.standard_normal(shape))
    kg = kWaveGrid(Vector(list(shape)), Vector(list(spacing)))
    med = kWaveMedium(sound_speed=c, density=1000.0, alpha_coeff=0.75, alpha_power=y)
    nab1, nab2, tau, eta = create_absorption_variables(kg, copy.deepcopy(med), "absorbing")
    S = setup_of(shape, spacing, 2e-8, c, 0.75, y, 4)
    ks = np.meshgrid(*[S.tables[("k", a)].astype(np.float64) for a in range(len(shape))], indexing="ij")
    kmag = np.sqrt(sum(k * k for k in ks))
    with np.errstate(divide="ignore"):
        mine1 = np.where(kmag == 0, 0.0, kmag ** (y - 2))
        mine2 = np.where(kmag == 0, 0.0, kmag ** (y - 1))
    for legacy, mine in ((nab1, mine1), (nab2, mine2)):
        legacy = np.asarray(legacy, dtype=np.float64)
        assert legacy.shape == mine.shape
        assert np.max(np.abs(mine - legacy)) <= 1e-6 * np.max(np.abs(legacy))
    assert np.max(np.abs(S.fields["tau"] - tau)) <= 1e-6 * np.max(np.abs(tau))
    assert np.max(np.abs(S.fields["eta"] - eta)) <= 1e-6 * np.max(np.abs(eta))


def test_pml_profiles(ref):
    from kwave.utils.pml import get_pml

    shape, spacing, dt, pml = (50, 44), (1e-4, 1.1e-4), 2e-8, 10
    S = setup_of(shape, spacing, dt, 1500.0, 0.0, 1.5, pml)
    for a, (n, d) in enumerate(zip(shape, spacing)):
        for name, stag in (("pml", False), ("pml_sg", True)):
            legacy = np.asarray(get_pml(n, d, dt, S.c_ref, pml, 2.0, stag, 1), dtype=np.float64).ravel()
            assert np.max(np.abs(S.tables[(name, a)] - legacy)) <= 1e-6, (a, name)
