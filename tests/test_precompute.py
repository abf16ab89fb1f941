"""Host-side FP64 setup (kwave_gb300.precompute) against the oracle's own
quantities, and the Hermitian-part identity that lets the device use
half-spectrum transforms.  CPU only."""
import numpy as np
import pytest

from fixtures import case_names, load_case
from kwave_gb300.precompute import build_setup, hermitian_part
from oracle.kspace_oracle import OracleSimulation


@pytest.mark.parametrize("name", case_names())
def test_setup_matches_oracle(name):
    prob, _, _, _ = load_case(name)
    S = build_setup(prob)
    o = OracleSimulation(prob, dtype=np.float32).setup()
    assert S.ndim == o.ndim and S.shape == o.grid_shape
    assert S.c_ref == o.c_ref
    for a in range(S.ndim):
        np.testing.assert_array_equal(S.tables[("pml", a)], o.pml_list[a].ravel())
        np.testing.assert_array_equal(S.tables[("pml_sg", a)], o.pml_sg_list[a].ravel())
        np.testing.assert_array_equal(S.tables[("k", a)], o.k_list[a].ravel())
        dtr = S.fields[f"dtrsg{a}"]
        ref = o.dt_over_rho0[a]
        np.testing.assert_allclose(np.broadcast_to(dtr, ref.shape), ref, rtol=2e-7)
    assert S.record_start == o.record_start_index
    assert S.requested == o._requested_record
    assert S.n_points == o.n_sensor_points
    if o.sensor_kind == "binary":
        np.testing.assert_array_equal(S.slots, o.sensor_index)
    if o.tau is not None:
        np.testing.assert_allclose(np.broadcast_to(S.fields["tau"], o.tau.shape), o.tau, rtol=1e-6)
    if o.eta is not None:
        np.testing.assert_allclose(np.broadcast_to(S.fields["eta"], o.eta.shape), o.eta, rtol=1e-6)
    if o._p0_initial is not None and S.smooth is None:
        np.testing.assert_allclose(S.fields["p0"], o._p0_initial, rtol=0, atol=2e-6 * np.abs(o._p0_initial).max())


@pytest.mark.parametrize("shape", [(128, 128), (48, 40), (45, 27), (32, 24, 20), (15, 16, 17)])
def test_smoothing_tables_reproduce_reference_window(shape):
    """The device window (linear interpolation of the 1-D samples at the
    per-axis squared coordinates) equals ifftshift(rotated Blackman window)."""
    from kwave_gb300.precompute import smoothing_tables
    from oracle.kspace_oracle import blackman_window_rotated

    win, radius, coords = smoothing_tables(shape)
    r2 = sum(np.asarray(c, np.float64).reshape([-1 if i == a else 1 for i in range(len(shape))])
             for a, c in enumerate(coords))
    r = np.minimum(np.sqrt(r2), radius)
    pos = (r + radius) / (2 * radius) * (len(win) - 1)
    i0 = np.minimum(pos.astype(int), len(win) - 2)
    f = pos - i0
    w = win[i0] + f * (win[i0 + 1] - win[i0])
    ref = np.fft.ifftshift(np.abs(blackman_window_rotated(shape)))
    np.testing.assert_allclose(w, ref, rtol=0, atol=2e-6)


@pytest.mark.parametrize("name", ["src2d_dirichlet", "src2d_velocity", "vel2d_dirichlet", "src2d_additive"])
def test_source_scaling_matches_oracle(name):
    prob, _, _, _ = load_case(name)
    S = build_setup(prob)
    o = OracleSimulation(prob, dtype=np.float32).setup()
    # inject one step into a zero field with both implementations' scalings
    for src in S.sources:
        t = 3
        field = np.zeros(o.grid_shape, np.float32)
        if src.slot < 3:
            op = o._source_p_ops[src.slot]
        else:
            op = o._source_u_ops[src.slot - 3]
        if src.mode == "additive":
            continue  # k-space corrected: compared end to end on the GPU
        ref = op(t, field).ravel()
        got = np.zeros_like(ref)
        rows = src.signal[:, t] if src.signal.shape[0] > 1 else np.full(src.index.size, src.signal[0, t])
        got[src.index] = rows
        np.testing.assert_allclose(got, ref, rtol=2e-7, atol=1e-30)


def test_cartesian_stencil_matches_oracle_interpolation():
    prob, _, _, _ = load_case("stokes3d_cart")
    S = build_setup(prob)
    o = OracleSimulation(prob, dtype=np.float64).setup()
    f = np.random.default_rng(0).standard_normal(o.grid_shape)
    ref = o._extract(f)
    vals = f.ravel()[S.slots]
    got = np.sum(S.interp_w * vals[S.interp_slot], axis=1)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("shape", [(16, 12), (15, 9), (8, 6, 10), (9, 5, 7)])
@pytest.mark.parametrize("use_sg", [True, False])
def test_half_spectrum_with_hermitian_ops_equals_reference_diff(shape, use_sg):
    """irfftn(op_h * rfftn(f)) == Re(ifftn(op * fftn(f))) for the gradient ops."""
    rng = np.random.default_rng(1)
    f = rng.standard_normal(shape)
    d = 1e-4
    ks = [2 * np.pi * np.fft.fftfreq(n, d) for n in shape]
    grids = np.meshgrid(*ks, indexing="ij")
    kmag = np.sqrt(sum(g ** 2 for g in grids))
    kappa = np.sinc(1500 * kmag * 2e-8 / 2 / np.pi)
    for a in range(len(shape)):
        k = ks[a]
        f1 = 1j * k * np.exp(1j * k * d / 2) if use_sg else 1j * k
        sh = [1] * len(shape)
        sh[a] = -1
        op = f1.reshape(sh) * kappa
        ref = np.real(np.fft.ifftn(op * np.fft.fftn(f)))
        oph = hermitian_part(f1).reshape(sh) * kappa
        H = shape[-1] // 2 + 1
        ax = tuple(range(len(shape)))
        got = np.fft.irfftn(oph[..., :H] * np.fft.rfftn(f, axes=ax), s=shape, axes=ax)
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-10 * np.abs(ref).max())
