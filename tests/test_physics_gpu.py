"""Physics variants of the register (power-of-two) kernels against the oracle.

The golden cases fix the reference's outputs on a few problems; these cases
cover the remaining branches of the power-of-two row stages and operator
passes on 3-D and 2-D grids: power law with and without dispersion, with
and without B/A, heterogeneous media, Stokes absorption, lossless nonlinear,
and additive k-space corrected sources together with power-law absorption.
The oracle runs the reference's algorithm in float32 (bit-identical to the
reference solver in float32 on every golden case), so the bar is the parity
bar: 1e-5 relative L2 on the recorded pressure and on the final fields.
"""
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def blobs(shape, rng, n=3):
    g = np.meshgrid(*[np.arange(s) for s in shape], indexing="ij")
    out = np.zeros(shape)
    for _ in range(n):
        c = [rng.uniform(s / 4, 3 * s / 4) for s in shape]
        out += rng.uniform(1, 5) * np.exp(-sum((gi - ci) ** 2 for gi, ci in zip(g, c)) / (2 * rng.uniform(1.5, 3) ** 2))
    return out


def field(shape, rng, base, rel):
    return base * (1 + rel * np.tanh(rng.standard_normal(shape)))


def problem(kind, shape, rng):
    nd = len(shape)
    prob = dict(shape=shape, spacing=(1e-4,) * nd, dt=1.5e-8, Nt=14, sound_speed=1500.0, density=1000.0,
                pml_size=(6,) * nd, pml_alpha=(2.0,) * nd, use_sg=True, use_kspace=True, smooth_p0=True,
                sensor_mask=(rng.random(shape) < 0.02), record=("p", "p_final"))
    if kind in ("powerlaw", "powerlaw_nodisp", "stokes", "lossless_nl", "powerlaw_src"):
        prob["sound_speed"] = field(shape, rng, 1500.0, 0.05)
        prob["density"] = field(shape, rng, 1000.0, 0.05)
    if kind == "powerlaw":
        prob.update(alpha_coeff=0.75, alpha_power=1.5, BonA=6.0)
    elif kind == "powerlaw_nodisp":
        prob.update(alpha_coeff=field(shape, rng, 0.5, 0.3), alpha_power=1.3, alpha_mode="no_dispersion")
    elif kind == "stokes":
        prob.update(alpha_coeff=0.5, alpha_power=2.0, BonA=5.0)
    elif kind == "lossless_nl":
        prob.update(BonA=field(shape, rng, 6.0, 0.2))
    if kind == "powerlaw_src":
        prob.update(alpha_coeff=0.75, alpha_power=1.5, BonA=6.0)
        mask = np.zeros(shape, bool)
        mask[tuple(s // 2 for s in shape[:-1])] = True
        prob.update(p_mask=mask, p_mode="additive",
                    p=1e3 * np.sin(2 * np.pi * 1e6 * 1.5e-8 * np.arange(prob["Nt"]))[None, :])
    else:
        prob["p0"] = blobs(shape, rng)
    return prob


CASES = [("powerlaw", (64, 32, 64)), ("powerlaw_nodisp", (32, 64, 128)), ("stokes", (64, 32, 64)),
         ("lossless_nl", (32, 32, 128)), ("powerlaw_src", (64, 32, 64)), ("powerlaw", (128, 256)),
         ("powerlaw_nodisp", (256, 64))]


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()


@pytest.mark.parametrize("kind,shape", CASES, ids=[f"{k}-{'x'.join(map(str, s))}" for k, s in CASES])
def test_power_of_two_physics(kind, shape):
    from kwave_gb300.solver import Simulation
    from oracle.kspace_oracle import OracleSimulation

    rng = np.random.default_rng(zlib.crc32(f"{kind}{shape}".encode()))
    prob = problem(kind, shape, rng)
    sim = Simulation.from_problem(prob)
    try:
        got = sim.run()
        fields = {"u": [u.copy() for u in sim.u], "rho": [r.copy() for r in sim.rho_split]}
    finally:
        sim.close()
    o = OracleSimulation(prob, np.float32)
    ref = o.run()
    for k in ("p", "p_final"):
        e = rel_l2(got[k], ref[k])
        print(f"{kind} {shape} {k}: {e:.2e}")
        assert e <= TOL, (k, e)
    for name, mine, theirs in (("u", fields["u"], o.u), ("rho", fields["rho"], o.rho_split)):
        for a, (x, y) in enumerate(zip(mine, theirs)):
            e = rel_l2(x, y)
            assert e <= TOL, (name, a, e)


@pytest.mark.parametrize("kind,shape", [("powerlaw", (64, 32, 64)), ("stokes", (48, 40)),
                                        ("powerlaw_nodisp", (32, 64, 128))])
def test_device_derived_medium(kind, shape):
    """dt/rho_sg, tau and eta formed on the device (kw_plan_derive_medium)
    against the same grids formed on the host in FP64: the two runs agree to
    float32 rounding of the medium arrays."""
    from kwave_gb300.precompute import build_setup
    from kwave_gb300.solver import DevicePlan
    from kwave_gb300 import _lib as K

    rng = np.random.default_rng(zlib.crc32(f"derive{kind}{shape}".encode()))
    prob = problem(kind, shape, rng)
    outs = []
    for dev in (False, True):
        S = build_setup(prob, derive_on_device=dev)
        assert bool(S.derive) == dev
        plan = DevicePlan(S)
        try:
            plan.run(S.Nt)
            plan.sync()
            outs.append([plan.read_field(K.KW_FLD_P)] + [plan.read_field(K.KW_FLD_U0 + a) for a in range(len(shape))])
        finally:
            plan.close()
    for a, b in zip(*outs):
        assert rel_l2(b, a) <= 2e-6, rel_l2(b, a)
