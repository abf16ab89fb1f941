"""Golden cases for the entry points built on the solver: the unified
``kspaceFirstOrder`` (kwave/kspaceFirstOrder.py) and ``TimeReversal``
(kwave/reconstruction/time_reversal.py), produced by the unmodified reference
on a host that holds its checkout (``KWAVE_REFERENCE_ROOT``, or a ``reference``
directory beside this repository):

    python tests/golden/make_api_golden.py

Cases land in ``tests/golden/api/``.  ``in:`` keys hold the user-level
problem (before any PML expansion), ``meta:`` keys the call's options.

* unified cases: the reference's ``kspaceFirstOrder(..., backend="python")``
  with ``dtype=np.float32`` (ref32) and ``np.float64`` (ref64);
* time reversal: a forward run records p on a binary line; the reference's
  ``TimeReversal`` then runs with its stock legacy ``kspaceFirstOrder2D``
  (python backend, which computes in float64: ref64) and with a legacy-
  signature function that runs the reference ``Simulation`` in float32
  (ref32).
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

import kwave_shim  # noqa: E402
from fixtures import save_case  # noqa: E402
from make_golden import gaussian_blobs, smooth_random_field, tone_burst_rows  # noqa: E402

SUBDIR = "api"


def _objects(prob):
    from kwave.kgrid import kWaveGrid
    from kwave.kmedium import kWaveMedium
    from kwave.ksensor import kSensor
    from kwave.ksource import kSource

    kg = kWaveGrid(list(prob["shape"]), list(prob["spacing"]))
    kg.setTime(int(prob["Nt"]), float(prob["dt"]))
    med = kWaveMedium(sound_speed=prob["sound_speed"])
    for k in ("density", "alpha_coeff", "alpha_power", "alpha_mode", "BonA"):
        if prob.get(k) is not None:
            setattr(med, k, prob[k])
    src = kSource()
    for k in ("p0", "p_mask", "p", "p_mode", "u_mask", "ux", "uy", "uz", "u_mode"):
        if prob.get(k) is not None:
            setattr(src, k, prob[k])
    sensor = None
    if prob.get("sensor_mask") is not None:
        sensor = kSensor(mask=prob["sensor_mask"], record=list(prob["record"]) if prob.get("record") else None)
    return kg, med, src, sensor


def run_unified(prob, opts, dtype):
    kwave_shim.install()
    from kwave.kspaceFirstOrder import kspaceFirstOrder

    kg, med, src, sen = _objects(prob)
    return kspaceFirstOrder(kg, med, src, sen, backend="python", device="cpu", dtype=dtype, quiet=True, **opts)


def unified_case(name, prob, opts):
    r32 = run_unified(prob, opts, np.float32)
    r64 = run_unified(prob, opts, np.float64)
    meta = {f"opt_{k}": v for k, v in opts.items()}
    save_case(name, prob, r32, r64, meta=meta, subdir=SUBDIR)
    print(name, {k: v.shape for k, v in r32.items()})


def case_unified2d_pml_outside():
    """Heterogeneous absorbing nonlinear 2-D medium, p0 smoothed after the
    grid is grown by 2 x 8 PML points, binary sensor circle."""
    rng = np.random.default_rng(101)
    shape = (56, 48)
    yy, xx = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    r = np.hypot(yy - 27.5, xx - 23.5)
    prob = dict(shape=shape, spacing=(1e-4, 1.2e-4), Nt=140, dt=1.5e-8,
                sound_speed=smooth_random_field(shape, rng, rel=0.04),
                density=smooth_random_field(shape, rng, rel=0.05, base=1000.0),
                alpha_coeff=0.75, alpha_power=1.5, BonA=6.0,
                p0=gaussian_blobs(shape, 3, rng, margin=10),
                sensor_mask=(np.abs(r - 20.0) < 0.6), record=("p", "p_final", "p_max", "p_rms", "ux", "uy"))
    return prob, dict(pml_size=8, pml_alpha=2.0, pml_inside=False, smooth_p0=True)


def case_unified3d_auto():
    """3-D, pml_size='auto' (44 x 40 x 36 grown by 10/12/14 points per side
    to 64^3), additive pressure source on a binary patch, Cartesian sensors."""
    rng = np.random.default_rng(102)
    shape = (44, 40, 36)
    dx = 1e-4
    dt = 1.5e-8
    m = np.zeros(shape, bool)
    m[22, 18:22, 16:20] = True
    n_src = int(m.sum())
    sig = tone_burst_rows(1, 40, dt, 1.2e6, 3, rng, max_delay=1)
    pts = rng.uniform(-0.6, 0.6, size=(3, 12)) * np.array([[s * dx / 2] for s in shape])
    prob = dict(shape=shape, spacing=(dx, dx, dx), Nt=40, dt=dt, sound_speed=1500.0, density=1000.0,
                p_mask=m, p=sig * 1e3, sensor_mask=pts, record=("p", "p_max", "p_final"))
    assert n_src > 0
    return prob, dict(pml_size="auto", pml_inside=False, smooth_p0=True)


def case_unified2d_pml_inside():
    """PML inside the grid with per-axis sizes and a short pml_alpha tuple,
    no smoothing, velocity and final-field recording."""
    rng = np.random.default_rng(103)
    shape = (48, 40)
    mask = np.zeros(shape, bool)
    mask[::4, ::3] = True
    prob = dict(shape=shape, spacing=(1e-4, 1e-4), Nt=90, dt=1.8e-8, sound_speed=1500.0, density=1000.0,
                p0=gaussian_blobs(shape, 2, rng, margin=12), sensor_mask=mask,
                record=("p", "ux", "uy", "p_final", "ux_final", "p_min"))
    return prob, dict(pml_size=(6, 9), pml_alpha=(1.5,), pml_inside=True, smooth_p0=False)


# ---------------------------------------------------------------------------
# time reversal
# ---------------------------------------------------------------------------

def _sim_f32(kgrid, source, sensor, medium, simulation_options, execution_options):
    """Legacy-signature run of the reference Simulation in float32."""
    from kwave.solvers.kspace_solver import Simulation

    return Simulation(kgrid, medium, source, sensor, use_sg=True, use_kspace=True,
                      smooth_p0=simulation_options.smooth_p0, pml_size=tuple(simulation_options.pml_size),
                      pml_alpha=tuple(simulation_options.pml_alpha), dtype=np.float32, quiet=True).run()


def case_tr2d():
    """Photoacoustic forward run (64 x 64, PML 10 inside) recorded on the line
    x = 12; time reversal from that line back to p0."""
    kwave_shim.install()
    from kwave.kspaceFirstOrder2D import kspaceFirstOrder2D
    from kwave.options.simulation_execution_options import SimulationExecutionOptions
    from kwave.options.simulation_options import SimulationOptions
    from kwave.reconstruction.time_reversal import TimeReversal
    from kwave.solvers.kspace_solver import Simulation

    rng = np.random.default_rng(104)
    shape = (64, 64)
    prob = dict(shape=shape, spacing=(1e-4, 1e-4), Nt=150, dt=2e-8, sound_speed=1500.0, density=1000.0)
    p0 = gaussian_blobs(shape, 3, rng, margin=20)
    mask = np.zeros(shape, bool)
    mask[12, 10:54] = True
    kg, med, _, _ = _objects(prob)
    from kwave.ksensor import kSensor
    from kwave.ksource import kSource

    src = kSource()
    src.p0 = p0
    fwd = Simulation(kg, med, src, kSensor(mask=mask, record=["p"]), smooth_p0=True, pml_size=(10, 10),
                     pml_alpha=(2.0, 2.0), dtype=np.float64, quiet=True).run()
    recorded = np.asarray(fwd["p"])
    opts = SimulationOptions(pml_inside=True, pml_size=[10, 10], pml_alpha=[2.0, 2.0], smooth_p0=True)
    exe = SimulationExecutionOptions(is_gpu_simulation=False, backend="python")
    outs = {}
    for tag, fn in (("32", _sim_f32), ("64", kspaceFirstOrder2D)):
        sensor = kSensor(mask=mask, record=["p"])
        sensor.recorded_pressure = recorded
        tr = TimeReversal(kg, med, sensor, compensation_factor=2.0)
        outs[tag] = {"p0_recon": np.asarray(tr(fn, opts, exe))}
    case = dict(prob, sensor_mask=mask, recorded_pressure=recorded, p0_true=p0)
    meta = dict(opt_pml_size=(10, 10), opt_pml_alpha=(2.0, 2.0), opt_compensation_factor=2.0)
    save_case("tr2d", case, outs["32"], outs["64"], meta=meta, subdir=SUBDIR)
    print("tr2d", outs["32"]["p0_recon"].shape)


CASES = {
    "unified2d_pml_outside": case_unified2d_pml_outside,
    "unified3d_auto": case_unified3d_auto,
    "unified2d_pml_inside": case_unified2d_pml_inside,
}


def main(names=None):
    for name, fn in CASES.items():
        if names and name not in names:
            continue
        prob, opts = fn()
        unified_case(name, prob, opts)
    if not names or "tr2d" in names:
        case_tr2d()


if __name__ == "__main__":
    main(sys.argv[1:])
