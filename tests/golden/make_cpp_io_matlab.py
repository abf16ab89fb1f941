"""Golden checks of the legacy C++ route's input files, from the reference's
own fixtures: ``tests/reference_outputs/*.json`` of the reference hold, for
input files that MATLAB k-Wave wrote for its examples, every dataset's dtype,
shape, attributes and SHA-256 checksums of its values rounded to 6..16
decimals (tests/h5_summary.py:18-33 of the reference); the reference's tests
(e.g. tests/test_ivp_homogeneous_medium.py) compare the files of its legacy
``kspaceFirstOrder2DC/3DC(..., save_to_disk=True)`` with them
(tests/diff_utils.py, precision 8, ``Nt`` and the creator/date/description
attributes excluded).

For each example this script builds the inputs with the reference's own
functions (grids and ``makeTime``/``setTime``, ``make_disc``, ``make_ball``,
``make_circle``, ``make_cart_circle``, ``filter_time_series``, ``smooth``) on a
host that holds the reference checkout (``KWAVE_REFERENCE_ROOT``, or a
``reference`` directory beside this repository), and stores them with the
summary entries at precision 8:

    python tests/golden/make_cpp_io_matlab.py

Cases land in ``tests/golden/cpp_io_matlab/``: ``<case>.npz`` with the
inputs (``in:<key>``) and simulation options (``opt:<name>``), and
``<case>.json`` with the expected summary.
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
OUT = HERE / "cpp_io_matlab"


def _reference():
    import kwave_shim

    kwave_shim.install()
    return kwave_shim.REFERENCE_ROOT


def _summary(root, name):
    """The reference's summary of one file, trimmed to what its comparison
    reads: dtype, shape, attributes, the precision-8 checksum; the root
    group's attributes other than creator, date and description."""
    src = json.loads((root / "tests" / "reference_outputs" / f"{name}.json").read_text())
    out = {}
    for k, v in src.items():
        if k == "root":
            out[k] = {"attrs": {a: s for a, s in v["attrs"].items()
                                if a not in ("created_by", "creation_date", "file_description")}}
        elif k != "Nt":
            out[k] = {"dtype": v["dtype"], "shape": v["shape"], "attrs": v["attrs"],
                      "checksum8": v["checksums"]["8"]}
    return out


def _store(case, ref_name, root, kgrid, medium, source, sensor_mask, **opts):
    arrs = {"in:shape": np.asarray([int(n) for n in kgrid.N]), "in:spacing": np.asarray(kgrid.spacing, float),
            "in:Nt": np.asarray(int(kgrid.Nt)), "in:dt": np.asarray(float(kgrid.dt))}
    for k, v in {**medium, **source}.items():
        arrs[f"in:{k}"] = np.asarray(v)
    arrs["in:sensor_mask"] = np.asarray(sensor_mask)
    for k, v in opts.items():
        arrs[f"opt:{k}"] = np.asarray(v)
    OUT.mkdir(exist_ok=True)
    np.savez_compressed(OUT / f"{case}.npz", **arrs)
    (OUT / f"{case}.json").write_text(json.dumps(_summary(root, ref_name), indent=1, sort_keys=True) + "\n")
    print(case)


def main():
    root = _reference()
    from kwave.data import Vector
    from kwave.kgrid import kWaveGrid
    from kwave.kmedium import kWaveMedium
    from kwave.utils.filters import filter_time_series, smooth
    from kwave.utils.mapgen import make_ball, make_cart_circle, make_circle, make_disc

    def grid(n, d, c=None, nt=None, dt=None):
        kg = kWaveGrid(Vector(list(n)), Vector(list(d)))
        if nt is not None:
            kg.setTime(nt, dt)
        else:
            kg.makeTime(c)
        return kg

    def discs(n):
        N = Vector(list(n))
        return 5 * make_disc(N, Vector([50, 50]), 8) + 3 * make_disc(N, Vector([80, 60]), 5)

    # 128^2 initial value problems, default options (PML 20 inside, p0 smoothed)
    absorbing = dict(sound_speed=1500.0, alpha_coeff=0.75, alpha_power=1.5)
    kg = grid((128, 128), (1e-4, 1e-4), 1500)
    _store("ivp_homogeneous_medium", "out_ivp_homogeneous_medium", root, kg, absorbing, dict(p0=discs((128, 128))),
           make_cart_circle(4e-3, 50))
    c = 1500 * np.ones((128, 128))
    c[:64] = 1800
    rho = 1000 * np.ones((128, 128))
    rho[:, 31:] = 1200
    _store("ivp_heterogeneous_medium", "out_ivp_heterogeneous_medium", root, grid((128, 128), (1e-4, 1e-4), c),
           dict(sound_speed=c, density=rho), dict(p0=discs((128, 128))), make_cart_circle(4e-3, 50))
    _store("ivp_binary_sensor_mask", "out_ivp_binary_sensor_mask", root, kg, absorbing, dict(p0=discs((128, 128))),
           make_circle(Vector([128, 128]), Vector([64, 64]), 42, 3 * np.pi / 2))
    for i, opts in enumerate((dict(pml_alpha=0.0), dict(pml_alpha=1e6), dict(pml_size=2), dict(pml_inside=False))):
        _store(f"na_controlling_the_PML_{i + 1}", f"out_na_controlling_the_PML/input_{i + 1}", root, kg,
               dict(sound_speed=1500.0), dict(p0=discs((128, 128))), make_cart_circle(4e-3, 50), **opts)

    # time-varying point sources on a 50 mm grid: pressure (monopole), velocity (dipole)
    d2 = 50e-3 / 128
    kg = grid((128, 128), (d2, d2), 1500)
    mask = np.zeros((128, 128))
    mask[95, 63] = 1
    sens = np.zeros((128, 128))
    sens[31, 63] = 1
    sig = filter_time_series(kg, kWaveMedium(**absorbing), 2 * np.sin(2 * np.pi * 0.25e6 * kg.t_array))
    _store("tvsp_homogeneous_medium_monopole", "out_tvsp_homogeneous_medium_monopole", root, kg, absorbing,
           dict(p_mask=mask, p=sig), sens)
    dense = dict(absorbing, density=1000.0)
    ux = filter_time_series(kg, kWaveMedium(**dense), -(2 / 1.5e6) * np.sin(2 * np.pi * 0.25e6 * kg.t_array))
    _store("tvsp_homogeneous_medium_dipole", "out_tvsp_homogeneous_medium_dipole", root, kg, dense,
           dict(u_mask=mask, ux=ux), sens)

    # a source moving along a line: 88 rows, each point driven in turn
    nd, dd = (64, 128), (10e-3 / 64, 20e-3 / 128)
    kg = grid(nd, dd, nt=4500, dt=20e-9)
    sp = filter_time_series(kg, kWaveMedium(**absorbing), 3 * np.sin(2 * np.pi * 0.75e6 * kg.t_array))
    pm = np.zeros(nd)
    pm[38, 20:108] = 1
    n = int(pm.sum())
    rows = np.zeros((n, kg.t_array.size))
    k, t = 1, 0
    while t < kg.t_array.size and k < n - 1:
        if kg.t_array[0, t] > k * dd[1] / 150:
            k += 1
        ratio = (k * dd[1] - 150 * kg.t_array[0, t]) / dd[1]
        rows[k - 1, t] = ratio * sp[0, t]
        rows[k, t] = (1 - ratio) * sp[0, t]
        t += 1
    sens = np.zeros(nd)
    sens[33, 63] = 1
    _store("tvsp_doppler_effect", "out_tvsp_doppler_effect", root, kg, absorbing, dict(p_mask=pm, p=rows), sens)

    # PML outside the user's grid, p0 smoothed by the caller
    n2 = (88, 216)
    p0 = smooth(5 * make_disc(Vector(list(n2)), Vector([30, 110]), 8)
                + 5 * make_disc(Vector(list(n2)), Vector([60, 140]), 5), True)
    line = np.zeros(n2)
    line[0, :] = 1
    kg = grid(n2, (1e-4, 1e-4), 1500)
    for case in ("pr_2D_FFT_line_sensor", "pr_2D_TR_line_sensor"):
        _store(case, f"out_{case}", root, kg, dict(sound_speed=1500.0), dict(p0=p0), line, pml_inside=False,
               pml_size=(20, 20), smooth_p0=False)

    # 3-D: heterogeneous media with Cartesian sensors mapped to grid points
    n3 = (64, 64, 64)
    c3 = 1500 * np.ones(n3)
    c3[:32] = 1800
    r3 = 1000 * np.ones(n3)
    r3[:, 15:, :] = 1200
    kg = grid(n3, (1e-4,) * 3, c3)
    N3 = Vector(list(n3))
    p03 = 10 * make_ball(N3, Vector([38, 32, 32]), 5) + 10 * make_ball(N3, Vector([20, 20, 20]), 3)
    x = np.arange(-22, 23, 2) * 1e-4
    _store("ivp_3D_simulation", "out_ivp_3D_simulation", root, kg, dict(sound_speed=c3, density=r3), dict(p0=p03),
           np.vstack([x, 22e-4 * np.ones_like(x), x]))
    pm3 = np.zeros(n3)
    pm3[15, 26:37, 26:37] = 1
    sig3 = filter_time_series(kg, kWaveMedium(sound_speed=c3, density=r3), np.sin(2 * np.pi * 2e6 * kg.t_array))
    yz = np.arange(-20, 21, 2) * 1e-4
    _store("tvsp_3D_simulation", "out_tvsp_3D_simulation", root, kg, dict(sound_speed=c3, density=r3),
           dict(p_mask=pm3, p=sig3), np.array([20e-4 * np.ones(yz.shape), yz, yz]))
    # small photoacoustic sources, 1 mm grids of 64 points, set time axis
    for d, maker in ((2, make_disc), (3, make_ball)):
        n = (64,) * d
        kgp = grid(n, (1e-3 / 64,) * d, nt=round(300e-9 / 2e-9) + 1, dt=2e-9)
        sens = np.zeros(n)
        sens[(21,) + (31,) * (d - 1)] = 1
        _store(f"ivp_photoacoustic_waveforms_{d}d", f"out_ivp_photoacoustic_waveforms/input_{d - 1}", root, kgp,
               dict(sound_speed=1500.0), dict(p0=maker(Vector(list(n)), Vector(list(n)) / 2, 2)), sens)
    # the sensor frequency response is applied to the recorded data, not stored
    kgf = grid((128, 128), (1e-4, 1e-4), 1500)
    for i in (1, 2):
        _store(f"ivp_sensor_frequency_response_{i}", f"out_ivp_sensor_frequency_response/input_{i}", root, kgf,
               absorbing, dict(p0=discs((128, 128))), make_cart_circle(4e-3, 50))
    # binary sensor from cart2grid, time axis to 6 us, PML switched off / outside
    from kwave.utils.conversion import cart2grid

    kgm = kWaveGrid(Vector([128, 128]), Vector([1e-4, 1e-4]))
    kgm.makeTime(1500, 0.3, 6e-6)
    bm = cart2grid(kgm, make_cart_circle(6.3e-3, 50))[0]
    for i, opts in ((1, dict(pml_alpha=0.0)), (2, dict(pml_inside=False))):
        _store(f"ivp_comparison_modelling_functions_{i}", f"out_ivp_comparison_modelling_functions/input_{i}", root,
               kgm, dict(sound_speed=1500.0), dict(p0=discs((128, 128))), bm, **opts)
    # 256 x 128 x 64 absorbing medium with a ball, a pressure patch source and a sensor plane
    nr = (256, 128, 64)
    kgr = grid(nr, (1e-4,) * 3, nt=1200, dt=15e-9)
    ball = make_ball(Vector(list(nr)), Vector(list(nr)) / 2 + Vector([40, 0, 0]), 20)
    cr = 1500 * np.ones(nr)
    rr = 1000 * np.ones(nr)
    cr[ball == 1] = 1800
    rr[ball == 1] = 1200
    med = dict(sound_speed=cr, density=rr, alpha_coeff=0.75, alpha_power=1.5)
    pmr = np.zeros(nr)
    pmr[10, 33:94, 16:47] = 1
    sigr = filter_time_series(kgr, kWaveMedium(**med), 0.5e6 * np.sin(2 * np.pi * 2e6 * kgr.t_array))
    plane = np.zeros(nr)
    plane[:, :, 31] = 1
    _store("cpp_running_simulations", "out_cpp_running_simulations", root, kgr, med, dict(p_mask=pmr, p=sigr),
           plane, pml_size=(10, 10, 10))
    n3b = (12, 44, 44)
    kg = grid(n3b, (2e-4,) * 3, 1500)
    p0b = smooth(10 * make_ball(Vector(list(n3b)), Vector(list(n3b)) / 2, 3), True)
    plane = np.zeros(n3b)
    plane[0] = 1
    _store("pr_3D_FFT_planar_sensor", "out_pr_3D_FFT_planar_sensor", root, kg, dict(sound_speed=1500.0),
           dict(p0=p0b), plane, pml_inside=False, pml_size=(10, 10, 10), smooth_p0=False)


if __name__ == "__main__":
    main()
