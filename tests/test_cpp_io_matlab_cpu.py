"""Input files of the legacy C++ route (``kspaceFirstOrder2DC/3DC`` with
``save_to_disk``), on the CPU, against the reference's own fixtures of files
that MATLAB k-Wave wrote for its examples (``tests/golden/cpp_io_matlab``,
made by ``tests/golden/make_cpp_io_matlab.py`` from the reference's
``tests/reference_outputs``).

* Every dataset of the file matches the fixture as the reference's
  comparison does it (tests/diff_utils.py and tests/h5_summary.py of the
  reference): the same names, dtypes, shapes and attributes, and the same
  SHA-256 checksum of the values rounded to 8 decimals; the root group's
  file type and version; ``Nt`` and the creator, date and description
  attributes are not compared.  The cases cover 2-D and 3-D grids,
  heterogeneous sound speed and density (staggered densities), Cartesian,
  binary-arc and line/plane sensors, smoothed p0, the PML inside and outside
  the grid and its size/alpha options, and pressure and velocity sources of
  one and of many rows (scaled source signals).
* Reading such a file back with ``scaled_sources=True`` gives the caller's
  source signals again (the scaling divided out, rows in C order), and the
  problem read back is the simulation the file was written for: the float64
  oracle runs both to the same sensor data within 1e-5 relative L2 (1e-6
  measured: the file holds dt and the signals in float32).
"""
import hashlib
import json
from pathlib import Path
from types import SimpleNamespace as NS

import numpy as np
import pytest

from kwave_gb300 import backend, cpp_io, h5io

GOLDEN = Path(__file__).resolve().parent / "golden" / "cpp_io_matlab"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))
MEDIUM = ("sound_speed", "density", "alpha_coeff", "alpha_power", "BonA")
SOURCE = ("p0", "p_mask", "p", "p_mode", "u_mask", "ux", "uy", "uz", "u_mode")


def _load(name):
    z = np.load(GOLDEN / f"{name}.npz", allow_pickle=False)
    inp = {k[3:]: z[k] for k in z.files if k.startswith("in:")}
    opts = {k[4:]: (z[k].item() if z[k].ndim == 0 else tuple(z[k].tolist())) for k in z.files if k.startswith("opt:")}
    return inp, opts, json.loads((GOLDEN / f"{name}.json").read_text())


def _objects(inp):
    shape = tuple(int(n) for n in inp["shape"])
    kgrid = NS(N=np.array(shape), spacing=np.array(inp["spacing"], float), Nt=int(inp["Nt"]), dt=float(inp["dt"]),
               dim=len(shape))
    medium = NS(**{k: (inp[k].item() if k in inp and inp[k].ndim == 0 else inp.get(k)) for k in MEDIUM})
    source = NS(**{k: inp.get(k) for k in SOURCE})
    sensor = NS(mask=inp["sensor_mask"], record=None, record_start_index=None)
    return kgrid, medium, source, sensor


def _write(name, tmp_path):
    inp, opts, expected = _load(name)
    kgrid, medium, source, sensor = _objects(inp)
    so = NS(save_to_disk=True, save_to_disk_exit=True, data_path=str(tmp_path), input_filename=f"{name}.h5", **opts)
    run = backend.kspaceFirstOrder2DC if kgrid.dim == 2 else backend.kspaceFirstOrder3DC
    assert run(kgrid, source, sensor, medium, so) is None
    return tmp_path / f"{name}.h5", inp, expected


def _summary(path):
    """What the reference's H5Summary records of a file (tests/h5_summary.py:
    dtype, attributes as the str() of h5py's bytes values, shape, SHA-256 of
    the values rounded to 8 decimals plus 0, which folds -0 into 0)."""
    ds, at, root = h5io.read_file(path)
    out = {}
    for k, v in ds.items():
        a = np.array(v)
        out[k] = {"dtype": str(a.dtype), "shape": list(a.shape),
                  "attrs": {n: str(np.bytes_(s.encode())) for n, s in at.get(k, {}).items()},
                  "checksum8": hashlib.sha256(a.round(8) + 0).hexdigest()}
    out["root"] = {"attrs": {n: str(np.bytes_(s.encode())) for n, s in root.items()}}
    return out


@pytest.mark.parametrize("name", CASES)
def test_legacy_input_file_matches_matlab_fixture(name, tmp_path):
    path, _, expected = _write(name, tmp_path)
    got = _summary(path)
    assert set(got) - {"Nt"} == set(expected), sorted(set(got) ^ set(expected))
    for k, want in expected.items():
        if k == "root":
            for a, v in want["attrs"].items():
                assert got["root"]["attrs"][a] == v, (a, got["root"]["attrs"][a], v)
            continue
        g = got[k]
        assert (g["dtype"], g["shape"], g["attrs"]) == (want["dtype"], want["shape"], want["attrs"]), k
        assert g["checksum8"] == want["checksum8"], k


def test_fixtures_cover_the_legacy_features():
    """The fixture set holds what the test above claims to cover."""
    kinds = set()
    for name in CASES:
        inp, opts, expected = _load(name)
        kinds.add(f"{len(inp['shape'])}-D")
        if np.asarray(inp["sound_speed"]).size > 1:
            kinds.add("heterogeneous")
        m = np.asarray(inp["sensor_mask"])
        kinds.add("cartesian" if m.ndim == 2 and m.shape[0] == len(inp["shape"]) and m.shape != tuple(inp["shape"])
                  else "binary")
        kinds.add("pml outside" if opts.get("pml_inside") is False else "pml inside")
        for f in ("p", "ux", "p0"):
            if f in inp:
                kinds.add(f"{f} rows {min(np.atleast_2d(inp[f]).shape[0], 2)}" if f != "p0" else "p0")
        assert "p_source_input" not in expected or "p" in inp
    assert kinds >= {"2-D", "3-D", "heterogeneous", "cartesian", "binary", "pml outside", "pml inside", "p0",
                     "p rows 1", "p rows 2", "ux rows 1"}, kinds


@pytest.mark.parametrize("name", ["tvsp_homogeneous_medium_monopole", "tvsp_homogeneous_medium_dipole",
                                  "tvsp_doppler_effect", "tvsp_3D_simulation"])
def test_scaled_sources_read_back(name, tmp_path):
    """The legacy file's scaled signals, read with ``scaled_sources=True``,
    are the caller's signals (rows in C order of the mask's points) to
    float32 rounding; read without it they carry the scaling."""
    path, inp, _ = _write(name, tmp_path)
    shape = tuple(int(n) for n in inp["shape"])
    prob = cpp_io.problem_from_input_file(path, scaled_sources=True)
    raw = cpp_io.problem_from_input_file(path)
    for f in ("p", "ux"):
        if f not in inp:
            continue
        want = np.atleast_2d(np.asarray(inp[f], dtype=np.float64))
        idx = cpp_io._fortran_index(inp["p_mask" if f == "p" else "u_mask"], shape)
        want = cpp_io._rows_to_c_order(want, idx, shape)
        got = np.asarray(prob[f], dtype=np.float64)
        assert got.shape == want.shape
        scale = np.max(np.abs(want))
        assert np.max(np.abs(got - want)) <= 1e-6 * scale, (f, float(np.max(np.abs(got - want))), scale)
        assert np.max(np.abs(np.asarray(raw[f], np.float64) - want)) > 1e-3 * scale


def test_legacy_route_refusals(tmp_path):
    inp, _, _ = _load("ivp_heterogeneous_medium")
    kgrid, medium, source, sensor = _objects(inp)
    with pytest.raises(ValueError, match="save_to_disk"):
        backend.kspaceFirstOrder2DC(kgrid, source, sensor, medium, NS(save_to_disk=False))
    medium.density = None
    with pytest.raises(ValueError, match="density"):
        backend.kspaceFirstOrder2DC(kgrid, source, sensor, medium,
                                    NS(save_to_disk=True, save_to_disk_exit=True, data_path=str(tmp_path)))
    with pytest.raises(ValueError, match="3-D"):
        backend.kspaceFirstOrder3DC(kgrid, source, sensor, medium, NS(save_to_disk=True))
    medium.density = np.ones(7)
    with pytest.raises(ValueError, match="density has 7 elements"):
        backend.kspaceFirstOrder2DC(kgrid, source, sensor, medium, NS(save_to_disk=True, data_path=str(tmp_path)))
    medium.density = 1000.0
    with pytest.raises(ValueError, match="too large"):
        backend.kspaceFirstOrder2DC(kgrid, source, sensor, medium,
                                    NS(save_to_disk=True, data_path=str(tmp_path), pml_size=64))


MAKETIME_CASES = ["ivp_homogeneous_medium", "ivp_heterogeneous_medium", "ivp_binary_sensor_mask", "ivp_3D_simulation",
                  "tvsp_homogeneous_medium_monopole", "tvsp_3D_simulation", "pr_2D_FFT_line_sensor",
                  "pr_3D_FFT_planar_sensor", "na_controlling_the_PML_1", "ivp_sensor_frequency_response_1"]


@pytest.mark.parametrize("name", MAKETIME_CASES)
def test_make_time_matches_kgrid(name):
    """cpp_io.make_time gives the Nt and dt the reference's kWaveGrid.makeTime
    gave for these grids and media (stored by the fixture script)."""
    inp, _, _ = _load(name)
    Nt, dt = cpp_io.make_time(tuple(inp["shape"]), tuple(inp["spacing"]), inp["sound_speed"])
    assert (Nt, dt) == (int(inp["Nt"]), float(inp["dt"]))


def test_legacy_route_makes_the_time_axis(tmp_path):
    """A grid without a time axis gets makeTime's, as the legacy route gives
    it (the reference's homogeneous-medium example passes such a grid): the
    file still matches MATLAB's, dt included."""
    inp, opts, expected = _load("ivp_homogeneous_medium")
    kgrid, medium, source, sensor = _objects(inp)
    kgrid.Nt = kgrid.dt = "auto"
    so = NS(save_to_disk=True, save_to_disk_exit=True, data_path=str(tmp_path), input_filename="auto.h5", **opts)
    backend.kspaceFirstOrder2DC(kgrid, source, sensor, medium, so)
    got = _summary(tmp_path / "auto.h5")
    assert got["dt"]["checksum8"] == expected["dt"]["checksum8"]
    assert int(np.asarray(h5io.read_file(tmp_path / "auto.h5")[0]["Nt"]).reshape(-1)[0]) == int(inp["Nt"])


def _direct_problem(name):
    """The problem the legacy route writes for a fixture, as the time loop
    takes it (source rows in C order of the mask's points)."""
    inp, opts, _ = _load(name)
    kgrid, medium, source, sensor = _objects(inp)
    prob = cpp_io.legacy_problem(kgrid, medium, source, sensor, pml_size=opts.get("pml_size", 20),
                                 pml_alpha=opts.get("pml_alpha", 2.0), pml_inside=opts.get("pml_inside", True))
    shape = tuple(prob["shape"])
    for f in ("p", "ux"):
        if prob.get(f) is not None:
            m = prob["p_mask" if f == "p" else "u_mask"]
            prob[f] = cpp_io._rows_to_c_order(np.atleast_2d(prob[f]), cpp_io._fortran_index(m, shape), shape)
    prob.update(record=("p",), record_start_index=1)
    return prob


@pytest.mark.parametrize("name", ["tvsp_homogeneous_medium_monopole", "tvsp_homogeneous_medium_dipole",
                                  "ivp_heterogeneous_medium"])
def test_legacy_file_is_the_same_simulation(name, tmp_path):
    from oracle.kspace_oracle import OracleSimulation

    path, _, _ = _write(name, tmp_path)
    from_file = cpp_io.problem_from_input_file(path, scaled_sources=True)
    direct = _direct_problem(name)
    a = OracleSimulation(from_file, np.float64).run()["p"]
    b = OracleSimulation(direct, np.float64).run()["p"]
    e = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    assert a.shape == b.shape and e <= 1e-5, e


@pytest.mark.parametrize("name", ["ivp_3D_simulation", "tvsp_doppler_effect", "ivp_heterogeneous_medium"])
def test_compressed_legacy_file(name, tmp_path):
    """``hdf_compression_level`` deflates the grids and many-row signals
    (kwave/utils/io.py:78-106); the values, and so the checksums, stay those
    of MATLAB's file, and the file shrinks."""
    inp, opts, expected = _load(name)
    kgrid, medium, source, sensor = _objects(inp)
    sizes = {}
    for level in (0, 6):
        so = NS(save_to_disk=True, save_to_disk_exit=True, data_path=str(tmp_path), input_filename=f"z{level}.h5",
                hdf_compression_level=level, **opts)
        (backend.kspaceFirstOrder2DC if kgrid.dim == 2 else backend.kspaceFirstOrder3DC)(kgrid, source, sensor,
                                                                                          medium, so)
        sizes[level] = (tmp_path / f"z{level}.h5").stat().st_size
    got = _summary(tmp_path / "z6.h5")
    for k, want in expected.items():
        if k != "root":
            assert got[k]["checksum8"] == want["checksum8"] and got[k]["shape"] == want["shape"], k
    assert sizes[6] < 0.5 * sizes[0], sizes
    with pytest.raises(ValueError, match="hdf_compression_level"):
        (backend.kspaceFirstOrder2DC if kgrid.dim == 2 else backend.kspaceFirstOrder3DC)(
            kgrid, source, sensor, medium, NS(save_to_disk=True, data_path=str(tmp_path), hdf_compression_level=12))


def test_record_flags_of_the_run(tmp_path):
    """The sensor's record list and start index reach the problem the file
    runs as (the binary's command-line flags); by default ``p`` alone, as the
    binary records; whole-grid aggregates are refused."""
    path, _, _ = _write("ivp_homogeneous_medium", tmp_path)
    assert cpp_io.problem_from_input_file(path)["record"] == ("p",)
    prob = cpp_io.problem_from_input_file(path, record=["p", "p_max", "u_final"], record_start_index=5)
    assert prob["record"] == ("p", "p_max", "u_final") and prob["record_start_index"] == 5
    assert cpp_io.problem_from_input_file(path, record="p_final")["record"] == ("p_final",)
    with pytest.raises(NotImplementedError, match="p_max_all"):
        cpp_io.problem_from_input_file(path, record=["p", "p_max_all"])
