"""HDF5 input files of the k-Wave C++ binary: written from a problem
(``kspaceFirstOrder(..., save_only=True, data_path=...)``) and run on the
GB300 time loop (:func:`run_input_file`).

The input file holds what kwave/solvers/cpp_simulation.py:139-318
(``CppSimulation._write_hdf5``) writes: grid, time step, PML sizes and
alphas, flags, medium scalars or grids, the staggered densities, sources with
their 1-based Fortran-order index lists, the sensor's index list and the file
attributes of kwave/utils/io.py:191-243.  Each matrix has the layout of
kwave/utils/io.py:52-188 (``write_matrix``): a 3-D array is stored
transposed (Fortran order) with dimensions (Nz, Ny, Nx) of the C array, a
2-D array as (1, Ny, Nx), a scalar as (1, 1, 1); float32 carries the
attributes ``data_type = float``, uint64 ``data_type = long``, both
``domain_type = real``.  The file container is :mod:`kwave_gb300.h5io`.

Running an input file maps it back onto the problem dict of the native
solver's time loop (C-order grids and masks, source rows in C order of the
mask's points): the same p0, medium, sources and sensor points, recording
``p`` as the C++ binary does by default.  Two things differ from the C++
binary and follow the native solver instead: the staggered densities are
derived from ``rho0`` as the native solver derives them (the file's
``rho0_sg*`` are not read), and the time loop is the native solver's.
"""
from __future__ import annotations

import os
import platform
from datetime import datetime

import numpy as np

from . import h5io
from .precompute import blackman_rotated

SOURCE_MODES = {"dirichlet": 0, "additive-no-correction": 1, "additive": 2}
MODE_NAMES = {v: k for k, v in SOURCE_MODES.items()}
FILE_MAJOR_VERSION, FILE_MINOR_VERSION = "1", "2"


def matrix(a):
    """(stored array, attributes) of one matrix in the layout of
    kwave/utils/io.py:52-188 (real float32 or uint64 only)."""
    a = np.asarray(a)
    if np.iscomplexobj(a):
        raise NotImplementedError("complex matrices are not written")
    if a.dtype == np.float32:
        dtype_c = "float"
    elif a.dtype == np.uint64:
        dtype_c = "long"
    else:
        raise ValueError("Input matrix must be of type single or uint64.")
    if a.ndim == 3:
        m = a.transpose(2, 1, 0)
        shape = m.shape
    elif a.ndim == 2:
        m = a.T
        shape = (1,) + m.shape
    elif a.size == 1:
        m, shape = a, (1, 1, 1)
    else:
        raise ValueError(f"a {a.ndim}-D matrix of {a.size} values has no layout in the k-Wave HDF5 format "
                         "(pass source signals as 2-D arrays)")
    return np.ascontiguousarray(m).reshape(shape), {"domain_type": "real", "data_type": dtype_c}


def unmatrix(stored, ndim):
    """Inverse of :func:`matrix` for a grid of ``ndim`` dimensions, a
    (rows, columns) array or a scalar."""
    s = np.asarray(stored)
    if s.size == 1:
        return s.reshape(())
    if ndim == 3:
        return s.transpose(2, 1, 0)
    return s.reshape(s.shape[-2:]).T


def smooth_host(p0):
    """p0 smoothed with the rotated Blackman window and its maximum restored,
    in float64 (kwave/utils/filters.py:549-615 as the unified entry point
    calls it, kwave/kspaceFirstOrder.py:241-245)."""
    a = np.asarray(p0, dtype=np.float64)
    win = blackman_rotated(a.shape)
    a_sm = np.real(np.fft.ifftn(np.fft.fftn(a) * np.fft.ifftshift(win)))
    return (np.abs(a).max() / np.abs(a_sm).max()) * a_sm


def _fortran_index(mask, shape):
    """1-based Fortran-order indices of a mask's points (uint64, (n, 1))."""
    m = np.asarray(mask).astype(bool).reshape(shape)
    return (np.where(m.flatten(order="F") != 0)[0] + 1).astype(np.uint64).reshape(-1, 1)


def _num_dim2(x):
    sz = np.squeeze(np.asarray(x)).shape
    return len(sz) if len(sz) > 2 else int(np.sum(np.array(sz) > 1))


def _absorbing_flag(prob):
    ac = prob.get("alpha_coeff")
    if ac is None or np.all(np.asarray(ac) == 0):
        return 0
    ap = prob.get("alpha_power")
    if ap is not None and abs(float(np.asarray(ap).flat[0]) - 2.0) < 1e-10:
        return 2
    return 1


def file_attributes(description=None):
    """Root attributes of an input file (kwave/utils/io.py:191-243)."""
    try:
        import kwave

        version = f"k-Wave {kwave.__version__}"
    except Exception:
        version = "k-Wave kwave-gb300"
    if description is None:
        user = os.environ.get("USERNAME")
        description = f"Input data created by {user} running MATLAB N/A on {platform.system()}"
    return {"major_version": FILE_MAJOR_VERSION, "minor_version": FILE_MINOR_VERSION, "created_by": version,
            "file_description": description, "file_type": "input",
            "creation_date": datetime.now().strftime("%d-%b-%Y-%H-%M-%S")}


def input_datasets(prob):
    """Datasets and their attributes of the input file for a problem dict
    whose grid already holds the PML and whose p0 is final (smoothed or not).
    The set, names, types and values of
    kwave/solvers/cpp_simulation.py:139-318."""
    shape = tuple(int(n) for n in prob["shape"])
    ndim = len(shape)
    spacing = [float(d) for d in prob["spacing"]]
    Nx = shape[0]
    Ny = shape[1] if ndim >= 2 else 1
    Nz = shape[2] if ndim >= 3 else 1
    pml_size = [int(p) for p in prob["pml_size"]]
    pml_alpha = [float(a) for a in prob["pml_alpha"]]

    c0 = np.atleast_1d(np.asarray(prob["sound_speed"], dtype=np.float32))
    dens = prob.get("density")
    rho0 = np.atleast_1d(np.asarray(dens if dens is not None else 1000.0, dtype=np.float32))
    c_ref = float(np.max(c0))
    if rho0.size == 1 or not prob.get("use_sg", True):
        rho0_sg = [rho0] * ndim
    else:
        rho0_sg = [0.5 * (rho0 + np.roll(rho0, -1, axis=axis)) for axis in range(ndim)]

    p0 = prob.get("p0")
    has_p0 = p0 is not None and bool(np.any(np.asarray(p0) != 0))
    ps = prob.get("p")
    has_p = ps is not None and bool(np.any(np.asarray(ps) != 0))
    vel = {v: prob.get(v) for v in ("ux", "uy", "uz")[:ndim]}
    has_u = {v: s is not None for v, s in vel.items()}

    mask = prob.get("sensor_mask")
    if mask is None:
        sensor_index = np.arange(1, int(np.prod(shape)) + 1, dtype=np.uint64)
    else:
        m = np.asarray(mask)
        if m.ndim == 2 and m.shape[0] == ndim and m.shape != shape:
            raise ValueError("Cartesian sensor masks are not supported by the cpp backend. "
                             "Use a binary (grid-shaped) mask or switch to backend='python'.")
        sensor_index = _fortran_index(m, shape)

    BonA = prob.get("BonA")
    nonlinear = BonA is not None and bool(np.any(np.asarray(BonA) != 0))
    ints = {"Nx": Nx, "Ny": Ny, "Nz": Nz, "Nt": int(prob["Nt"]),
            "pml_x_size": pml_size[0], "pml_y_size": pml_size[1] if ndim >= 2 else 0,
            "pml_z_size": pml_size[2] if ndim >= 3 else 0,
            # the C++ binary takes the number of time points of a source signal here
            "p_source_flag": np.asarray(ps).shape[-1] if has_p else 0,
            "p0_source_flag": int(has_p0),
            "ux_source_flag": np.asarray(vel["ux"]).shape[-1] if has_u.get("ux") else 0,
            "uy_source_flag": np.asarray(vel["uy"]).shape[-1] if has_u.get("uy") else 0,
            "uz_source_flag": np.asarray(vel["uz"]).shape[-1] if has_u.get("uz") else 0,
            "sxx_source_flag": 0, "syy_source_flag": 0, "szz_source_flag": 0, "sxy_source_flag": 0,
            "sxz_source_flag": 0, "syz_source_flag": 0, "transducer_source_flag": 0, "nonuniform_grid_flag": 0,
            "nonlinear_flag": int(nonlinear), "absorbing_flag": _absorbing_flag(prob), "elastic_flag": 0,
            "axisymmetric_flag": 0, "sensor_mask_type": 0}
    out = {}
    for k, v in ints.items():
        out[k] = matrix(np.array(v, dtype=np.uint64))
    out["sensor_mask_index"] = matrix(np.asarray(sensor_index, dtype=np.uint64).reshape(-1, 1))

    floats = {"dx": spacing[0], "dt": float(prob["dt"]), "c0": c0, "c_ref": c_ref, "rho0": rho0}
    if ndim >= 2:
        floats["dy"] = spacing[1]
        floats["pml_y_alpha"] = pml_alpha[1]
    if ndim >= 3:
        floats["dz"] = spacing[2]
        floats["pml_z_alpha"] = pml_alpha[2]
    floats["pml_x_alpha"] = pml_alpha[0]
    for i, name in enumerate(("rho0_sgx", "rho0_sgy", "rho0_sgz")[:ndim]):
        floats[name] = rho0_sg[i]
    if nonlinear:
        floats["BonA"] = np.asarray(BonA, dtype=np.float32)
    if prob.get("alpha_coeff") is not None:
        floats["alpha_coeff"] = np.asarray(prob["alpha_coeff"], dtype=np.float32)
    if prob.get("alpha_power") is not None:
        floats["alpha_power"] = np.float32(np.asarray(prob["alpha_power"]).flat[0])
    for k, v in floats.items():
        out[k] = matrix(np.atleast_1d(np.asarray(v, dtype=np.float32)))

    if has_p0:
        out["p0_source_input"] = matrix(np.asarray(p0, dtype=np.float32).reshape(shape))
    if has_p:
        p_data = np.asarray(ps, dtype=np.float32)
        out["p_source_input"] = matrix(p_data)
        pm = np.asarray(prob["p_mask"])
        if pm.ndim == 2 and pm.shape[0] == ndim and pm.shape != shape:
            raise ValueError("Cartesian source masks (p_mask) are not supported by the cpp backend. "
                             "Use a binary (grid-shaped) mask or switch to backend='python'.")
        out["p_source_index"] = matrix(_fortran_index(pm, shape))
        out["p_source_mode"] = matrix(np.array(SOURCE_MODES.get(prob.get("p_mode") or "additive", 2),
                                               dtype=np.uint64))
        out["p_source_many"] = matrix(np.array(int(_num_dim2(p_data) > 1), dtype=np.uint64))
    for v, on in has_u.items():
        if on:
            out[f"{v}_source_input"] = matrix(np.asarray(vel[v], dtype=np.float32))
    if any(has_u.values()):
        um = np.asarray(prob["u_mask"])
        if um.ndim == 2 and um.shape[0] == ndim and um.shape != shape:
            raise ValueError("Cartesian source masks (u_mask) are not supported by the cpp backend. "
                             "Use a binary (grid-shaped) mask or switch to backend='python'.")
        out["u_source_index"] = matrix(_fortran_index(um, shape))
        out["u_source_mode"] = matrix(np.array(SOURCE_MODES.get(prob.get("u_mode") or "additive", 2),
                                               dtype=np.uint64))
        first = next(vel[v] for v in ("ux", "uy", "uz")[:ndim] if has_u.get(v))
        out["u_source_many"] = matrix(np.array(int(_num_dim2(first) > 1), dtype=np.uint64))
    return out


def write_input_file(path, prob, description=None):
    """Write the input file of a (PML-holding, final-p0) problem dict."""
    ds = input_datasets(prob)
    h5io.write_file(path, {k: v[0] for k, v in ds.items()}, {k: v[1] for k, v in ds.items()},
                    file_attributes(description))


def save_input_files(prob, data_path):
    """``save_only``: write ``kwave_input.h5`` into data_path (created if
    needed; an existing input file is not overwritten) and return the input
    and output file names, as kwave/solvers/cpp_simulation.py:47-61."""
    os.makedirs(data_path, exist_ok=True)
    input_file = os.path.join(data_path, "kwave_input.h5")
    output_file = os.path.join(data_path, "kwave_output.h5")
    if os.path.exists(input_file):
        raise FileExistsError(f"{input_file!r} already exists. Delete it or choose a different data_path to avoid "
                              "overwriting previous simulation inputs.")
    write_input_file(input_file, prob)
    return input_file, output_file


# ---------------------------------------------------------------------------
# running an input file
# ---------------------------------------------------------------------------

def _scalar(ds, name, cast=float):
    return cast(np.asarray(ds[name]).reshape(-1)[0])


def _grid_or_scalar(ds, name, ndim):
    a = unmatrix(ds[name], ndim)
    return float(a) if a.ndim == 0 else np.ascontiguousarray(a, dtype=np.float32)


def _mask_from_index(idx, shape):
    m = np.zeros(int(np.prod(shape)), dtype=bool)
    m[np.asarray(idx, dtype=np.int64).reshape(-1) - 1] = True
    return m.reshape(shape, order="F")


def _rows_to_c_order(rows, idx, shape):
    """Source rows ordered by the Fortran-order index list -> rows in C
    order of the same points (the native solver's order)."""
    rows = np.asarray(rows)
    if rows.shape[0] == 1:
        return rows
    f = np.asarray(idx, dtype=np.int64).reshape(-1) - 1
    c = np.ravel_multi_index(np.unravel_index(f, shape, order="F"), shape)
    return rows[np.argsort(c, kind="stable")]


def problem_from_input_file(path):
    """Problem dict of the native solver's time loop for an input file (PML
    inside the grid, p0 used as stored, ``p`` recorded)."""
    ds, _, root = h5io.read_file(path)
    if root.get("file_type", "input") != "input":
        raise ValueError(f"{path}: file_type {root.get('file_type')!r}, expected 'input'")
    for flag in ("elastic_flag", "axisymmetric_flag", "transducer_source_flag", "nonuniform_grid_flag"):
        if flag in ds and _scalar(ds, flag, int):
            raise NotImplementedError(f"{flag} set: not part of the first-order fluid time loop")
    for s in ("sxx", "syy", "szz", "sxy", "sxz", "syz"):
        if f"{s}_source_flag" in ds and _scalar(ds, f"{s}_source_flag", int):
            raise NotImplementedError("stress sources belong to the elastic code")
    if "sensor_mask_type" in ds and _scalar(ds, "sensor_mask_type", int) != 0:
        raise NotImplementedError("cuboid-corner sensor masks")
    Nx, Ny, Nz = (_scalar(ds, k, int) for k in ("Nx", "Ny", "Nz"))
    ndim = 3 if Nz > 1 else 2
    shape = (Nx, Ny, Nz)[:ndim]
    spacing = tuple(_scalar(ds, k) for k in ("dx", "dy", "dz")[:ndim])
    prob = dict(shape=shape, spacing=spacing, Nt=_scalar(ds, "Nt", int), dt=_scalar(ds, "dt"),
                pml_size=tuple(_scalar(ds, f"pml_{a}_size", int) for a in "xyz"[:ndim]),
                pml_alpha=tuple(_scalar(ds, f"pml_{a}_alpha") for a in "xyz"[:ndim]),
                use_sg=True, use_kspace=True, smooth_p0=False, record=("p",), record_start_index=1)
    prob["sound_speed"] = _grid_or_scalar(ds, "c0", ndim)
    prob["density"] = _grid_or_scalar(ds, "rho0", ndim)
    if "c_ref" in ds:
        prob["c_ref"] = _scalar(ds, "c_ref")
    absorbing = _scalar(ds, "absorbing_flag", int) if "absorbing_flag" in ds else 0
    if absorbing:
        prob["alpha_coeff"] = _grid_or_scalar(ds, "alpha_coeff", ndim)
        prob["alpha_power"] = _scalar(ds, "alpha_power")
    if "nonlinear_flag" in ds and _scalar(ds, "nonlinear_flag", int):
        prob["BonA"] = _grid_or_scalar(ds, "BonA", ndim)
    if "p0_source_flag" in ds and _scalar(ds, "p0_source_flag", int):
        prob["p0"] = np.ascontiguousarray(unmatrix(ds["p0_source_input"], ndim), dtype=np.float32)
    if "p_source_flag" in ds and _scalar(ds, "p_source_flag", int):
        idx = ds["p_source_index"]
        prob["p_mask"] = _mask_from_index(idx, shape)
        prob["p"] = _rows_to_c_order(unmatrix(ds["p_source_input"], 2), idx, shape)
        prob["p_mode"] = MODE_NAMES[_scalar(ds, "p_source_mode", int)] if "p_source_mode" in ds else "additive"
    vel = [v for v in ("ux", "uy", "uz")[:ndim] if f"{v}_source_flag" in ds and _scalar(ds, f"{v}_source_flag", int)]
    if vel:
        idx = ds["u_source_index"]
        prob["u_mask"] = _mask_from_index(idx, shape)
        for v in vel:
            prob[v] = _rows_to_c_order(unmatrix(ds[f"{v}_source_input"], 2), idx, shape)
        prob["u_mode"] = MODE_NAMES[_scalar(ds, "u_source_mode", int)] if "u_source_mode" in ds else "additive"
    prob["sensor_mask"] = _mask_from_index(ds["sensor_mask_index"], shape)
    return prob


def run_input_file(path, stream=None):
    """Run an input file of the C++ binary on the GB300 time loop; returns
    the result dict of the native solver (``p`` as (n_sensor, Nt) with the
    sensor points in C order)."""
    from .solver import Simulation

    sim = Simulation.from_problem(problem_from_input_file(path), stream=stream)
    try:
        return sim.run()
    finally:
        sim.close()
