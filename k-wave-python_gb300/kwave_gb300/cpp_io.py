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


def legacy_staggered(rho0, axis):
    """rho0 at the staggered points x_axis + d/2 as the legacy route
    interpolates it (kwave/kspaceFirstOrder2D.py:246-249 and the 3-D
    counterpart, linear ``interpolate2d``/``interpolate3d`` of
    kwave/utils/interp.py): the mean of each point and its neighbour along
    ``axis``; the last point's query lies outside the grid and keeps rho0
    (no wrap-around), in float64."""
    r = np.asarray(rho0, dtype=np.float64)
    out = r.copy()
    lo = [slice(None)] * r.ndim
    hi = list(lo)
    lo[axis], hi[axis] = slice(0, -1), slice(1, None)
    out[tuple(lo)] = 0.5 * (r[tuple(lo)] + r[tuple(hi)])
    return out


def _c0_at(c0, idx, rows):
    """Sound speed at the first ``rows`` points of a 1-based Fortran-order
    index list (one value for a homogeneous medium)."""
    c = np.asarray(c0, dtype=np.float64)
    if c.size == 1:
        return np.full(rows, float(c.reshape(-1)[0]))
    return c.ravel(order="F")[np.asarray(idx, dtype=np.int64).reshape(-1)[:rows] - 1]


def legacy_source_factors(prob, field):
    """Per-row factors by which the legacy route scales a source signal before
    storing it, in units the C++ binary adds to its split fields as they are
    (kwave/kWaveSimulation_helper/scale_source_terms_func.py:89-190 and
    :262-330, the MATLAB k-Wave convention of its input files):

    * pressure, additive modes: 2 dt / (N c0 dx), dirichlet: 1 / (N c0^2),
      with N the number of dimensions and dx the x spacing;
    * velocity component ``u_a``, additive modes: 2 c0 dt / d_a, dirichlet: 1.

    c0 is the sound speed at each row's source point (row i belongs to the
    i-th point of the Fortran-order index list) in a heterogeneous medium."""
    shape = tuple(int(n) for n in prob["shape"])
    ndim = len(shape)
    dt = float(prob["dt"])
    spacing = [float(d) for d in prob["spacing"]]
    rows = np.asarray(prob[field]).reshape(-1, np.asarray(prob[field]).shape[-1]).shape[0]
    if field == "p":
        c = _c0_at(prob["sound_speed"], _fortran_index(prob["p_mask"], shape), rows)
        if (prob.get("p_mode") or "additive") == "dirichlet":
            return 1.0 / (ndim * c ** 2)
        return 2.0 * dt / (ndim * c * spacing[0])
    if (prob.get("u_mode") or "additive") == "dirichlet":
        return np.ones(rows)
    c = _c0_at(prob["sound_speed"], _fortran_index(prob["u_mask"], shape), rows)
    return 2.0 * c * dt / spacing[("ux", "uy", "uz").index(field)]


def input_datasets(prob, legacy=False):
    """Datasets and their attributes of the input file for a problem dict
    whose grid already holds the PML and whose p0 is final (smoothed or not).
    The set, names, types and values of
    kwave/solvers/cpp_simulation.py:139-318; with ``legacy`` those of the
    legacy route (kspaceFirstOrder2DC/3DC with ``save_to_disk``,
    kwave/kWaveSimulation_helper/save_to_disk_func.py), which are the MATLAB
    k-Wave input files: density 1 when unset, staggered densities by
    :func:`legacy_staggered`, source signals scaled by
    :func:`legacy_source_factors` (rows in the order of the Fortran-order
    index list, as the caller gives them)."""
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
    if dens is None:
        dens = 1.0 if legacy else 1000.0
    rho0 = np.atleast_1d(np.asarray(dens, dtype=np.float32))
    c_ref = float(np.max(c0))
    if rho0.size == 1 or not prob.get("use_sg", True):
        rho0_sg = [rho0] * ndim
    elif legacy:
        rho0_sg = [legacy_staggered(np.asarray(dens, dtype=np.float64), axis) for axis in range(ndim)]
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
        if legacy:
            sig = np.asarray(ps, dtype=np.float64)
            sig = sig.reshape(-1, sig.shape[-1]) if sig.ndim != 2 else sig
            p_data = (sig * legacy_source_factors(prob, "p")[:, None]).astype(np.float32)
        else:
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
            if legacy:
                sig = np.asarray(vel[v], dtype=np.float64)
                sig = sig.reshape(-1, sig.shape[-1]) if sig.ndim != 2 else sig
                out[f"{v}_source_input"] = matrix((sig * legacy_source_factors(prob, v)[:, None]).astype(np.float32))
            else:
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


def _deflate_chunks(stored):
    """Chunk shape for a deflated matrix, or None for one stored as is:
    kwave/utils/io.py:78-106 compresses grids and many-row signals (two or
    more axes longer than 1) and vectors of more than 1 MB of doubles, the
    rest not.  The chunks split the first axis longer than 1 into at most
    64 pieces (one B-tree node of chunks)."""
    a = np.asarray(stored)
    long_axes = [i for i, n in enumerate(a.shape) if n > 1]
    if len(long_axes) < 2 and a.size <= (1024 ** 2) // 8:
        return None
    ch = list(a.shape)
    ax = long_axes[0]
    ch[ax] = -(-a.shape[ax] // 64)
    return tuple(ch)


def write_input_file(path, prob, description=None, legacy=False, compression_level=0):
    """Write the input file of a (PML-holding, final-p0) problem dict
    (``legacy``: the legacy route's values, see :func:`input_datasets`).
    ``compression_level`` 1-9 deflates the matrices that
    kwave/utils/io.py:52-188 compresses at ``hdf_compression_level``."""
    ds = input_datasets(prob, legacy=legacy)
    data = {k: v[0] for k, v in ds.items()}
    chunks, comp = {}, {}
    if compression_level:
        for k, a in data.items():
            ch = _deflate_chunks(a)
            if ch is not None:
                chunks[k], comp[k] = ch, int(compression_level)
    h5io.write_file(path, data, {k: v[1] for k, v in ds.items()}, file_attributes(description), chunks=chunks,
                    compression=comp)


def _time_unset(v):
    return v is None or isinstance(v, str) or (np.ndim(v) == 0 and np.isnan(float(v)))


def make_time(shape, spacing, c, cfl=0.3, t_end=None):
    """(Nt, dt) of kWaveGrid.makeTime (kwave/kgrid.py:455-495): dt = cfl x
    the smallest spacing / the largest sound speed; by default the time to
    cross the grid's diagonal at the smallest sound speed, Nt = floor(t_end /
    dt) + 1, one more when t_end / dt is not whole but MATLAB's rem(t_end,
    dt) is zero."""
    c = np.asarray(c, dtype=np.float64)
    size = np.asarray(shape, dtype=np.float64) * np.asarray(spacing, dtype=np.float64)
    if t_end is None:
        t_end = float(np.linalg.norm(size, ord=2)) / float(np.min(c))
    dt = cfl * float(np.min(spacing)) / float(np.max(c))
    q = t_end / dt
    Nt = int(np.floor(q) + 1)
    if np.floor(q) != np.ceil(q) and t_end - np.trunc(q) * dt == 0:
        Nt += 1
    return Nt, dt


def legacy_problem(kgrid, medium, source, sensor, *, pml_size=20, pml_alpha=2.0, pml_inside=True, smooth_p0=True,
                   use_sg=True):
    """The problem dict whose legacy input file the legacy route writes for
    these arguments (kwave/kspaceFirstOrder2D.py:142-384 with
    ``save_to_disk``): a homogeneous medium without a density gets density
    1 (kwave/kWaveSimulation.py:596-602; a heterogeneous one must set it),
    Cartesian sensor points are mapped to their nearest grid points, p0 is
    smoothed with its maximum restored before the grid is grown by the PML
    (kwave/kWaveSimulation.py:1209-1253), and with ``pml_inside=False`` the
    grid, medium, p0, masks and sensor grow by ``pml_size`` on every side
    (kwave/kWaveSimulation_helper/expand_grid_matrices.py).  Source rows stay
    in the caller's order, the Fortran order of the mask's points."""
    from types import SimpleNamespace

    from .conversion import cart2grid
    from .precompute import _get, grid_shape_of, problem_from_kwave
    from .unified import _is_cartesian, expand_problem, normalize_pml

    shape, spacing = grid_shape_of(kgrid)
    Nt, dt = _get(kgrid, "Nt"), _get(kgrid, "dt")
    if _time_unset(Nt) or _time_unset(dt):
        # kwave/kWaveSimulation.py:1038-1041: a grid without a time axis gets makeTime at the k-space CFL
        c = _get(medium, "sound_speed")
        if c is None:
            raise ValueError("medium.sound_speed must be defined")
        Nt, dt = make_time(shape, spacing, c)
    kgrid = SimpleNamespace(N=np.array(shape), spacing=np.array(spacing), Nt=int(Nt), dt=float(dt), dim=len(shape))
    prob = problem_from_kwave(kgrid, medium, source, sensor, smooth_p0=False, use_sg=use_sg)
    ndim = len(shape)
    if ndim not in (2, 3):
        raise NotImplementedError("the C++ input file holds 2-D and 3-D grids")
    pml_size = tuple(int(p) for p in normalize_pml(pml_size, ndim))
    pml_alpha = tuple(float(a) for a in normalize_pml(pml_alpha, ndim, "pml_alpha"))
    n = int(np.prod(shape))
    for k in ("sound_speed", "density", "alpha_coeff", "BonA", "p0", "p_mask", "u_mask"):
        v = prob.get(k)
        if v is not None and np.asarray(v).size not in (1, n):
            raise ValueError(f"{k} has {np.asarray(v).size} elements but the grid has {n} points")
    if pml_inside and any(2 * p >= N for p, N in zip(pml_size, shape)):
        raise ValueError(f"pml_size {pml_size} is too large for the grid {shape} with the PML inside")
    if prob.get("density") is None:
        if np.asarray(prob["sound_speed"]).size > 1:
            raise ValueError("medium.density must be defined for a heterogeneous medium")
        prob["density"] = 1.0
    m = prob.get("sensor_mask")
    if m is not None and _is_cartesian(m, ndim):
        kg = SimpleNamespace(N=np.array(shape), spacing=np.array(prob["spacing"]), dim=ndim)
        prob["sensor_mask"] = cart2grid(kg, np.asarray(m), order="C")[0]
    p0 = prob.get("p0")
    if smooth_p0 and p0 is not None and np.asarray(p0).size > 1:
        prob["p0"] = smooth_host(np.asarray(p0, dtype=np.float64).reshape(shape))
    if not pml_inside:
        prob = expand_problem(prob, pml_size)
    prob.update(pml_size=pml_size, pml_alpha=pml_alpha, smooth_p0=False)
    return prob


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


def problem_from_input_file(path, scaled_sources=False, record=None, record_start_index=None):
    """Problem dict of the native solver's time loop for an input file (PML
    inside the grid, p0 used as stored).  It records ``p``, as the C++ binary
    does by default, or the ``record`` list of a sensor, whose flags the
    binary takes on its command line
    (kwave/options/simulation_execution_options.py:276-305); the binary's
    whole-grid aggregates (``*_all``) are not recorded by the time loop and
    are refused.  ``record_start_index`` is the binary's ``-s``.
    ``scaled_sources``:
    the file's source signals carry the legacy route's scaling (files of
    MATLAB k-Wave and of kspaceFirstOrder2DC/3DC with ``save_to_disk``, see
    :func:`legacy_source_factors`), which is divided out again; files of
    ``kspaceFirstOrder(..., save_only=True)`` hold the signals unscaled.  The
    two kinds carry the same attributes, so the caller says which it is."""
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
    if scaled_sources:
        _unscale_sources(prob, ds)
    if record is not None:
        rec = (record,) if isinstance(record, str) else tuple(record)
        whole = [k for k in rec if k.endswith("_all")]
        if whole:
            raise NotImplementedError(f"{whole}: whole-grid aggregates of the C++ binary are not recorded by the "
                                      "time loop")
        prob["record"] = rec
    if record_start_index is not None:
        prob["record_start_index"] = int(record_start_index)
    return prob


def _unscale_sources(prob, ds):
    """Divide the legacy scaling out of the source rows of a problem read
    from a file (rows already in C order: the factors are taken in the
    file's Fortran order and permuted the same way)."""
    shape = tuple(prob["shape"])
    for field, idx_name in (("p", "p_source_index"), ("ux", "u_source_index"), ("uy", "u_source_index"),
                            ("uz", "u_source_index")):
        if field not in prob:
            continue
        mask_key = "p_mask" if field == "p" else "u_mask"
        fprob = dict(prob, p=None, ux=None, uy=None, uz=None)
        fprob[field] = unmatrix(ds[f"{field}_source_input"], 2)
        fprob[mask_key] = prob[mask_key]
        f = legacy_source_factors(fprob, field)
        rows = np.asarray(prob[field], dtype=np.float64)
        if rows.shape[0] > 1:
            f = _rows_to_c_order(f[:, None], ds[idx_name], shape)[:, 0]
        prob[field] = (rows / f[:, None]).astype(np.float32)


def run_input_file(path, stream=None, scaled_sources=False, record=None, record_start_index=None):
    """Run an input file of the C++ binary on the GB300 time loop; returns
    the result dict of the native solver (``p`` as (n_sensor, Nt) with the
    sensor points in C order).  ``scaled_sources``, ``record`` and
    ``record_start_index`` as for :func:`problem_from_input_file`."""
    from .solver import Simulation

    prob = problem_from_input_file(path, scaled_sources=scaled_sources, record=record,
                                   record_start_index=record_start_index)
    sim = Simulation.from_problem(prob, stream=stream)
    try:
        return sim.run()
    finally:
        sim.close()
