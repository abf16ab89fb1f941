"""``kspaceFirstOrder(..., backend="gb300")``: the unified entry point.

Mirrors kwave/kspaceFirstOrder.py:119-325 (argument names, defaults where the
reference has no GPU-specific meaning, validation messages, PML expansion,
p0 smoothing after expansion and the stripping of full-grid outputs) and
sends the time loop to the GB300 device plan.

The pre-processing works on the plain problem dict that
:func:`kwave_gb300.precompute.problem_from_kwave` collects, so it needs
neither ``kwave`` nor its grid classes:

* ``pml_inside=False`` grows the grid by ``2 * pml_size`` per axis; grid-
  shaped medium maps are edge-extended, p0 and the binary source/sensor
  masks zero-padded, Cartesian sensor points kept (they are physical
  coordinates on a grid that stays centred) — kspaceFirstOrder.py:42-65;
* p0 smoothing (restore-max Blackman window) then runs on the device over
  the expanded grid, which is the reference's order (kspaceFirstOrder.py
  :234-238: smooth after expansion);
* full-grid outputs ending in ``_max``/``_min``/``_rms`` (and the ``_all``
  forms) are cropped back (kspaceFirstOrder.py:68-77, :318-322); ``*_final``
  fields come back cropped from the solver already.

Differences, all stated where they apply: the computation is float32 (a
float64 ``dtype`` only draws a warning, as ``backend="cpp"`` does in the
reference, :262-268); ``device`` must be ``"gpu"``; ``binary_path`` is
refused.  ``save_only=True`` writes the HDF5 input file of the C++ binary
into ``data_path``, as ``backend="cpp"`` does (:mod:`kwave_gb300.cpp_io`),
instead of running.
"""
from __future__ import annotations

import warnings
from types import SimpleNamespace

import numpy as np

from .precompute import grid_of, problem_from_kwave

BACKEND = "gb300"

_FULL_GRID_SUFFIXES = ("_max", "_min", "_rms", "_max_all", "_min_all", "_rms_all")
_MEDIUM_EDGE = ("sound_speed", "density", "alpha_coeff", "BonA")
_SOURCE_ZERO = ("p0", "p_mask", "u_mask")


# ---------------------------------------------------------------------------
# argument handling (kwave/kspaceFirstOrder.py:16-28, :80-112)
# ---------------------------------------------------------------------------

def normalize_pml(val, ndim, name="pml_size"):
    """Scalar -> per-axis tuple; a shorter sequence repeats its last entry
    (kspaceFirstOrder.py:16-24)."""
    if isinstance(val, str):
        valid = "an integer, tuple of integers, or 'auto'" if name == "pml_size" else "a float or tuple of floats"
        raise ValueError(f"{name} must be {valid}, got {val!r}")
    if isinstance(val, (int, float, np.integer, np.floating)):
        return (val,) * ndim
    t = tuple(val)
    if len(t) == 0 or len(t) > ndim:
        raise ValueError(f"{name} must be a scalar or 1-to-{ndim}-element sequence, got {len(t)} elements")
    return t + (t[-1],) * (ndim - len(t))


def resolve_dtype(value):
    """dtype-like -> np.float32 / np.float64 (kspaceFirstOrder.py:80-112);
    ``None`` and ``"off"`` mean float64 as in the reference."""
    if value is None or (isinstance(value, str) and value == "off"):
        return np.float64
    try:
        resolved = np.dtype(value).type
    except TypeError as e:
        framework = getattr(type(value), "__module__", "").split(".")[0]
        hint = ""
        if framework in ("torch", "jax", "jaxlib", "tensorflow"):
            hint = f" {framework}.dtype objects aren't supported; pass the equivalent numpy dtype (np.float32 / np.float64)."
        raise ValueError(
            f"dtype must be a numpy dtype, type, or string (e.g. 'float32', 'single'), got {value!r}.{hint}") from e
    if resolved is np.float32:
        return np.float32
    if resolved is np.float64:
        return np.float64
    raise ValueError(f"dtype must resolve to float32 or float64; got {resolved.__name__} from {value!r}")


def largest_prime_factor(n: int) -> int:
    n = int(n)
    best, p = 1, 2
    while p * p <= n:
        while n % p == 0:
            best, n = p, n // p
        p += 1
    return max(best, n) if n > 1 else best


def get_optimal_pml_size(grid_size, pml_range=None):
    """Per axis, the PML size in ``pml_range`` (default 10..40) whose expanded
    length N + 2 * pml has the smallest largest prime factor; ties go to the
    smallest size (kwave/utils/pml.py:76-159, non-axisymmetric form)."""
    shape = grid_of(grid_size)[0] if not isinstance(grid_size, (tuple, list, np.ndarray)) else tuple(
        int(n) for n in grid_size)
    if not 1 <= len(shape) <= 3:
        raise ValueError("Grid dimensions must be given as a 1, 2, or 3 element vector.")
    lo, hi = (10, 40) if pml_range is None else (int(round(pml_range[0])), int(round(pml_range[1])))
    if lo < 0 or hi < 0:
        raise ValueError("Optional input pml_range must be positive.")
    if hi <= lo:
        raise ValueError("The second value for pml_range must be greater than the first.")
    sizes = np.arange(lo, hi + 1)
    out = []
    for n in shape:
        facs = [largest_prime_factor(n + 2 * int(s)) for s in sizes]
        out.append(int(sizes[int(np.argmin(facs))]))
    return np.array(out, dtype=int)


# ---------------------------------------------------------------------------
# validation (kwave/solvers/validation.py:6-127), on the problem dict
# ---------------------------------------------------------------------------

def _is_cartesian(mask, ndim):
    a = np.asarray(mask)
    return a.ndim == 2 and a.shape[0] == ndim


def validate_problem(prob, pml_size):
    shape = tuple(prob["shape"])
    ndim, n = len(shape), int(np.prod(shape))
    Nt, dt = prob["Nt"], prob["dt"]
    if isinstance(Nt, str) or isinstance(dt, str):
        raise ValueError("kgrid.Nt and kgrid.dt must be set before calling kspaceFirstOrder. "
                         "Call kgrid.makeTime(medium.sound_speed) or kgrid.setTime(Nt, dt) first.")
    if int(Nt) < 1:
        raise ValueError(f"kgrid.Nt must be >= 1, got {Nt}")
    if float(dt) <= 0:
        raise ValueError(f"kgrid.dt must be > 0, got {dt}")
    # medium
    c = np.atleast_1d(np.asarray(prob.get("sound_speed")))
    if c.size > 1 and c.size != n:
        raise ValueError(f"medium.sound_speed has {c.size} elements but grid has {n} points.")
    if np.any(c <= 0):
        raise ValueError("medium.sound_speed must be positive everywhere.")
    if prob.get("density") is not None:
        rho = np.atleast_1d(np.asarray(prob["density"]))
        if rho.size > 1 and rho.size != n:
            raise ValueError(f"medium.density has {rho.size} elements but grid has {n} points.")
        if np.any(rho <= 0):
            raise ValueError("medium.density must be positive everywhere.")
    if prob.get("alpha_coeff") is not None:
        if np.any(np.atleast_1d(np.asarray(prob["alpha_coeff"])) < 0):
            raise ValueError("medium.alpha_coeff must be non-negative.")
        if prob.get("alpha_power") is not None:
            power = float(np.asarray(prob["alpha_power"]).flat[0])
            if power < 0 or power > 3:
                warnings.warn(f"medium.alpha_power={power} is outside typical range [0, 3].", stacklevel=4)
    # PML
    for i in range(ndim):
        N, pml = int(shape[i]), int(pml_size[i])
        if pml < 0:
            raise ValueError(f"pml_size[{i}] must be non-negative, got {pml}")
        if 2 * pml >= N:
            raise ValueError(f"pml_size[{i}]={pml} is too large for grid size N[{i}]={N} (2*pml must be < N).")
    # CFL (Tabei et al., JASA 2002, eq. 11)
    cfl = float(np.max(c)) * float(dt) / float(np.min(prob["spacing"]))
    limit = 2 / (np.pi * np.sqrt(ndim))
    if cfl > limit:
        warnings.warn(f"CFL number = {cfl:.3f} exceeds pseudospectral stability limit "
                      f"{limit:.3f} for {ndim}D. Reduce dt or increase grid spacing.", stacklevel=4)
    # source
    if prob.get("p0") is not None:
        p0 = np.asarray(prob["p0"])
        if p0.size != n and p0.size != 0:
            raise ValueError(f"source.p0 has {p0.size} elements but grid has {n} points.")
    if prob.get("p") is not None and prob.get("p_mask") is None:
        raise ValueError("source.p requires source.p_mask to be set.")
    for key in ("p_mask", "u_mask"):
        if prob.get(key) is not None:
            m = np.asarray(prob[key])
            if not _is_cartesian(m, ndim) and m.size != n:
                raise ValueError(f"source.{key} has {m.size} elements but grid has {n} points.")
    vel = [v for v in ("ux", "uy", "uz") if prob.get(v) is not None]
    for v in vel:
        if prob.get("u_mask") is None:
            raise ValueError(f"source.{v} requires source.u_mask to be set.")
    many = {np.squeeze(np.asarray(prob[v])).ndim > 1 for v in vel}
    if len(many) > 1:
        raise ValueError("All velocity source components must either be single (1D) or many (2D) time series.")
    # sensor
    if prob.get("sensor_mask") is not None:
        m = np.asarray(prob["sensor_mask"])
        if not _is_cartesian(m, ndim) and m.size != 1 and m.size != n:
            raise ValueError(f"sensor.mask has {m.size} elements but grid has {n} points.")


# ---------------------------------------------------------------------------
# PML outside the user domain (kspaceFirstOrder.py:33-77)
# ---------------------------------------------------------------------------

def _pad(val, shape, pml_size, zero):
    arr = np.asarray(val)
    if arr.size <= 1:  # homogeneous values broadcast: left as they are
        return val
    if arr.size == int(np.prod(shape)):
        arr = arr.reshape(shape)
    widths = [(int(p), int(p)) for p in pml_size]
    if zero:
        return np.pad(arr, widths, mode="constant", constant_values=0)
    return np.pad(arr, widths, mode="edge")


def expand_problem(prob, pml_size):
    """Problem on the grid grown by ``2 * pml_size`` (PML outside the domain)."""
    shape = tuple(int(n) for n in prob["shape"])
    out = dict(prob)
    out["shape"] = tuple(n + 2 * int(p) for n, p in zip(shape, pml_size))
    for k in _MEDIUM_EDGE:
        if out.get(k) is not None:
            out[k] = _pad(out[k], shape, pml_size, zero=False)
    for k in _SOURCE_ZERO:
        if out.get(k) is not None:
            out[k] = _pad(out[k], shape, pml_size, zero=True)
    m = out.get("sensor_mask")
    if m is not None and not _is_cartesian(m, len(shape)):
        out["sensor_mask"] = _pad(m, shape, pml_size, zero=True)
    return out


def strip_pml(result, pml_size, ndim, suffixes=_FULL_GRID_SUFFIXES):
    """Crop the PML from full-grid outputs whose key ends in one of
    ``suffixes`` and whose rank equals the grid's (kspaceFirstOrder.py:68-77)."""
    sl = tuple(slice(int(p), -int(p) if int(p) else None) for p in pml_size[:ndim])
    return {k: (v[sl] if isinstance(v, np.ndarray) and v.ndim == ndim and any(k.endswith(s) for s in suffixes) else v)
            for k, v in result.items()}


def reshape_to_grid(data, grid_shape):
    """(n_sensor, Nt) -> (*grid_shape, Nt); (n_sensor,) -> grid_shape
    (kspaceFirstOrder.py:328-349)."""
    data = np.asarray(data)
    if data.ndim == 2:
        return data.reshape(*grid_shape, data.shape[1])
    if data.ndim == 1:
        return data.reshape(grid_shape)
    return data


# ---------------------------------------------------------------------------
# entry point
# ---------------------------------------------------------------------------

def prepare_problem(kgrid, medium, source, sensor, *, pml_size=20, pml_alpha=2.0, pml_inside=False, use_sg=True,
                    use_kspace=True, smooth_p0=True):
    """The problem dict the time loop runs for these arguments, and the
    per-axis PML size: ``"auto"`` sizing, normalisation, validation and
    (``pml_inside=False``) expansion, as kspaceFirstOrder.py:220-238 does
    before dispatch."""
    shape = grid_of(kgrid)[0]
    ndim = len(shape)
    if isinstance(pml_size, str) and pml_size.lower() == "auto":
        pml_size = tuple(int(x) for x in get_optimal_pml_size(shape))
    pml_size = tuple(int(p) for p in normalize_pml(pml_size, ndim))
    pml_alpha = tuple(float(a) for a in normalize_pml(pml_alpha, ndim, "pml_alpha"))

    prob = problem_from_kwave(kgrid, medium, source, sensor, pml_size=pml_size, pml_alpha=pml_alpha,
                              use_sg=use_sg, use_kspace=use_kspace, smooth_p0=smooth_p0)
    validate_problem(prob, pml_size)
    if not pml_inside:
        prob = expand_problem(prob, pml_size)
    return prob, pml_size


def kspaceFirstOrder(kgrid, medium, source, sensor=None, *, pml_size=20, pml_alpha=2.0, pml_inside=False,
                     use_sg=True, use_kspace=True, smooth_p0=True, backend=BACKEND, device="gpu", dtype=None,
                     save_only=False, data_path=None, quiet=False, debug=False, num_threads=None, device_num=None,
                     binary_path=None, stream=None) -> dict:
    """Run a k-Wave simulation on the GB300 time loop.

    Same arguments and result dict as kwave/kspaceFirstOrder.py:119-325 for
    ``backend="gb300"``: 2-D and 3-D grids; time series are
    ``(n_sensor, Nt)`` with sensor points in C order, aggregates
    ``(n_sensor,)``, ``*_final`` fields on the user's grid.  ``stream`` is an
    optional CUDA stream handle (int) for the device plan.  ``save_only=True``
    writes ``data_path/kwave_input.h5`` (the C++ binary's input file) and
    returns ``{"input_file", "output_file"[, "pml_size"]}`` without running.
    """
    if backend != BACKEND:
        raise ValueError(f"Unknown backend: {backend!r}. This entry point runs backend={BACKEND!r}; "
                         "use kwave.kspaceFirstOrder.kspaceFirstOrder for 'python' or 'cpp'.")
    if device != "gpu":
        raise ValueError(f"device must be 'gpu' for backend={BACKEND!r}, got {device!r}")
    if binary_path is not None:
        raise NotImplementedError("external binaries belong to backend='cpp'")
    if device_num not in (None, 0):
        raise NotImplementedError("backend='gb300' runs on the current CUDA device; select it with "
                                  "CUDA_VISIBLE_DEVICES")
    explicit = dtype is not None
    if resolve_dtype(dtype) is not np.float32 and explicit:
        warnings.warn(f"dtype={np.dtype(dtype).name!r} has no effect with backend='gb300'; the time loop "
                      "computes in float32.", stacklevel=2)
    if any(isinstance(getattr(kgrid, a, None), str) for a in ("Nt", "dt")):
        raise ValueError("kgrid.Nt and kgrid.dt must be set before calling kspaceFirstOrder. "
                         "Call kgrid.makeTime(medium.sound_speed) or kgrid.setTime(Nt, dt) first.")
    shape = grid_of(kgrid)[0]
    ndim = len(shape)
    if ndim not in (2, 3):
        raise NotImplementedError("backend='gb300' runs 2-D and 3-D grids")
    prob, pml_size = prepare_problem(kgrid, medium, source, sensor, pml_size=pml_size, pml_alpha=pml_alpha,
                                     pml_inside=pml_inside, use_sg=use_sg, use_kspace=use_kspace,
                                     smooth_p0=smooth_p0)
    if save_only:
        return _save_input_files(prob, pml_size, pml_inside, sensor, data_path)

    from .solver import Simulation

    sim = Simulation.from_problem(prob, stream=stream)
    try:
        result = sim.run()
    finally:
        sim.close()
    if not pml_inside:
        result = strip_pml(result, pml_size, ndim)
    return result


_NO_CPP_ALPHA_MODES = ("no_absorption", "no_dispersion", "stokes")


def _save_input_files(prob, pml_size, pml_inside, sensor, data_path):
    """``save_only=True``: the HDF5 input file of the C++ binary for this
    problem in ``data_path`` (kwave/kspaceFirstOrder.py:271-316 with
    backend='cpp'): p0 smoothed on the host as that path does, Cartesian
    sensor points mapped to grid points; returns the file names (and the PML
    size when it lies outside the user's grid)."""
    from . import cpp_io
    from .conversion import cart2grid

    if data_path is None:
        raise ValueError("data_path must be provided when save_only=True (the HDF5 files must persist for cluster "
                         "submission).")
    if prob.get("alpha_mode") in _NO_CPP_ALPHA_MODES:
        raise ValueError(f"medium.alpha_mode={prob['alpha_mode']!r} cannot be stored: the HDF5 input format of the "
                         "C++ binary has no alpha_mode, and the binary applies power-law absorption and dispersion.")
    if sensor is not None and getattr(sensor, "record", None) is not None:
        warnings.warn("sensor.record is not stored in the HDF5 input file; the C++ binary records its default "
                      "fields.", stacklevel=3)
    rsi = getattr(sensor, "record_start_index", 1) if sensor is not None else 1
    if rsi not in (None, 1):
        warnings.warn("sensor.record_start_index is not stored in the HDF5 input file; the C++ binary records from "
                      "the first time step.", stacklevel=3)
    shape = tuple(int(n) for n in prob["shape"])
    prob = dict(prob)
    m = prob.get("sensor_mask")
    if m is not None and _is_cartesian(m, len(shape)):
        kg = SimpleNamespace(N=np.array(shape), spacing=np.array(prob["spacing"]), dim=len(shape))
        prob["sensor_mask"] = cart2grid(kg, np.asarray(m), order="C")[0]
    if prob.get("smooth_p0", True) and prob.get("p0") is not None and np.asarray(prob["p0"]).size > 1 \
            and len(shape) >= 2:
        prob["p0"] = cpp_io.smooth_host(np.asarray(prob["p0"], dtype=float).reshape(shape))
    input_file, output_file = cpp_io.save_input_files(prob, data_path)
    result = {"input_file": input_file, "output_file": output_file}
    if not pml_inside:
        result["pml_size"] = pml_size
    return result


def install():
    """Let ``kwave.kspaceFirstOrder.kspaceFirstOrder(..., backend="gb300")``
    reach :func:`kspaceFirstOrder` (other backends go to the original).

    Patches the module attribute, so it reaches callers that look the
    function up through the module after this call.  Idempotent.
    """
    import kwave.kspaceFirstOrder as mod

    orig = mod.kspaceFirstOrder
    if getattr(orig, "_gb300_dispatch", False):
        return orig

    def dispatch(kgrid, medium, source, sensor=None, **kwargs):
        if kwargs.get("backend") == BACKEND:
            return kspaceFirstOrder(kgrid, medium, source, sensor, **kwargs)
        return orig(kgrid, medium, source, sensor, **kwargs)

    dispatch._gb300_dispatch = True
    dispatch._original = orig
    dispatch.__doc__ = orig.__doc__
    mod.kspaceFirstOrder = dispatch
    return dispatch


def uninstall():
    import kwave.kspaceFirstOrder as mod

    orig = getattr(mod.kspaceFirstOrder, "_original", None)
    if orig is not None:
        mod.kspaceFirstOrder = orig

