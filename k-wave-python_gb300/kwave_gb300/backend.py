"""Drop-in boundary: the ``"gb300"`` backend behind kspaceFirstOrder2D/3D.

The legacy entry points (kwave/kspaceFirstOrder2D.py:215-218,
kwave/kspaceFirstOrder3D.py:208-211) import
``kwave.solvers.native.run_python_backend`` at call time when
``execution_options.is_python_backend`` is true.  ``install()`` replaces that
attribute with a dispatcher: execution options whose backend is ``"gb300"``
go to :func:`run_gb300_backend`, everything else to the original function.

The reference's option setter accepts only None/"OMP"/"CUDA"/"python"
(kwave/options/simulation_execution_options.py:114-119), so
:func:`execution_options` builds a subclass that also accepts ``"gb300"`` and
reports ``is_python_backend`` (the switch the legacy functions test).
"""
from __future__ import annotations

import numpy as np

from .precompute import grid_of
from .solver import Simulation

BACKEND = "gb300"


def is_gb300(execution_options) -> bool:
    return getattr(execution_options, "backend", None) == BACKEND


def _per_axis(val, dim, default, cast):
    """native.py:9-18, plus broadcasting of a length-1 sequence (the form that
    SimulationOptions stores a scalar pml_size in, simulation_options.py:178-179)."""
    if val is None:
        return (default,) * dim
    if not hasattr(val, "__len__"):
        return (cast(val),) * dim
    seq = [cast(v) for v in np.asarray(val).ravel()]
    if len(seq) == 1:
        seq = seq * dim
    if len(seq) != dim:
        raise ValueError(f"expected {dim} per-axis values, got {len(seq)}")
    return tuple(seq)


def run_gb300_backend(kgrid, medium, source, sensor, simulation_options, execution_options=None):
    """GB300 counterpart of ``run_python_backend`` (kwave/solvers/native.py:6-30).

    Same defaults as the reference bridge: PML size 20 and alpha 2.0 per axis
    when unset, ``use_sg``/``use_kspace``/``smooth_p0`` from the simulation
    options.  Differences: the computation is float32 (the reference bridge
    always runs float64 because it never passes ``data_cast``), and a scalar
    ``pml_size`` is broadcast instead of failing with IndexError.
    """
    dim = len(grid_of(kgrid)[0])
    pml_size = _per_axis(getattr(simulation_options, "pml_size", None), dim, 20, int)
    pml_alpha = _per_axis(getattr(simulation_options, "pml_alpha", None), dim, 2.0, float)
    sim = Simulation(
        kgrid, medium, source, sensor, device="gpu",
        use_sg=getattr(simulation_options, "use_sg", True),
        use_kspace=getattr(simulation_options, "use_kspace", True),
        smooth_p0=getattr(simulation_options, "smooth_p0", True),
        pml_size=pml_size, pml_alpha=pml_alpha, quiet=True,
    )
    try:
        return sim.run()
    finally:
        sim.close()


def _legacy(ndim_expected, name):
    def run(kgrid, source, sensor, medium, simulation_options, execution_options=None):
        dim = len(grid_of(kgrid)[0])
        if dim != ndim_expected:
            raise ValueError(f"{name} needs a {ndim_expected}-D grid, got {dim}-D")
        return run_gb300_backend(kgrid, medium, source, sensor, simulation_options, execution_options)

    run.__name__ = run.__qualname__ = name
    run.__doc__ = (f"{name}(kgrid, source, sensor, medium, simulation_options, execution_options) on the GB300 "
                   "time loop: the legacy signature (kwave/kspaceFirstOrder2D.py:140-148, "
                   "kwave/kspaceFirstOrder3D.py) taking the python-backend branch "
                   "(kwave/kspaceFirstOrder2D.py:215-218) straight to :func:`run_gb300_backend`.  "
                   "``simulation_options`` is read for pml_size, pml_alpha, use_sg, use_kspace and "
                   "smooth_p0; ``execution_options`` is accepted and ignored.")
    return run


kspaceFirstOrder2D = _legacy(2, "kspaceFirstOrder2D")
kspaceFirstOrder3D = _legacy(3, "kspaceFirstOrder3D")


def _input_path(simulation_options):
    """The input file name of the options: ``input_filename`` inside
    ``data_path`` (kwave/options/simulation_options.py:111-112 and :189,
    which join the two unless the name is already absolute)."""
    import os
    import tempfile

    name = getattr(simulation_options, "input_filename", None) or "kwave_input.h5"
    if os.path.isabs(name):
        return name
    return os.path.join(getattr(simulation_options, "data_path", None) or tempfile.gettempdir(), name)


def _legacy_cpp(ndim_expected, name):
    def run(kgrid, source, sensor, medium, simulation_options, execution_options=None):
        from . import cpp_io
        from .precompute import grid_shape_of

        dim = len(grid_shape_of(kgrid)[0])
        if dim != ndim_expected:
            raise ValueError(f"{name} needs a {ndim_expected}-D grid, got {dim}-D")
        if not getattr(simulation_options, "save_to_disk", False):
            raise ValueError("CPU simulation requires saving to disk. Please set SimulationOptions.save_to_disk=True")
        prob = cpp_io.legacy_problem(
            kgrid, medium, source, sensor,
            # the legacy default PML: 20 points in 2-D, 10 in 3-D (simulation_options.py:264-287)
            pml_size=_per_axis(getattr(simulation_options, "pml_size", None), dim, 20 if dim == 2 else 10, int),
            pml_alpha=_per_axis(getattr(simulation_options, "pml_alpha", None), dim, 2.0, float),
            pml_inside=getattr(simulation_options, "pml_inside", True),
            smooth_p0=getattr(simulation_options, "smooth_p0", True),
            use_sg=getattr(simulation_options, "use_sg", True))
        path = _input_path(simulation_options)
        level = getattr(simulation_options, "hdf_compression_level", None) or 0
        if not (isinstance(level, (int, np.integer)) and 0 <= level <= 9):
            raise ValueError("Optional input ''hdf_compression_level'' must be an integer between 0 and 9.")
        cpp_io.write_input_file(path, prob, legacy=True, compression_level=int(level))
        if getattr(simulation_options, "save_to_disk_exit", False):
            return None
        # the sensor's record list and start index, which the reference hands to the binary as flags
        return cpp_io.run_input_file(path, scaled_sources=True, record=getattr(sensor, "record", None),
                                     record_start_index=getattr(sensor, "record_start_index", None))

    run.__name__ = run.__qualname__ = name
    run.__doc__ = (f"{name}(kgrid, source, sensor, medium, simulation_options, execution_options): the legacy "
                   "C++ route (kwave/kspaceFirstOrder2D.py:82-139 and :221-384) with ``save_to_disk``.  Writes "
                   "the input file the legacy route writes (``cpp_io.legacy_problem`` and "
                   "``cpp_io.input_datasets(legacy=True)``) to ``input_filename`` in ``data_path``; returns None "
                   "with ``save_to_disk_exit``, otherwise runs that file on the GB300 time loop in place of the "
                   "C++ binary and returns the native solver's result dict (``cpp_io.run_input_file``).  "
                   "``simulation_options`` is read for save_to_disk, save_to_disk_exit, data_path, "
                   "input_filename, hdf_compression_level, pml_size, pml_alpha, pml_inside, smooth_p0 and use_sg.")
    return run


kspaceFirstOrder2DC = _legacy_cpp(2, "kspaceFirstOrder2DC")
kspaceFirstOrder3DC = _legacy_cpp(3, "kspaceFirstOrder3DC")


_installed = {}


def install():
    """Route ``backend="gb300"`` through the legacy kspaceFirstOrder2D/3D calls.

    Requires the reference package (``kwave``) to be importable.  Idempotent.
    """
    import kwave.solvers.native as native

    if getattr(native.run_python_backend, "_gb300_dispatch", False):
        return native.run_python_backend
    original = native.run_python_backend

    def run_python_backend(kgrid, medium, source, sensor, simulation_options, execution_options):
        if is_gb300(execution_options):
            return run_gb300_backend(kgrid, medium, source, sensor, simulation_options, execution_options)
        return original(kgrid, medium, source, sensor, simulation_options, execution_options)

    run_python_backend._gb300_dispatch = True
    run_python_backend._original = original
    native.run_python_backend = run_python_backend
    _installed["native"] = (native, original)
    return run_python_backend


def uninstall():
    if "native" in _installed:
        native, original = _installed.pop("native")
        native.run_python_backend = original


def execution_options(**kwargs):
    """SimulationExecutionOptions with ``backend="gb300"`` (needs ``kwave``)."""
    from kwave.options.simulation_execution_options import SimulationExecutionOptions

    class GB300ExecutionOptions(SimulationExecutionOptions):
        @property
        def backend(self):
            return self._backend

        @backend.setter
        def backend(self, value):
            if value not in (None, "OMP", "CUDA", "python", BACKEND):
                raise ValueError(f"Backend must be one of [None, 'OMP', 'CUDA', 'python', '{BACKEND}'], got '{value}'")
            self._backend = value

        @property
        def is_python_backend(self):
            return self._backend in ("python", BACKEND)

    kwargs.setdefault("backend", BACKEND)
    kwargs.setdefault("is_gpu_simulation", True)
    return GB300ExecutionOptions(**kwargs)
