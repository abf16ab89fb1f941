"""Time-reversal reconstruction on the GB300 time loop.

:class:`TimeReversal` mirrors kwave/reconstruction/time_reversal.py:19-150:
the recorded sensor pressure, reversed in time, drives a Dirichlet pressure
source on the sensor mask; the final pressure field of that run, times the
compensation factor and clipped at zero, is the initial-pressure estimate.

The reversed run is an ordinary device simulation with a many-signal
Dirichlet source (the sensor points), so it uses the same kernels as the
forward problem.  By default it runs through
:func:`kwave_gb300.backend.kspaceFirstOrder2D` / ``3D``; any function with
the legacy signature ``f(kgrid, source, sensor, medium, simulation_options,
execution_options)`` may be passed instead, as in the reference.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np

from .precompute import grid_of


def _source_and_sensor(mask, p, record):
    """kSource / kSensor objects when ``kwave`` is importable (so that a
    reference simulation function accepts them), plain namespaces otherwise."""
    try:
        from kwave.ksensor import kSensor
        from kwave.ksource import kSource
    except Exception:
        src = SimpleNamespace(p0=None, p_mask=mask, p=p, p_mode="dirichlet", u_mask=None, ux=None, uy=None, uz=None,
                              u_mode=None)
        return src, SimpleNamespace(mask=mask, record=record, record_start_index=1)
    src = kSource()
    src.p_mask = mask
    src.p = p
    src.p_mode = "dirichlet"
    return src, kSensor(mask=mask, record=record)


class TimeReversal:
    """Time-reversal reconstruction of an initial pressure distribution.

    Args:
        kgrid: grid (``N``, ``spacing``, ``Nt``, ``dt`` and an explicit
            ``t_array``).
        medium: medium of the reconstruction run.
        sensor: sensor with a binary ``mask`` of the grid's shape and, before
            the call, ``recorded_pressure`` of shape (n_sensor, Nt).
        compensation_factor: > 0, 2.0 compensates for recording on a
            half-plane (default).

    Raises ``ValueError`` for the same invalid inputs as the reference
    (time_reversal.py:56-92).  Unlike the reference, the sensor's ``record``
    list is copied before ``"p_final"`` is added to it rather than extended
    in place.
    """

    def __init__(self, kgrid, medium, sensor, compensation_factor: float = 2.0) -> None:
        self.kgrid = kgrid
        self.medium = medium
        self.sensor = sensor
        self.compensation_factor = compensation_factor
        self._source = None
        self._new_sensor = None
        mask = getattr(sensor, "mask", None)
        if mask is None:
            raise ValueError("Sensor mask must be set for time reversal. Use sensor.mask = ...")
        t_array = getattr(kgrid, "t_array", None)
        if t_array is None:
            raise ValueError("t_array must be explicitly set for time reversal")
        if isinstance(t_array, str):
            if t_array == "auto":
                raise ValueError("t_array must be explicitly set for time reversal")
            raise ValueError(f"Invalid t_array value: {t_array}")
        if compensation_factor <= 0:
            raise ValueError("compensation_factor must be positive")
        if not np.any(mask):
            raise ValueError("Sensor mask must have at least one active point")
        shape = grid_of(kgrid)[0]
        if not np.array_equal(np.shape(mask), shape):
            raise ValueError(f"Sensor mask shape {np.shape(mask)} does not match grid dimensions {shape}")
        record = getattr(sensor, "record", None)
        self._passed_record = list(record) if record is not None else []
        if "p_final" not in self._passed_record:
            self._passed_record.append("p_final")

    def __call__(self, simulation_function=None, simulation_options=None, execution_options=None) -> np.ndarray:
        """Run the reversed simulation; returns the compensated, non-negative
        p_final, transposed as the reference returns it (time_reversal.py:150).

        ``simulation_function`` defaults to the GB300 legacy entry point of the
        grid's dimension and ``simulation_options`` to the reference's
        defaults (PML 20 points, alpha 2, staggered grid, k-space correction,
        p0 smoothing — which has no p0 to act on here).
        """
        recorded = getattr(self.sensor, "recorded_pressure", None)
        if recorded is None:
            raise ValueError("Sensor must have recorded pressure data. Run a forward simulation first.")
        if simulation_function is None:
            from .backend import kspaceFirstOrder2D, kspaceFirstOrder3D

            ndim = len(grid_of(self.kgrid)[0])
            simulation_function = {2: kspaceFirstOrder2D, 3: kspaceFirstOrder3D}.get(ndim)
            if simulation_function is None:
                raise NotImplementedError("the GB300 time loop runs 2-D and 3-D grids")
        if simulation_options is None:
            simulation_options = SimpleNamespace(pml_size=None, pml_alpha=None, use_sg=True, use_kspace=True,
                                                 smooth_p0=True)
        self._source, self._new_sensor = _source_and_sensor(self.sensor.mask, np.flip(recorded, axis=1),
                                                            self._passed_record)
        result = simulation_function(self.kgrid, self._source, self._new_sensor, self.medium, simulation_options,
                                     execution_options)
        p0_recon = result["p_final"] if isinstance(result, dict) else result
        p0_recon = self.compensation_factor * p0_recon
        p0_recon[p0_recon < 0] = 0
        return p0_recon.T
