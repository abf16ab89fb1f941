"""kwave_gb300: the k-space first-order time loop of k-wave-python on one GB300.

Entry points:
  * ``backend.install()`` + ``backend.execution_options()`` — select the GPU
    time loop from the legacy ``kspaceFirstOrder2D/3D`` call;
  * ``backend.run_gb300_backend`` — the bridge itself (the counterpart of
    ``kwave.solvers.native.run_python_backend``);
  * ``solver.Simulation`` — the counterpart of
    ``kwave.solvers.kspace_solver.Simulation``;
  * ``unified.kspaceFirstOrder`` — the unified entry point
    (``kwave.kspaceFirstOrder.kspaceFirstOrder``) for ``backend="gb300"``;
  * ``backend.kspaceFirstOrder2D`` / ``3D`` — the legacy signatures;
  * ``backend.kspaceFirstOrder2DC`` / ``3DC`` — the legacy C++ route with
    ``save_to_disk``: the C++ binary's input file as the legacy route and
    MATLAB k-Wave write it, run on the GPU time loop in place of the binary;
  * ``reconstruction.TimeReversal`` — time-reversal reconstruction, with
    ``conversion.cart2grid`` for Cartesian sensors;
  * ``solver.SimulationBatch`` / ``solver.run_batch`` — many independent
    simulations of any sizes advanced together, one graph launch per step.
"""
__version__ = "0.1.0"

from .backend import (BACKEND, execution_options, install, kspaceFirstOrder2D, kspaceFirstOrder2DC,  # noqa: F401
                      kspaceFirstOrder3D, kspaceFirstOrder3DC, run_gb300_backend, uninstall)
from .conversion import cart2grid  # noqa: F401
from .reconstruction import TimeReversal  # noqa: F401
from .solver import Simulation, SimulationBatch, run_batch, run_problem  # noqa: F401
from .unified import get_optimal_pml_size, kspaceFirstOrder, reshape_to_grid  # noqa: F401
