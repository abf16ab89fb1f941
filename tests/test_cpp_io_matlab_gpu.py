"""The legacy C++ route run on the GPU in place of the binary
(``kspaceFirstOrder2DC/3DC`` with ``save_to_disk`` and without
``save_to_disk_exit``): the legacy input file of a pressure point source,
its scaled signal divided out again, runs to the same sensor data as the
problem it was written from run directly, within 1e-5 relative L2 (the
file stores dt and the signal in float32; measured 1.7e-6, and 1.9e-6 for
the float32 oracle on the same two problems).  That the file describes the
same simulation is checked for more cases, and in float64, on the CPU
(``test_cpp_io_matlab_cpu.py``).
"""
from types import SimpleNamespace as NS

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib

    _lib.require_device()


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", ["tvsp_homogeneous_medium_monopole"])
def test_legacy_route_runs_its_file(name, tmp_path):
    from test_cpp_io_matlab_cpu import _load, _objects

    from kwave_gb300 import backend, cpp_io
    from kwave_gb300.solver import run_problem

    inp, opts, _ = _load(name)
    kgrid, medium, source, sensor = _objects(inp)
    so = NS(save_to_disk=True, save_to_disk_exit=False, data_path=str(tmp_path), input_filename="run.h5", **opts)
    got = backend.kspaceFirstOrder2DC(kgrid, source, sensor, medium, so)
    prob = cpp_io.legacy_problem(kgrid, medium, source, sensor, pml_size=opts.get("pml_size", 20),
                                 pml_alpha=opts.get("pml_alpha", 2.0), pml_inside=opts.get("pml_inside", True))
    for f in ("p", "ux"):
        if f in prob and prob[f] is not None:
            # the direct run takes the caller's rows in C order of the mask's points, as the file reader gives them
            m = prob["p_mask" if f == "p" else "u_mask"]
            shape = tuple(prob["shape"])
            prob[f] = cpp_io._rows_to_c_order(np.atleast_2d(prob[f]), cpp_io._fortran_index(m, shape), shape)
    prob.update(record=("p",), record_start_index=1)
    ref = run_problem(prob)
    e = rel_l2(got["p"], ref["p"])
    print(f"{name}: legacy file run vs direct run, p rel L2 {e:.2e}")
    assert got["p"].shape == ref["p"].shape
    assert e <= 1e-5, e
