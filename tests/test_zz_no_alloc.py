"""kw_gradient_noalloc, the entry point for callers that cannot let a library
allocate device memory (framework custom operators that own all device memory,
real-time pipelines that forbid allocation once running).

It must give what the plan API gives for the same spectral derivative: a plan
with p0 = f, rho0 = 1 and dt = 2 holds u_a = (dt / rho0 / 2) Re F^-1[op_grad_a
F[f]] = Re F^-1[op_grad_a F[f]] after its first step
(kwave/solvers/kspace_solver.py:729-733), with kappa from c_ref dt / 2 = c0.
Two calls in a row, on different grids and axes, check that the shared static
scratch carries nothing from one call into the next.  Kept in its own file so
it is collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative L2, as in the parity tests
KAPPA_COEF = float(np.float32(1e-5))  # c_ref * dt / 2 with c0 = 1e-5 m/s, dt = 2 s


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(np.asarray(b, np.float64)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib

    _lib.require_device()
    return _lib.lib()


def plan_gradient(f, spacing, axis, use_sg=True, use_kspace=True):
    from kwave_gb300.solver import Simulation

    nd = f.ndim
    prob = dict(shape=f.shape, spacing=spacing, dt=2.0, Nt=1, sound_speed=KAPPA_COEF, density=1.0, p0=f,
                smooth_p0=False, sensor_mask=None, record=("p",), pml_size=(0,) * nd, pml_alpha=(0.0,) * nd,
                use_sg=use_sg, use_kspace=use_kspace)
    sim = Simulation.from_problem(prob).setup()
    try:
        sim.step()
        return sim.u[axis]
    finally:
        sim.close()


def noalloc_gradient(lib, f, spacing, axis, use_sg=True, kappa_coef=KAPPA_COEF):
    import torch

    fd = torch.from_numpy(np.ascontiguousarray(f, np.float32)).cuda()
    out = torch.full_like(fd, float("nan"))
    shape = (C.c_int32 * 3)(*f.shape, *([1] * (3 - f.ndim)))
    d = (C.c_double * 3)(*spacing, *([1.0] * (3 - f.ndim)))
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.kw_gradient_noalloc(C.c_void_p(fd.data_ptr()), C.c_void_p(out.data_ptr()), f.ndim, shape, d, axis,
                                 kappa_coef, int(use_sg), C.c_void_p(stream))
    assert rc == 0, lib.kw_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_gradient_matches_plan_on_two_calls_in_a_row(lib):
    rng = np.random.default_rng(3)
    cases = [(np.float32(rng.standard_normal((24, 20, 16))), (1e-4, 1.2e-4, 1e-4), 0),
             (np.float32(rng.standard_normal((48, 30))), (1e-4, 0.8e-4), 1)]
    for f, spacing, axis in cases:
        got = noalloc_gradient(lib, f, spacing, axis)
        ref = plan_gradient(f.astype(np.float64), spacing, axis)
        assert np.all(np.isfinite(got))
        err = rel_l2(got, ref)
        assert err <= TOL, (f.shape, axis, err)


@pytest.mark.parametrize("shape,spacing,axis,use_sg,use_kspace", [
    ((21, 15), (1e-4, 1.1e-4), 1, True, True),          # odd last axis: full complex row FFT
    ((14, 12, 9), (1e-4, 0.9e-4, 1.2e-4), 2, True, True),  # 3-D, odd last axis, derivative along it
    ((20, 18, 10), (1e-4, 1e-4, 1e-4), 2, True, True),   # 3-D, even last axis, axis 2
    ((30, 25), (1e-4, 1e-4), 0, False, True),            # no staggered-grid shift
    ((16, 12, 14), (1e-4, 1e-4, 1e-4), 1, True, False),  # kappa_coef = 0 (no k-space correction)
])
def test_noalloc_gradient_options_match_plan(lib, shape, spacing, axis, use_sg, use_kspace):
    """Odd and even last axes, each axis in 3-D, use_sg off and kappa off,
    each against the plan built with the same options."""
    rng = np.random.default_rng(sum(shape) + axis)
    f = np.float32(rng.standard_normal(shape))
    got = noalloc_gradient(lib, f, spacing, axis, use_sg=use_sg, kappa_coef=KAPPA_COEF if use_kspace else 0.0)
    ref = plan_gradient(f.astype(np.float64), spacing, axis, use_sg=use_sg, use_kspace=use_kspace)
    assert np.all(np.isfinite(got))
    err = rel_l2(got, ref)
    assert err <= TOL, (shape, axis, use_sg, use_kspace, err)


def test_noalloc_rejects_grids_beyond_the_static_scratch(lib):
    import torch

    from kwave_gb300 import _lib

    buf = torch.zeros(4, device="cuda")
    shape = (C.c_int32 * 3)(4096, 4096, 1)  # 4096 * 2050 spectrum values > 2,097,152
    d = (C.c_double * 3)(1e-4, 1e-4, 1.0)
    rc = lib.kw_gradient_noalloc(C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), 2, shape, d, 0, 0.0, 1, None)
    assert rc == _lib.KW_ERR_UNSUPPORTED
    assert b"static scratch" in lib.kw_last_error()
