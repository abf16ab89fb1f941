"""Step-by-step state of the device time loop against the oracle, on small
grids covering even/odd last axes, 2-D and 3-D, with and without PML.  After
the first step with p0 the velocity is (dt / 2 rho_sg) Re F^-1[op_grad F[p0]]
(kwave/solvers/kspace_solver.py:729-733), so step 0 checks the spectral
gradient alone; later steps check the whole update."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# generic shared-memory transforms (any 2,3,5,7-smooth length) ...
SHAPES = [(16, 15), (15, 16), (16, 16), (8, 8), (2, 4), (12, 20), (30, 18), (8, 6, 10), (9, 5, 7), (6, 10, 12),
          # ... and register transforms (power-of-two lengths 64..1024 along x/y, 128..2048 along the last axis)
          (128, 128), (64, 512), (512, 128), (1024, 120), (64, 128, 256), (16, 64, 2048), (20, 256, 30)]


def rel_max(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("pml", [0, 2])
def test_state_after_each_step(shape, pml):
    from kwave_gb300.solver import Simulation
    from oracle.kspace_oracle import OracleSimulation

    rng = np.random.default_rng(sum(shape) + pml)
    prob = dict(shape=shape, spacing=(1e-4,) * len(shape), dt=2e-8, Nt=4, sound_speed=1500.0, density=1000.0,
                p0=rng.standard_normal(shape), smooth_p0=False, sensor_mask=None, record=("p",),
                pml_size=(pml,) * len(shape), pml_alpha=(2.0,) * len(shape), use_sg=True, use_kspace=True)
    sim = Simulation.from_problem(prob).setup()
    o = OracleSimulation(prob, np.float32).setup()
    try:
        for t in range(4):
            sim.step()
            o.step()
            for a, b in zip(sim.u, o.u):
                assert rel_max(a, b) < 2e-6, ("u", t)
            for a, b in zip(sim.rho_split, o.rho_split):
                assert rel_max(a, b) < 2e-6, ("rho", t)
            assert rel_max(sim.p, o.p) < 2e-6, ("p", t)
    finally:
        sim.close()
