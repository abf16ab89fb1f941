"""Golden outputs of the 256^3 heterogeneous absorbing IVP (the headline
workload, ``bench.ivp3d_problem(n=256, seed=0)``) from the unmodified
reference solver, float32 and float64.

Run on a host that holds the k-wave-python checkout (``KWAVE_REFERENCE_ROOT``,
or a ``reference`` directory beside this repository):

    python tests/golden/make_golden_256.py float32 &
    python tests/golden/make_golden_256.py float64 &

One 256^3 reference step takes about 20 s on one core (numpy's FFT is
single-threaded), so a 1000-step run takes hours.  The script therefore
drives the reference's own ``Simulation.setup()`` / ``Simulation.step()``
(kwave/solvers/kspace_solver.py:205-747) and writes a fixture at each of the
checkpoints 100, 250, 500 and 1000 steps; the first t steps of the 1000-step
problem are the whole of a t-step problem, because Nt changes nothing in a
step.  Aggregates come from the reference's ``_compute_aggregates``
(:824-837) over the first t columns.

The inputs are not stored (c0, rho0 and p0 are 64 MiB each): the test
regenerates them with ``bench.ivp3d_problem`` and checks them against the
sums stored here.  Outputs are stored reduced, to keep the fixtures small:

* ``p_max``   -- all 65,536 sensor points of the z = 20 plane;
* ``p_sub``   -- the p series of every 16th sensor point in x and y of the
                 plane (256 points, C order of the plane) for every step;
* ``pfin_sub``-- the final pressure field on the interior (PML stripped, as
                 ``p_final``), every 8th cell along each axis.

Files: ``ivp3d_256/ref32_t0100.npz`` ... ``ivp3d_256/ref64_t1000.npz``.
"""
import sys
import time
from pathlib import Path
from types import SimpleNamespace as NS

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

import kwave_shim  # noqa: E402

OUT_DIR = HERE / "ivp3d_256"
CHECKPOINTS = (100, 250, 500, 1000)
SENSOR_STRIDE = 16
FIELD_STRIDE = 8
SEED = 0
N = 256


def sensor_subset(n=N, stride=SENSOR_STRIDE):
    """Rows of the sensor series kept in ``p_sub``: the binary z-plane mask
    enumerates (x, y) in C order, so row = x * n + y."""
    xs = np.arange(0, n, stride)
    return (xs[:, None] * n + xs[None, :]).ravel()


def field_subset(interior_shape, stride=FIELD_STRIDE):
    return tuple(slice(0, s, stride) for s in interior_shape)


def input_sums(prob):
    out = {}
    for k in ("sound_speed", "density", "p0"):
        a = np.asarray(prob[k], np.float64)
        out[f"sum_{k}"] = np.array([a.sum(), (a * a).sum()])
    return out


def main(dtype_name):
    from bench import ivp3d_problem

    dtype = {"float32": np.float32, "float64": np.float64}[dtype_name]
    tag = {"float32": "ref32", "float64": "ref64"}[dtype_name]
    kwave_shim.install()
    from kwave.solvers.kspace_solver import Simulation, _compute_aggregates

    prob = ivp3d_problem(n=N, nt=max(CHECKPOINTS), seed=SEED)
    kg = NS(Nx=N, Ny=N, Nz=N, dx=prob["spacing"][0], dy=prob["spacing"][1], dz=prob["spacing"][2],
            Nt=int(prob["Nt"]), dt=float(prob["dt"]))
    medium = NS(sound_speed=prob["sound_speed"], density=prob["density"], alpha_coeff=prob["alpha_coeff"],
                alpha_power=prob["alpha_power"], BonA=prob["BonA"])
    source = NS(p0=prob["p0"])
    sensor = NS(mask=prob["sensor_mask"], record=prob["record"], record_start_index=None)
    sim = Simulation(kg, medium, source, sensor, use_sg=True, use_kspace=True, smooth_p0=True,
                     pml_size=prob["pml_size"], pml_alpha=prob["pml_alpha"], dtype=dtype, quiet=True)
    t0 = time.time()
    sim.setup()
    print(f"{tag}: setup {time.time() - t0:.1f} s", flush=True)
    sums = input_sums(prob)
    rows = sensor_subset()
    interior = tuple(slice(s, n - s) for s, n in zip(prob["pml_size"], prob["shape"]))
    OUT_DIR.mkdir(exist_ok=True)
    t0 = time.time()
    for t_end in CHECKPOINTS:
        while sim.t < t_end:
            sim.step()
            if sim.t % 10 == 0:
                print(f"{tag}: step {sim.t} {(time.time() - t0) / sim.t:.2f} s/step", flush=True)
        series = np.asarray(sim.sensor_data["p"][:, :t_end])
        agg = _compute_aggregates({"p": series}, 3, ("p", "p_max"))
        pint = np.asarray(sim.p[interior])
        arrs = dict(p_max=agg["p_max"], p_sub=series[rows], pfin_sub=pint[field_subset(pint.shape)],
                    rows=rows, nt=np.array(t_end), seed=np.array(SEED), n=np.array(N),
                    sensor_stride=np.array(SENSOR_STRIDE), field_stride=np.array(FIELD_STRIDE), **sums)
        path = OUT_DIR / f"{tag}_t{t_end:04d}.npz"
        np.savez_compressed(path, **arrs)
        print(f"{tag}: wrote {path.name} after {time.time() - t0:.0f} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "float32")
