"""Golden HDF5 input files of the k-Wave C++ binary, as the unmodified
reference writes them: ``kspaceFirstOrder(..., backend="cpp",
save_only=True, data_path=...)`` (kwave/kspaceFirstOrder.py:271-316 ->
kwave/solvers/cpp_simulation.py:139-318 -> kwave/utils/io.py:52-243), on a
host that holds the reference checkout (``KWAVE_REFERENCE_ROOT``, or a
``reference`` directory beside this repository):

    python tests/golden/make_cpp_io_golden.py

h5py is not installed here, so a recording stand-in for the h5py calls that
writer makes (``File(name, "a")`` as a context manager, ``create_dataset``,
``attrs.create``) captures every dataset (name, shape, dtype, values) and
attribute instead of writing a file; the container format itself is not part
of these fixtures.  Cases land in ``tests/golden/cpp_io/`` with the keys
``in:<problem key>``, ``meta:opt_<option>``, ``h5:<dataset>``,
``h5attr:<dataset>:<attribute>`` and ``h5root:<attribute>``.
"""
import sys
import tempfile
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

SUBDIR = "cpp_io"


class _Attrs(dict):
    def create(self, name, data, shape=None, dtype=None):
        self[name] = np.asarray(data, dtype=dtype)


class _Dataset:
    def __init__(self, arr):
        self.data = arr
        self.attrs = _Attrs()


class _File:
    store = {}

    def __init__(self, name, mode="r"):
        self.rec = _File.store.setdefault(str(name), {"datasets": {}, "attrs": _Attrs()})
        self.attrs = self.rec["attrs"]

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def create_dataset(self, name, shape=None, data=None, dtype=None, chunks=None, compression=None):
        name = name.lstrip("/")
        if name in self.rec["datasets"]:
            raise ValueError(f"dataset {name} exists")
        arr = np.asarray(data, dtype=np.dtype(dtype) if dtype is not None else None).reshape(tuple(shape))
        ds = _Dataset(arr)
        self.rec["datasets"][name] = ds
        return ds

    def __getitem__(self, name):
        return self.rec["datasets"][name.lstrip("/")]


def _install_recorder():
    h5 = types.ModuleType("h5py")
    h5.File = _File
    sys.modules["h5py"] = h5
    import kwave_shim

    kwave_shim.install()


def save_only(prob, opts):
    """Run the reference's save_only path; returns the captured file."""
    _install_recorder()
    from kwave.kspaceFirstOrder import kspaceFirstOrder
    from make_api_golden import _objects

    kg, med, src, sen = _objects(prob)
    with tempfile.TemporaryDirectory() as d:
        res = kspaceFirstOrder(kg, med, src, sen, backend="cpp", save_only=True, data_path=d, **opts)
        rec = _File.store.pop(res["input_file"])
    return rec, res


def case(name, prob, opts):
    rec, res = save_only(prob, opts)
    arrs = {f"in:{k}": np.asarray(v) for k, v in prob.items() if v is not None}
    arrs.update({f"meta:opt_{k}": np.asarray(v) for k, v in opts.items()})
    for k, ds in rec["datasets"].items():
        arrs[f"h5:{k}"] = ds.data
        for a, v in ds.attrs.items():
            arrs[f"h5attr:{k}:{a}"] = v
    for a, v in rec["attrs"].items():
        arrs[f"h5root:{a}"] = v
    if "pml_size" in res:
        arrs["meta:ret_pml_size"] = np.asarray(res["pml_size"])
    (HERE / SUBDIR).mkdir(exist_ok=True)
    np.savez_compressed(HERE / SUBDIR / f"{name}.npz", **arrs)
    print(name, len(rec["datasets"]), "datasets")


def case_ivp2d():
    """Heterogeneous absorbing nonlinear 2-D medium, p0 smoothed after the
    grid grows by 2 x 8 PML points, binary sensor points."""
    from make_golden import gaussian_blobs, smooth_random_field

    rng = np.random.default_rng(201)
    shape = (40, 40)  # 56 x 56 with the PML: lengths the device FFTs take
    prob = dict(shape=shape, spacing=(1e-4, 1.2e-4), Nt=60, dt=1.5e-8,
                sound_speed=smooth_random_field(shape, rng, rel=0.04),
                density=smooth_random_field(shape, rng, rel=0.05, base=1000.0),
                alpha_coeff=0.75, alpha_power=1.5, BonA=6.0, p0=gaussian_blobs(shape, 2, rng, margin=8),
                sensor_mask=rng.random(shape) < 0.05)
    return prob, dict(pml_size=8, pml_alpha=2.0, pml_inside=False, smooth_p0=True)


def case_src3d():
    """3-D additive pressure source with two signals on a patch, scalar
    medium, no sensor (every grid point), PML inside."""
    from make_golden import tone_burst_rows

    rng = np.random.default_rng(202)
    shape = (20, 18, 16)
    dt = 1.5e-8
    m = np.zeros(shape, bool)
    m[10, 6:8, 5:8] = True
    sig = np.vstack([tone_burst_rows(1, 30, dt, 1.2e6, 3, rng, max_delay=1) for _ in range(int(m.sum()))]) * 1e3
    prob = dict(shape=shape, spacing=(1e-4, 1e-4, 1e-4), Nt=30, dt=dt, sound_speed=1500.0, density=1000.0,
                p_mask=m, p=sig)
    return prob, dict(pml_size=(4, 5, 6), pml_alpha=(2.0, 1.5, 1.0), pml_inside=True, smooth_p0=False)


def case_vel2d():
    """2-D Dirichlet velocity source on a line (one signal per component),
    Stokes absorption, Cartesian sensor points mapped to the grid."""
    from make_golden import tone_burst_rows

    rng = np.random.default_rng(203)
    shape = (32, 30)
    dt = 1.8e-8
    um = np.zeros(shape, bool)
    um[8, 6:24] = True
    ux = tone_burst_rows(1, 40, dt, 1.0e6, 2, rng, max_delay=1) * 0.1
    uy = tone_burst_rows(1, 40, dt, 1.0e6, 2, rng, max_delay=1) * 0.05
    pts = rng.uniform(-1.2e-3, 1.2e-3, size=(2, 10))
    prob = dict(shape=shape, spacing=(1e-4, 1e-4), Nt=40, dt=dt, sound_speed=1500.0, density=1000.0,
                alpha_coeff=0.5, alpha_power=2.0, u_mask=um, ux=ux, uy=uy, u_mode="dirichlet", sensor_mask=pts)
    return prob, dict(pml_size=6, pml_alpha=2.0, pml_inside=False, smooth_p0=True)


if __name__ == "__main__":
    for fn in (case_ivp2d, case_src3d, case_vel2d):
        prob, opts = fn()
        case(fn.__name__[5:], prob, opts)
