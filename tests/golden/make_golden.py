"""Generate the golden cases under tests/golden/ from the unmodified reference.

Run on a host that holds the k-wave-python checkout (``KWAVE_REFERENCE_ROOT``,
or a ``reference`` directory beside this repository):

    python tests/golden/make_golden.py

Each case is a seeded problem description; the script runs the reference's
native ``Simulation`` (kwave/solvers/kspace_solver.py) with dtype float32 and
float64 through ``kwave_shim`` and stores inputs and outputs with
``fixtures.save_case``.  The GPU machine never runs this script; it only reads the
committed ``.npz`` files.
"""
import sys
from pathlib import Path
from types import SimpleNamespace as NS

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(HERE.parent.parent))

import kwave_shim  # noqa: E402
from fixtures import save_case  # noqa: E402


# ---------------------------------------------------------------------------
# seeded input generators (synthetic stand-ins for the reference's examples)
# ---------------------------------------------------------------------------

def gaussian_blobs(shape, n, rng, sigma=(1.5, 4.0), amp=(1.0, 10.0), margin=2):
    grids = np.meshgrid(*[np.arange(s) for s in shape], indexing="ij")
    out = np.zeros(shape)
    for _ in range(n):
        c = [rng.uniform(margin, s - 1 - margin) for s in shape]
        s = rng.uniform(*sigma)
        a = rng.uniform(*amp)
        r2 = sum((g - ci) ** 2 for g, ci in zip(grids, c))
        out += a * np.exp(-r2 / (2 * s * s))
    return out


def smooth_random_field(shape, rng, rel=0.05, base=1500.0, corr=3.0):
    noise = rng.standard_normal(shape)
    k = np.meshgrid(*[np.fft.fftfreq(s) for s in shape], indexing="ij")
    filt = np.exp(-0.5 * sum((ki * corr * 2 * np.pi) ** 2 for ki in k))
    f = np.real(np.fft.ifftn(np.fft.fftn(noise) * filt))
    f /= f.std() + 1e-30
    return base * (1.0 + rel * f)


def tone_burst_rows(n_rows, length, dt, f0, cycles, rng, max_delay=8):
    t = np.arange(length) * dt
    rows = []
    for _ in range(n_rows):
        d = rng.integers(0, max_delay) * dt
        tt = t - d
        env = np.where((tt >= 0) & (tt <= cycles / f0), np.sin(np.pi * f0 * np.clip(tt, 0, None) / cycles) ** 2, 0.0)
        rows.append(env * np.sin(2 * np.pi * f0 * tt))
    return np.array(rows)


# ---------------------------------------------------------------------------
# running the reference
# ---------------------------------------------------------------------------

def _ns_objects(prob):
    shape, spacing = prob["shape"], prob["spacing"]
    kg = {}
    for ax, (n, d) in zip("xyz", zip(shape, spacing)):
        kg[f"N{ax}"] = int(n)
        kg[f"d{ax}"] = float(d)
    kg["Nt"] = int(prob["Nt"])
    kg["dt"] = float(prob["dt"])
    medium = NS(**{k: prob[k] for k in ("sound_speed", "density", "alpha_coeff", "alpha_power", "alpha_mode", "BonA") if prob.get(k) is not None})
    src = NS(**{k: prob[k] for k in ("p0", "p_mask", "p", "p_mode", "u_mask", "ux", "uy", "uz", "u_mode") if prob.get(k) is not None})
    if prob.get("sensor_mask") is None and prob.get("record") is None:
        sensor = None
    else:
        sensor = NS(mask=prob.get("sensor_mask"), record=prob.get("record"), record_start_index=prob.get("record_start_index"))
    return NS(**kg), medium, src, sensor


def run_reference(prob, dtype):
    kwave_shim.install()
    from kwave.solvers.kspace_solver import Simulation

    kg, med, src, sen = _ns_objects(prob)
    sim = Simulation(
        kg, med, src, sen,
        use_sg=prob.get("use_sg", True), use_kspace=prob.get("use_kspace", True),
        smooth_p0=prob.get("smooth_p0", True),
        pml_size=prob.get("pml_size"), pml_alpha=prob.get("pml_alpha"),
        dtype=dtype, quiet=True,
    )
    return sim.run()


def base(shape, spacing, dt, Nt, **kw):
    d = dict(shape=tuple(shape), spacing=tuple(spacing), dt=dt, Nt=Nt, sound_speed=1500.0, density=1000.0,
             pml_size=(10,) * len(shape), pml_alpha=(2.0,) * len(shape), use_sg=True, use_kspace=True,
             smooth_p0=True)
    d.update(kw)
    return d


# ---------------------------------------------------------------------------
# cases
# ---------------------------------------------------------------------------

def case_ivp2d_128_circle():
    """2-D homogeneous IVP, 128^2, two discs, 50-point Cartesian circle."""
    kwave_shim.install()
    from kwave.data import Vector
    from kwave.kgrid import kWaveGrid
    from kwave.utils.mapgen import make_cart_circle, make_disc

    N, d = Vector([128, 128]), Vector([1e-4, 1e-4])
    kgrid = kWaveGrid(N, d)
    kgrid.makeTime(1500.0, 0.3)
    p0 = 5.0 * make_disc(N, Vector([64, 64]), 5) + 3.0 * make_disc(N, Vector([54, 84]), 3)
    cart = make_cart_circle(4e-3, 50)
    return base((128, 128), (1e-4, 1e-4), float(kgrid.dt), int(kgrid.Nt), p0=p0.astype(float),
                sensor_mask=np.asarray(cart, float), record=("p", "p_final"), pml_size=(20, 20))


def case_het2d():
    rng = np.random.default_rng(11)
    sh = (48, 40)
    c = smooth_random_field(sh, rng, rel=0.06)
    rho = smooth_random_field(sh, rng, rel=0.05, base=1000.0)
    mask = np.zeros(sh, bool)
    mask.ravel()[rng.choice(mask.size, 30, replace=False)] = True
    return base(sh, (1e-4, 1e-4), 2e-8, 60, sound_speed=c, density=rho, alpha_coeff=0.75, alpha_power=1.5, BonA=6.0,
                p0=gaussian_blobs(sh, 5, rng), smooth_p0=False, sensor_mask=mask,
                record=("p", "p_max", "p_min", "p_rms", "p_final"), pml_size=(8, 8))


def case_src_additive():
    rng = np.random.default_rng(12)
    sh = (64, 60)
    c = smooth_random_field(sh, rng, rel=0.05)
    pmask = np.zeros(sh, bool)
    pmask[12, 20:40:2] = True
    sig = tone_burst_rows(int(pmask.sum()), 40, 2e-8, 3e6, 2, rng)
    smask = np.zeros(sh, bool)
    smask[20, 10:50] = True
    return base(sh, (1e-4, 1e-4), 2e-8, 70, sound_speed=c, p_mask=pmask, p=sig, p_mode="additive",
                sensor_mask=smask, record=("p", "p_final"))


def case_src_dirichlet():
    rng = np.random.default_rng(13)
    sh = (50, 45)
    pmask = np.zeros(sh, bool)
    pmask[20:23, 20:23] = True
    sig = tone_burst_rows(1, 30, 2e-8, 2e6, 2, rng, max_delay=1)[0]
    smask = np.zeros(sh, bool)
    smask[5:45:5, 30] = True
    return base(sh, (1e-4, 1.2e-4), 2e-8, 55, sound_speed=1540.0, density=1020.0, alpha_coeff=0.5, alpha_power=1.1,
                p_mask=pmask, p=sig, p_mode="dirichlet", sensor_mask=smask, record=("p", "p_rms"))


def case_src_velocity():
    rng = np.random.default_rng(14)
    sh = (40, 36)
    umask = np.zeros(sh, bool)
    umask[10, 10:26] = True
    n = int(umask.sum())
    ux = tone_burst_rows(n, 25, 2e-8, 3e6, 2, rng) * 1e-3
    uy = tone_burst_rows(1, 25, 2e-8, 3e6, 2, rng, max_delay=1) * 5e-4
    pmask = np.zeros(sh, bool)
    pmask[30, 5] = True
    smask = np.zeros(sh, bool)
    smask[13:18, 12:22] = True
    return base(sh, (1e-4, 1e-4), 2e-8, 50, sound_speed=smooth_random_field(sh, rng, rel=0.04),
                u_mask=umask, ux=ux, uy=uy, u_mode="additive",
                p_mask=pmask, p=tone_burst_rows(1, 20, 2e-8, 3e6, 2, rng, max_delay=1), p_mode="additive-no-correction",
                sensor_mask=smask, record=("p", "ux", "uy", "ux_staggered", "uy_staggered", "u_max", "p_final", "ux_final"))


def case_vel_dirichlet():
    rng = np.random.default_rng(15)
    sh = (32, 40)
    umask = np.zeros(sh, bool)
    umask[8:10, 12:20] = True
    n = int(umask.sum())
    uy = tone_burst_rows(n, 20, 2e-8, 3e6, 2, rng) * 1e-3
    smask = np.zeros(sh, bool)
    smask[13, :] = True
    return base(sh, (1e-4, 1e-4), 2e-8, 40, u_mask=umask, uy=uy, u_mode="dirichlet",
                sensor_mask=smask, record=("p", "uy_staggered"))


def case_het3d():
    rng = np.random.default_rng(21)
    sh = (32, 24, 20)
    c = smooth_random_field(sh, rng, rel=0.06)
    rho = smooth_random_field(sh, rng, rel=0.05, base=1000.0)
    mask = np.zeros(sh, bool)
    mask[:, :, 5] = True
    return base(sh, (1e-4,) * 3, 2e-8, 40, sound_speed=c, density=rho, alpha_coeff=0.75, alpha_power=1.5, BonA=6.0,
                p0=gaussian_blobs(sh, 6, rng, sigma=(1.5, 3.0)), smooth_p0=True, sensor_mask=mask,
                record=("p", "p_max", "p_final"), pml_size=(4, 4, 4))


def case_stokes3d():
    rng = np.random.default_rng(22)
    sh = (20, 20, 24)
    cart = rng.uniform(-6e-4, 6e-4, size=(3, 10))
    return base(sh, (1e-4,) * 3, 2e-8, 30, sound_speed=1500.0, alpha_coeff=0.5, alpha_power=2.0,
                p0=gaussian_blobs(sh, 3, rng, sigma=(1.5, 3.0)), smooth_p0=False, sensor_mask=cart,
                record=("p", "p_final"), pml_size=(4, 4, 4))


def case_opts2d():
    rng = np.random.default_rng(23)
    sh = (36, 36)
    mask = np.zeros(sh, bool)
    mask[18, :] = True
    return base(sh, (1e-4, 1e-4), 2e-8, 40, use_sg=False, use_kspace=False, record_start_index=10,
                p0=gaussian_blobs(sh, 3, rng), smooth_p0=True, sensor_mask=mask, record=("p", "p_min", "p_final"),
                sound_speed=smooth_random_field(sh, rng, rel=0.03))


def case_nodisp2d():
    rng = np.random.default_rng(24)
    sh = (32, 32)
    mask = np.zeros(sh, bool)
    mask[::4, 5] = True
    return base(sh, (1e-4, 1e-4), 2e-8, 40, alpha_coeff=0.5, alpha_power=1.05, alpha_mode="no_dispersion",
                p0=gaussian_blobs(sh, 2, rng), sensor_mask=mask, record=("p",), pml_size=(6, 6))


def case_nosensor2d():
    rng = np.random.default_rng(25)
    sh = (24, 20)
    return base(sh, (1e-4, 1e-4), 2e-8, 10, p0=gaussian_blobs(sh, 2, rng), pml_size=(4, 4))


def case_intensity2d():
    """p0 with velocity and intensity recording (non-staggered u from t = 0)."""
    rng = np.random.default_rng(31)
    sh = (48, 40)
    mask = np.zeros(sh, bool)
    mask[30:34, 10:30:3] = True
    return base(sh, (1e-4, 1e-4), 2e-8, 50, p0=gaussian_blobs(sh, 3, rng), sensor_mask=mask,
                record=("p", "u", "I", "I_avg", "ux_rms"), sound_speed=smooth_random_field(sh, rng, rel=0.04),
                pml_size=(8, 8))


def case_src3d():
    """3-D k-space corrected pressure and velocity sources, non-staggered u, record_start_index."""
    rng = np.random.default_rng(32)
    sh = (24, 20, 16)
    pmask = np.zeros(sh, bool)
    pmask[8, 6:14:2, 8] = True
    umask = np.zeros(sh, bool)
    umask[14, 10, 4:12] = True
    smask = np.zeros(sh, bool)
    smask[4:20:3, 10, 8] = True
    return base(sh, (1e-4,) * 3, 2e-8, 40, sound_speed=smooth_random_field(sh, rng, rel=0.04),
                density=smooth_random_field(sh, rng, rel=0.03, base=1000.0),
                p_mask=pmask, p=tone_burst_rows(int(pmask.sum()), 25, 2e-8, 3e6, 2, rng), p_mode="additive",
                u_mask=umask, ux=tone_burst_rows(1, 20, 2e-8, 3e6, 2, rng, max_delay=1) * 1e-3, u_mode="additive",
                sensor_mask=smask, record=("p", "ux", "uz_staggered", "p_final"), record_start_index=5,
                pml_size=(4, 4, 4))


def case_pow2_2d_src():
    """Power-of-two grid (register/TMA kernels): additive corrected p source, dirichlet u source."""
    rng = np.random.default_rng(33)
    sh = (64, 128)
    pmask = np.zeros(sh, bool)
    pmask[20, 40:80:4] = True
    umask = np.zeros(sh, bool)
    umask[40:42, 60:64] = True
    smask = np.zeros(sh, bool)
    smask[30, :] = True
    return base(sh, (1e-4, 1e-4), 2e-8, 60, sound_speed=smooth_random_field(sh, rng, rel=0.04),
                alpha_coeff=0.5, alpha_power=1.1,
                p_mask=pmask, p=tone_burst_rows(int(pmask.sum()), 30, 2e-8, 3e6, 2, rng), p_mode="additive",
                u_mask=umask, uy=tone_burst_rows(1, 20, 2e-8, 3e6, 2, rng, max_delay=1) * 1e-3, u_mode="dirichlet",
                sensor_mask=smask, record=("p", "u", "p_max", "p_final"), pml_size=(8, 8))


def case_pow2_3d():
    """Power-of-two 3-D grid with the headline physics plus Cartesian sensors and u."""
    rng = np.random.default_rng(34)
    sh = (64, 64, 64)
    c = smooth_random_field(sh, rng, rel=0.05)
    rho = smooth_random_field(sh, rng, rel=0.04, base=1000.0)
    cart = rng.uniform(-2.5e-3, 2.5e-3, size=(3, 12))
    return base(sh, (1e-4,) * 3, 2e-8, 30, sound_speed=c, density=rho, alpha_coeff=0.75, alpha_power=1.5, BonA=6.0,
                p0=gaussian_blobs(sh, 5, rng, sigma=(2.0, 4.0)), smooth_p0=True, sensor_mask=cart,
                record=("p", "u", "p_rms", "p_final"), pml_size=(10, 10, 10))


def case_ivp3d_48_absorbing():
    """The 256^3 absorbing IVP physics (heterogeneous, power law y=1.5, BonA 6, 10-pt PML, z-plane sensor) at 48^3."""
    from bench import ivp3d_problem

    return ivp3d_problem(n=48, nt=40, seed=7, plane_z=12)


CASES = {
    "ivp2d_128_circle": case_ivp2d_128_circle,
    "het2d_abs_nl": case_het2d,
    "src2d_additive": case_src_additive,
    "src2d_dirichlet": case_src_dirichlet,
    "src2d_velocity": case_src_velocity,
    "vel2d_dirichlet": case_vel_dirichlet,
    "het3d_abs_nl": case_het3d,
    "stokes3d_cart": case_stokes3d,
    "opts2d_nosg": case_opts2d,
    "nodisp2d": case_nodisp2d,
    "nosensor2d": case_nosensor2d,
    "ivp3d_48_absorbing": case_ivp3d_48_absorbing,
    "intensity2d": case_intensity2d,
    "src3d_additive": case_src3d,
    "pow2_2d_src": case_pow2_2d_src,
    "pow2_3d": case_pow2_3d,
}


def main(names=None):
    for name, fn in CASES.items():
        if names and name not in names:
            continue
        prob = fn()
        r32 = run_reference(prob, np.float32)
        r64 = run_reference(prob, np.float64)
        save_case(name, prob, r32, r64)
        print(name, {k: v.shape for k, v in r32.items()})


if __name__ == "__main__":
    main(sys.argv[1:])
