"""Benchmark: k-space first-order time loop on one GB300 (placeholder; generators only)."""
import numpy as np


def _random_rotation(rng):
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def config2_problem(n=256, nt=1000, seed=0, plane_z=20, pml=10):
    """3-D heterogeneous absorbing IVP: n^3 grid including a ``pml``-point PML,
    dx = 0.1 mm, 8 random ellipsoids (c ~ U(1400,1800) m/s, rho ~ U(900,1200)
    kg/m^3, semi-axes 8-30 px at n=256, scaled with n), power-law absorption
    0.75 dB/(MHz^y cm) with y = 1.5, B/A = 6, p0 = 20 Gaussian blobs
    (sigma 2-6 px at n=256, amplitude U(1,10) Pa), binary sensor on the
    z = ``plane_z`` plane recording p and p_max.  dt from the CFL-0.3 rule of
    ``kWaveGrid.makeTime`` (kwave/kgrid.py:455-495) at the maximum sound speed."""
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    scale = n / 256.0
    c = np.full(shape, 1500.0)
    rho = np.full(shape, 1000.0)
    lo, hi = pml, n - pml
    for _ in range(8):
        ctr = rng.uniform(lo, hi, size=3)
        semi = rng.uniform(8, 30, size=3) * scale
        R = _random_rotation(rng)
        cv = rng.uniform(1400, 1800)
        rv = rng.uniform(900, 1200)
        r = int(np.ceil(semi.max())) + 1
        sl = tuple(slice(max(0, int(ci) - r), min(n, int(ci) + r + 1)) for ci in ctr)
        g = np.meshgrid(*[np.arange(s.start, s.stop) for s in sl], indexing="ij")
        x = np.stack([gi - ci for gi, ci in zip(g, ctr)], axis=-1) @ R
        inside = np.sum((x / semi) ** 2, axis=-1) <= 1.0
        c[sl][inside] = cv
        rho[sl][inside] = rv
    p0 = np.zeros(shape)
    for _ in range(20):
        ctr = rng.uniform(lo, hi, size=3)
        sig = rng.uniform(2, 6) * scale
        amp = rng.uniform(1, 10)
        r = int(np.ceil(5 * sig)) + 1
        sl = tuple(slice(max(0, int(ci) - r), min(n, int(ci) + r + 1)) for ci in ctr)
        g = np.meshgrid(*[np.arange(s.start, s.stop) for s in sl], indexing="ij")
        r2 = sum((gi - ci) ** 2 for gi, ci in zip(g, ctr))
        p0[sl] += amp * np.exp(-r2 / (2 * sig * sig))
    dx = 1e-4
    dt = 0.3 * dx / float(c.max())
    mask = np.zeros(shape, bool)
    mask[:, :, plane_z] = True
    return dict(shape=shape, spacing=(dx, dx, dx), dt=dt, Nt=nt, sound_speed=c, density=rho,
                alpha_coeff=0.75, alpha_power=1.5, BonA=6.0, p0=p0, smooth_p0=True,
                sensor_mask=mask, record=("p", "p_max"), pml_size=(pml,) * 3, pml_alpha=(2.0,) * 3,
                use_sg=True, use_kspace=True)
