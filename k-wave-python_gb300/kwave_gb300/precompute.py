"""Host-side setup of the GB300 time loop: computed once in FP64, stored in FP32.

Restates the setup half of ``Simulation`` (kwave/solvers/kspace_solver.py
:205-689) for the device plan:

* grid/medium parsing and scalar-vs-grid handling (:205-241, :48-57);
* sensor parsing: binary masks, Cartesian points as multilinear stencils,
  ``record`` expansion and ``record_start_index`` (:243-361);
* PML vectors (kwave/utils/pml.py:6-64), k vectors, operator tables
  (:408-447), absorption/dispersion/nonlinearity coefficients (:449-550,
  kwave/utils/conversion.py:20-35);
* source scaling (:552-645, :60-114) and the staggered density (:647-666,
  :798-809);
* p0 smoothing with the rotated Blackman window (kwave/utils/filters.py
  :549-615, kwave/utils/signals.py:58-283).

Spectral operators are handed to the device as 1-D tables without kappa;
kappa and |k|^a are evaluated per cell on the device.  Each 1-D complex table
is replaced by its Hermitian part (it differs from the reference table only at
an even-length Nyquist bin, where the value becomes real).  With that, the
half-spectrum real inverse transform returns exactly Re(ifftn(op * fftn(f)))
as the reference computes it (:705, :796).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

AXES = "xyz"


# ---------------------------------------------------------------------------
# reading kwave-style objects
# ---------------------------------------------------------------------------

def _get(obj, name, default=None):
    if obj is None:
        return default
    if isinstance(obj, dict):
        return obj.get(name, default)
    return getattr(obj, name, default)


def _enabled(x) -> bool:
    """Zero scalars/arrays mean 'disabled' (kspace_solver.py:23-24)."""
    if x is None:
        return False
    if hasattr(x, "__len__"):
        # any non-zero (NaN included), without a temporary mask; grids in slabs on the pool
        return bool(_par_reduce(np.asarray(x), np.any, any))
    return x != 0


_PAR_MIN = 1 << 20  # elements below which a reduction runs on the calling thread


def _par_reduce(arr, fn, combine):
    """``fn`` over ``arr`` as ``combine`` of ``fn`` over slabs along axis 0
    on the worker pool (exact for max, min, any: no rounding involved)."""
    if arr.ndim == 0 or arr.size < _PAR_MIN or arr.shape[0] < 2:
        return fn(arr)
    n0 = arr.shape[0]
    nslab = min(n0, 4 * (_pool()._max_workers))
    bounds = [(i * n0 // nslab, (i + 1) * n0 // nslab) for i in range(nslab)]
    return combine(_pool().map(lambda ab: fn(arr[ab[0]:ab[1]]), [ab for ab in bounds if ab[1] > ab[0]]))


def grid_of(kgrid):
    """(shape, spacing, Nt, dt) from a kWaveGrid (N/spacing) or an Nx/dx namespace
    (kspace_solver.py:210-226)."""
    shape, spacing = grid_shape_of(kgrid)
    return shape, spacing, int(_get(kgrid, "Nt")), float(_get(kgrid, "dt"))


def grid_shape_of(kgrid):
    """(shape, spacing) of a kWaveGrid or an Nx/dx namespace, whatever its
    time axis holds."""
    if _get(kgrid, "N") is not None and _get(kgrid, "spacing") is not None:
        shape = tuple(int(n) for n in np.atleast_1d(_get(kgrid, "N")))
        spacing = tuple(float(d) for d in np.atleast_1d(_get(kgrid, "spacing")))
    else:
        shape, spacing = [], []
        for ax in AXES:
            n, d = _get(kgrid, f"N{ax}"), _get(kgrid, f"d{ax}")
            if n is None or d is None:
                break
            shape.append(int(n))
            spacing.append(float(d))
        shape, spacing = tuple(shape), tuple(spacing)
    return shape, spacing


def problem_from_kwave(kgrid, medium, source, sensor, *, pml_size=None, pml_alpha=None, use_sg=True,
                       use_kspace=True, smooth_p0=True):
    """Collect the inputs the time loop reads into one plain dict."""
    shape, spacing, Nt, dt = grid_of(kgrid)
    prob = dict(shape=shape, spacing=spacing, Nt=Nt, dt=dt, pml_size=pml_size, pml_alpha=pml_alpha,
                use_sg=bool(use_sg), use_kspace=bool(use_kspace), smooth_p0=bool(smooth_p0))
    for k in ("sound_speed", "density", "alpha_coeff", "alpha_power", "alpha_mode", "BonA"):
        v = _get(medium, k)
        if v is not None:
            prob[k] = v.value if hasattr(v, "value") and not isinstance(v, np.ndarray) else v
    for k in ("p0", "p_mask", "p", "p_mode", "u_mask", "ux", "uy", "uz", "u_mode"):
        v = _get(source, k)
        if v is not None:
            prob[k] = v
    prob["sensor_mask"] = _get(sensor, "mask")
    prob["record"] = _get(sensor, "record")
    prob["record_start_index"] = _get(sensor, "record_start_index")
    return prob


# ---------------------------------------------------------------------------
# FP64 formulas
# ---------------------------------------------------------------------------

def expand_to_grid(val, shape, name):
    """kspace_solver.py:48-57; returns a Python float for scalars."""
    if val is None:
        raise ValueError(f"Missing required parameter: {name}")
    raw = np.asarray(val)
    n = int(np.prod(shape))
    if raw.size == 1:
        return float(np.asarray(raw, dtype=np.float64).ravel()[0])
    if raw.size == n:
        if raw.dtype == np.float64:
            return raw.reshape(shape)
        src = raw.reshape(shape)
        return _par_fill(tuple(shape), lambda i, j: src[i:j], dtype=np.float64)
    raise ValueError(f"{name} size {raw.size} incompatible with grid size {n}")


def pml_profile(N, dx, dt, c, size, alpha, staggered):
    """kwave/utils/pml.py:6-64 (1-D, FP64)."""
    x = np.arange(1, size + 1, dtype=np.float64)
    if staggered:
        left = alpha * (c / dx) * ((((x + 0.5) - size - 1) / (0 - size)) ** 4)
        right = alpha * (c / dx) * (((x + 0.5) / size) ** 4)
    else:
        left = alpha * (c / dx) * (((x - size - 1) / (0 - size)) ** 4)
        right = alpha * (c / dx) * ((x / size) ** 4)
    out = np.ones(N)
    out[:size] = np.exp(-left * dt / 2)
    out[N - size:] = np.exp(-right * dt / 2)
    return out


def db2neper(alpha, y):
    """kwave/utils/conversion.py:20-35."""
    return 100.0 * alpha * (1e-6 / (2.0 * math.pi)) ** y / (20.0 * math.log10(math.e))


def hermitian_part(table):
    """(f(k) + conj f(-k)) / 2 for a 1-D table in FFT order."""
    n = table.shape[0]
    neg = np.conj(table[(-np.arange(n)) % n])
    return 0.5 * (table + neg)


def blackman_rotated(shape):
    """Rotated Blackman window of kwave/utils/signals.py:222-283 as used by
    kwave/utils/filters.py:586-596 (even sizes enlarged by one, then trimmed)."""
    N = np.array(shape, dtype=int)
    sym = (N % 2).astype(bool)
    Ne = N + (1 - sym.astype(int))
    L = int(Ne.max())
    n = np.arange(L)
    a = 0.16
    win_lin = (1 - a) / 2 - 0.5 * np.cos(2 * np.pi * n / (L - 1)) + (a / 2) * np.cos(4 * np.pi * n / (L - 1))
    radius = (L - 1) / 2
    ll = np.linspace(-radius, radius, L)
    r2 = None
    for ax, m in enumerate(Ne):
        c = np.linspace(-radius, radius, int(m)) ** 2
        sh = [1] * len(Ne)
        sh[ax] = int(m)
        c = c.reshape(sh)
        r2 = c if r2 is None else r2 + c
    r = np.sqrt(r2)
    r = np.minimum(r, radius)
    win = np.interp(r, ll, win_lin)
    return np.abs(win[tuple(slice(0, int(m)) for m in N)])


def smoothing_tables(shape):
    """1-D description of the rotated Blackman window of kwave/utils/signals.py
    :222-283 as used by kwave/utils/filters.py:586-601 (even sizes enlarged by
    one, then trimmed; applied after ifftshift): the window samples on
    [-radius, radius] and, per axis, the squared coordinate of every FFT index.
    The device evaluates window(min(sqrt(sum c^2), radius)) per cell."""
    N = np.array(shape, dtype=int)
    sym = (N % 2).astype(bool)
    Ne = N + (1 - sym.astype(int))
    L = int(Ne.max())
    n = np.arange(L)
    a = 0.16
    win_lin = (1 - a) / 2 - 0.5 * np.cos(2 * np.pi * n / (L - 1)) + (a / 2) * np.cos(4 * np.pi * n / (L - 1))
    radius = (L - 1) / 2
    coords = []
    for m, ne in zip(N, Ne):
        xx = np.linspace(-radius, radius, int(ne))[: int(m)]
        idx = (np.arange(m) + m // 2) % m  # ifftshift
        coords.append((xx[idx] ** 2).astype(np.float32))
    return np.abs(win_lin).astype(np.float32), float(radius), coords


# ---------------------------------------------------------------------------
# slab-parallel evaluation of the per-cell set-up arrays
# ---------------------------------------------------------------------------

_POOL = None


def _pool():
    """Thread pool for the per-cell set-up arrays (NumPy releases the GIL on
    large array operations, so slabs along axis 0 run in parallel)."""
    global _POOL
    if _POOL is None:
        from concurrent.futures import ThreadPoolExecutor

        _POOL = ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)))
    return _POOL


def _par_fill(shape, fn, dtype=np.float32):
    """Array of ``shape`` and ``dtype`` (float32 by default) whose slabs [a, b)
    along axis 0 are ``fn(a, b)`` (each evaluated in FP64 and cast), computed
    in parallel."""
    out = np.empty(shape, dtype=dtype)
    n0 = shape[0]
    nslab = min(n0, 4 * (_pool()._max_workers))
    bounds = [(i * n0 // nslab, (i + 1) * n0 // nslab) for i in range(nslab)]

    def run(ab):
        a, b = ab
        if b > a:
            out[a:b] = fn(a, b)

    list(_pool().map(run, bounds))
    return out


def _stagger_slab(arr, axis, a, b):
    """``stagger(arr, axis)[a:b]`` computed from the slab (and, along axis 0,
    the next plane)."""
    if axis != 0:
        return stagger(arr[a:b], axis)
    n0 = arr.shape[0]
    hi_end = min(b + 1, n0)
    lo = arr[a:min(b, n0 - 1)]
    hi = arr[a + 1:hi_end]
    avg = 0.5 * (lo + hi)
    if b == n0:
        return np.concatenate([avg, arr[n0 - 1:n0]], axis=0)
    return avg


def stagger(arr, axis):
    """Neighbour mean along ``axis``, last plane copied (kspace_solver.py:798-809)."""
    lo = [slice(None)] * arr.ndim
    hi = [slice(None)] * arr.ndim
    lo[axis], hi[axis] = slice(None, -1), slice(1, None)
    avg = 0.5 * (arr[tuple(lo)] + arr[tuple(hi)])
    last = [slice(None)] * arr.ndim
    last[axis] = slice(-1, None)
    return np.concatenate([avg, arr[tuple(last)]], axis=axis)


# ---------------------------------------------------------------------------
# the setup record
# ---------------------------------------------------------------------------

@dataclass
class SourceSpec:
    slot: int                 # 0..2 pressure into rho_i, 3..5 velocity u_i
    mode: str
    index: np.ndarray         # int64 flat C-order mask indices
    signal: np.ndarray        # float32 (n_rows, length), pre-scaled


@dataclass
class Setup:
    shape: tuple
    spacing: tuple
    dt: float
    Nt: int
    ndim: int
    c_ref: float
    use_sg: bool
    use_kspace: bool
    fields: dict = field(default_factory=dict)        # name -> float32 grid or python float
    tables: dict = field(default_factory=dict)        # (kind, axis) -> float32 1-D (complex as interleaved)
    absorb_mode: int = 0
    dispersion: int = 0
    nonlinear: int = 0
    alpha_power: float = 0.0
    sources: list = field(default_factory=list)
    # medium grids left to the device (kw_plan_derive_medium): bit 0 dt/rho_sg,
    # bit 1 tau, bit 2 eta; with the absorption-coefficient grid (float32) or
    # scalar and the absorption mode
    derive: int = 0
    derive_alpha: object = None
    derive_alpha_s: float = 0.0
    sensor_kind: str = "all"                          # all | binary | cartesian
    slots: np.ndarray = None                          # int64 flat indices sampled every recorded step
    n_points: int = 0
    interp_slot: np.ndarray = None                    # int32 (n_points, 2^D)
    interp_w: np.ndarray = None                       # float64 (n_points, 2^D)
    record: set = field(default_factory=set)          # internal record set (with dependencies)
    requested: set = field(default_factory=set)       # user-requested keys
    record_start: int = 0
    pml_sizes: tuple = ()
    has_p0: bool = False
    smooth: tuple = None                              # (window, radius, coords) when p0 is smoothed


def parse_record(record, ndim):
    """Record-key expansion of kspace_solver.py:280-316."""
    record = record or ("p", "p_final")
    if isinstance(record, str):
        record = (record,)
    rec = set(record)
    axes = AXES[:ndim]
    if "u" in rec:
        rec.discard("u")
        rec.update(f"u{a}" for a in axes)
    if "u_staggered" in rec:
        rec.discard("u_staggered")
        rec.update(f"u{a}_staggered" for a in axes)
    for suf in ("_max", "_min", "_rms", "_final"):
        if f"u{suf}" in rec:
            rec.discard(f"u{suf}")
            rec.update(f"u{a}{suf}" for a in axes)
    if "I" in rec:
        rec.discard("I")
        rec.update(f"I{a}" for a in axes)
    if "I_avg" in rec:
        rec.discard("I_avg")
        rec.update(f"I{a}_avg" for a in axes)
    requested = set(rec)
    for key in list(rec):
        for suf in ("_max", "_min", "_rms"):
            if key.endswith(suf):
                rec.add(key[: -len(suf)])
    if any(k.startswith("I") for k in requested):
        rec.update(["p"] + [f"u{a}" for a in axes])
    return rec, requested


def _cartesian_stencil(cart, shape, spacing):
    """Multilinear stencil of RegularGridInterpolator(method='linear',
    bounds_error=True) on axes (arange(N) - N//2) * d (kspace_solver.py:341-359)."""
    ndim = len(shape)
    npts = cart.shape[1]
    idx, w = [], []
    for d in range(ndim):
        g = (np.arange(shape[d]) - shape[d] // 2) * spacing[d]
        x = cart[d]
        if np.any(x < g[0]) or np.any(x > g[-1]):
            raise ValueError(f"One of the requested xi is out of bounds in dimension {d}")
        i = np.clip(np.searchsorted(g, x) - 1, 0, len(g) - 2)
        idx.append(i)
        w.append((x - g[i]) / (g[i + 1] - g[i]))
    nc = 1 << ndim
    flat = np.zeros((npts, nc), np.int64)
    wt = np.ones((npts, nc))
    for c in range(nc):
        lin = np.zeros(npts, np.int64)
        for d in range(ndim):
            bit = (c >> d) & 1
            wt[:, c] *= w[d] if bit else (1.0 - w[d])
            lin = lin * shape[d] + (idx[d] + bit)
        flat[:, c] = lin
    slots, inv = np.unique(flat.ravel(), return_inverse=True)
    return slots.astype(np.int64), inv.reshape(npts, nc).astype(np.int32), wt


def build_setup(prob, derive_on_device=False) -> Setup:
    """FP64 precompute of everything the device plan needs.  With
    ``derive_on_device`` the grids of dt/rho0 on the staggered grids and of
    tau / eta are left to the device (``Setup.derive``), which forms them from
    the uploaded float32 c0 / rho0 / alpha as the reference does."""
    shape = tuple(int(n) for n in prob["shape"])
    spacing = tuple(float(d) for d in prob["spacing"])
    ndim = len(shape)
    if ndim not in (2, 3):
        raise NotImplementedError("the GB300 backend runs 2-D and 3-D grids (kspaceFirstOrder2D/3D)")
    dt, Nt = float(prob["dt"]), int(prob["Nt"])
    c0 = expand_to_grid(prob.get("sound_speed"), shape, "sound_speed")
    dens = prob.get("density")
    rho0 = expand_to_grid(dens if dens is not None else 1000.0, shape, "density")
    def f32(a):
        if isinstance(a, float):
            return a
        arr = np.asarray(a)
        return _par_fill(arr.shape, lambda i, j: arr[i:j])

    c0_32 = f32(c0)
    # c_ref = max(c0) of the FP32-cast medium (kspace_solver.py:228-231)
    c_ref = float(np.float32(c0_32)) if isinstance(c0_32, float) else float(_par_reduce(c0_32, np.max, max))
    if prob.get("c_ref") is not None:
        # held fixed by the sound-speed gradient (the reference has no such
        # input: c_ref is always max(c0)), so that PML and kappa do not move with c0
        c_ref = float(np.float32(prob["c_ref"]))
    S = Setup(shape=shape, spacing=spacing, dt=dt, Nt=Nt, ndim=ndim, c_ref=c_ref,
              use_sg=bool(prob.get("use_sg", True)), use_kspace=bool(prob.get("use_kspace", True)))
    S.fields["c0"] = c0_32
    S.fields["rho0"] = f32(rho0)

    # --- sensor (kspace_solver.py:243-361) ---
    numel = int(np.prod(shape))
    mask_raw = prob.get("sensor_mask")
    if mask_raw is None:
        S.sensor_kind = "all"
        S.slots = np.arange(numel, dtype=np.int64)
        S.n_points = numel
    else:
        m = np.asarray(mask_raw)
        if m.ndim == 2 and m.shape[0] == ndim:
            S.sensor_kind = "cartesian"
            m = np.asarray(m, dtype=float)
            S.slots, S.interp_slot, S.interp_w = _cartesian_stencil(m, shape, spacing)
            S.n_points = m.shape[1]
        elif m.size == 1 or m.size == numel:
            b = (m.ravel() if m.dtype == bool else (m != 0).ravel())
            if b.size == 1:
                b = np.full(numel, bool(b[0]))
            S.sensor_kind = "binary"
            S.slots = np.flatnonzero(b).astype(np.int64)
            S.n_points = int(S.slots.size)
        else:
            raise ValueError(f"Sensor mask shape {m.shape} is neither binary (numel={numel}) nor Cartesian ({ndim}, N_points)")
    S.record, S.requested = parse_record(prob.get("record"), ndim)
    rs = prob.get("record_start_index")
    rs = int(rs) if rs is not None else 1
    if rs < 1:
        raise ValueError(f"sensor.record_start_index must be >= 1 (1-based, MATLAB convention), got {rs}")
    if rs > Nt:
        raise ValueError(f"sensor.record_start_index ({rs}) exceeds Nt ({Nt})")
    S.record_start = rs - 1

    # --- PML (kspace_solver.py:363-406) ---
    psz, pal = prob.get("pml_size"), prob.get("pml_alpha")
    sizes = []
    for a in range(ndim):
        n = shape[a]
        ps = int(psz[a]) if psz is not None else 0
        pa = float(pal[a]) if pal is not None else 0.0
        sizes.append(ps if pa != 0 else 0)
        if ps == 0 or pa == 0:
            pml = pml_sg = np.ones(n)
        else:
            pml = pml_profile(n, spacing[a], dt, c_ref, ps, pa, staggered=False)
            pml_sg = pml_profile(n, spacing[a], dt, c_ref, ps, pa, staggered=True)
        S.tables[("pml", a)] = pml.astype(np.float32)
        S.tables[("pml_sg", a)] = pml_sg.astype(np.float32)
    S.pml_sizes = tuple(sizes)

    # --- k-space tables (kspace_solver.py:408-447, 677) ---
    for a in range(ndim):
        n, d = shape[a], spacing[a]
        k = 2 * np.pi * np.fft.fftfreq(n, d=d)
        k32 = k.astype(np.float32)
        kk = k32.astype(np.float64)
        if S.use_sg:
            fg = 1j * kk * np.exp(1j * kk * d / 2)
            fd = 1j * kk * np.exp(-1j * kk * d / 2)
        else:
            fg = 1j * kk
            fd = 1j * kk
        us = np.exp(-1j * kk * d / 2)
        S.tables[("k", a)] = k32
        for name, tb in (("op_grad", fg), ("op_div", fd), ("unstag", us)):
            h = hermitian_part(tb)
            S.tables[(name, a)] = np.stack([h.real, h.imag], axis=-1).astype(np.float32).ravel()

    # --- absorption / dispersion / nonlinearity (kspace_solver.py:449-550) ---
    ac = prob.get("alpha_coeff", 0)
    mode = prob.get("alpha_mode", None)
    if _enabled(ac):
        y = float(np.asarray(prob.get("alpha_power", 1.5), dtype=np.float64).ravel()[0])
        alpha = expand_to_grid(ac, shape, "alpha_coeff")
        S.alpha_power = y
        stokes = abs(y - 2.0) < 1e-10
        if mode == "no_absorption":
            S.absorb_mode = 0
        else:
            S.absorb_mode = 2 if stokes else 1
            S.dispersion = int(not stokes and mode not in ("no_absorption", "no_dispersion"))
            grid_in = not (isinstance(alpha, float) and isinstance(c0, float))
            if derive_on_device and grid_in:
                S.derive |= 2 | (4 if S.dispersion else 0)
                if isinstance(alpha, float):
                    S.derive_alpha_s = alpha
                else:
                    S.derive_alpha = _par_fill(tuple(shape), lambda i, j: alpha[i:j])
            elif stokes:
                a_np = db2neper(alpha, y) if isinstance(alpha, float) else db2neper(np.asarray(alpha), y)
                S.fields["tau"] = _cell_field(shape, lambda sl: -2 * _sl(a_np, sl) * _sl(c0, sl), a_np, c0)
            else:
                a_np = db2neper(alpha, y) if isinstance(alpha, float) else db2neper(np.asarray(alpha), y)
                S.fields["tau"] = _cell_field(
                    shape, lambda sl: -2 * _sl(a_np, sl) * _pow(_sl(c0, sl), y - 1), a_np, c0)
                if S.dispersion:
                    tn = math.tan(math.pi * y / 2)
                    S.fields["eta"] = _cell_field(
                        shape, lambda sl: 2 * _sl(a_np, sl) * _pow(_sl(c0, sl), y) * tn, a_np, c0)
    B = prob.get("BonA", 0)
    if _enabled(B):
        S.nonlinear = 1
        S.fields["BonA"] = f32(expand_to_grid(B, shape, "BonA"))

    # --- dt / rho0 on the staggered grids (kspace_solver.py:655-666) ---
    if derive_on_device and not isinstance(rho0, float):
        S.derive |= 1
    for a in range(ndim):
        if S.derive & 1:
            continue
        if isinstance(rho0, float):
            S.fields[f"dtrsg{a}"] = dt / rho0
        elif not S.use_sg:
            S.fields[f"dtrsg{a}"] = _par_fill(shape, lambda i, j: dt / rho0[i:j])
        else:
            S.fields[f"dtrsg{a}"] = _par_fill(shape, lambda i, j, a=a: dt / _stagger_slab(rho0, a, i, j))

    # --- sources (kspace_solver.py:552-645) ---
    S.sources = _build_sources(prob, shape, spacing, dt, c0, ndim)
    S.source_c0 = c0  # the sound speed the source scalings use (for later signal updates)

    # --- p0 (kspace_solver.py:679-689) ---
    p0r = prob.get("p0", 0)
    if _enabled(p0r):
        p0 = expand_to_grid(p0r, shape, "p0")
        if isinstance(p0, float):
            p0 = np.full(shape, p0)
        if prob.get("smooth_p0", True) and ndim >= 2:
            # smoothed on the device before the first step (kwave/utils/filters.py:549-615)
            S.smooth = smoothing_tables(shape)
        S.fields["p0"] = _par_fill(tuple(shape), lambda i, j: p0[i:j])
        S.has_p0 = True
    return S


def _sl(x, sl):
    """Slab of a grid array, or the scalar itself."""
    return x if np.ndim(x) == 0 else x[sl]


def _pow(x, e):
    return x ** e if np.ndim(x) == 0 else np.power(x, e)


def _cell_field(shape, fn, *inputs):
    """Python float when every input is a scalar, else the float32 grid of
    fn(slab) evaluated slab-parallel along axis 0."""
    if all(np.ndim(x) == 0 for x in inputs):
        return float(fn(slice(None)))
    return _par_fill(tuple(shape), lambda i, j: np.broadcast_to(fn(slice(i, j)), (j - i,) + tuple(shape[1:])))


def _fv(x):
    """Python float for scalars, C-contiguous float32 grid otherwise."""
    if np.ndim(x) == 0:
        return float(x)
    return np.ascontiguousarray(x, dtype=np.float32)


def _mask_index(mask_raw, shape):
    m = np.asarray(mask_raw, dtype=bool).ravel()
    if m.size == 1:
        m = np.full(int(np.prod(shape)), bool(m[0]))
    return np.flatnonzero(m).astype(np.int64)


def _signal_rows(sig_raw):
    s = np.asarray(sig_raw, dtype=np.float64)
    if s.ndim == 1:
        s = s.reshape(1, -1)
    elif s.ndim > 2:
        s = s.reshape(-1, s.shape[-1])
    return s


def _build_sources(prob, shape, spacing, dt, c0, ndim):
    out = []
    n = ndim

    def c_at(idx):
        return np.full(idx.size, c0) if isinstance(c0, float) else np.asarray(c0).ravel()[idx]

    pm, ps = prob.get("p_mask", 0), prob.get("p", 0)
    pmode = prob.get("p_mode", None) or "additive"
    if _enabled(pm) and _enabled(ps):
        if pmode not in ("dirichlet", "additive", "additive-no-correction"):
            raise ValueError(f"Unknown source mode: {pmode!r}. Use 'additive', 'additive-no-correction', or 'dirichlet'.")
        idx = _mask_index(pm, shape)
        sig = _signal_rows(ps)
        c = c_at(idx)
        if pmode == "additive":
            # one field 2 dt / (n c0) s; the device adds F^-1[source_kappa F[.]] / d_i to rho_i
            out.append(SourceSpec(0, pmode, idx, _scaled(sig, 2 * dt / (n * c), idx.size)))
        else:
            for i in range(n):
                scale = 1.0 / (n * c ** 2) if pmode == "dirichlet" else 2 * dt / (n * c * spacing[i])
                out.append(SourceSpec(i, pmode, idx, _scaled(sig, scale, idx.size)))
    um = prob.get("u_mask", 0)
    umode = prob.get("u_mode", None) or "additive"
    for i, v in enumerate(("ux", "uy", "uz")[:n]):
        us = prob.get(v, 0)
        if _enabled(um) and _enabled(us):
            if umode not in ("dirichlet", "additive", "additive-no-correction"):
                raise ValueError(f"Unknown source mode: {umode!r}. Use 'additive', 'additive-no-correction', or 'dirichlet'.")
            idx = _mask_index(um, shape)
            c = c_at(idx)
            scale = np.ones_like(c) if umode == "dirichlet" else 2 * c * dt / spacing[i]
            out.append(SourceSpec(3 + i, umode, idx, _scaled(_signal_rows(us), scale, idx.size)))
    return out


def _scaled(sig, scale, n_src):
    """signal * scale[:, None] (kspace_solver.py:80-88); one row if it broadcasts to one."""
    scale = np.atleast_1d(np.asarray(scale, dtype=np.float64))
    s = sig * scale[:, None]
    if s.shape[0] not in (1, n_src):
        raise ValueError(f"source signal rows ({sig.shape[0]}) do not match mask points ({n_src})")
    return np.ascontiguousarray(s, dtype=np.float32)
