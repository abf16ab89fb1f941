"""GB300 counterpart of ``kwave.solvers.kspace_solver.Simulation``.

Same constructor arguments, same ``setup() / step() / run()`` split and the
same result dictionary as the reference class (kwave/solvers/kspace_solver.py
:122-778); the time loop runs on the GPU through libkwave_gb300 (ctypes).  The
arithmetic type is float32; the sensor series and running aggregates stay on
the device until ``run()`` returns.
"""
from __future__ import annotations

import ctypes as C
import warnings

import numpy as np

from . import _lib as K
from .precompute import AXES, Setup, build_setup, problem_from_kwave

_TABLES = {"k": K.KW_T_K, "pml": K.KW_T_PML, "pml_sg": K.KW_T_PMLSG, "op_grad": K.KW_T_OPGRAD,
           "op_div": K.KW_T_OPDIV, "unstag": K.KW_T_UNSTAG}
_FIELDS = {"c0": K.KW_F_C0, "rho0": K.KW_F_RHO0, "dtrsg0": K.KW_F_DTRSG0, "dtrsg1": K.KW_F_DTRSG1,
           "dtrsg2": K.KW_F_DTRSG2, "BonA": K.KW_F_BONA, "tau": K.KW_F_TAU, "eta": K.KW_F_ETA, "p0": K.KW_F_P0}


def _series_id(key, ndim):
    if key == "p":
        return K.KW_R_P
    for i, a in enumerate(AXES[:ndim]):
        if key == f"u{a}_staggered":
            return K.KW_R_UX_ST + i
        if key == f"u{a}":
            return K.KW_R_UX + i
    return None


STATS = {"h2d_bytes": 0, "d2h_bytes": 0}


class DevicePlan:
    """Owns one kw_plan (device state of one simulation)."""

    def __init__(self, S: Setup, stream=None, generic_fft=False):
        lib = K.lib()
        K.require_device()
        self.S = S
        self.lib = lib
        self.stream = stream
        d = K.KwGridDesc()
        d.ndim = S.ndim
        for a in range(3):
            d.shape[a] = S.shape[a] if a < S.ndim else 1
            d.spacing[a] = S.spacing[a] if a < S.ndim else 1.0
        d.Nt = S.Nt
        d.record_start = S.record_start
        d.dt = S.dt
        d.c_ref = S.c_ref
        d.use_sg = int(S.use_sg)
        d.use_kspace = int(S.use_kspace)
        d.absorb_mode = S.absorb_mode
        d.dispersion = S.dispersion
        d.nonlinear = S.nonlinear
        d.alpha_power = S.alpha_power
        d.flags = K.KW_DESC_GENERIC_FFT if generic_fft else 0
        self._h = C.c_void_p()
        K.check(lib.kw_plan_create(C.byref(d), C.byref(self._h)))
        try:
            self._upload()
            K.check(lib.kw_plan_finalize(self._h))
        except BaseException:
            lib.kw_plan_destroy(self._h)
            self._h = None
            raise

    def _upload(self):
        S, lib, h = self.S, self.lib, self._h
        nbytes = 0
        for name, fid in _FIELDS.items():
            v = S.fields.get(name)
            if v is None:
                continue
            if isinstance(v, float):
                K.check(lib.kw_plan_set_field(h, fid, None, 0, C.c_float(v)))
            else:
                a = np.ascontiguousarray(v, dtype=np.float32).ravel()
                nbytes += a.nbytes
                K.check(lib.kw_plan_set_field(h, fid, K.ptr(a), a.size, C.c_float(0.0)))
        if S.derive:
            al = S.derive_alpha
            if al is not None:
                al = np.ascontiguousarray(al, dtype=np.float32).ravel()
                nbytes += al.nbytes
            K.check(lib.kw_plan_derive_medium(h, S.derive, K.ptr(al) if al is not None else None,
                                              0 if al is None else al.size, C.c_double(S.derive_alpha_s),
                                              C.c_double(S.alpha_power), S.absorb_mode))
        for (name, axis), tb in S.tables.items():
            a = np.ascontiguousarray(tb, dtype=np.float32)
            nbytes += a.nbytes
            K.check(lib.kw_plan_set_table(h, _TABLES[name], axis, K.ptr(a), a.size))
        for src in S.sources:
            idx = np.ascontiguousarray(src.index, dtype=np.int64)
            sig = np.ascontiguousarray(src.signal, dtype=np.float32)
            nbytes += idx.nbytes + sig.nbytes
            K.check(lib.kw_plan_set_source(h, src.slot, K.SRC_MODES[src.mode], K.ptr(idx), idx.size, K.ptr(sig),
                                           sig.shape[0], sig.shape[1]))
        mask = 0
        for key in S.record:
            sid = _series_id(key, S.ndim)
            if sid is not None:
                mask |= 1 << sid
        slots = np.ascontiguousarray(S.slots, dtype=np.int64)
        nbytes += slots.nbytes
        self.record_mask = mask
        K.check(lib.kw_plan_set_sensor(h, K.ptr(slots), slots.size, mask))
        if S.sensor_kind == "cartesian":
            sl = np.ascontiguousarray(S.interp_slot, dtype=np.int32)
            w = np.ascontiguousarray(S.interp_w, dtype=np.float64)
            nbytes += sl.nbytes + w.nbytes
            K.check(lib.kw_plan_set_sensor_interp(h, sl.shape[0], sl.shape[1], K.ptr(sl), K.ptr(w)))
        if S.smooth is not None:
            win, radius, coords = S.smooth
            for axis, cw in enumerate(coords):
                a = np.ascontiguousarray(cw, dtype=np.float32)
                nbytes += a.nbytes
                K.check(lib.kw_plan_set_table(h, K.KW_T_WCOORD, axis, K.ptr(a), a.size))
            w = np.ascontiguousarray(win, dtype=np.float32)
            nbytes += w.nbytes
            K.check(lib.kw_plan_set_p0_smoothing(h, K.ptr(w), w.size, C.c_double(radius)))
        self.h2d_bytes = nbytes
        STATS["h2d_bytes"] = nbytes

    @property
    def handle(self):
        return self._h

    def run(self, nsteps):
        st = C.c_void_p(self.stream) if self.stream is not None else None
        K.check(self.lib.kw_plan_run(self._h, int(nsteps), st))

    def sync(self):
        st = C.c_void_p(self.stream) if self.stream is not None else None
        K.check(self.lib.kw_plan_sync(self._h, st))

    def autotune(self, nsteps=6):
        """Pick the launch geometry of the run-time-length FFT kernels by timing
        the first ``nsteps`` steps for each candidate (kw_plan_autotune); the
        plan is left at t = 0 and results do not depend on the choice.
        Returns (tile columns, rows per block)."""
        st = C.c_void_p(self.stream) if self.stream is not None else None
        T, R = C.c_int32(), C.c_int32()
        K.check(self.lib.kw_plan_autotune(self._h, int(nsteps), st, C.byref(T), C.byref(R)))
        return T.value, R.value

    def adjoint_p0(self, residual):
        """Transposed time loop applied to a residual at the recorded grid
        points (n_slots, Nt - record_start): the gradient with respect to p0
        of sum(residual * recorded slot values) (kw_plan_adjoint_p0).  For a
        Cartesian sensor, ``adjoint.slot_residual`` maps point residuals to
        slots.  The plan is reset."""
        r = np.ascontiguousarray(residual, dtype=np.float32)
        g = np.empty(self.S.shape, np.float32)
        st = C.c_void_p(self.stream) if self.stream is not None else None
        K.check(self.lib.kw_plan_adjoint_p0(self._h, K.ptr(r), r.size, K.ptr(g), st))
        return g

    def update_p0(self, p0):
        """New initial pressure for this plan (kw_plan_update_p0); rewinds to t = 0."""
        a = np.ascontiguousarray(p0, dtype=np.float32).ravel()
        K.check(self.lib.kw_plan_update_p0(self._h, K.ptr(a), a.size))
        STATS["h2d_bytes"] += a.nbytes

    def update_sources(self, prob):
        """New source signals from problem dict ``prob`` (same masks and modes
        as this plan's), scaled as at set-up (kw_plan_update_source); rewinds
        the plan to t = 0."""
        from .precompute import _build_sources

        S = self.S
        for src in _build_sources(prob, S.shape, S.spacing, S.dt, S.source_c0, S.ndim):
            sig = np.ascontiguousarray(src.signal, dtype=np.float32)
            K.check(self.lib.kw_plan_update_source(self._h, src.slot, K.ptr(sig), sig.shape[0], sig.shape[1]))
            STATS["h2d_bytes"] += sig.nbytes
        K.check(self.lib.kw_plan_reset(self._h))

    def set_checkpoints(self, interval):
        """Keep the carried state every ``interval`` steps of the coming
        forward run (kw_plan_set_checkpoints); 0 turns them off."""
        K.check(self.lib.kw_plan_set_checkpoints(self._h, int(interval)))

    def adjoint(self, residual, grad_c=False):
        """kw_plan_adjoint: (gradient w.r.t. p0, gradient w.r.t. c0 or None) of
        sum(residual * recorded slot values).  ``grad_c`` needs this plan's
        forward run to Nt with p0 set and checkpoints on.  The plan is reset."""
        r = np.ascontiguousarray(residual, dtype=np.float32)
        g = np.empty(self.S.shape, np.float32)
        gc = np.empty(self.S.shape, np.float32) if grad_c else None
        st = C.c_void_p(self.stream) if self.stream is not None else None
        K.check(self.lib.kw_plan_adjoint(self._h, K.ptr(r), r.size, K.ptr(g), K.ptr(gc) if grad_c else None, st))
        return g, gc

    def set_radix_order(self, order):
        """Radix schedule of the run-time-length FFTs (kw_plan_set_radix_order)."""
        K.check(self.lib.kw_plan_set_radix_order(self._h, int(order)))

    def set_graphs(self, enable):
        """Run repeated steps as replayed CUDA graphs (default) or as plain launches."""
        K.check(self.lib.kw_plan_set_graphs(self._h, int(bool(enable))))

    def time_index(self):
        t = C.c_int32()
        K.check(self.lib.kw_plan_time_index(self._h, C.byref(t)))
        return t.value

    def read_series(self, sid):
        n_rec = self.S.Nt - self.S.record_start
        out = np.empty((self.S.n_points, n_rec), np.float32)
        K.check(self.lib.kw_plan_read_series(self._h, sid, K.ptr(out), out.size))
        STATS["d2h_bytes"] += out.nbytes
        return out

    def read_aggregate(self, sid, kind):
        out = np.empty(self.S.n_points, np.float32)
        K.check(self.lib.kw_plan_read_aggregate(self._h, sid, kind, K.ptr(out), out.size))
        STATS["d2h_bytes"] += out.nbytes
        return out

    def read_field(self, fid):
        out = np.empty(self.S.shape, np.float32)
        K.check(self.lib.kw_plan_read_field(self._h, fid, K.ptr(out), out.size))
        STATS["d2h_bytes"] += out.nbytes
        return out

    def close(self):
        if getattr(self, "_h", None):
            self.lib.kw_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Simulation:
    """GB300 k-space pseudospectral propagator with the reference's interface.

    ``Simulation(kgrid, medium, source, sensor, *, device, use_sg, use_kspace,
    smooth_p0, pml_size, pml_alpha, quiet, dtype).run()`` mirrors
    kwave/solvers/kspace_solver.py:135-203; ``device`` is accepted for
    signature compatibility and must be "gpu" (there is no CPU path).
    """

    def __init__(self, kgrid, medium, source, sensor, *, device="gpu", use_sg=True, use_kspace=True, smooth_p0=True,
                 pml_size=None, pml_alpha=None, quiet=False, dtype=None, stream=None):
        if device not in ("gpu", "cuda", "auto"):
            raise ValueError(f"Unknown device {device!r}. The GB300 backend runs on the GPU only.")
        if dtype is not None and np.dtype(dtype) != np.float32:
            raise NotImplementedError("the GB300 backend computes in float32 (dtype=np.float32)")
        if pml_size is None and hasattr(kgrid, "N"):
            warnings.warn("Simulation received a kWaveGrid without explicit pml_size; PML will be disabled.",
                          UserWarning, stacklevel=2)
        self.prob = problem_from_kwave(kgrid, medium, source, sensor, pml_size=pml_size, pml_alpha=pml_alpha,
                                       use_sg=use_sg, use_kspace=use_kspace, smooth_p0=smooth_p0)
        self.quiet = quiet
        self.stream = stream
        self._plan = None
        self.t = 0

    @classmethod
    def from_problem(cls, prob, stream=None):
        obj = cls.__new__(cls)
        obj.prob = dict(prob)
        obj.quiet = True
        obj.stream = stream
        obj._plan = None
        obj.t = 0
        return obj

    # -- setup / stepping ---------------------------------------------------
    def setup(self, generic_fft=False, autotune=False):
        """Host set-up and device plan.  ``generic_fft`` runs every pass with
        the run-time-length FFT kernels (what lets a batch group the plan's
        passes with other plans); the default picks the fastest kernels for
        the grid.  ``autotune`` times the candidate launch geometries of the
        run-time-length kernels on the first steps and keeps the fastest."""
        self.S = build_setup(self.prob, derive_on_device=True)
        self._plan = DevicePlan(self.S, stream=self.stream, generic_fft=generic_fft)
        if autotune:
            self.tuned = self._plan.autotune()
        self.t = 0
        return self

    @property
    def Nt(self):
        return self.S.Nt

    def step(self):
        if self._plan is None:
            self.setup()
        if self.t < self.S.Nt:
            self._plan.run(1)
            self.t = self._plan.time_index()
        return self

    def run(self):
        if self._plan is None:
            self.setup()
        self._plan.run(self.S.Nt - self.t)
        self._plan.sync()
        self.t = self._plan.time_index()
        return self.results()

    # -- fields (host copies) -------------------------------------------------
    @property
    def p(self):
        return self._plan.read_field(K.KW_FLD_P)

    @property
    def u(self):
        return [self._plan.read_field(K.KW_FLD_U0 + i) for i in range(self.S.ndim)]

    @property
    def rho_split(self):
        return [self._plan.read_field(K.KW_FLD_RHO0 + i) for i in range(self.S.ndim)]

    # -- results (kspace_solver.py:763-778) --------------------------------------
    def results(self):
        S, plan = self.S, self._plan
        out = {}
        for key in sorted(S.record):
            sid = _series_id(key, S.ndim)
            if sid is None:
                continue
            if key in S.requested:
                out[key] = plan.read_series(sid)
            for suf, kind in (("_max", K.KW_AGG_MAX), ("_min", K.KW_AGG_MIN), ("_rms", K.KW_AGG_RMS)):
                if key + suf in S.requested:
                    out[key + suf] = plan.read_aggregate(sid, kind)
        if any(k.startswith("I") for k in S.requested):
            series = {"p": plan.read_series(K.KW_R_P)}
            for i, a in enumerate(AXES[: S.ndim]):
                series[f"u{a}"] = plan.read_series(K.KW_R_UX + i)
            out.update(acoustic_intensity(series))
        interior = tuple(slice(s, N - s if s else None) for s, N in zip(S.pml_sizes, S.shape))
        if "p_final" in S.requested:
            out["p_final"] = plan.read_field(K.KW_FLD_P)[interior].copy()
        for i, a in enumerate(AXES[: S.ndim]):
            if f"u{a}_final" in S.requested:
                out[f"u{a}_final"] = plan.read_field(K.KW_FLD_U0 + i)[interior].copy()
        return {k: v for k, v in out.items() if k in S.requested}

    def close(self):
        if self._plan is not None:
            self._plan.close()
            self._plan = None


def acoustic_intensity(result):
    """Intensity from the recorded p and non-staggered u series: u is shifted
    forward half a time step by a temporal Fourier interpolant, then I = p u
    and its time average (kwave/solvers/kspace_solver.py:840-862).  This is
    post-processing of the returned series, done on the host as in the
    reference."""
    p = result["p"]
    n = p.shape[-1]
    freq = 2 * np.pi * np.arange(-(n // 2), n - n // 2) / n
    shift = np.fft.ifftshift(np.exp(1j * freq * 0.5))
    out = {}
    for a in "xyz":
        u = result.get(f"u{a}")
        if u is None:
            continue
        us = np.real(np.fft.ifft(shift * np.fft.fft(u, axis=-1), axis=-1))
        out[f"I{a}"] = p * us
        out[f"I{a}_avg"] = np.mean(out[f"I{a}"], axis=-1)
    return out


class SimulationBatch:
    """Independent simulations advanced together on one stream (kw_batch).

    Each member keeps its own grid size, medium, sources, sensor and results.
    Every step of all members is one CUDA graph launch.  By default each
    member uses the kernels picked for its grid and joins that graph as a
    parallel branch holding its own step graph.  With ``grouped=True`` the
    members set up here use the run-time-length FFT kernels, and the k-th pass
    of every member runs in one grouped launch over all of them (a handful of
    launches per step whatever the batch size).  ``autotune=True`` times
    candidate launch geometries of the run-time-length FFT kernels on the
    batch's first steps and keeps the fastest (results do not depend on it).
    The reference has no batch object: it runs ``Simulation.run()``
    (kwave/solvers/kspace_solver.py:749-778) once per simulation, and a loop
    over members here gives the same results.
    """

    def __init__(self, sims, stream=None, grouped=False, autotune=False, radix=False):
        self.sims = list(sims)
        if not self.sims:
            raise ValueError("SimulationBatch needs at least one simulation")
        self.stream = stream
        for s in self.sims:
            if s._plan is None:
                s.stream = stream
                s.setup(generic_fft=grouped)
        lib = K.lib()
        self.lib = lib
        handles = (C.c_void_p * len(self.sims))(*[s._plan.handle for s in self.sims])
        self._h = C.c_void_p()
        K.check(lib.kw_batch_create(handles, len(self.sims), C.byref(self._h)))
        self.tuned = None
        if autotune:
            self.tuned = self.autotune()
        self.radix_order = 0
        if radix:
            self.radix_order = self.autotune_radix()

    def autotune(self, nsteps=8):
        """One launch geometry of the run-time-length kernels for all members,
        timed on the batch itself (kw_batch_autotune); every member must be at
        t = 0 and is rewound there.  Returns (tile columns, rows-per-block factor)."""
        st = C.c_void_p(self.stream) if self.stream is not None else None
        T, num, den = C.c_int32(), C.c_int32(), C.c_int32()
        K.check(self.lib.kw_batch_autotune(self._h, int(nsteps), st, C.byref(T), C.byref(num), C.byref(den)))
        for s in self.sims:
            s.t = s._plan.time_index()
        return T.value, num.value / den.value

    def set_radix_order(self, order):
        """The same FFT schedule for every member (kw_batch_set_radix_order;
        0-2 Stockham radix orders, 3 the two-level schedule)."""
        K.check(self.lib.kw_batch_set_radix_order(self._h, int(order)))
        self.radix_order = int(order)

    def autotune_radix(self, nsteps=8):
        """One radix schedule of the run-time-length FFTs for all members,
        timed on the batch itself (kw_batch_autotune_radix); every member must
        be at t = 0 and is rewound there.  Schedules differ in rounding, within
        the parity bar.  Returns the schedule index."""
        st = C.c_void_p(self.stream) if self.stream is not None else None
        o = C.c_int32()
        K.check(self.lib.kw_batch_autotune_radix(self._h, int(nsteps), st, C.byref(o)))
        for s in self.sims:
            s.t = s._plan.time_index()
        return o.value

    @classmethod
    def from_problems(cls, problems, stream=None, grouped=False, autotune=False, radix=False):
        return cls([Simulation.from_problem(p, stream=stream) for p in problems], stream=stream, grouped=grouped,
                   autotune=autotune, radix=radix)

    def launch_count(self):
        c = C.c_int64()
        K.check(self.lib.kw_batch_launch_count(self._h, C.byref(c)))
        return c.value

    def graph_launches(self):
        """Graph launches of the batch's steps so far (kw_batch_graph_launches)."""
        c = C.c_int64()
        K.check(self.lib.kw_batch_graph_launches(self._h, C.byref(c)))
        return c.value

    def set_loops(self, enable):
        """Runs of steps with one launch sequence as one device-side loop
        launch (default) or one launch per step (kw_batch_set_loops)."""
        K.check(self.lib.kw_batch_set_loops(self._h, int(bool(enable))))

    def run_steps(self, nsteps):
        st = C.c_void_p(self.stream) if self.stream is not None else None
        K.check(self.lib.kw_batch_run(self._h, int(nsteps), st))
        for s in self.sims:
            s.t = s._plan.time_index()

    def run(self):
        """Run every member to its Nt and return the list of result dictionaries."""
        self.run_steps(max(s.S.Nt - s.t for s in self.sims))
        self.sims[0]._plan.sync()
        return [s.results() for s in self.sims]

    def close(self):
        if getattr(self, "_h", None):
            self.lib.kw_batch_destroy(self._h)
            self._h = None
        for s in self.sims:
            s.close()

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                self.lib.kw_batch_destroy(self._h)
                self._h = None
        except Exception:
            pass


def run_batch(problems, stream=None, grouped=False, autotune=False, radix=False):
    """Set up, run together and close the simulations described by plain problem dicts."""
    b = SimulationBatch.from_problems(problems, stream=stream, grouped=grouped, autotune=autotune, radix=radix)
    try:
        return b.run()
    finally:
        b.close()


def run_problem(prob, stream=None):
    """Set up, run and close one simulation described by a plain problem dict."""
    sim = Simulation.from_problem(prob, stream=stream)
    try:
        return sim.run()
    finally:
        sim.close()
