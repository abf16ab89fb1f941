"""Gradients of sensor-data misfits with respect to the initial pressure and the sound speed.

The reference has no adjoint.  These functions run the transposed time loop
of the lossless, source-free step (kwave/solvers/kspace_solver.py:691-747
with alpha = 0, B/A = 0) on the GPU (``kw_plan_adjoint_p0``).  It is exact
to float32 rounding, because the transpose of every spectral operator of the
step is another operator of the step (G_i^T = -D_i).

* ``p0_gradient(prob, p0, d_obs)`` returns the misfit 1/2 ||d(p0) - d_obs||^2
  and its gradient with respect to p0, for a problem dict with a sensor
  recording p and ``smooth_p0`` False.  A Cartesian sensor records grid
  points ("slots") on the device and interpolates them multilinearly at the
  end; its residual goes back to the slots through the transpose of that
  interpolation (``slot_residual``) before the device adjoint.
* ``SensorData`` is a ``torch.autograd.Function`` with p0 mapped to the
  recorded pressure; its backward is the adjoint.
* ``misfit_gradients(prob, p0, d_obs, c)`` adds the gradient with respect to
  the sound speed (c_ref held fixed).  The transposed step needs the forward
  density sum of every step; the forward run keeps its carried state every K
  steps and the adjoint regenerates each segment from its checkpoint
  (``kw_plan_set_checkpoints`` / ``kw_plan_adjoint``).  ``SensorDataPC`` is
  the autograd Function of (p0, c0).
"""
from __future__ import annotations

import numpy as np

from .solver import Simulation


def _require_unsmoothed(prob, who):
    """The adjoint is the transpose of the linear map p0 -> recorded p; the
    restore-max smoothing of p0 (kwave/utils/filters.py:549-615) is not
    linear, and an unset ``smooth_p0`` means True (kspace_solver.py:145)."""
    if prob.get("smooth_p0", True):
        raise ValueError(f"{who} needs smooth_p0=False (restore-max smoothing is not linear)")


def _plan_for(prob):
    q = dict(prob)
    q["p0"] = None
    q["record"] = ("p",)
    sim = Simulation.from_problem(q)
    sim.setup()
    return sim


def forward_p0(prob, p0):
    """Recorded pressure (n_points, Nt - record_start) for initial pressure p0."""
    q = dict(prob)
    q["p0"] = np.asarray(p0, np.float64)
    q["record"] = ("p",)
    sim = Simulation.from_problem(q)
    try:
        return sim.run()["p"]
    finally:
        sim.close()


def slot_residual(S, residual):
    """Residual at the sensor's recorded grid points: the identity for binary
    sensors; for Cartesian ones the transpose of the multilinear
    interpolation (``Setup.interp_slot`` / ``interp_w``, the weights of
    kspace_solver.py:341-359)."""
    r = np.asarray(residual, np.float64)
    if S.sensor_kind != "cartesian":
        return r
    npts, nc = S.interp_slot.shape
    if r.shape[0] != npts:
        raise ValueError(f"residual has {r.shape[0]} rows, the sensor {npts} points")
    out = np.zeros((S.slots.size, r.shape[1]))
    np.add.at(out, S.interp_slot.ravel(), (S.interp_w[:, :, None] * r[:, None, :]).reshape(npts * nc, -1))
    return out


def adjoint_p0(prob, residual):
    """Gradient with respect to p0 of sum(residual * recorded p)."""
    _require_unsmoothed(prob, "adjoint_p0")
    sim = _plan_for(prob)
    try:
        return sim._plan.adjoint_p0(slot_residual(sim.S, residual))
    finally:
        sim.close()


def p0_gradient(prob, p0, d_obs):
    """(misfit, gradient) of 1/2 ||d(p0) - d_obs||^2 with respect to p0."""
    _require_unsmoothed(prob, "p0_gradient")
    d = forward_p0(prob, p0)
    r = d.astype(np.float64) - np.asarray(d_obs, np.float64)
    return 0.5 * float(np.sum(r * r)), adjoint_p0(prob, r)


def fixed_c_ref(prob):
    """c_ref of the base problem, max(c0) of the float32 medium
    (kspace_solver.py:228-231); the sound-speed gradient holds it fixed."""
    c = prob.get("sound_speed")
    return float(np.max(np.asarray(c, np.float32)))


def default_checkpoint_interval(nt, ndim):
    """Interval K that minimises checkpoint memory (Nt / K slots of 2 D + 2
    fields) plus the segment buffer (K fields): K = sqrt(Nt (2 D + 2))."""
    return max(1, int(round(np.sqrt(nt * (2 * ndim + 2)))))


def _forward_plan(prob, p0, c, checkpoint_interval):
    q = dict(prob)
    q["p0"] = np.asarray(p0, np.float64)
    q["record"] = ("p",)
    q["c_ref"] = fixed_c_ref(prob)
    if c is not None:
        q["sound_speed"] = np.asarray(c, np.float64)
    sim = Simulation.from_problem(q).setup()
    K = checkpoint_interval or default_checkpoint_interval(sim.S.Nt, sim.S.ndim)
    sim._plan.set_checkpoints(int(K))
    return sim, sim.run()["p"]


def misfit_gradients(prob, p0, d_obs, c=None, checkpoint_interval=None):
    """(misfit, gradient w.r.t. p0, gradient w.r.t. c0) of 1/2 ||d(p0, c) -
    d_obs||^2 on the GPU: one forward run keeping checkpoints every
    ``checkpoint_interval`` steps (default ``default_checkpoint_interval``),
    then the transposed loop, which regenerates the forward density sums from
    the checkpoints segment by segment (kw_plan_adjoint).  ``c`` defaults to
    the problem's sound speed; c_ref (PML, kappa) stays at the problem's
    max(c0), so the gradient is that of the map with c_ref fixed."""
    _require_unsmoothed(prob, "misfit_gradients")
    sim, d = _forward_plan(prob, p0, c, checkpoint_interval)
    try:
        r = d.astype(np.float64) - np.asarray(d_obs, np.float64)
        g_p0, g_c = sim._plan.adjoint(slot_residual(sim.S, r), grad_c=True)
    finally:
        sim.close()
    return 0.5 * float(np.sum(r * r)), g_p0, g_c


def steepest_descent_p0(forward, adjoint, d_obs, p_init, iterations, p_true=None):
    """Steepest descent on the quadratic misfit 1/2 ||F p - d_obs||^2 with the
    exact line search of a linear F: g = F^T r, alpha = |g|^2 / |F g|^2,
    p <- p - alpha g, r <- r - alpha F g.  Two passes per iteration (one
    adjoint, one forward).  ``forward``/``adjoint`` map p0 -> recorded data
    and residual -> gradient (``forward_p0`` / ``adjoint_p0`` bound to a
    problem on the GPU).  Returns p and the history of (misfit, relative p
    error or None)."""
    p = np.array(p_init, np.float64)
    r = np.asarray(forward(p), np.float64) - np.asarray(d_obs, np.float64)
    hist = []
    for _ in range(int(iterations)):
        g = np.asarray(adjoint(r), np.float64)
        fg = np.asarray(forward(g), np.float64)
        den = float(np.sum(fg * fg))
        if den == 0.0:
            break
        alpha = float(np.sum(g * g)) / den
        p -= alpha * g
        r -= alpha * fg
        err = None if p_true is None else float(np.linalg.norm(p - p_true) / np.linalg.norm(p_true))
        hist.append((0.5 * float(np.sum(r * r)), err))
    return p, hist


class LinearP0:
    """The linear map p0 -> recorded p of one problem (lossless, source-free,
    smoothing off) on ONE device plan kept for many passes: ``forward(p0)``
    uploads p0 into the plan (kw_plan_update_p0) and runs it, ``adjoint(r)``
    runs the transposed loop on the same plan (kw_plan_adjoint).  What the
    reconstruction drivers call, without a host set-up per pass."""

    def __init__(self, prob, stream=None):
        _require_unsmoothed(prob, "LinearP0")
        q = dict(prob)
        q["p0"] = np.ones(tuple(prob["shape"]))  # a grid placeholder (zero means "no p0"); every pass replaces it
        q["record"] = ("p",)
        self.sim = Simulation.from_problem(q, stream=stream).setup()
        self.plan = self.sim._plan
        self.S = self.sim.S
        self.passes = 0

    def forward(self, p0):
        self.plan.update_p0(np.asarray(p0, np.float64))
        self.plan.run(self.S.Nt)
        self.plan.sync()
        self.passes += 1
        return self.sim.results()["p"]

    def adjoint(self, residual):
        self.passes += 1
        return self.plan.adjoint(slot_residual(self.S, residual))[0]

    def close(self):
        self.sim.close()


def cgls_p0(forward, adjoint, d_obs, p_init, iterations, p_true=None, on_iteration=None):
    """Conjugate gradients on the normal equations (CGLS) of the linear
    least-squares problem min 1/2 ||F p - d_obs||^2 -- the same two passes
    per iteration as steepest descent (one adjoint, one forward), with
    search directions conjugate in F^T F:

        r = d_obs - F p,  s = F^T r,  q = s,  gamma = |s|^2
        loop: w = F q,  alpha = gamma / |w|^2,  p += alpha q,  r -= alpha w,
              s = F^T r,  beta = |s|^2 / gamma,  gamma = |s|^2,  q = s + beta q

    Returns p and the history of (misfit, relative p error or None).
    ``on_iteration(i, p)`` is called after each iteration when given."""
    p = np.array(p_init, np.float64)
    r = np.asarray(d_obs, np.float64) - np.asarray(forward(p), np.float64)
    s = np.asarray(adjoint(r), np.float64)
    q = s.copy()
    gamma = float(np.sum(s * s))
    hist = []
    for i in range(int(iterations)):
        if gamma == 0.0:
            break
        w = np.asarray(forward(q), np.float64)
        den = float(np.sum(w * w))
        if den == 0.0:
            break
        alpha = gamma / den
        p += alpha * q
        r -= alpha * w
        err = None if p_true is None else float(np.linalg.norm(p - p_true) / np.linalg.norm(p_true))
        hist.append((0.5 * float(np.sum(r * r)), err))
        if on_iteration is not None:
            on_iteration(i, p)
        if i + 1 == int(iterations):
            break
        s = np.asarray(adjoint(r), np.float64)
        g_new = float(np.sum(s * s))
        q = s + (g_new / gamma) * q
        gamma = g_new
    return p, hist


try:
    import torch

    class SensorData(torch.autograd.Function):
        """p0 (grid tensor) -> recorded pressure (n_points, n_rec); backward
        through the GPU adjoint.  ``prob`` is a problem dict with a binary
        sensor recording p and smooth_p0 False."""

        @staticmethod
        def forward(ctx, p0, prob):
            _require_unsmoothed(prob, "SensorData")
            ctx.prob = prob
            ctx.device = p0.device
            d = forward_p0(prob, p0.detach().cpu().double().numpy())
            return torch.as_tensor(d, dtype=p0.dtype, device=p0.device)

        @staticmethod
        def backward(ctx, grad_d):
            g = adjoint_p0(ctx.prob, grad_d.detach().cpu().double().numpy())
            return torch.as_tensor(g, dtype=grad_d.dtype, device=ctx.device), None

    class SensorDataPC(torch.autograd.Function):
        """(p0, c0) grid tensors -> recorded pressure (n_points, n_rec), c_ref
        held at the problem's max(c0); backward gives both gradients through
        the checkpointed GPU adjoint.  The forward keeps its plan (with the
        checkpoints) until backward runs."""

        @staticmethod
        def forward(ctx, p0, c, prob, checkpoint_interval=None):
            _require_unsmoothed(prob, "SensorDataPC")
            sim, d = _forward_plan(prob, p0.detach().cpu().double().numpy(), c.detach().cpu().double().numpy(),
                                   checkpoint_interval)
            ctx.sim = sim
            ctx.device = p0.device
            return torch.as_tensor(d, dtype=p0.dtype, device=p0.device)

        @staticmethod
        def backward(ctx, grad_d):
            sim = ctx.sim
            try:
                g_p0, g_c = sim._plan.adjoint(slot_residual(sim.S, grad_d.detach().cpu().double().numpy()),
                                              grad_c=True)
            finally:
                sim.close()
            return (torch.as_tensor(g_p0, dtype=grad_d.dtype, device=ctx.device),
                    torch.as_tensor(g_c, dtype=grad_d.dtype, device=ctx.device), None, None)
except ImportError:  # pragma: no cover - torch is part of the host stack
    SensorData = SensorDataPC = None
