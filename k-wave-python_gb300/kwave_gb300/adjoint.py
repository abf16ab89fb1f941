"""Gradients of sensor-data misfits with respect to the initial pressure.

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
except ImportError:  # pragma: no cover - torch is part of the host stack
    SensorData = None
