"""CPU adjoint oracle for the lossless k-space time loop.

TEST INFRASTRUCTURE ONLY.  Like ``kspace_oracle`` this module is a checker:
only ``tests/`` may import it, and nothing in ``kwave_gb300`` imports or
calls it.  It fixes in FP64 what a GPU adjoint of the time loop has to
reproduce.  The reference has no adjoint: this is the exact transpose of its
discrete step.

The forward map is the reference's step (kwave/solvers/kspace_solver.py
:691-747) for a lossless medium without sources, from p0 to the recorded
pressure d_t = S p_t.  ``forward`` reproduces ``OracleSimulation(prob,
float64)`` to rounding.

    u_i'   = sg_i (sg_i u_i - a_i G_i p)          G_i f = Re F^-1[op_grad_i F f], a_i = dt / rho_sg_i
    rho_i' = m_i (m_i rho_i - b D_i u_i')         D_i f = Re F^-1[op_div_i F f],  b = dt rho0
    p'     = c^2 sum_i rho_i'

The t = 0 initial-condition override (:725-733) sets the state after step 0:

    p = p0,  rho_i = p0 / (c^2 D),  u_i = (a_i / 2) G_i p0

For real fields the transpose of Re F^-1[o F .] is Re F^-1[conj(o) F .], and
conj(op_grad_i) = -op_div_i, so G_i^T = -D_i and D_i^T = -G_i.  The adjoint
step, with lambda the adjoint of the state after the step, is

    lr_i' += c^2 lp'
    lu_i' += G_i (b m_i lr_i')
    lr_i   = m_i^2 lr_i'
    lu_i   = sg_i^2 lu_i'
    lp     = sum_i D_i (a_i sg_i lu_i')

The recorded misfit enters as lp += S^T r_t at every recorded step.  The
gradient with respect to p0 is the transpose of the t = 0 override:

    g_p0 = lp + sum_i lr_i / (c^2 D) - sum_i D_i ((a_i / 2) lu_i)

The gradient with respect to c2 = c^2 adds, from every step t >= 1,
(sum_i rho_i') lp' and, from the override, -sum_i p0 lr_i / (c2^2 D).  c_ref
(PML, kappa) is held at the base problem's value.

Requirements: no absorption, no B/A, no sources, and ``smooth_p0`` False
(restore_max smoothing is not linear).  The sensor is binary or Cartesian;
S is formed as a dense matrix by probing the oracle's own extraction, so
this is for small grids.
"""
from __future__ import annotations

import numpy as np

from .kspace_oracle import OracleSimulation, is_enabled


class AdjointOracle:
    def __init__(self, prob: dict):
        for key in ("alpha_coeff", "BonA", "p_mask", "u_mask"):
            if is_enabled(prob.get(key, 0)):
                raise ValueError(f"the adjoint oracle covers the lossless source-free loop ({key} set)")
        if prob.get("smooth_p0", True):
            raise ValueError("the adjoint oracle needs smooth_p0=False")
        base = dict(prob)
        base["p0"] = None
        base["record"] = ("p",)
        sim = OracleSimulation(base, np.float64).setup()
        self.sim = sim
        self.shape = sim.grid_shape
        self.ndim = sim.ndim
        self.Nt = sim.Nt
        self.rs = sim.record_start_index
        self.og = sim.op_grad_list
        self.od = sim.op_div_list
        self.m = sim.pml_list
        self.sg = sim.pml_sg_list
        self.a = sim.dt_over_rho0
        self.b = sim.dt * sim.rho0
        self.c = sim.c0.copy()
        numel = int(np.prod(self.shape))
        S = np.zeros((sim.n_sensor_points, numel))
        e = np.zeros(numel)
        for j in range(numel):
            e[j] = 1.0
            S[:, j] = sim._extract(e.reshape(self.shape))
            e[j] = 0.0
        self.S = S

    # -- operators ---------------------------------------------------------------
    def _G(self, i, f):
        return np.real(np.fft.ifftn(self.og[i] * np.fft.fftn(f)))

    def _D(self, i, f):
        return np.real(np.fft.ifftn(self.od[i] * np.fft.fftn(f)))

    def _rec(self, p):
        return self.S @ p.ravel()

    def _rec_T(self, r):
        return (self.S.T @ r).reshape(self.shape)

    # -- forward -----------------------------------------------------------------
    def forward(self, p0, c=None, keep=False):
        """Recorded pressure (n_points, Nt - record_start); with ``keep`` also
        the per-step sums of the density components (t >= 1)."""
        D = self.ndim
        c2 = (self.c if c is None else np.asarray(c, float)) ** 2
        p0 = np.asarray(p0, float)
        p = p0.copy()
        rho = [p0 / (c2 * D) for _ in range(D)]
        u = [(self.a[i] / 2) * self._G(i, p0) for i in range(D)]
        d = np.zeros((self.S.shape[0], self.Nt - self.rs))
        sums = [None] * self.Nt
        if self.rs == 0:
            d[:, 0] = self._rec(p)
        for t in range(1, self.Nt):
            for i in range(D):
                u[i] = self.sg[i] * (self.sg[i] * u[i] - self.a[i] * self._G(i, p))
            for i in range(D):
                rho[i] = self.m[i] * (self.m[i] * rho[i] - self.b * self._D(i, u[i]))
            s = rho[0]
            for r in rho[1:]:
                s = s + r
            if keep:
                sums[t] = s
            p = c2 * s
            if t >= self.rs:
                d[:, t - self.rs] = self._rec(p)
        return (d, sums) if keep else d

    # -- adjoint -----------------------------------------------------------------
    def adjoint(self, r, c=None, sums=None, p0=None):
        """Transpose of ``forward`` applied to r (same shape as its output):
        returns g_p0, and with ``sums`` and ``p0`` also g_c2 (the derivative
        of <r, forward> with respect to c^2)."""
        D = self.ndim
        c2 = (self.c if c is None else np.asarray(c, float)) ** 2
        lp = np.zeros(self.shape)
        lu = [np.zeros(self.shape) for _ in range(D)]
        lr = [np.zeros(self.shape) for _ in range(D)]
        gc2 = np.zeros(self.shape) if sums is not None else None
        for t in range(self.Nt - 1, 0, -1):
            if t >= self.rs:
                lp = lp + self._rec_T(r[:, t - self.rs])
            if gc2 is not None:
                gc2 += sums[t] * lp
            lr = [lr[i] + c2 * lp for i in range(D)]
            lu = [lu[i] + self._G(i, self.b * self.m[i] * lr[i]) for i in range(D)]
            lp = np.zeros(self.shape)
            for i in range(D):
                lp = lp + self._D(i, self.a[i] * self.sg[i] * lu[i])
            lr = [self.m[i] * self.m[i] * lr[i] for i in range(D)]
            lu = [self.sg[i] * self.sg[i] * lu[i] for i in range(D)]
        if self.rs == 0:
            lp = lp + self._rec_T(r[:, 0])
        g = lp.copy()
        for i in range(D):
            g += lr[i] / (c2 * D) - self._D(i, (self.a[i] / 2) * lu[i])
        if gc2 is None:
            return g
        for i in range(D):
            gc2 += -np.asarray(p0, float) * lr[i] / (c2 * c2 * D)
        return g, gc2

    def misfit_gradient(self, p0, d_obs, c=None):
        """L = 1/2 ||forward(p0, c) - d_obs||^2 and its gradients with respect
        to p0 and c (c_ref held fixed)."""
        c = self.c if c is None else np.asarray(c, float)
        d, sums = self.forward(p0, c, keep=True)
        r = d - d_obs
        g_p0, g_c2 = self.adjoint(r, c, sums, p0)
        return 0.5 * float(np.sum(r * r)), g_p0, 2 * c * g_c2
