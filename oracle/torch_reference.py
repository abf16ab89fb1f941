"""FP64 PyTorch autograd reference of the lossless time loop.

TEST INFRASTRUCTURE ONLY (like the other modules of ``oracle/``): only
``tests/`` may import it.  It runs the reference's step
(kwave/solvers/kspace_solver.py:691-747 with alpha = 0, B/A = 0, no sources)
and its t = 0 initial-condition override (:725-733) in torch float64, so that
autograd gives the gradients of a sensor-data misfit with respect to p0 and
the sound speed c.  c_ref (PML, kappa) stays at the base problem's value.
The operators, PML profiles and the sensor matrix are the adjoint oracle's.
This is the "FP64 autograd reference" that a GPU adjoint is checked against
on small grids.
"""
from __future__ import annotations

import numpy as np

from .adjoint_oracle import AdjointOracle


def misfit_and_grads(prob: dict, p0, d_obs, c=None):
    """(L, dL/dp0, dL/dc) of L = 1/2 ||S p_t - d_obs||^2 over the recorded steps,
    by torch autograd in float64."""
    import torch

    A = AdjointOracle(prob)
    T = lambda a: torch.as_tensor(np.asarray(a), dtype=torch.float64)  # noqa: E731
    Tc = lambda a: torch.as_tensor(np.asarray(a), dtype=torch.complex128)  # noqa: E731
    og, od = [Tc(o) for o in A.og], [Tc(o) for o in A.od]
    m, sg, a = [T(x) for x in A.m], [T(x) for x in A.sg], [T(x) for x in A.a]
    b, S = T(A.b), T(A.S)
    p0_t = T(p0).requires_grad_(True)
    c_t = T(A.c if c is None else c).requires_grad_(True)
    c2 = c_t * c_t
    D = A.ndim

    def G(i, f):
        return torch.fft.ifftn(og[i] * torch.fft.fftn(f)).real

    def Dv(i, f):
        return torch.fft.ifftn(od[i] * torch.fft.fftn(f)).real

    p = p0_t
    rho = [p0_t / (c2 * D) for _ in range(D)]
    u = [(a[i] / 2) * G(i, p0_t) for i in range(D)]
    rec = []
    if A.rs == 0:
        rec.append(S @ p.reshape(-1))
    for t in range(1, A.Nt):
        u = [sg[i] * (sg[i] * u[i] - a[i] * G(i, p)) for i in range(D)]
        rho = [m[i] * (m[i] * rho[i] - b * Dv(i, u[i])) for i in range(D)]
        s = rho[0]
        for r in rho[1:]:
            s = s + r
        p = c2 * s
        if t >= A.rs:
            rec.append(S @ p.reshape(-1))
    d = torch.stack(rec, dim=1)
    loss = 0.5 * ((d - T(d_obs)) ** 2).sum()
    loss.backward()
    return float(loss.item()), p0_t.grad.numpy(), c_t.grad.numpy()
