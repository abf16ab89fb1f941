"""FP64 PyTorch autograd reference of the lossless time loop.

TEST INFRASTRUCTURE ONLY (like the other modules of ``oracle/``): only
``tests/`` may import it.  It runs the reference's step
(kwave/solvers/kspace_solver.py:691-747 with alpha = 0, B/A = 0, no sources)
and its t = 0 initial-condition override (:725-733) in torch float64, so that
autograd gives the gradients of a sensor-data misfit with respect to p0 and
the sound speed c.  c_ref (PML, kappa) stays at the base problem's value.
With ``operators="oracle"`` the operators, PML profiles and the sensor
matrix are the adjoint oracle's; with ``operators="independent"`` they are
built here in torch from the reference's formulas (binary sensors only), so
that a test comparing the two also checks the oracle's operator
construction.  This is the "FP64 autograd reference" that a GPU adjoint is
checked against on small grids.
"""
from __future__ import annotations

import numpy as np

from .adjoint_oracle import AdjointOracle


def _pml_1d(n, dx, dt, c, size, alpha, staggered):
    """kwave/utils/pml.py:43-58 (get_pml) in torch float64."""
    import torch

    x = torch.arange(1, size + 1, dtype=torch.float64)
    if staggered:
        left = alpha * (c / dx) * ((((x + 0.5) - size - 1) / (0 - size)) ** 4)
        right = alpha * (c / dx) * (((x + 0.5) / size) ** 4)
    else:
        left = alpha * (c / dx) * (((x - size - 1) / (0 - size)) ** 4)
        right = alpha * (c / dx) * ((x / size) ** 4)
    out = torch.ones(n, dtype=torch.float64)
    if size > 0:
        out[:size] = torch.exp(-left * dt / 2)
        out[n - size:] = torch.exp(-right * dt / 2)
    return out


def _stagger(a, axis):
    """Mean of neighbours along axis, last plane copied (kspace_solver.py:798-809)."""
    import torch

    if a.numel() == 1:
        return a
    lo = a.narrow(axis, 0, a.shape[axis] - 1)
    hi = a.narrow(axis, 1, a.shape[axis] - 1)
    return torch.cat([0.5 * (lo + hi), a.narrow(axis, a.shape[axis] - 1, 1)], dim=axis)


def independent_operators(prob: dict):
    """Operators of the lossless step built here from the reference's
    formulas, not taken from the oracle: k = 2 pi fftfreq(N, d) and
    kappa = sinc(c_ref |k| dt / 2) (kspace_solver.py:419-431), the shifted
    gradient / divergence operators (:440-447), the PML profiles (pml.py via
    :363-406), dt / rho0 on the staggered grids (:657-666) and the binary
    sensor's C-order indices (:268-274).  Returns a namespace like
    AdjointOracle's (og, od, m, sg, a, b, c, ndim, Nt, rs, S)."""
    import types

    import torch

    shape = tuple(int(n) for n in prob["shape"])
    D = len(shape)
    dt = float(prob["dt"])
    sp = [float(d) for d in prob["spacing"]]
    c = torch.as_tensor(np.broadcast_to(np.asarray(prob["sound_speed"], float), shape).copy())
    rho0 = torch.as_tensor(np.broadcast_to(np.asarray(prob.get("density", 1000.0), float), shape).copy())
    c_ref = float(c.max())
    ks = []
    for ax, (n, d) in enumerate(zip(shape, sp)):
        view = [1] * D
        view[ax] = n
        ks.append((2 * np.pi * torch.fft.fftfreq(n, d=d, dtype=torch.float64)).reshape(view))
    kmag = torch.sqrt(sum(k * k for k in ks))
    arg = c_ref * kmag * dt / 2
    kappa = torch.where(arg == 0, torch.ones_like(arg), torch.sin(arg) / torch.where(arg == 0, torch.ones_like(arg), arg))
    use_sg = prob.get("use_sg", True)
    og, od, m, sg, a = [], [], [], [], []
    ps = prob.get("pml_size") or (20,) * D
    pa = prob.get("pml_alpha") or (2.0,) * D
    for ax, (n, d) in enumerate(zip(shape, sp)):
        k = ks[ax]
        sh = torch.exp(1j * k * d / 2) if use_sg else torch.ones_like(k, dtype=torch.complex128)
        og.append(1j * k * sh * kappa)
        od.append(1j * k * torch.conj(sh) * kappa)
        view = [1] * D
        view[ax] = n
        m.append(_pml_1d(n, d, dt, c_ref, int(ps[ax]), float(pa[ax]), False).reshape(view))
        sg.append(_pml_1d(n, d, dt, c_ref, int(ps[ax]), float(pa[ax]), True).reshape(view))
        a.append(dt / _stagger(rho0, ax))
    mask = np.asarray(prob["sensor_mask"], bool)
    if mask.shape != shape:
        raise ValueError("independent operators cover binary sensor masks only")
    idx = np.flatnonzero(mask.ravel())
    S = torch.zeros((idx.size, int(np.prod(shape))), dtype=torch.float64)
    S[torch.arange(idx.size), torch.as_tensor(idx)] = 1.0
    rs = max(int(prob.get("record_start_index") or 1) - 1, 0)
    return types.SimpleNamespace(og=og, od=od, m=m, sg=sg, a=a, b=dt * rho0, c=c.numpy(), ndim=D, Nt=int(prob["Nt"]),
                                 rs=rs, S=S)


def misfit_and_grads(prob: dict, p0, d_obs, c=None, operators="oracle"):
    """(L, dL/dp0, dL/dc) of L = 1/2 ||S p_t - d_obs||^2 over the recorded steps,
    by torch autograd in float64."""
    import torch

    A = AdjointOracle(prob) if operators == "oracle" else independent_operators(prob)
    T = lambda a: torch.as_tensor(np.asarray(a), dtype=torch.float64) if not torch.is_tensor(a) else a  # noqa: E731
    Tc = lambda a: torch.as_tensor(np.asarray(a), dtype=torch.complex128) if not torch.is_tensor(a) else a  # noqa: E731
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
