"""Learned warm start of initial-pressure reconstruction.

A small BF16 U-Net (FP32 accumulation on the tensor cores, kw_unet.cu) maps
a time-reversal image to an estimate of p0; adjoint iterations (CGLS on the
GPU time loop, ``adjoint.cgls_p0``) refine it, with plain adjoint iterations
from zero as fallback and as the yardstick of its error.  The reference has no such
component; the network's input is the reference's time-reversal image
(kwave/reconstruction/time_reversal.py:129-150: the recorded pressure,
reversed in time, drives a Dirichlet source on the sensor mask; the final
pressure times the compensation factor 2, clipped at zero).

Everything the network computes runs in this library's kernels: the 3x3
convolutions and their data and weight gradients on tcgen05, pooling,
upsampling (read through the convolution's input gather), ReLU, the loss and
Adam.  torch only holds the device buffers.

Network (4 levels, 32 base channels, 256 x 256 input, NHWC bf16):

    e1: conv(8->32), conv(32->32)              256^2   (input: the image in channel 0 of 8)
    e2: pool, conv(32->64), conv(64->64)       128^2
    e3: pool, conv(64->128), conv(128->128)     64^2
    b : pool, conv(128->256), conv(256->256)    32^2
    d3: conv([e3, up(b)] 384->128), conv(128->128)   64^2
    d2: conv([e2, up(d3)] 192->64), conv(64->64)    128^2
    d1: conv([e1, up(d2)] 96->32), conv(32->32)     256^2
    out: conv(32->16), channel 0;  p0_hat = s * image + out_0

with ReLU after every convolution but the last, 2 x 2 average pooling and
nearest-neighbour upsampling.  s is a fixed input scale (least-squares fit of
the training targets by the images); the network learns the correction.
"""
from __future__ import annotations

import time

import numpy as np

from . import unet_ops as U
from .adjoint import LinearP0, cgls_p0
from .conversion import cart2grid
from .phantoms import circle_points, vessel_phantom
from .solver import Simulation, SimulationBatch

# (name, full-resolution input channels, upsampled input channels, output channels, ReLU)
LAYERS = [
    ("e1a", 8, 0, 32, True), ("e1b", 32, 0, 32, True),
    ("e2a", 32, 0, 64, True), ("e2b", 64, 0, 64, True),
    ("e3a", 64, 0, 128, True), ("e3b", 128, 0, 128, True),
    ("ba", 128, 0, 256, True), ("bb", 256, 0, 256, True),
    ("d3a", 128, 256, 128, True), ("d3b", 128, 0, 128, True),
    ("d2a", 64, 128, 64, True), ("d2b", 64, 0, 64, True),
    ("d1a", 32, 64, 32, True), ("d1b", 32, 0, 32, True),
    ("out", 32, 0, 16, False),
]
IN_CH = 8
SPEC = {layer[0]: layer for layer in LAYERS}


# ---------------------------------------------------------------------------
# training pairs from the forward solver and time reversal
# ---------------------------------------------------------------------------
def pair_problem(seed, n=256, nt=800, n_sensor=128, radius=5e-3, dx=5e-5, pml=20):
    """Forward problem of one training pair: the vessel phantom of ``seed`` as
    p0 on an n x n grid (PML inside, homogeneous water, lossless), the binary
    mask of ``n_sensor`` points on a circle of ``radius`` (nearest grid points,
    ``cart2grid``) recording p for ``nt`` steps of dt = 0.3 dx / c."""
    p0 = vessel_phantom(n, np.random.default_rng(seed), pml)
    kg = type("G", (), {"N": np.array([n, n]), "spacing": np.array([dx, dx])})()
    mask = cart2grid(kg, circle_points(n_sensor, radius), order="C")[0].astype(bool)
    return dict(shape=(n, n), spacing=(dx, dx), dt=0.3 * dx / 1500.0, Nt=nt, sound_speed=1500.0, density=1000.0,
                p0=p0, smooth_p0=False, sensor_mask=mask, record=("p",), pml_size=(pml, pml), pml_alpha=(2.0, 2.0),
                use_sg=True, use_kspace=True)


def noisy(d, rng, level=0.01):
    """Recorded data plus Gaussian noise of ``level`` times its standard deviation."""
    return d + level * float(np.std(d)) * rng.standard_normal(d.shape)


def tr_problem(prob, data):
    """The time-reversal run of ``data`` (n_sensor, Nt) recorded on the binary
    mask of ``prob``: a Dirichlet pressure source on the mask driven by the
    time-reversed data, no p0, and a sensor on the same mask that records
    only ``p_final`` (time_reversal.py:94-98,129-135).  The image is the
    final pressure field; recording adds no work per step (a sensor on every
    grid point recording p, the solver's default without a mask, wrote the
    whole field into the time series at each step)."""
    q = {k: v for k, v in prob.items() if k not in ("p0", "sensor_mask", "record", "record_start_index")}
    q.update(p_mask=prob["sensor_mask"], p=np.ascontiguousarray(np.flip(data, axis=1)), p_mode="dirichlet",
             sensor_mask=prob["sensor_mask"], record=("p_final",))
    return q


def _tr_image(sim, compensation_factor):
    img = compensation_factor * sim.p
    img[img < 0] = 0
    return img


def time_reversal_images(probs, datas, stream=None, compensation_factor=2.0):
    """Time-reversal images of several recordings in one batch: the whole
    final pressure field of each reversed run times the compensation factor,
    clipped at zero (the reference returns the same field without the PML)."""
    b = SimulationBatch.from_problems([tr_problem(p, d) for p, d in zip(probs, datas)], stream=stream)
    try:
        b.run()
        return [_tr_image(s, compensation_factor) for s in b.sims]
    finally:
        b.close()


class PairGenerator:
    """Forward and time-reversal runs of many pairs on two persistent batches
    of ``batch`` plans each: the forward plans get each new phantom with
    kw_plan_update_p0 and the time-reversal plans each new reversed recording
    with kw_plan_update_source, so the host set-up and the plan creation are
    paid once, not per pair.  All pairs share the grid, medium and sensor."""

    def __init__(self, batch=256, noise=0.01, compensation_factor=2.0, grouped=False, **kw):
        self.kw = kw
        self.noise = noise
        self.cf = compensation_factor
        self.batch = batch
        probs = [pair_problem(s, **kw) for s in range(batch)]
        self.fwd = SimulationBatch.from_problems(probs, grouped=grouped)
        ones = np.ones((int(probs[0]["sensor_mask"].sum()), probs[0]["Nt"]))
        self.tr = SimulationBatch.from_problems([tr_problem(p, ones) for p in probs], grouped=grouped)

    def run(self, seeds, rng):
        """(images, phantoms) of the given phantom seeds (at most ``batch``)."""
        probs = [pair_problem(s, **self.kw) for s in seeds]
        sims = self.fwd.sims[: len(probs)]
        for sim, pr in zip(sims, probs):
            sim._plan.update_p0(pr["p0"])
            sim.t = 0
        self.fwd.run_steps(max(s.S.Nt for s in sims))
        sims[0]._plan.sync()
        datas = [noisy(s.results()["p"].astype(np.float64), rng, self.noise) for s in sims]
        tsims = self.tr.sims[: len(probs)]
        for sim, pr, d in zip(tsims, probs, datas):
            sim._plan.update_sources(tr_problem(pr, d))
            sim.t = 0
        self.tr.run_steps(max(s.S.Nt for s in tsims))
        tsims[0]._plan.sync()
        return [_tr_image(s, self.cf) for s in tsims], [p["p0"] for p in probs]

    def close(self):
        self.fwd.close()
        self.tr.close()


def generate_pairs(n_pairs, seed0=1000, batch=256, noise=0.01, grouped=True, **kw):
    """(images, targets): time-reversal images of noisy recordings and the
    phantoms that made them, float32 (n_pairs, n, n), generated ``batch``
    pairs at a time on persistent batches of plans (PairGenerator).  With
    ``grouped`` (the default) each pass of all members is one grouped launch
    of the run-time-length kernels: 512 pairs at 256^2 in 9 s against 34 s
    with each member's own step graph as a branch."""
    gen = PairGenerator(batch=min(batch, n_pairs), noise=noise, grouped=grouped, **kw)
    imgs, p0s = [], []
    try:
        for g0 in range(0, n_pairs, gen.batch):
            seeds = list(range(seed0 + g0, seed0 + min(n_pairs, g0 + gen.batch)))
            a, b = gen.run(seeds, np.random.default_rng(seed0 + g0 + 7))
            imgs += a
            p0s += b
    finally:
        gen.close()
    return np.asarray(imgs, np.float32), np.asarray(p0s, np.float32)


# ---------------------------------------------------------------------------
# the network
# ---------------------------------------------------------------------------
class UNet:
    """Parameters (f32 masters, bf16 copies, Adam moments, gradients) and the
    forward / backward passes of the network above, on CUDA tensors."""

    def __init__(self, seed=0, device="cuda", in_scale=1.0):
        import torch

        self.device = device
        self.in_scale = float(in_scale)
        g = torch.Generator().manual_seed(seed)
        self.p = {}
        for name, c1, c2, co, _ in LAYERS:
            cin = c1 + c2
            fan = 9 * (1 if name == "e1a" else cin)
            std = np.sqrt(2.0 / fan) if name != "out" else 1e-2 / np.sqrt(fan)
            w = torch.randn((co, 9, cin), generator=g) * std
            if name == "e1a":
                w[:, :, 1:] = 0.0  # only channel 0 of the input carries the image
            self.p[name] = {"w": w.to(device), "b": torch.zeros(co, device=device)}
        self.state = {}
        for name, prm in self.p.items():
            self.state[name] = {k: {"m": torch.zeros_like(v), "v": torch.zeros_like(v), "g": torch.zeros_like(v)}
                                for k, v in prm.items()}
        self.wb = {name: prm["w"].to(torch.bfloat16).contiguous() for name, prm in self.p.items()}
        self.step_count = 0

    # -- forward ---------------------------------------------------------------
    def _conv(self, name, x1, x2=None, yf=None):
        import torch

        spec = SPEC[name]
        relu = spec[4]
        if yf is not None:
            U.conv3x3(x1, self.wb[name], self.p[name]["b"], relu=relu, x2=x2, yf=yf)
            return yf
        y = torch.empty((*x1.shape[:3], spec[3]), dtype=torch.bfloat16, device=x1.device)
        U.conv3x3(x1, self.wb[name], self.p[name]["b"], relu=relu, x2=x2, y=y)
        return y

    def forward(self, images, keep=False):
        """images: f32 (nb, n, n) CUDA tensor -> f32 (nb, n, n) estimate of p0."""
        import torch

        nb, n, _ = images.shape
        a = {}
        x0 = torch.empty((nb, n, n, IN_CH), dtype=torch.bfloat16, device=images.device)
        U.image_to_nhwc(images.contiguous(), x0, self.in_scale)
        a["x0"] = x0
        a["e1a"] = self._conv("e1a", x0)
        a["e1b"] = self._conv("e1b", a["e1a"])
        a["p1"] = U.avgpool2(a["e1b"])
        a["e2a"] = self._conv("e2a", a["p1"])
        a["e2b"] = self._conv("e2b", a["e2a"])
        a["p2"] = U.avgpool2(a["e2b"])
        a["e3a"] = self._conv("e3a", a["p2"])
        a["e3b"] = self._conv("e3b", a["e3a"])
        a["p3"] = U.avgpool2(a["e3b"])
        a["ba"] = self._conv("ba", a["p3"])
        a["bb"] = self._conv("bb", a["ba"])
        a["d3a"] = self._conv("d3a", a["e3b"], a["bb"])
        a["d3b"] = self._conv("d3b", a["d3a"])
        a["d2a"] = self._conv("d2a", a["e2b"], a["d3b"])
        a["d2b"] = self._conv("d2b", a["d2a"])
        a["d1a"] = self._conv("d1a", a["e1b"], a["d2b"])
        a["d1b"] = self._conv("d1b", a["d1a"])
        out = torch.empty((nb, n, n, 16), dtype=torch.float32, device=images.device)
        self._conv("out", a["d1b"], yf=out)
        a["out"] = out
        if keep:
            self.acts = a
        return U.residual_out(out, images, self.in_scale)

    # -- backward ----------------------------------------------------------------
    def _layer_back(self, name, dy, x1, x2=None, need_dx=True):
        """Gradients of one convolution layer from the gradient of its output."""
        import torch

        _, c1, c2, co, relu = SPEC[name]
        y = self.acts[name]
        dz = U.relu_grad(dy, y) if relu else dy
        st = self.state[name]
        U.conv3x3_wgrad(x1, dz, st["w"]["g"], x2=x2)
        U.bias_grad(dz, st["b"]["g"])
        if not need_dx:
            return None
        wt = U.flip_weights(self.wb[name])
        dcat = torch.empty((*dz.shape[:3], c1 + c2), dtype=torch.bfloat16, device=dz.device)
        U.conv3x3(dz, wt, None, relu=False, y=dcat)
        return dcat

    def backward(self, dout):
        """dout: bf16 (nb, n, n, 16) gradient of the output layer; fills the
        parameter gradients (zeroed first)."""
        a = self.acts
        for st in self.state.values():
            for s in st.values():
                s["g"].zero_()
        d = self._layer_back("out", dout, a["d1b"])
        d = self._layer_back("d1b", d, a["d1a"])
        dcat = self._layer_back("d1a", d, a["e1b"], a["d2b"])
        d_e1b_skip, d = U.split_concat_grad(dcat, 32)
        d = self._layer_back("d2b", d, a["d2a"])
        dcat = self._layer_back("d2a", d, a["e2b"], a["d3b"])
        d_e2b_skip, d = U.split_concat_grad(dcat, 64)
        d = self._layer_back("d3b", d, a["d3a"])
        dcat = self._layer_back("d3a", d, a["e3b"], a["bb"])
        d_e3b_skip, d = U.split_concat_grad(dcat, 128)
        d = self._layer_back("bb", d, a["ba"])
        d = self._layer_back("ba", d, a["p3"])
        d = U.avgpool2_bwd(d, add=d_e3b_skip)
        d = self._layer_back("e3b", d, a["e3a"])
        d = self._layer_back("e3a", d, a["p2"])
        d = U.avgpool2_bwd(d, add=d_e2b_skip)
        d = self._layer_back("e2b", d, a["e2a"])
        d = self._layer_back("e2a", d, a["p1"])
        d = U.avgpool2_bwd(d, add=d_e1b_skip)
        d = self._layer_back("e1b", d, a["e1a"])
        self._layer_back("e1a", d, a["x0"], need_dx=False)

    def loss_and_grad(self, images, targets, loss):
        """Adds the summed squared error of the estimate against targets (f32
        (nb, n, n) CUDA tensors) to the device scalar ``loss`` and fills the
        parameter gradients of the mean squared error."""
        import torch

        self.forward(images, keep=True)
        nb, n, _ = images.shape
        dout = torch.empty((nb, n, n, 16), dtype=torch.bfloat16, device=images.device)
        U.mse_grad(self.acts["out"], images, self.in_scale, targets, dout, 2.0 / (nb * n * n), loss)
        self.backward(dout)

    def adam_step(self, lr):
        self.step_count += 1
        for name, prm in self.p.items():
            st = self.state[name]
            U.adam(prm["w"], st["w"]["m"], st["w"]["v"], st["w"]["g"], self.wb[name], lr, self.step_count)
            U.adam(prm["b"], st["b"]["m"], st["b"]["v"], st["b"]["g"], None, lr, self.step_count)

    def train(self, images, targets, epochs=4, batch=16, lr=1e-3, seed=0, log=None):
        """Adam on the mean squared error over (images, targets) float32
        (N, n, n) host arrays, batches drawn without replacement; the learning
        rate falls by a cosine to lr/20.  Returns the mean loss per pixel of
        each epoch."""
        import torch

        rng = np.random.default_rng(seed)
        N, n = len(images), images.shape[1]
        nbatch = max(1, N // batch)
        steps = epochs * nbatch
        hist = []
        k = 0
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        for ep in range(epochs):
            order = rng.permutation(N)
            loss.zero_()
            for i in range(nbatch):
                sel = order[i * batch:(i + 1) * batch]
                x = torch.from_numpy(np.ascontiguousarray(images[sel])).pin_memory().to(self.device, non_blocking=True)
                y = torch.from_numpy(np.ascontiguousarray(targets[sel])).pin_memory().to(self.device, non_blocking=True)
                self.loss_and_grad(x, y, loss)
                frac = k / max(1, steps - 1)
                self.adam_step(lr * (0.05 + 0.95 * 0.5 * (1 + np.cos(np.pi * frac))))
                k += 1
            hist.append(float(loss.item()) / (nbatch * batch * n * n))
            if log:
                log(f"epoch {ep}: loss {hist[-1]:.4e}")
        return hist

    def predict(self, images, batch=16):
        """Estimates of p0 for (N, n, n) host images (an array or a list of
        (n, n) arrays, converted to float32)."""
        import torch

        out = []
        for i in range(0, len(images), batch):
            x = torch.as_tensor(np.ascontiguousarray(images[i:i + batch], dtype=np.float32), device=self.device)
            out.append(self.forward(x).cpu().numpy())
        return np.concatenate(out)

    def state_dict(self):
        return {f"{n}.{k}": v.detach().cpu().numpy() for n, prm in self.p.items() for k, v in prm.items()}


def fit_input_scale(images, targets):
    """Least-squares scale s of targets ~ s * images."""
    a = np.asarray(images, np.float64).ravel()
    b = np.asarray(targets, np.float64).ravel()
    return float(a @ b / max(a @ a, 1e-300))


# ---------------------------------------------------------------------------
# refinement and the plain iterations it is measured against
# ---------------------------------------------------------------------------
def refine(prob, d_obs, p_init, iterations, p_true=None):
    """CGLS from p_init on the problem's linear map p0 -> recorded p (one plan
    reused for every pass); returns (p, history of (misfit, p error), seconds
    after each iteration)."""
    op = LinearP0(prob)
    stamps = []
    t0 = time.perf_counter()
    try:
        p, hist = cgls_p0(op.forward, op.adjoint, d_obs, p_init, iterations, p_true=p_true,
                          on_iteration=lambda i, p: stamps.append(time.perf_counter() - t0))
    finally:
        op.close()
    return p, hist, stamps


def time_to(errors, stamps, level, start=0.0):
    """Seconds until the relative p0 error first reaches ``level`` (None if never)."""
    for e, s in zip(errors, stamps):
        if e is not None and e <= level:
            return start + s
    return None
