"""The learned warm start's network as a whole: forward and parameter
gradients against the same network in plain PyTorch FP32 on the CPU, a
training run that lowers the loss, and the trained network beating the
time-reversal image it starts from on held-out pairs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib

    _lib.require_device()


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _rounders():
    """Autograd functions that round to bf16 where the kernels store bf16:
    R rounds the values in both directions (an activation written in bf16 and
    the gradient that arrives at it, also written in bf16), G only the
    gradient (the f32 output layer, whose gradient is written in bf16)."""
    import torch

    class R(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x):
            return x.to(torch.bfloat16).float()

        @staticmethod
        def backward(ctx, g):
            return g.to(torch.bfloat16).float()

    class G(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x):
            return x.clone()

        @staticmethod
        def backward(ctx, g):
            return g.to(torch.bfloat16).float()

    return R.apply, G.apply


def torch_reference(net, images, targets):
    """The network of kwave_gb300.warmstart in torch.nn.functional (NCHW,
    FP32 arithmetic, weights rounded to bf16 as the kernels read them, and
    activations and their gradients rounded to bf16 at the points where the
    kernels store them); returns the estimate, the loss and the gradients of
    every parameter."""
    import torch
    import torch.nn.functional as F

    from kwave_gb300.warmstart import LAYERS

    R, G = _rounders()

    W, B = {}, {}
    for name, c1, c2, co, _ in LAYERS:
        w = net.p[name]["w"].detach().cpu().to(torch.bfloat16).float()
        W[name] = w.reshape(co, 3, 3, c1 + c2).permute(0, 3, 1, 2).contiguous().requires_grad_(True)
        B[name] = net.p[name]["b"].detach().cpu().clone().requires_grad_(True)
    img = torch.as_tensor(images).float()
    x = torch.zeros((img.shape[0], 8, img.shape[1], img.shape[2]))
    x[:, 0] = (img * net.in_scale).to(torch.bfloat16).float()

    def conv(name, a, b=None, relu=True):
        if b is not None:
            a = torch.cat([a, F.interpolate(b, scale_factor=2, mode="nearest")], 1)
        y = F.conv2d(R(a), W[name], B[name], padding=1)
        return R(torch.relu(y)) if relu else G(y)

    def pool(a):
        return R(F.avg_pool2d(a, 2))

    e1 = conv("e1b", conv("e1a", x))
    e2 = conv("e2b", conv("e2a", pool(e1)))
    e3 = conv("e3b", conv("e3a", pool(e2)))
    b = conv("bb", conv("ba", pool(e3)))
    d3 = conv("d3b", conv("d3a", e3, b))
    d2 = conv("d2b", conv("d2a", e2, d3))
    d1 = conv("d1b", conv("d1a", e1, d2))
    out = conv("out", d1, relu=False)
    est = out[:, 0] + net.in_scale * img
    loss = ((est - torch.as_tensor(targets).float()) ** 2).mean()
    loss.backward()
    grads = {}
    for name, c1, c2, co, _ in LAYERS:
        grads[name] = (W[name].grad.permute(0, 2, 3, 1).reshape(co, 9, c1 + c2).numpy(), B[name].grad.numpy())
    return est.detach().numpy(), float(loss.detach()), grads


def smooth_images(nb, n, seed):
    rng = np.random.default_rng(seed)
    g = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    out = np.zeros((nb, n, n))
    for i in range(nb):
        for _ in range(4):
            cx, cy, s = rng.uniform(4, n - 4), rng.uniform(4, n - 4), rng.uniform(1.5, 4)
            out[i] += rng.uniform(0.5, 2) * np.exp(-((g[0] - cx) ** 2 + (g[1] - cy) ** 2) / (2 * s * s))
    return out.astype(np.float32)


def test_network_forward_and_gradients_match_torch():
    """Whole-network estimate and every parameter gradient against torch
    autograd, the reference rounding activations and gradients to bf16 where
    the kernels store them.  Weights are scaled down and biases set to 1 so
    that every pre-activation stays positive: a ReLU mask that flips on a
    value near zero (its sign set by FP32 summation order) would otherwise
    dominate the comparison of the deep layers' gradients.  What remains is
    summation order and the odd bf16 rounding-boundary flip: 1e-2 relative L2
    for the estimate, the loss and every gradient.  The mask itself is checked
    exactly in the per-operation tests, which pin each kernel at 1e-5."""
    import torch

    from kwave_gb300.warmstart import LAYERS, UNet

    net = UNet(seed=3, in_scale=0.8)
    for name, *_ in LAYERS:  # a non-trivial output layer, so that every gradient is exercised
        net.p[name]["w"].mul_(0.15 if name != "out" else 30.0)
        net.p[name]["b"].fill_(1.0 if name != "out" else 0.0)
        net.wb[name] = net.p[name]["w"].to(torch.bfloat16).contiguous()
    imgs = smooth_images(2, 32, 1)
    tgts = 1.5 * smooth_images(2, 32, 2)
    est_ref, loss_ref, g_ref = torch_reference(net, imgs, tgts)
    x = torch.as_tensor(imgs, device="cuda")
    y = torch.as_tensor(tgts, device="cuda")
    loss = torch.zeros(1, device="cuda")
    net.loss_and_grad(x, y, loss)
    est = net.forward(x).cpu().numpy()
    torch.cuda.synchronize()
    e_est = rel(est, est_ref)
    e_loss = abs(float(loss) / imgs.size - loss_ref) / loss_ref
    neg = sum(int((net.acts[name].float() <= 0).sum()) for name, *_ in LAYERS if name != "out")
    print(f"estimate {e_est:.2e}, loss {e_loss:.2e}, non-positive hidden activations {neg}")
    assert e_est <= 1e-2 and e_loss <= 1e-2
    worst = 0.0
    for name, *_ in LAYERS:
        gw = net.state[name]["w"]["g"].cpu().numpy()
        gb = net.state[name]["b"]["g"].cpu().numpy()
        ew, eb = rel(gw, g_ref[name][0]), rel(gb, g_ref[name][1])
        print(f"{name}: weight grad {ew:.2e}, bias grad {eb:.2e}")
        worst = max(worst, ew, eb)
    assert worst <= 1e-2, worst


def test_training_lowers_the_loss():
    """Adam steps on a fixed smooth-image-to-target map bring the loss down."""
    from kwave_gb300.warmstart import UNet

    imgs = smooth_images(64, 32, 5)
    tgts = np.maximum(1.3 * imgs - 0.3, 0).astype(np.float32)
    net = UNet(seed=1, in_scale=1.0)
    hist = net.train(imgs, tgts, epochs=6, batch=8, lr=2e-3)
    print("loss per epoch", hist)
    assert hist[-1] < 0.5 * hist[0], hist


def test_trained_network_beats_time_reversal():
    """Training pairs from the device forward solver and time reversal
    (vessel phantoms, 128^2, 64-point circle, 400 steps, 1 % noise): after
    training on 384 pairs, the network's estimate is closer to the held-out
    phantoms than the time-reversal image scaled by its least-squares factor."""
    from kwave_gb300.warmstart import UNet, fit_input_scale, generate_pairs

    kw = dict(n=128, nt=400, n_sensor=64, radius=2.4e-3)
    imgs, p0s = generate_pairs(384, seed0=10, batch=128, **kw)
    timgs, tp0s = generate_pairs(16, seed0=5000, batch=16, **kw)
    s = fit_input_scale(imgs, p0s)
    net = UNet(seed=0, in_scale=s)
    hist = net.train(imgs, p0s, epochs=12, batch=16, lr=1e-3)
    est = net.predict(timgs)
    e_net = np.mean([rel(e, t) for e, t in zip(est, tp0s)])
    e_tr = np.mean([rel(s * i, t) for i, t in zip(timgs, tp0s)])
    print(f"held-out relative p0 error: network {e_net:.3f}, scaled time reversal {e_tr:.3f}; losses {hist}")
    assert e_net < e_tr


def test_pair_generator_reuses_plans_exactly():
    """Training pairs from the persistent plan batches (new p0 and new
    time-reversal signals uploaded into finalized plans) equal those of fresh
    simulations per pair, bit for bit, including a partial last group."""
    from kwave_gb300.solver import run_batch
    from kwave_gb300.warmstart import generate_pairs, noisy, pair_problem, time_reversal_images

    kw = dict(n=64, nt=120, n_sensor=32, radius=5e-4)
    imgs, p0s = generate_pairs(6, seed0=3, batch=4, grouped=False, **kw)
    for g0, seeds in ((0, [3, 4, 5, 6]), (4, [7, 8])):
        probs = [pair_problem(s, **kw) for s in seeds]
        rng = np.random.default_rng(3 + g0 + 7)
        datas = [noisy(r["p"].astype(np.float64), rng) for r in run_batch(probs)]
        ref = time_reversal_images(probs, datas)
        for i, (r, pr) in enumerate(zip(ref, probs)):
            assert np.array_equal(imgs[g0 + i], r.astype(np.float32))
            assert np.array_equal(p0s[g0 + i], pr["p0"].astype(np.float32))
    # grouped launches run the run-time-length kernels: the same pairs to rounding
    gimgs, gp0s = generate_pairs(6, seed0=3, batch=4, grouped=True, **kw)
    assert np.array_equal(gp0s, p0s)
    for a, b in zip(gimgs, imgs):
        assert rel(a, b) <= 1e-5


def test_time_reversal_image_independent_of_recording():
    """The time-reversal runs record p_final alone on the sensor mask, as the
    reference's time reversal does; the image (the final pressure field) is
    bit-identical to that of the same run recording p on every grid point at
    every step, and no time series is kept."""
    from kwave_gb300.solver import Simulation, run_batch
    from kwave_gb300.warmstart import noisy, pair_problem, time_reversal_images, tr_problem

    kw = dict(n=64, nt=120, n_sensor=32, radius=5e-4)
    probs = [pair_problem(s, **kw) for s in (11, 12)]
    datas = [noisy(r["p"].astype(np.float64), np.random.default_rng(1)) for r in run_batch(probs)]
    imgs = time_reversal_images(probs, datas)
    for pr, d, img in zip(probs, datas, imgs):
        q = tr_problem(pr, d)
        sim = Simulation.from_problem(q).setup()
        try:
            res = sim.run()
            assert set(res) == {"p_final"}, sorted(res)
        finally:
            sim.close()
        full = dict(q, sensor_mask=None, record=None)
        sim = Simulation.from_problem(full).setup()
        try:
            res_full = sim.run()
            p_full = sim.p
        finally:
            sim.close()
        assert res_full["p"].shape[0] == 64 * 64
        ref = 2.0 * p_full
        ref[ref < 0] = 0
        assert np.array_equal(img, ref)
        assert np.array_equal(res["p_final"], res_full["p_final"])
