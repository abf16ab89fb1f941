"""Benchmark of the GB300 k-space first-order time loop.

Workload (the headline configuration): 3-D heterogeneous absorbing IVP on a
256^3 grid including a 10-point PML, dx = 0.1 mm, power-law absorption
(0.75 dB/(MHz^y cm), y = 1.5), B/A = 6, 8 random ellipsoids, 20 Gaussian p0
blobs, a binary sensor on the z = 20 plane recording p and p_max; seeded
synthetic inputs of those shapes.

A bench "step" is one time step of that simulation over the whole grid
(16.8 M cells).  ``value`` = cells x timed steps / device time (CUDA events on
the launching stream), state resident in HBM, steps run as ``kw_plan_run``
runs them (replayed step graphs).  Per-kernel durations for the roofline come
from a second, instrumented pass over the same steps (every launch bracketed
by CUDA events).  ``--workload transmit`` measures 128 batched 2-D transmit
events through ``SimulationBatch`` instead.  ``e2e`` = the same metric
through the public bridge (``run_gb300_backend``, the kspaceFirstOrder3D
path) for a full 1000-step simulation from host numpy inputs to host results,
host set-up and host<->device copies included.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``--impl reference`` times the reference's CPU implementation of the same
workload (the oracle restatement, bit-identical to kwave's native NumPy
solver) on a bounded sample of time steps.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path
from types import SimpleNamespace

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (str(ROOT), str(ROOT / "k-wave-python_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Mcell-steps/s vs native solver; time to 1% p0 error, learned+adjoint vs plain"
UNIT = "Mcell-steps/s"
WORKLOAD = ("3-D heterogeneous absorbing IVP, 256^3 incl. 10-pt PML, dx=0.1 mm, 1000 steps, "
            "power law 0.75 dB/(MHz^y cm) y=1.5, B/A=6, 8 ellipsoids, 20 p0 blobs, z=20 plane sensor p+p_max")
A_MODEL_BYTES_PER_CELL_STEP = 168  # algorithmic bytes per cell-step of this configuration


# ---------------------------------------------------------------------------
# synthetic workloads
# ---------------------------------------------------------------------------

def _random_rotation(rng):
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def ivp3d_problem(n=256, nt=1000, seed=0, plane_z=20, pml=10):
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


def _five_smooth(lo, hi):
    out = []
    for n in range(lo, hi + 1):
        m = n
        for f in (2, 3, 5):
            while m % f == 0:
                m //= f
        if m == 1:
            out.append(n)
    return out


def transmit_problem(shape, seed, nt=2000, dx=5e-5, pml=20, n_elem=32, pitch=4, width=3, cycles=3, f0=1.5e6):
    """One 2-D transmit event: a seeded speckle medium (c = 1540 (1 + 0.02 N(0,1))
    m/s, rho = 1000 (1 + 0.02 N(0,1)) kg/m^3) with 3 random discs of +-10 % c,
    power-law absorption 0.5 dB/(MHz^y cm) with y = 1.1, a linear array of
    ``n_elem`` elements (``width`` px wide, ``pitch`` px apart, two points
    inside the PML edge along x) driving a ``cycles``-cycle ``f0`` tone burst
    (Gaussian envelope) steered at a random angle in [-30, 30] degrees as an
    additive (k-space corrected) pressure source, and the array's points as a
    binary sensor recording p.  dt from the CFL-0.3 rule at the maximum sound speed."""
    rng = np.random.default_rng(seed)
    nx, ny = shape
    c = 1540.0 * (1 + 0.02 * rng.standard_normal(shape))
    rho = 1000.0 * (1 + 0.02 * rng.standard_normal(shape))
    gx, gy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    for _ in range(3):
        cx, cy = rng.uniform(pml + 10, nx - pml - 10), rng.uniform(pml + 10, ny - pml - 10)
        r = rng.uniform(5, 20)
        c[(gx - cx) ** 2 + (gy - cy) ** 2 <= r * r] *= 1 + rng.choice([-0.1, 0.1])
    dt = 0.3 * dx / float(c.max())
    x0 = pml + 2
    aperture = n_elem * pitch
    y0 = (ny - aperture) // 2
    theta = np.deg2rad(rng.uniform(-30, 30))
    yc = (np.arange(n_elem) * pitch + 0.5 * width) * dx
    delays = (yc - yc.mean()) * np.sin(theta) / 1540.0
    delays -= delays.min()
    burst = cycles / f0
    length = int(np.ceil((burst + delays.max()) / dt)) + 1
    t = np.arange(length) * dt
    mask = np.zeros(shape, bool)
    elem_of = np.full(shape, -1)
    for e in range(n_elem):
        ys = slice(y0 + e * pitch, y0 + e * pitch + width)
        mask[x0, ys] = True
        elem_of[x0, ys] = e
    points = elem_of[mask]  # element of each source point, C order
    tt = t[None, :] - delays[points][:, None]
    env = np.exp(-((tt - burst / 2) / (burst / 4)) ** 2) * ((tt >= 0) & (tt <= burst))
    sig = 1e4 * env * np.sin(2 * np.pi * f0 * tt)
    return dict(shape=tuple(shape), spacing=(dx, dx), dt=dt, Nt=nt, sound_speed=c, density=rho,
                alpha_coeff=0.5, alpha_power=1.1, p_mask=mask, p=sig, p_mode="additive", sensor_mask=mask.copy(),
                record=("p",), pml_size=(pml, pml), pml_alpha=(2.0, 2.0), use_sg=True, use_kspace=True, smooth_p0=False)


def transmit_problems(n_inst=128, nt=2000, seed=0, sizes=None):
    """``n_inst`` transmit events with grid sizes drawn from the 5-smooth sizes in
    [192, 512] per axis (20-point PML inside), dx = 0.05 mm."""
    rng = np.random.default_rng(seed)
    sizes = sizes or _five_smooth(192, 512)
    return [transmit_problem((int(rng.choice(sizes)), int(rng.choice(sizes))), seed * 100003 + i, nt=nt)
            for i in range(n_inst)]


def vessel_problem(n=512, nt=1500, seed=0, pml=20, n_sensor=256, radius=11e-3, dx=5e-5):
    """Initial-pressure reconstruction case: n^2 grid including a ``pml``-point
    PML, dx = 0.05 mm, homogeneous c = 1500 m/s, rho = 1000 kg/m^3, lossless;
    p0 of 15 smoothed line segments (width 1-4 px) and 5 discs with amplitudes
    U(0.5, 2); ``n_sensor`` Cartesian points on a circle of ``radius``; p0
    smoothing off (the reconstruction variable is p0 itself)."""
    from kwave_gb300.phantoms import circle_points, vessel_phantom

    p0 = vessel_phantom(n, np.random.default_rng(seed), pml)
    sensor = circle_points(n_sensor, radius)
    return dict(shape=(n, n), spacing=(dx, dx), dt=0.3 * dx / 1500.0, Nt=nt, sound_speed=1500.0, density=1000.0,
                p0=p0, smooth_p0=False, sensor_mask=sensor, record=("p",), pml_size=(pml, pml),
                pml_alpha=(2.0, 2.0), use_sg=True, use_kspace=True)


def kwave_objects(prob):
    """The same problem as the objects the legacy kspaceFirstOrder3D call takes."""
    kgrid = SimpleNamespace(N=np.array(prob["shape"]), spacing=np.array(prob["spacing"]), Nt=prob["Nt"], dt=prob["dt"],
                            dim=len(prob["shape"]))
    medium = SimpleNamespace(sound_speed=prob["sound_speed"], density=prob["density"], alpha_coeff=prob["alpha_coeff"],
                             alpha_power=prob["alpha_power"], alpha_mode=None, BonA=prob["BonA"])
    source = SimpleNamespace(p0=prob["p0"])
    sensor = SimpleNamespace(mask=prob["sensor_mask"], record=prob["record"], record_start_index=1)
    opts = SimpleNamespace(pml_size=prob["pml_size"], pml_alpha=prob["pml_alpha"], use_sg=True, use_kspace=True,
                           smooth_p0=prob["smooth_p0"])
    return kgrid, medium, source, sensor, opts


# ---------------------------------------------------------------------------
# measurement helpers
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]
        return False

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes (read + write) per launch of each kernel class, measured with ncu
# (dram__bytes_read.sum + dram__bytes_write.sum) on the 256^3 headline
# workload.
NCU_TRAFFIC_256 = {"rows_rho": 909.6e6, "rows_u": 956.3e6, "rows_eos": 530.1e6, "axis_ops": 269.2e6,
                   "axis_plain": 262.7e6}


def launch_bytes(S):
    """Algorithmic bytes per launch of each kernel class for a set-up problem:
    every array a launch must read or write, counted once (fp32 reals, complex64
    half spectra)."""
    D = S.ndim
    ntot = int(np.prod(S.shape))
    L = S.shape[-1]
    H = L // 2 + 1
    spec = (ntot // L) * H * 8  # half spectrum, without the row padding to an even length
    real = ntot * 4
    grid = lambda name: isinstance(S.fields.get(name), np.ndarray)  # noqa: E731
    powerlaw = S.absorb_mode == 1
    nb = 1 + S.dispersion
    by = {}
    # axis passes with operators: grad (1 in, D out), div (D in, D out), fractional Laplacians (nb in/out)
    ops = [(1 + D) * spec, 2 * D * spec] + ([2 * nb * spec] if powerlaw else [])
    by["axis_ops"] = sum(ops) / len(ops)
    plain = [2 * D * spec, 2 * D * spec, 2 * D * spec] + ([2 * nb * spec, 2 * nb * spec] if powerlaw else []) + [2 * spec]
    by["axis_plain"] = sum(plain) / len(plain) if D == 3 else 0.0
    by["rows_u"] = D * (2 * spec + 2 * real) + sum(real for a in range(D) if grid(f"dtrsg{a}"))
    rho = D * (spec + 2 * real) + (real if grid("rho0") else 0)
    if powerlaw:
        rho += real + nb * spec
    else:
        rho += spec + (real if grid("c0") else 0) + (real if grid("BonA") else 0)
    by["rows_rho"] = rho
    eos = nb * spec + real + spec
    for name in ("c0", "tau", "eta", "rho0", "BonA"):
        if grid(name) and (name != "eta" or S.dispersion) and (name not in ("rho0", "BonA") or S.nonlinear):
            eos += real
    by["rows_eos"] = eos if powerlaw else 0.0
    return by


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(ms, device="cuda"):
    """The largest of the ranks' timed-region lengths (all_reduce MAX over the
    process group); ``ms`` itself outside a group of more than one rank."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms)
    t = torch.tensor([float(ms)], device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(cells, steps, ms_max, ws):
    """Whole-job Mcell-steps/s of ``ws`` independent replicas of ``cells``
    cells over ``steps`` steps, timed by the slowest rank."""
    return ws * cells * steps / (ms_max / 1e3) / 1e6


def cpu_baseline_sample(n=256, steps=1, warm=1):
    """Oracle (the reference's CPU implementation, restated) on the same
    workload: set-up and ``warm`` untimed steps (the first is the t=0 step),
    then ``steps`` timed steps."""
    from oracle.kspace_oracle import OracleSimulation

    warm = max(1, int(warm))
    prob = ivp3d_problem(n=n, nt=warm + steps)
    sim = OracleSimulation(prob, dtype=np.float32).setup()
    for _ in range(warm):
        sim.step()
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.step()
    dt = time.perf_counter() - t0
    return n ** 3 * steps / dt / 1e6, dt


def headline_config(n, nt):
    """The workload description both arms print (identical for the same grid and step count)."""
    return {"workload": WORKLOAD, "grid": [n] * 3, "nt": nt,
            "l2": "inputs larger than L2 (state + medium ~1.1 GB per step at 256^3)"}


def headline_parity(e2e_result=None):
    """Relative L2 errors of the headline result against the unmodified
    reference's float32 and float64 runs of the same seeded problem
    (tests/golden/ivp3d_256, made by tests/golden/make_golden_256.py): the
    1000-step result of the e2e run when that golden exists, otherwise a
    fresh run of the longest problem that has one."""
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    import ivp3d_256
    from kwave_gb300.solver import run_problem

    cps = ivp3d_256.checkpoints()
    if not cps:
        return None
    t = cps[-1]
    if e2e_result is not None and t == 1000:
        got = e2e_result
    else:
        prob = ivp3d_problem(n=256, nt=t, seed=0)
        ivp3d_256.check_inputs(prob, ivp3d_256.load(t)["ref32"])
        prob["record"] = ("p", "p_max", "p_final")
        got = run_problem(prob)
    return {"steps_compared": t, "tolerance_vs_f32": 1e-5, "rel_l2": ivp3d_256.parity(got, t),
            "what": "p_max on all 65,536 plane points, the p series of 256 plane points, every 8th cell of the "
                    "final interior p (when recorded); against the reference solver in float32 and float64"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    steps = max(1, min(args.steps, 3))
    warm = min(args.warmup, 3)
    value, secs = cpu_baseline_sample(args.n, steps, warm)
    cpu = {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
           "sample": f"{steps} time step(s) of the 256^3 workload after set-up and {warm} untimed steps "
                     f"({secs:.1f} s); "
                     "NumPy pocketfft is single-threaded, so the reference path uses one core "
                     f"(host has {os.cpu_count()})"}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": steps,
            "warmup": warm, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, shapes of the named workload)",
            "config": headline_config(args.n, max(1000, args.steps + args.warmup)),
            "timed_steps": f"{warm}..{warm + steps - 1} (a bounded sample of the GPU arm's steps)",
            "cpu_baseline": cpu, "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib as K
    from kwave_gb300.backend import run_gb300_backend
    from kwave_gb300.precompute import build_setup
    from kwave_gb300.solver import DevicePlan

    n = args.n
    K_steps, W = args.steps, args.warmup
    nt = max(1000, K_steps + W)
    prob = ivp3d_problem(n=n, nt=nt, seed=rank)
    S = build_setup(prob)
    stream = torch.cuda.current_stream()
    plan = DevicePlan(S, stream=stream.cuda_stream)
    lib = K.lib()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # warm-up (includes the t = 0 initial-condition step)
    plan.run(W)
    torch.cuda.synchronize()
    cnt0 = C_int64()
    lib.kw_plan_launch_count(plan.handle, ctypes.byref(cnt0))
    barrier()
    torch.cuda.synchronize()
    # timed region: K steps as kw_plan_run runs them (replayed step graphs)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        plan.run(K_steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    cnt1 = C_int64()
    lib.kw_plan_launch_count(plan.handle, ctypes.byref(cnt1))
    # instrumented pass over the same steps: every launch bracketed by CUDA
    # events on the launching stream, for the per-kernel durations
    K.check(lib.kw_plan_reset(plan.handle))
    plan.run(W)
    torch.cuda.synchronize()
    K.check(lib.kw_plan_set_timing(plan.handle, 1))
    ev0.record(stream)
    plan.run(K_steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms_instr = ev0.elapsed_time(ev1)
    kms = (ctypes.c_double * 6)()
    kcnt = (ctypes.c_int64 * 6)()
    K.check(lib.kw_plan_read_timing(plan.handle, kms, kcnt))
    K.check(lib.kw_plan_set_timing(plan.handle, 0))
    ms_max = max_over_ranks(ms)
    cells = int(np.prod(S.shape))
    value = replica_throughput(cells, K_steps, ms_max, ws)

    # roofline of the dominant kernel class (algorithmic bytes / average launch time)
    names = K.KW_K_NAMES
    by = launch_bytes(S)
    dom = max(range(6), key=lambda i: kms[i])
    avg_ms = kms[dom] / max(kcnt[dom], 1)
    peak, peak_kind = measured_peaks()
    achieved = by.get(names[dom], 0.0) / (avg_ms / 1e3) / 1e9
    kernels = {names[i]: {"launches": int(kcnt[i]), "ms_total": kms[i], "share": kms[i] / max(sum(kms), 1e-30),
                          "alg_bytes_per_launch": by.get(names[i], 0.0),
                          "gbs": (by.get(names[i], 0.0) / (kms[i] / max(kcnt[i], 1) / 1e3) / 1e9) if kcnt[i] else None}
               for i in range(6) if kcnt[i]}
    step_gbs = A_MODEL_BYTES_PER_CELL_STEP * cells * K_steps / (ms / 1e3) / 1e9
    # measured DRAM bytes of one step: ncu bytes per launch x launches per step
    ncu_step = (sum(NCU_TRAFFIC_256[names[i]] * kcnt[i] for i in range(6) if kcnt[i] and names[i] in NCU_TRAFFIC_256)
                / K_steps) if n == 256 else None
    plan.close()
    del plan

    # end to end through the public bridge (host inputs -> host results), one full simulation
    e2e = None
    if not args.no_e2e:
        prob_e2e = ivp3d_problem(n=n, nt=1000, seed=rank)
        kg, med, src, sen, opts = kwave_objects(prob_e2e)
        from kwave_gb300.solver import STATS

        torch.cuda.synchronize()
        barrier()
        STATS["d2h_bytes"] = 0
        t0 = time.perf_counter()
        res = run_gb300_backend(kg, med, src, sen, opts)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        assert set(res) == {"p", "p_max"}
        h2d, d2h = STATS["h2d_bytes"], STATS["d2h_bytes"]
        e2e = {"value": cells * 1000 / (t1 - t0) / 1e6, "unit": UNIT, "h2d_bytes_per_step": h2d / 1000,
               "d2h_bytes_per_step": d2h / 1000, "seconds": t1 - t0}

    if rank != 0:
        return 0
    parity = None if (args.no_parity or n != 256) else headline_parity(res if e2e else None)
    cpu = None
    if not args.no_cpu_baseline:
        cv, secs = cpu_baseline_sample(256, 1)
        cpu = {"value": cv, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"1 time step of the 256^3 workload after set-up and the t=0 step ({secs:.1f} s), "
                         "oracle restatement (bit-identical to kwave's native NumPy solver), single-threaded"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K_steps, "warmup": W,
        "ms_per_step": ms_max / K_steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded ellipsoids and Gaussian blobs with the named shapes and ranges)",
        "config": headline_config(n, nt),
        "timed_steps": f"{W}..{W + K_steps - 1}",
        "parallelism": "replicas" if ws > 1 else "single GPU",
        "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": NCU_TRAFFIC_256.get(names[dom]) if n == 256 else None,
                     "traffic_source": "ncu dram bytes per launch, 256^3 headline",
                     "peak_source": peak_kind},
        "step_roofline": {"model_bytes_per_cell_step": A_MODEL_BYTES_PER_CELL_STEP, "achieved": step_gbs,
                          "peak": peak, "frac": step_gbs / peak, "unit": "GB/s",
                          "ncu_dram_bytes_per_step": ncu_step,
                          "ncu_dram_over_model": None if ncu_step is None else
                          ncu_step / (A_MODEL_BYTES_PER_CELL_STEP * cells)},
        "kernels": kernels,
        "instrumented_pass": {"ms_per_step": ms_instr / K_steps,
                              "note": "the same K steps as plain launches, each bracketed by CUDA events: source of "
                                      "the per-kernel durations in roofline and kernels"},
        "parity": parity,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk.summary(),
        "gpu_launches": int(cnt1.value - cnt0.value),
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


TRANSMIT_WORKLOAD = ("batched 2-D transmit events: 128 simulations, grid sizes drawn from the 5-smooth sizes in "
                     "[192,512]^2 incl. 20-pt PML, dx=0.05 mm, speckle c/rho +-2 % + 3 discs +-10 % c, power law "
                     "0.5 dB/(MHz^y cm) y=1.1, 32-element array, steered 3-cycle 1.5 MHz burst (additive source), "
                     "array points recording p, 2000 steps")
TRANSMIT_A_MODEL = 132  # algorithmic bytes per cell-step of this configuration


def run_transmit(args):
    """Batched 2-D transmit events through ``SimulationBatch``: every step of
    all members is one graph launch.  ``value`` = summed cells x timed steps /
    device time; ``one_by_one`` = the same members and steps run one simulation
    after another on the same stream; ``e2e`` = problem dicts in, results out
    (set-up, uploads, the whole run and the result reads) for the full batch."""
    import torch

    import __graft_entry__ as g

    g.build()
    from kwave_gb300.solver import SimulationBatch, run_batch

    ninst, K_steps, W = args.instances, args.steps, args.warmup
    nt = max(2000, W + K_steps + 1)
    probs = transmit_problems(ninst, nt=nt, seed=1)
    cells = sum(int(np.prod(p["shape"])) for p in probs)
    stream = torch.cuda.current_stream()
    t_setup = time.perf_counter()
    b = SimulationBatch.from_problems(probs, stream=stream.cuda_stream, grouped=args.grouped, autotune=args.autotune,
                                      radix=args.radix)
    if args.fft_schedule is not None:
        b.set_radix_order(args.fft_schedule)
    t_setup = time.perf_counter() - t_setup
    tuned = b.tuned
    radix_order = b.radix_order

    def launches():
        return b.launch_count()

    b.run_steps(W)
    torch.cuda.synchronize()
    l0 = launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record(stream)
        b.run_steps(K_steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    nlaunch = launches() - l0
    value = cells * K_steps / (ms / 1e3) / 1e6
    b.close()
    del b
    # the same members one after another, each with the kernels picked for its
    # grid and its own step graphs
    from kwave_gb300.solver import Simulation

    k1 = min(K_steps, 100)
    sims = [Simulation.from_problem(p, stream=stream.cuda_stream).setup() for p in probs]
    for s in sims:
        s._plan.run(W)
    torch.cuda.synchronize()
    ev0.record(stream)
    for s in sims:
        s._plan.run(k1)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms1 = ev0.elapsed_time(ev1)
    one_by_one = cells * k1 / (ms1 / 1e3) / 1e6
    for s in sims:
        s.close()
    del sims
    e2e = None
    if not args.no_e2e:
        probs_e2e = transmit_problems(ninst, nt=2000, seed=2)
        cells_e2e = sum(int(np.prod(p["shape"])) for p in probs_e2e)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = run_batch(probs_e2e, grouped=args.grouped, autotune=args.autotune, radix=args.radix)
        t1 = time.perf_counter()
        assert len(res) == ninst and all(r["p"].shape[1] == 2000 for r in res)
        h2d = sum(sum(np.asarray(v).nbytes for v in (p["sound_speed"], p["density"], p["p"], p["p_mask"]))
                  for p in probs_e2e)
        d2h = sum(r["p"].nbytes for r in res)
        e2e = {"value": cells_e2e * 2000 / (t1 - t0) / 1e6, "unit": UNIT, "h2d_bytes_per_step": h2d / 2000,
               "d2h_bytes_per_step": d2h / 2000, "seconds": t1 - t0}
    cpu = None
    if not args.no_cpu_baseline:
        from oracle.kspace_oracle import OracleSimulation

        prob = transmit_problem((352, 352), 7, nt=40)
        sim = OracleSimulation(prob, dtype=np.float32).setup()
        sim.step()
        t0 = time.perf_counter()
        for _ in range(30):
            sim.step()
        secs = time.perf_counter() - t0
        cpu = {"value": 352 * 352 * 30 / secs / 1e6, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"30 steps of one 352^2 transmit event ({secs:.1f} s), oracle restatement, single-threaded"}
    peak, peak_kind = measured_peaks()
    step_gbs = TRANSMIT_A_MODEL * cells * K_steps / (ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": K_steps, "warmup": W,
        "ms_per_step": ms / K_steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded speckle media, discs, steering angles and grid sizes of the named ranges)",
        "config": {"workload": TRANSMIT_WORKLOAD, "instances": ninst, "cells_per_step": cells, "nt": nt,
                   "batch": "grouped launches" if args.grouped else "members as parallel graph branches",
                   "autotune": bool(args.autotune), "tuned": tuned, "radix_autotune": bool(args.radix),
                   "radix_order": radix_order, "setup_seconds": t_setup,
                   "l2": f"inputs larger than L2 ({cells * 4 * 12 / 1e9:.1f} GB of state, medium and spectra)"},
        "step_roofline": {"model_bytes_per_cell_step": TRANSMIT_A_MODEL, "achieved": step_gbs, "peak": peak,
                          "frac": step_gbs / peak, "unit": "GB/s", "peak_source": peak_kind},
        "one_by_one": {"value": one_by_one, "unit": UNIT, "steps": k1},
        "cpu_baseline": cpu, "e2e": e2e, "clocks": clk.summary(), "gpu_launches": int(nlaunch),
    }
    print(json.dumps(line), flush=True)
    return 0


ADJOINT_WORKLOAD = ("p0 reconstruction: 512^2 incl. 20-pt PML, dx=0.05 mm, c=1500, lossless, vessel phantom "
                    "(15 segments + 5 discs), 256-point Cartesian circle r=11 mm, 1500 steps, data + 1 % noise, "
                    "CGLS (conjugate gradients on the normal equations) from zero")


def run_adjoint(args):
    """p0 reconstruction by plain adjoint iterations (CGLS): each iteration is
    one GPU adjoint (transposed time loop) and one forward pass on one device
    plan (``adjoint.LinearP0``).  ``value`` = cell-steps of all passes / wall
    time of the iterations, host inputs and outputs of every pass included
    (what ``e2e`` also reports); the line gives seconds per iteration, the
    relative p0 error per iteration, the time to 1 % and, under
    ``gradient_p0_c``, one checkpointed misfit gradient with respect to p0
    and c (the sound-speed gradient of the same problem)."""
    import torch

    import __graft_entry__ as g

    g.build()
    from kwave_gb300.adjoint import LinearP0, cgls_p0, default_checkpoint_interval, misfit_gradients

    prob = vessel_problem(nt=1500)
    rng = np.random.default_rng(11)
    op = LinearP0(prob)
    d_clean = op.forward(prob["p0"])
    d_obs = d_clean + 0.01 * np.std(d_clean) * rng.standard_normal(d_clean.shape)
    cgls_p0(op.forward, op.adjoint, d_obs, np.zeros(prob["shape"]), 1)  # warm-up (library, kernels, graphs)
    torch.cuda.synchronize()
    iters = max(1, args.steps if args.steps < 1000 else 20)
    p0 = op.passes
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        p, hist = cgls_p0(op.forward, op.adjoint, d_obs, np.zeros(prob["shape"]), iters, p_true=prob["p0"])
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
    passes = op.passes - p0
    op.close()
    cells = int(np.prod(prob["shape"]))
    errs = [h[1] for h in hist]
    to1 = next((i + 1 for i, e in enumerate(errs) if e <= 0.01), None)
    nslots = 256 * 4  # bilinear corners of the Cartesian points
    h2d = (cells * 4 + nslots * prob["Nt"] * 4) / 2  # p0 of a forward or residual of an adjoint, per pass
    d2h = (256 * prob["Nt"] * 4 + cells * 4) / 2     # series of a forward or gradient of an adjoint, per pass
    value = cells * prob["Nt"] * passes / secs / 1e6
    # one gradient with respect to p0 and c (checkpointed forward + adjoint)
    K = default_checkpoint_interval(prob["Nt"], 2)
    misfit_gradients(prob, 0.5 * prob["p0"], d_obs, checkpoint_interval=K)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    misfit_gradients(prob, 0.5 * prob["p0"], d_obs, checkpoint_interval=K)
    torch.cuda.synchronize()
    gsecs = time.perf_counter() - t0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
            "steps": iters, "warmup": 1, "ms_per_step": 1e3 * secs / iters, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic vessel phantom, 1 % noise",
            "config": {"workload": ADJOINT_WORKLOAD, "iterations": iters, "passes": passes,
                       "l2": "each pass streams the 512^2 state 1500 times; no flush between passes"},
            "seconds_per_iteration": secs / iters, "p0_rel_error": errs,
            "iterations_to_1pct": to1, "seconds_to_1pct": None if to1 is None else secs / iters * to1,
            "gradient_p0_c": {"seconds": gsecs, "checkpoint_interval": K,
                              "note": "forward with checkpoints every K steps, then the transposed loop regenerating "
                                      "each segment's forward density sums"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": h2d / prob["Nt"],
                    "d2h_bytes_per_step": d2h / prob["Nt"],
                    "note": "every pass takes host inputs and returns host outputs; a step is one time step"},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


WARMSTART_WORKLOAD = ("learned warm start: 4-level U-Net, 32 base channels, BF16 on tcgen05, trained on pairs (time-"
                      "reversal image, p0) from the device forward solver at 256^2 (vessel phantoms, 128-point circle "
                      "r=5 mm on the grid, 800 steps, 1 % noise); held-out problems refined by CGLS from the network's "
                      "estimate vs CGLS from zero")


def run_warmstart(args):
    """Learned warm start against plain adjoint iterations.  Generates the
    training pairs with the device solver (batched forward runs and batched
    time-reversal runs), trains the U-Net with the library's tcgen05 kernels,
    then on held-out problems runs CGLS from zero and CGLS from the network's
    estimate (inference time included) and reports the relative p0 error
    after each iteration, the time to 1 % and the time to reach the error
    that plain CGLS ends at."""
    import torch

    import __graft_entry__ as g

    g.build()
    from kwave_gb300.warmstart import UNet, fit_input_scale, generate_pairs, noisy, pair_problem, refine, time_to

    npairs, epochs, iters, ntest = args.pairs, args.epochs, args.iterations, args.test_problems
    t0 = time.perf_counter()
    imgs, p0s = generate_pairs(npairs, seed0=1000, batch=256, grouped=args.grouped)
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    s = fit_input_scale(imgs[: min(npairs, 512)], p0s[: min(npairs, 512)])
    net = UNet(seed=0, in_scale=s)
    t0 = time.perf_counter()
    hist = net.train(imgs, p0s, epochs=epochs, batch=16, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del imgs, p0s
    cells = 256 * 256
    results = []
    for j in range(ntest):
        prob = pair_problem(90000 + j)
        from kwave_gb300.adjoint import forward_p0

        d_obs = noisy(forward_p0(prob, prob["p0"]).astype(np.float64), np.random.default_rng(90000 + j))
        # each arm starts with the objects of the previous one collected, so
        # neither pays for the other's clean-up
        gc.collect()
        torch.cuda.synchronize()
        # plain: CGLS from zero
        _, h0, st0 = refine(prob, d_obs, np.zeros(prob["shape"]), iters, p_true=prob["p0"])
        # learned: time reversal + network + CGLS from its estimate
        gc.collect()
        torch.cuda.synchronize()
        tl = time.perf_counter()
        from kwave_gb300.warmstart import time_reversal_images

        img = time_reversal_images([prob], [d_obs])[0].astype(np.float32)
        torch.cuda.synchronize()
        t_tr = time.perf_counter() - tl
        est = net.predict(img[None])[0]
        torch.cuda.synchronize()
        t_net = time.perf_counter() - tl
        e_net = float(np.linalg.norm(est - prob["p0"]) / np.linalg.norm(prob["p0"]))
        _, h1, st1 = refine(prob, d_obs, est.astype(np.float64), iters, p_true=prob["p0"])
        e0 = [h[1] for h in h0]
        e1 = [h[1] for h in h1]
        target = min(e0)
        results.append({"plain_errors": e0, "learned_errors": e1, "network_error": e_net,
                        "tr_plus_network_seconds": t_net, "time_reversal_seconds": t_tr, "plain_seconds": st0[-1], "learned_seconds": t_net + st1[-1],
                        "plain_to_1pct": time_to(e0, st0, 0.01), "learned_to_1pct": time_to(e1, st1, 0.01, t_net),
                        "plain_to_plain_best": time_to(e0, st0, target),
                        "learned_to_plain_best": (t_net if e_net <= target else time_to(e1, st1, target, t_net))})
    ratios = [r["plain_to_plain_best"] / r["learned_to_plain_best"] for r in results
              if r["learned_to_plain_best"] is not None and r["plain_to_plain_best"] is not None]
    line = {"metric": METRIC, "impl": "gb300", "workload": "warmstart", "value": float(np.median(ratios)) if ratios else None,
            "unit": "x (time for plain CGLS to reach its own best p0 error / time for learned+CGLS to reach it)",
            "n_gpus": 1, "higher_is_better": True, "dtype": "bf16 network, f32 solver",
            "data": "synthetic vessel phantoms", "config": {"workload": WARMSTART_WORKLOAD, "pairs": npairs,
                                                            "grouped_generation": bool(args.grouped),
                                                            "epochs": epochs, "cgls_iterations": iters,
                                                            "test_problems": ntest},
            "generation_seconds": t_gen, "training_seconds": t_train, "train_loss_per_epoch": hist,
            "median_network_error": float(np.median([r["network_error"] for r in results])),
            "median_plain_final_error": float(np.median([r["plain_errors"][-1] for r in results])),
            "median_learned_final_error": float(np.median([r["learned_errors"][-1] for r in results])),
            "time_to_1pct": {"plain": [r["plain_to_1pct"] for r in results],
                             "learned": [r["learned_to_1pct"] for r in results]},
            "per_problem": results, "cell_steps_per_pass": cells * 800}
    print(json.dumps(line), flush=True)
    return 0


UNET_WORKLOAD = ("U-Net training step of the learned warm start: batch 16 of 256^2 images, 4 levels, 32 base "
                 "channels, BF16 activations and weights, FP32 accumulation on tcgen05; forward, data and weight "
                 "gradients, Adam")


def unet_step_flops(nb=16, n=256):
    """Algorithmic flops of one training step: 2 M N K per convolution for the
    forward pass, the data gradient (all layers but the first) and the weight
    gradient, M = pixels, N = output channels, K = 9 x input channels."""
    from kwave_gb300.warmstart import LAYERS

    res = {"e1": n, "e2": n // 2, "e3": n // 4, "ba": n // 8, "bb": n // 8, "d3": n // 4, "d2": n // 2, "d1": n,
           "ou": n}
    tot = 0.0
    for name, c1, c2, co, _ in LAYERS:
        h = res[name[:2]]
        f = 2.0 * nb * h * h * co * 9 * (c1 + c2)
        tot += f * (3 if name != "e1a" else 2)
    return tot


def run_unet(args):
    """Throughput of the U-Net training step on the tensor cores: ``value`` =
    images per second; the roofline is the convolution flops of a step over
    its device time against the measured bf16 tensor peak, and the dominant
    kernel (the tcgen05 convolution, ``k_conv_tma``) is timed alone on the
    largest layer for its own fraction."""
    import torch

    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import unet_ops as U
    from kwave_gb300.warmstart import UNet

    nb, n = 16, 256
    rng = np.random.default_rng(0)
    imgs = torch.as_tensor(rng.random((nb, n, n), dtype=np.float32), device="cuda")
    tgts = torch.as_tensor(rng.random((nb, n, n), dtype=np.float32), device="cuda")
    net = UNet(seed=0, in_scale=1.0)
    loss = torch.zeros(1, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(max(3, args.warmup)):
        net.loss_and_grad(imgs, tgts, loss)
        net.adam_step(1e-4)
    torch.cuda.synchronize()
    K_steps = args.steps if args.steps < 1000 else 20
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        ev0.record(stream)
        for _ in range(K_steps):
            net.loss_and_grad(imgs, tgts, loss)
            net.adam_step(1e-4)
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / K_steps
    flops = unet_step_flops(nb, n)
    # the dominant kernel alone: the 32 -> 32 convolution at 256^2 (batch 16)
    x = torch.randn((nb, n, n, 32), device="cuda").to(torch.bfloat16)
    w = (0.1 * torch.randn((32, 9, 32), device="cuda")).to(torch.bfloat16)
    y = torch.empty((nb, n, n, 32), dtype=torch.bfloat16, device="cuda")
    for _ in range(3):
        U.conv3x3(x, w, None, relu=True, y=y)
    torch.cuda.synchronize()
    reps = 20
    ev0.record(stream)
    for _ in range(reps):
        U.conv3x3(x, w, None, relu=True, y=y)
    ev1.record(stream)
    torch.cuda.synchronize()
    kms = ev0.elapsed_time(ev1) / reps
    kflops = 2.0 * nb * n * n * 32 * 9 * 32
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("bf16_tflops", 1900.0))
    step_tf = flops / (ms / 1e3) / 1e12
    k_tf = kflops / (kms / 1e3) / 1e12
    line = {"metric": METRIC, "impl": "gb300", "workload": "unet", "value": nb / (ms / 1e3), "unit": "images/s",
            "n_gpus": 1, "steps": K_steps, "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (f32 accumulation)", "data": "random images",
            "config": {"workload": UNET_WORKLOAD, "batch": nb, "image": n},
            "step_roofline": {"bound": "tensor", "flops_per_step": flops, "achieved": step_tf, "peak": peak,
                              "unit": "TFLOP/s", "frac": step_tf / peak, "peak_source": "measured" if peaks else "fallback"},
            "roofline": {"bound": "tensor", "kernel": "k_conv_tma (conv3x3 32->32, 16 x 256^2)", "achieved": k_tf,
                         "peak": peak, "unit": "TFLOP/s", "frac": k_tf / peak, "traffic": None,
                         "kernel_ms": kms},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


import ctypes  # noqa: E402

C_int64 = ctypes.c_int64


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=256, help="grid edge (the headline workload is 256)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the comparison with the 256^3 golden")
    ap.add_argument("--pairs", type=int, default=10000, help="warmstart workload: training pairs")
    ap.add_argument("--epochs", type=int, default=6, help="warmstart workload: training epochs")
    ap.add_argument("--iterations", type=int, default=20, help="warmstart workload: CGLS iterations per problem")
    ap.add_argument("--test-problems", type=int, default=4, help="warmstart workload: held-out problems")
    ap.add_argument("--workload", default="ivp3d", choices=["ivp3d", "transmit", "adjoint", "warmstart", "unet"],
                    help="ivp3d: the 256^3 headline; transmit: 128 batched 2-D transmit events; "
                         "adjoint: p0 reconstruction by adjoint iterations at 512^2")
    ap.add_argument("--instances", type=int, default=128, help="transmit workload: simulations per batch")
    ap.add_argument("--grouped", action="store_true",
                    help="transmit / warmstart workloads: grouped launches across the batch members")
    ap.add_argument("--autotune", action="store_true", help="transmit workload: autotune each member's launch geometry")
    ap.add_argument("--radix", action="store_true", help="transmit workload: autotune the FFT radix schedule too")
    ap.add_argument("--fft-schedule", type=int, default=None,
                    help="transmit workload: FFT schedule of every member (0-2 Stockham radix orders, 3 two-level)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "transmit":
        return run_transmit(args)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "warmstart":
        return run_warmstart(args)
    if args.workload == "unet":
        return run_unet(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
