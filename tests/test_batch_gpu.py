"""Step graphs and batches on the GPU.

* Replayed step graphs (the default of ``kw_plan_run``) give bit-identical
  results to plain per-step launches on every golden case: the captured
  launches are the same kernels with the same arguments, and only the step
  index comes from the device counter.
* ``SimulationBatch`` (``kw_batch``) runs members of different dimensions,
  sizes, step counts, sources and sensors together, with the passes of the
  members grouped into shared launches; every member's results are
  bit-identical to running it alone with the same kernels, also when the
  batch is advanced in uneven chunks or mixes grouped and ungrouped members,
  and meet the parity bar against the reference's golden outputs.
* Batched 2-D transmit events (linear array, steered tone burst, additive
  k-space corrected source, power-law absorption, uneven 5-smooth grid sizes,
  odd lengths included) agree with the oracle within 1e-5 relative L2.
"""
import numpy as np
import pytest

from fixtures import case_names, load_case

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def assert_same(name, got, ref):
    assert set(got) == set(ref), (name, sorted(got), sorted(ref))
    for k in ref:
        assert got[k].shape == ref[k].shape, (name, k)
        assert np.array_equal(got[k], ref[k]), (name, k, float(np.max(np.abs(got[k] - ref[k]))))


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()
    from kwave_gb300 import _lib

    _lib.require_device()


def plain_run(prob, generic_fft=False):
    from kwave_gb300.solver import Simulation

    sim = Simulation.from_problem(prob)
    sim.setup(generic_fft=generic_fft)
    sim._plan.set_graphs(False)
    try:
        return sim.run()
    finally:
        sim.close()


@pytest.fixture(scope="module")
def golden_plain():
    return {name: (load_case(name)[0], plain_run(load_case(name)[0])) for name in case_names()}


@pytest.fixture(scope="module")
def golden_generic():
    return {name: (load_case(name)[0], plain_run(load_case(name)[0], generic_fft=True)) for name in case_names()}


def test_step_graphs_bit_exact(golden_plain):
    from kwave_gb300.solver import run_problem

    for name, (prob, ref) in golden_plain.items():
        assert_same(name, run_problem(prob), ref)


def test_batch_bit_exact_and_parity(golden_generic):
    from kwave_gb300.solver import SimulationBatch

    names = sorted(golden_generic)
    b = SimulationBatch.from_problems([golden_generic[n][0] for n in names], grouped=True)
    try:
        got = b.run()
        launches = b.launch_count()
    finally:
        b.close()
    for name, res in zip(names, got):
        assert_same(name, res, golden_generic[name][1])
        _, r32, r64, _ = load_case(name)
        for k in r32:
            e32, gap = rel_l2(res[k], r32[k]), rel_l2(r32[k], r64[k])
            if gap > 0.5 * TOL:
                assert e32 <= TOL or rel_l2(res[k], r64[k]) <= 1.5 * gap + 1e-6, (name, k, e32, gap)
            else:
                assert e32 <= TOL, (name, k, e32)
    # grouped: far fewer launches than the members' steps would take one by one
    # (about a dozen each); device-side loop runs add one counting kernel per step
    steps = sum(golden_generic[n][0]["Nt"] for n in names)
    print(f"{len(names)} members, {steps} member-steps, {launches} launches")
    assert launches < 5 * steps


def test_batch_mixed_members(golden_plain, golden_generic):
    """Grouped members (generic FFT kernels) beside ungrouped ones (default
    kernels, joining as their own step graphs)."""
    from kwave_gb300.solver import Simulation, SimulationBatch

    names = sorted(golden_plain)[:8]
    sims = []
    for i, n in enumerate(names):
        sim = Simulation.from_problem(golden_plain[n][0])
        sim.setup(generic_fft=bool(i % 2))
        sims.append(sim)
    b = SimulationBatch(sims)
    try:
        for i, (n, res) in enumerate(zip(names, b.run())):
            assert_same(n, res, (golden_generic if i % 2 else golden_plain)[n][1])
    finally:
        b.close()


def test_batch_uneven_chunks(golden_generic):
    """Members with different Nt advanced in chunks of 1, 7 and 13 steps: the
    last step of every chunk is a plain step, members that reached Nt idle."""
    from kwave_gb300.solver import SimulationBatch

    names = sorted(golden_generic)[:6]
    b = SimulationBatch.from_problems([golden_generic[n][0] for n in names], grouped=True)
    try:
        for chunk in (1, 7, 13):
            b.run_steps(chunk)
        b.run()
        for name, sim in zip(names, b.sims):
            assert sim.t == sim.S.Nt
            assert_same(name, sim.results(), golden_generic[name][1])
    finally:
        b.close()


def test_autotune_bit_exact():
    """The autotuner changes only the launch geometry of the run-time-length
    kernels: results stay bit-identical, the plan is rewound to t = 0, and a
    power-of-two plan keeps its kernels."""
    import bench
    from kwave_gb300.solver import Simulation

    prob = bench.transmit_problem((90, 150), 11, nt=40, n_elem=6, pml=12)
    ref = plain_run(prob)
    sim = Simulation.from_problem(prob)
    sim.setup(autotune=True)
    try:
        T, R = sim.tuned
        assert T in (2, 4, 8, 16) and R >= 1, sim.tuned
        assert sim._plan.time_index() == 0
        assert_same("autotuned", sim.run(), ref)
    finally:
        sim.close()
    prob2 = bench.transmit_problem((64, 128), 12, nt=20, n_elem=6, pml=12)
    sim = Simulation.from_problem(prob2)
    sim.setup(autotune=True)
    try:
        assert_same("autotuned pow2", sim.run(), plain_run(prob2))
    finally:
        sim.close()


def test_batch_autotune_bit_exact(golden_generic):
    from kwave_gb300.solver import SimulationBatch

    names = sorted(golden_generic)[:6]
    for grouped in (False, True):
        b = SimulationBatch.from_problems([golden_generic[n][0] for n in names], grouped=grouped, autotune=True)
        try:
            T, f = b.tuned
            assert T in (0, 2, 4, 8, 16) and f in (0.5, 1.0, 2.0), b.tuned
            assert all(s.t == 0 for s in b.sims)
            for name, res in zip(names, b.run()):
                if grouped:
                    assert_same(name, res, golden_generic[name][1])
                else:
                    _, r32, r64, _ = load_case(name)
                    for k in r32:
                        e32, gap = rel_l2(res[k], r32[k]), rel_l2(r32[k], r64[k])
                        assert e32 <= TOL or rel_l2(res[k], r64[k]) <= 1.5 * gap + 1e-6, (name, k, e32)
        finally:
            b.close()


TRANSMIT = [((96, 120), 1), ((75, 135), 2), ((128, 100), 3), ((90, 144), 4), ((81, 96), 5), ((64, 128), 6)]


def test_transmit_events_batch_vs_oracle():
    import bench
    from kwave_gb300.solver import run_batch
    from oracle.kspace_oracle import OracleSimulation

    probs = [bench.transmit_problem(shape, seed, nt=90, n_elem=6, pml=12) for shape, seed in TRANSMIT]
    got = run_batch(probs)
    got_grouped = run_batch(probs, grouped=True)
    for (shape, _), prob, res, resg in zip(TRANSMIT, probs, got, got_grouped):
        ref = OracleSimulation(prob, np.float32).run()
        for mode, r in (("branches", res), ("grouped", resg)):
            e = rel_l2(r["p"], ref["p"])
            print(f"transmit {shape} {mode}: p rel L2 {e:.2e}")
            assert r["p"].shape == ref["p"].shape
            assert e <= TOL, (shape, mode, e)


def test_radix_schedules_vs_oracle():
    """Every radix schedule of the run-time-length FFTs, set on a plan or
    picked by the batch radix autotuner, keeps transmit events and the golden
    cases within the parity bar of the oracle / the reference (the schedules
    differ in rounding, so they are compared with the oracle, not bit for
    bit)."""
    import bench
    from kwave_gb300.solver import Simulation, SimulationBatch
    from oracle.kspace_oracle import OracleSimulation

    probs = [bench.transmit_problem(shape, seed, nt=90, n_elem=6, pml=12) for shape, seed in TRANSMIT[:3]]
    refs = [OracleSimulation(p, np.float32).run()["p"] for p in probs]
    for order in range(4):
        for prob, ref in zip(probs, refs):
            sim = Simulation.from_problem(prob).setup(generic_fft=True)
            try:
                sim._plan.set_radix_order(order)
                e = rel_l2(sim.run()["p"], ref)
            finally:
                sim.close()
            print(f"radix schedule {order} {prob['shape']}: {e:.2e}")
            assert e <= TOL, (order, prob["shape"], e)
    b = SimulationBatch.from_problems(probs, grouped=True, autotune=True, radix=True)
    try:
        res = b.run()
        print("tuned radix schedule", b.radix_order)
        for r, ref in zip(res, refs):
            assert rel_l2(r["p"], ref) <= TOL
    finally:
        b.close()
    name = "het2d_abs_nl"
    prob, r32, _, _ = load_case(name)
    for order in (1, 2, 3):
        sim = Simulation.from_problem(prob).setup(generic_fft=True)
        try:
            sim._plan.set_radix_order(order)
            res = sim.run()
        finally:
            sim.close()
        for k in r32:
            assert rel_l2(res[k], r32[k]) <= TOL, (name, order, k)


@pytest.mark.parametrize("grouped", [False, True])
def test_device_loop_runs_bit_exact(grouped):
    """Runs of steps with one launch sequence as one launch of a device-side
    loop graph (conditional while node over the batch's step graph) give the
    same results bit for bit as one graph launch per step, with far fewer
    graph launches."""
    import bench
    from kwave_gb300.solver import SimulationBatch

    probs = [bench.transmit_problem(shape, seed, nt=160, n_elem=6, pml=12) for shape, seed in TRANSMIT[:4]]
    out, counts = [], []
    for loops in (False, True):
        b = SimulationBatch.from_problems(probs, grouped=grouped)
        try:
            b.set_loops(loops)
            out.append(b.run())
            counts.append(b.graph_launches())
        finally:
            b.close()
    print(f"grouped={grouped}: graph launches per step {counts[0]} -> with loops {counts[1]}")
    for ra, rb in zip(*out):
        for k in ra:
            assert np.array_equal(ra[k], rb[k]), k
    assert counts[1] < counts[0] // 4, counts
