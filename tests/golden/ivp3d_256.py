"""Reader of the 256^3 headline golden (``ivp3d_256/ref{32,64}_tNNNN.npz``,
written by ``make_golden_256.py`` from the unmodified reference) and the
parity figures of a GPU result against it.

A GPU result is a dict with ``p`` (65,536 x T series of the z = 20 plane,
sensor-major), ``p_max`` and ``p_final`` (interior field) of the same
problem run for T steps.  Figures are relative L2 errors over the stored
reductions: all points of ``p_max``, the 256-point subset of the ``p``
series, and the every-8th-cell subset of ``p_final``.
"""
from pathlib import Path

import numpy as np

DIR = Path(__file__).resolve().parent / "ivp3d_256"


def checkpoints():
    """Step counts for which both the float32 and the float64 golden exist."""
    have = {}
    for f in DIR.glob("ref*_t*.npz"):
        tag, t = f.stem.split("_t")
        have.setdefault(int(t), set()).add(tag)
    return sorted(t for t, tags in have.items() if {"ref32", "ref64"} <= tags)


def load(t):
    out = {}
    for tag in ("ref32", "ref64"):
        z = np.load(DIR / f"{tag}_t{t:04d}.npz", allow_pickle=False)
        out[tag] = {k: z[k] for k in z.files}
    return out


def check_inputs(prob, ref):
    """The regenerated inputs must be those the golden was made from."""
    for k in ("sound_speed", "density", "p0"):
        a = np.asarray(prob[k], np.float64)
        got = np.array([a.sum(), (a * a).sum()])
        want = ref[f"sum_{k}"]
        if not np.allclose(got, want, rtol=1e-12, atol=0):
            raise AssertionError(f"regenerated {k} differs from the golden's input: {got} vs {want}")


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def parity(got, t):
    """Relative L2 errors of a GPU result against the float32 and float64
    reference for the t-step golden: {key: {"vs_f32", "vs_f64", "f32_vs_f64"}}."""
    g = load(t)
    r32, r64 = g["ref32"], g["ref64"]
    rows = r32["rows"]
    fs = int(r32["field_stride"])
    mine = {"p_max": np.asarray(got["p_max"]),
            "p_sub": np.asarray(got["p"])[rows, :t]}
    if "p_final" in got:
        pf = np.asarray(got["p_final"])
        mine["pfin_sub"] = pf[::fs, ::fs, ::fs]
    out = {}
    for k, v in mine.items():
        out[k] = {"vs_f32": _rel(v, r32[k]), "vs_f64": _rel(v, r64[k]), "f32_vs_f64": _rel(r32[k], r64[k])}
    return out
