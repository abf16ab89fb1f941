"""Rebuild user-level objects (grid, medium, source, sensor namespaces) and
call options from an ``api/`` golden case, for the unified entry point and
time-reversal tests."""
from types import SimpleNamespace as NS

import numpy as np

from fixtures import case_names, load_case

SUBDIR = "api"
MEDIUM_KEYS = ("sound_speed", "density", "alpha_coeff", "alpha_power", "alpha_mode", "BonA")
SOURCE_KEYS = ("p0", "p_mask", "p", "p_mode", "u_mask", "ux", "uy", "uz", "u_mode")


def names(prefix=""):
    return [n for n in case_names(SUBDIR) if n.startswith(prefix)]


def _opt(v):
    v = v.item() if v.ndim == 0 else tuple(v.tolist())
    return v


def load(name):
    prob, r32, r64, meta = load_case(name, SUBDIR)
    opts = {k[4:]: _opt(v) for k, v in meta.items() if k.startswith("opt_")}
    return prob, opts, r32, r64


def objects(prob):
    Nt, dt = int(prob["Nt"]), float(prob["dt"])
    kgrid = NS(N=np.array(prob["shape"]), spacing=np.array(prob["spacing"]), Nt=Nt, dt=dt,
               t_array=np.arange(Nt) * dt, dim=len(prob["shape"]))
    medium = NS(**{k: prob.get(k) for k in MEDIUM_KEYS})
    source = NS(**{k: prob.get(k) for k in SOURCE_KEYS})
    sensor = None
    if prob.get("sensor_mask") is not None:
        sensor = NS(mask=prob["sensor_mask"], record=list(prob["record"]) if prob.get("record") else None,
                    record_start_index=None)
    return kgrid, medium, source, sensor
