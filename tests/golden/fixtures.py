"""Load/save golden cases: a problem description plus reference outputs.

A case file ``<name>.npz`` holds
  * ``in:<key>``       problem inputs (see ``oracle/kspace_oracle.py`` for keys),
  * ``ref32:<key>``    outputs of the unmodified reference solver, dtype=float32,
  * ``ref64:<key>``    outputs of the unmodified reference solver, dtype=float64.
  * ``meta:<key>``     anything else the case needs (options of the call).
Strings and tuples are stored as 0-d/1-d numpy arrays; ``None`` is omitted.
Cases of the solver itself sit in this folder; cases of the entry points
built on it (unified ``kspaceFirstOrder``, ``TimeReversal``) in ``api/``.
"""
from pathlib import Path

import numpy as np

GOLDEN_DIR = Path(__file__).resolve().parent

_TUPLE_KEYS = ("shape", "spacing", "pml_size", "pml_alpha", "record")
_STR_KEYS = ("p_mode", "u_mode", "alpha_mode")
_BOOL_KEYS = ("use_sg", "use_kspace", "smooth_p0")


def _dir(subdir):
    return GOLDEN_DIR / subdir if subdir else GOLDEN_DIR


def save_case(name, prob, outs32, outs64, meta=None, subdir=None):
    arrs = {}
    for k, v in prob.items():
        if v is None:
            continue
        arrs[f"in:{k}"] = np.asarray(v)
    for k, v in outs32.items():
        arrs[f"ref32:{k}"] = np.asarray(v)
    for k, v in outs64.items():
        arrs[f"ref64:{k}"] = np.asarray(v)
    for k, v in (meta or {}).items():
        arrs[f"meta:{k}"] = np.asarray(v)
    _dir(subdir).mkdir(exist_ok=True)
    np.savez_compressed(_dir(subdir) / f"{name}.npz", **arrs)


def load_case(name, subdir=None):
    z = np.load(_dir(subdir) / f"{name}.npz", allow_pickle=False)
    prob, r32, r64, meta = {}, {}, {}, {}
    for key in z.files:
        kind, k = key.split(":", 1)
        v = z[key]
        if kind == "in":
            if k in _TUPLE_KEYS:
                v = tuple(v.tolist())
            elif k in _STR_KEYS:
                v = str(v)
            elif k in _BOOL_KEYS:
                v = bool(v)
            elif v.ndim == 0:
                v = v.item()
            prob[k] = v
        elif kind == "ref32":
            r32[k] = v
        elif kind == "ref64":
            r64[k] = v
        else:
            meta[k] = v
    return prob, r32, r64, meta


def case_names(subdir=None):
    return sorted(p.stem for p in _dir(subdir).glob("*.npz"))
