"""Import shim for the unmodified k-wave-python reference (test infrastructure only).

Used by ``make_golden.py`` and by the CPU tests that compare the oracle port
against the reference when the reference checkout is present.  It never ships
with the product path and nothing on the GPU side imports it.

Why a shim is needed (reference 0.6.3rc1):
  * ``kwave/__init__.py:293-294`` downloads the closed C++ binaries at import
    time; offline this raises ``URLError`` (only ``TimeoutError`` is caught).
    We register a pre-built ``kwave`` package object so ``__init__`` never runs.
  * ``beartype``, ``jaxtyping``, ``matplotlib``, ``cv2`` and ``h5py`` are not
    installed; the native solver path never calls them, so identity / ``Any``
    stubs suffice.
  * scipy >= 1.16 made ``RegularGridInterpolator.values`` read-only while
    ``kwave/solvers/kspace_solver.py:358`` assigns it every step; a setter is
    restored.
"""
import os
import sys
import types
import typing
from pathlib import Path

# The checkout is named by KWAVE_REFERENCE_ROOT; without it, a ``reference``
# directory beside the repository is used (the layout of the build host).
_BESIDE_REPO = Path(__file__).resolve().parents[3] / "reference"
REFERENCE_ROOT = Path(os.environ.get("KWAVE_REFERENCE_ROOT", str(_BESIDE_REPO)))


def reference_available() -> bool:
    return (REFERENCE_ROOT / "kwave" / "solvers" / "kspace_solver.py").exists()


class _AnySubscript:
    def __getitem__(self, item):
        return typing.Any

    def __call__(self, *a, **k):
        return typing.Any


def install():
    """Install the stubs and the package object.  Idempotent."""
    if "kwave" in sys.modules and getattr(sys.modules["kwave"], "_graft_shim", False):
        return sys.modules["kwave"]
    if not reference_available():
        raise RuntimeError(f"reference checkout not found at {REFERENCE_ROOT}")

    # beartype: decorator = identity, beartype.typing = typing
    bt = types.ModuleType("beartype")
    bt.beartype = lambda f=None, **k: (f if f is not None else (lambda g: g))
    bt.typing = typing
    sys.modules.setdefault("beartype", bt)
    sys.modules.setdefault("beartype.typing", typing)
    btv = types.ModuleType("beartype.vale")
    btv.Is = _AnySubscript()
    sys.modules.setdefault("beartype.vale", btv)
    btd = types.ModuleType("beartype.door")
    btd.is_bearable = lambda *a, **k: True
    sys.modules.setdefault("beartype.door", btd)

    jt = types.ModuleType("jaxtyping")
    for name in ("Float", "Num", "Real", "Bool", "Int", "Integer", "Complex", "Shaped", "UInt", "Inexact", "Array"):
        setattr(jt, name, _AnySubscript())
    sys.modules.setdefault("jaxtyping", jt)

    mpl = types.ModuleType("matplotlib")
    mpl.__path__ = []
    plt = types.ModuleType("matplotlib.pyplot")
    colors = types.ModuleType("matplotlib.colors")
    colors.ListedColormap = lambda *a, **k: None
    colors.LinearSegmentedColormap = types.SimpleNamespace(from_list=lambda *a, **k: None)
    cm = types.ModuleType("matplotlib.cm")
    anim = types.ModuleType("matplotlib.animation")
    mpl.pyplot, mpl.colors, mpl.cm, mpl.animation = plt, colors, cm, anim
    for n, m in (("matplotlib", mpl), ("matplotlib.pyplot", plt), ("matplotlib.colors", colors),
                 ("matplotlib.cm", cm), ("matplotlib.animation", anim)):
        sys.modules.setdefault(n, m)
    sys.modules.setdefault("cv2", types.ModuleType("cv2"))
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))

    kw = types.ModuleType("kwave")
    kw.__path__ = [str(REFERENCE_ROOT / "kwave")]
    kw.__file__ = str(REFERENCE_ROOT / "kwave" / "__init__.py")
    kw.__version__ = "0.6.3rc1"
    kw.PLATFORM = "linux"
    kw.BINARY_PATH = kw.BINARY_DIR = Path("/nonexistent")
    kw._graft_shim = True
    sys.modules["kwave"] = kw

    from scipy.interpolate import RegularGridInterpolator as RGI

    prop = getattr(RGI, "values", None)
    if isinstance(prop, property) and prop.fset is None:
        def _get(self):
            return self._values if hasattr(self, "_values") else prop.fget(self)

        def _set(self, v):
            self._values = v

        try:
            RGI.values = property(_get, _set)
        except Exception:
            pass
    return kw
