"""Import the reference's pure-Python block functions on the CPU.

Test infrastructure only: used by ``make_golden.py`` in a container that holds
the reference sources.  The reference is pure Python over CuPy and
``cupyx.scipy.ndimage``; this shim registers ``cupy -> numpy``,
``cupyx.scipy.ndimage -> scipy.ndimage`` and a stub ``dask.array`` in
``sys.modules`` and then imports the reference modules unchanged, so the golden
vectors are the reference's own code run through NumPy/SciPy.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np
import scipy.ndimage as _ndi



def reference_root() -> str:
    """The folder that holds the reference's ``FujiShaderGPU`` package, from the
    ``FSG_REFERENCE_ROOT`` environment variable (required; ``make_golden.py``
    sets it from its ``--reference`` argument)."""
    root = os.environ.get("FSG_REFERENCE_ROOT")
    if not root:
        raise RuntimeError("set FSG_REFERENCE_ROOT (or pass --reference to make_golden.py) to the folder "
                           "holding the reference's FujiShaderGPU package")
    if not os.path.isdir(os.path.join(root, "FujiShaderGPU")):
        raise RuntimeError(f"no FujiShaderGPU package under {root!r}")
    return root


def _install_shim() -> None:
    if "cupy" in sys.modules and getattr(sys.modules["cupy"], "_fsg_shim", False):
        return
    cp = types.ModuleType("cupy")
    cp._fsg_shim = True

    def _getattr(name):
        return getattr(np, name)

    cp.__getattr__ = _getattr  # type: ignore[attr-defined]
    cp.asnumpy = np.asarray
    cp.ndarray = np.ndarray

    class _Pool:
        def free_all_blocks(self):
            return None

        def used_bytes(self):
            return 0

    cp.get_default_memory_pool = lambda: _Pool()
    cp.get_default_pinned_memory_pool = lambda: _Pool()
    sys.modules["cupy"] = cp

    cupyx = types.ModuleType("cupyx")
    cupyx_scipy = types.ModuleType("cupyx.scipy")
    cupyx_scipy.ndimage = _ndi
    cupyx.scipy = cupyx_scipy
    sys.modules["cupyx"] = cupyx
    sys.modules["cupyx.scipy"] = cupyx_scipy
    sys.modules["cupyx.scipy.ndimage"] = _ndi

    dask = types.ModuleType("dask")
    dask_array = types.ModuleType("dask.array")

    class _Array:  # stand-in type for annotations only
        pass

    dask_array.Array = _Array
    dask.array = dask_array
    sys.modules["dask"] = dask
    sys.modules["dask.array"] = dask_array

    root = reference_root()
    if root not in sys.path:
        sys.path.insert(0, root)


def load():
    """Return a namespace with the reference functions the golden set uses."""
    _install_shim()
    import importlib

    mods = {}
    for name in (
        "FujiShaderGPU.algorithms._nan_utils",
        "FujiShaderGPU.algorithms._impl_hillshade",
        "FujiShaderGPU.algorithms._impl_slope",
        "FujiShaderGPU.algorithms._impl_curvature",
        "FujiShaderGPU.algorithms._impl_topousm_fast",
        "FujiShaderGPU.algorithms._impl_openness",
        "FujiShaderGPU.algorithms._impl_ambient_occlusion",
        "FujiShaderGPU.algorithms._normalization",
        "FujiShaderGPU.algorithms._global_stats",
        "FujiShaderGPU.algorithms.common.spatial_mode",
        "FujiShaderGPU.io.output_encoding",
    ):
        mods[name.rsplit(".", 1)[1]] = importlib.import_module(name)
    return types.SimpleNamespace(**mods)
