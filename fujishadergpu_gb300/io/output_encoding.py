"""float32 -> int16/uint8 output encoding parameters (io/output_encoding.py of
the reference, :39-175).  The encoding itself runs in the kernels' store
epilogue (``quantize`` in csrc/fsg_common.cuh)."""
from __future__ import annotations

from typing import Dict, Optional, Tuple

import math

NORM_HEADROOM = 1.176
OUTPUT_VALUE_RANGES: Dict[str, Tuple[float, float]] = {
    "topousm_fast": (-NORM_HEADROOM, NORM_HEADROOM),
    "hillshade": (0.0, 1.0),
    "curvature": (0.0, 1.0),
    "openness": (0.0, 1.0),
    "ambient_occlusion": (0.0, 1.0),
    "slope": (0.0, 90.0),
}
SUPPORTED_OUTPUT_DTYPES = ("float32", "int16", "uint8")
_INT_MAXPOS = {"int16": 32767, "uint8": 255}


def output_nodata_for_dtype(dtype: str) -> float:
    return float("nan") if str(dtype) == "float32" else 0.0


def resolve_output_range(algorithm: str, *, params: Optional[dict] = None, override=None):
    if override is not None:
        lo, hi = float(override[0]), float(override[1])
        if hi > lo:
            return lo, hi
        raise ValueError(f"output range must satisfy high > low, got ({lo!r}, {hi!r})")
    algo = str(algorithm).lower()
    if algo == "slope" and params is not None:
        unit = str(params.get("unit", "degree")).lower()
        if unit == "radian":
            return (0.0, float(math.pi / 2.0))
        if unit != "degree":
            return None
    return OUTPUT_VALUE_RANGES.get(algo)


def quantize_params(lo: float, hi: float, dtype: str) -> Dict[str, float]:
    lo, hi = float(lo), float(hi)
    dt = str(dtype).lower()
    maxpos = _INT_MAXPOS[dt]
    signed = lo < 0.0 < hi
    if signed:
        a = max(abs(lo), abs(hi)) or 1.0
        if dt == "int16":
            ac, bc, dmin, dmax = maxpos / a, 0.0, -maxpos, maxpos
        else:
            ac, bc, dmin, dmax = (maxpos - 1) / 2.0 / a, (maxpos + 1) / 2.0, 1, maxpos
    else:
        span = (hi - lo) if (hi - lo) > 0 else 1.0
        ac = (maxpos - 1) / span
        bc = 1.0 - ac * lo
        dmin, dmax = 1, maxpos
    return {"a_coef": float(ac), "b_coef": float(bc), "dn_min": int(dmin), "dn_max": int(dmax),
            "scale": float(1.0 / ac), "offset": float(-bc / ac), "nodata": 0.0, "signed": bool(signed)}
