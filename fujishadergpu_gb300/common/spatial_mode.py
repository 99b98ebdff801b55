"""--mode / --radii / --weights semantics (algorithms/common/spatial_mode.py,
algorithms/_nan_utils.py:77-154, core/tile_compute.py:9-90 of the reference)."""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Sequence, Tuple

AUTO_RADII_SEQUENCE: Tuple[int, ...] = (2, 8, 32, 128, 512, 2048)
AUTO_RADIUS_MAX = 2048
LOCAL_RADII = [1]
LOCAL_WEIGHTS = [1.0]


def auto_spatial_radii(short_side_px: Optional[float]) -> List[int]:
    """Geometric radii truncated to min(short_side/10, 2048); at least [2]."""
    limit = float(AUTO_RADIUS_MAX) if short_side_px is None else min(float(AUTO_RADIUS_MAX),
                                                                          float(short_side_px) / 10.0)
    out = [r for r in AUTO_RADII_SEQUENCE if float(r) <= limit]
    return out or [AUTO_RADII_SEQUENCE[0]]


def auto_spatial_weights(n: int) -> List[float]:
    """2**(n-1..0) normalised to 1 (nearer radii weigh more)."""
    if n <= 0:
        return []
    raw = [2.0 ** (n - 1 - i) for i in range(n)]
    s = sum(raw)
    return [w / s for w in raw]


def clean_normalized_weights(weights) -> Optional[List[float]]:
    """Non-finite / non-positive -> 0, L1-normalised; None if nothing positive."""
    vals = []
    for w in weights:
        try:
            x = float(w)
        except (TypeError, ValueError):
            return None
        vals.append(x if math.isfinite(x) and x > 0 else 0.0)
    s = sum(vals)
    return None if s <= 0 else [v / s for v in vals]


def _count_matches(weights, n) -> bool:
    if weights is None or isinstance(weights, (str, bytes)):
        return False
    try:
        return len(weights) == n
    except TypeError:
        return False


def resolve_spatial_radii_weights(radii, weights, pixel_size, short_side_px=None):
    """Spatial radii/weights resolution of the stencil/openness algorithms."""
    if radii is None:
        r = auto_spatial_radii(short_side_px)
        if _count_matches(weights, len(r)):
            u = clean_normalized_weights(weights)
            if u is not None:
                return r, u
        return r, auto_spatial_weights(len(r))
    out = []
    for v in radii:
        try:
            iv = int(round(float(v)))
        except (TypeError, ValueError):
            continue
        if iv > 0:
            out.append(iv)
    if not out:
        out = auto_spatial_radii(None)
    seen, ordered = set(), []
    for v in out:
        if v not in seen:
            seen.add(v)
            ordered.append(v)
    if _count_matches(weights, len(ordered)):
        u = clean_normalized_weights(weights)
        if u is not None:
            return ordered, u
    return ordered, auto_spatial_weights(len(ordered))


def deduplicate_radii_weights(radii: Sequence[int], weights) -> Tuple[List[int], Optional[List[float]]]:
    """Keep radius order; duplicate radii sum their (sanitised) weights; L1-normalise."""
    order: List[int] = []
    pos: Dict[int, int] = {}
    rl = list(radii)
    for r in rl:
        if r not in pos:
            pos[r] = len(order)
            order.append(r)
    if weights is None:
        return order, None
    wl = list(weights)
    if len(wl) != len(rl):
        return order, None
    agg = [0.0] * len(order)
    for r, v in zip(rl, wl):
        try:
            x = float(v)
        except (TypeError, ValueError):
            x = 0.0
        if not math.isfinite(x) or x <= 0:
            x = 0.0
        agg[pos[r]] += x
    t = sum(agg)
    return (order, None) if t <= 0 else (order, [x / t for x in agg])


def normalize_topousm_radii(manual_radii, manual_weights) -> Tuple[Optional[List[int]], Optional[List[float]]]:
    """Explicit topousm_fast radii: round, clamp to >= 1, dedup (core/tile_compute.py:42-90)."""
    if manual_radii is None:
        return None, None
    out = []
    for v in manual_radii:
        try:
            x = float(v)
        except (TypeError, ValueError):
            continue
        if math.isfinite(x):
            out.append(max(1, int(round(x))))
    if not out:
        return None, None
    return deduplicate_radii_weights(out, manual_weights)
