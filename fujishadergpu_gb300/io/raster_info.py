"""Metric pixel scales (io/raster_info.py:13-35 of the reference)."""
from __future__ import annotations

import math
from typing import Tuple


def meters_per_degree(lat_deg: float) -> Tuple[float, float]:
    """(m per degree longitude, m per degree latitude), WGS84 series."""
    lat = math.radians(float(lat_deg))
    m_lat = 111132.92 - 559.82 * math.cos(2.0 * lat) + 1.175 * math.cos(4.0 * lat) - 0.0023 * math.cos(6.0 * lat)
    m_lon = 111412.84 * math.cos(lat) - 93.5 * math.cos(3.0 * lat) + 0.118 * math.cos(5.0 * lat)
    return max(1e-6, float(m_lon)), float(m_lat)


def tile_pixel_scales(core_y: int, core_h: int, transform) -> Tuple[float, float]:
    """Signed metres per pixel at the latitude of a tile core's centre
    (core/tile_processor.py:910-932); ``transform`` = (a, b, c, d, e, f) affine."""
    a, _, _, _, e, f = transform
    top = f + core_y * e
    bottom = f + (core_y + core_h) * e
    lat = 0.5 * (top + bottom)
    mlon, mlat = meters_per_degree(lat)
    px = math.copysign(abs(a) * mlon, a if a != 0 else 1.0)
    py = math.copysign(abs(e) * mlat, e if e != 0 else -1.0)
    return float(px), float(py)
