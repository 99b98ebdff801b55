"""Slope (algorithms/_impl_slope.py of the reference)."""
from __future__ import annotations

from ._base import TileAlgorithm
from ._stencil import stencil_block


def compute_slope_block(block, *, unit="degree", pixel_size=1.0, pixel_scale_x=None, pixel_scale_y=None):
    """atan(|grad z|) in degree / percent / radian (_impl_slope.py:19-35)."""
    return stencil_block(block, ["slope"], unit=unit, pixel_size=pixel_size,
                         pixel_scale_x=pixel_scale_x, pixel_scale_y=pixel_scale_y)["slope"]


class SlopeAlgorithm(TileAlgorithm):
    """Tile adapter (algorithms/tile/slope.py, dask_bridge.py:114-124)."""

    def process(self, dem_gpu, **params):
        p = self._merged(params)
        if str(p.get("mode", "local")).lower() == "spatial":
            from ._spatial import spatial_stencil
            return spatial_stencil("slope", dem_gpu, p)
        return compute_slope_block(dem_gpu, unit=p.get("unit", "degree"), pixel_size=p.get("pixel_size", 1.0),
                                   pixel_scale_x=p.get("pixel_scale_x"), pixel_scale_y=p.get("pixel_scale_y"))

    def get_default_params(self):
        return {"unit": "degree", "pixel_size": 1.0, "mode": "local", "radii": None, "weights": None}
