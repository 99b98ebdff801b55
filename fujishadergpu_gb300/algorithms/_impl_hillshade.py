"""Hillshade (algorithms/_impl_hillshade.py of the reference).

``compute_hillshade_block`` keeps the reference signature
(_impl_hillshade.py:20-23) and runs the fused stencil kernel with only the
hillshade plane requested.
"""
from __future__ import annotations

from ._base import Constants, TileAlgorithm
from ._stencil import stencil_block


def compute_hillshade_block(block, *, azimuth=Constants.DEFAULT_AZIMUTH,
                            altitude=Constants.DEFAULT_ALTITUDE, z_factor=1.0,
                            pixel_size=1.0, pixel_scale_x=None, pixel_scale_y=None):
    """Lambertian hillshade in [0, 1] of one window (_impl_hillshade.py:20-54)."""
    return stencil_block(block, ["hillshade"], azimuth=azimuth, altitude=altitude, z_factor=z_factor,
                         pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                         pixel_scale_y=pixel_scale_y)["hillshade"]


class HillshadeAlgorithm(TileAlgorithm):
    """Tile adapter (algorithms/tile/hillshade.py, dask_bridge.py:72-111)."""

    def process(self, dem_gpu, **params):
        p = self._merged(params)
        mode = str(p.get("mode", "local")).lower()
        radii = p.get("radii", [1])
        if not isinstance(radii, (list, tuple)) or len(radii) == 0:
            radii = [1]
        multiscale = bool(p.get("multiscale", False) or len(radii) > 1)
        if mode == "spatial" or (multiscale and len(radii) > 1):
            from ._spatial import spatial_stencil
            return spatial_stencil("hillshade", dem_gpu, p)
        z = p.get("z_factor", 1.0)
        return compute_hillshade_block(
            dem_gpu, azimuth=p.get("azimuth", Constants.DEFAULT_AZIMUTH),
            altitude=p.get("altitude", Constants.DEFAULT_ALTITUDE), z_factor=1.0 if z is None else z,
            pixel_size=p.get("pixel_size", 1.0), pixel_scale_x=p.get("pixel_scale_x"),
            pixel_scale_y=p.get("pixel_scale_y"))

    def get_default_params(self):
        return {"azimuth": Constants.DEFAULT_AZIMUTH, "altitude": Constants.DEFAULT_ALTITUDE,
                "z_factor": 1.0, "pixel_size": 1.0, "multiscale": False, "radii": None,
                "weights": None, "agg": "mean", "mode": "local"}
