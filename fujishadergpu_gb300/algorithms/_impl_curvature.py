"""Curvature (algorithms/_impl_curvature.py of the reference)."""
from __future__ import annotations

from ._base import TileAlgorithm
from ._stencil import stencil_block

CURVATURE_TYPES = ("mean", "gaussian", "planform", "profile")


def compute_curvature_block(block, *, curvature_type="mean", pixel_size=1.0, pixel_scale_x=None,
                            pixel_scale_y=None):
    """Display-mapped curvature ((tanh(100k)+1)/2)^(1/2.2) (_impl_curvature.py:19-57).

    Any ``curvature_type`` other than mean/gaussian/planform selects profile,
    as the reference's final ``else`` branch does.
    """
    ct = curvature_type if curvature_type in ("mean", "gaussian", "planform") else "profile"
    name = "curvature_" + ct
    return stencil_block(block, [name], pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                         pixel_scale_y=pixel_scale_y)[name]


class CurvatureAlgorithm(TileAlgorithm):
    """Tile adapter (algorithms/tile/curvature.py, dask_bridge.py:141-151)."""

    def process(self, dem_gpu, **params):
        p = self._merged(params)
        if str(p.get("mode", "local")).lower() == "spatial":
            from ._spatial import spatial_stencil
            return spatial_stencil("curvature", dem_gpu, p)
        return compute_curvature_block(dem_gpu, curvature_type=p.get("curvature_type", "mean"),
                                       pixel_size=p.get("pixel_size", 1.0),
                                       pixel_scale_x=p.get("pixel_scale_x"), pixel_scale_y=p.get("pixel_scale_y"))

    def get_default_params(self):
        return {"curvature_type": "mean", "pixel_size": 1.0, "mode": "local", "radii": None, "weights": None}
