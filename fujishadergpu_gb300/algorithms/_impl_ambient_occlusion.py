"""Ambient occlusion (algorithms/_impl_ambient_occlusion.py of the reference).

``compute_ambient_occlusion_block`` keeps the reference signature
(:32-121) and runs ``fsg_ambient_occlusion`` with the whole block as one
window; ``compute_ambient_occlusion_spatial_block`` (:124-157) decimates for
large radii; ``AmbientOcclusionAlgorithm`` is the tile adapter
(algorithms/tile/ambient_occlusion.py -> dask_bridge._direct_ambient_occlusion
:190-203, and the Dask ``process`` :163-203 for ``mode='spatial'``).
"""
from __future__ import annotations

import ctypes as C

from .. import _arrays
from .. import _native as N
from ._base import TileAlgorithm
from ._stencil import make_plane
from ._stats import robust_unsigned_stretch_stat_func


def make_params(*, num_samples=16, radius=10.0, intensity=1.0, pixel_size=1.0, nodata=None,
                stretch=None) -> N.AoParams:
    p = N.AoParams()
    p.num_samples = int(num_samples)
    p.radius = float(radius)
    p.intensity = float(intensity)
    p.pixel_size = float(pixel_size if pixel_size else 1.0)
    p.has_nodata = 0 if nodata is None else 1
    p.nodata = float("nan") if nodata is None else float(nodata)
    if stretch is not None and len(stretch) >= 2 and float(stretch[1]) > 1e-12:
        p.stretch_lo, p.stretch_scale = float(stretch[0]), float(stretch[1])
    return p


def run_ambient_occlusion(view, tiles, params, plane, stream=None):
    tarr = (N.Tile * max(1, len(tiles)))(*tiles)
    s = _arrays.current_stream_handle() if stream is None else stream
    N.check(N.lib().fsg_ambient_occlusion(C.c_void_p(view.ptr), view.ld, view.h, view.w, tarr, len(tiles),
                                          C.byref(params), C.byref(plane), C.c_void_p(s)))


def _scales(pixel_size, pixel_scale_x, pixel_scale_y):
    # _impl_ambient_occlusion.py:59-60: |pixel_scale| or pixel_size
    sx = abs(float(pixel_scale_x)) if pixel_scale_x is not None else float(pixel_size)
    sy = abs(float(pixel_scale_y)) if pixel_scale_y is not None else float(pixel_size)
    return sx, sy


def whole_tile(h, w, sx, sy, core=None):
    t = N.Tile()
    t.win_y0, t.win_x0, t.win_h, t.win_w = 0, 0, h, w
    t.core_y0, t.core_x0, t.core_h, t.core_w = core if core is not None else (0, 0, h, w)
    t.out_y0, t.out_x0 = 0, 0
    t.pixel_scale_x, t.pixel_scale_y = sx, sy
    return t


def ambient_occlusion_plane(block, *, num_samples=16, radius=10.0, intensity=1.0, pixel_size=1.0,
                            pixel_scale_x=None, pixel_scale_y=None, stretch=None, out_dtype="float32", qp=None,
                            nodata=None):
    v = _arrays.as_device_f32_2d(block)
    sx, sy = _scales(pixel_size, pixel_scale_x, pixel_scale_y)
    params = make_params(num_samples=num_samples, radius=radius, intensity=intensity, pixel_size=pixel_size,
                         nodata=nodata, stretch=stretch)
    out = _arrays.empty(v.h, v.w, out_dtype, device=v.tensor.device)
    if v.h * v.w:
        run_ambient_occlusion(v, [whole_tile(v.h, v.w, sx, sy)], params, make_plane(out, out_dtype, qp))
    return out, v


def compute_ambient_occlusion_block(block, *, num_samples: int = 16, radius: float = 10.0, intensity: float = 1.0,
                                    pixel_size: float = 1.0, pixel_scale_x: float = None,
                                    pixel_scale_y: float = None):
    """AO in [0, 1] (_impl_ambient_occlusion.py:32-121)."""
    out, v = ambient_occlusion_plane(block, num_samples=num_samples, radius=radius, intensity=intensity,
                                     pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                                     pixel_scale_y=pixel_scale_y)
    return _arrays.wrap_result(out, v.origin)


def compute_ambient_occlusion_spatial_block(block, *, num_samples: int = 16, radius: float = 10.0,
                                            intensity: float = 1.0, pixel_size: float = 1.0,
                                            pixel_scale_x: float = None, pixel_scale_y: float = None):
    """_impl_ambient_occlusion.py:124-157: AO of the NaN-aware f x f decimation for large radii."""
    from ._spatial import spatial_block
    return spatial_block(block, "ambient_occlusion", radius, pixel_size=pixel_size, pixel_scale_x=pixel_scale_x,
                         pixel_scale_y=pixel_scale_y, num_samples=int(num_samples), intensity=float(intensity))


class AmbientOcclusionAlgorithm(TileAlgorithm):
    """Tile adapter: algorithms/tile/ambient_occlusion.py -> dask_bridge._direct_ambient_occlusion
    (:190-203); ``mode='spatial'`` runs the multiscale responses (_impl_ambient_occlusion.py:176-189)."""

    def process(self, dem_gpu, **params):
        p = self._merged(params)
        if str(p.get("mode", "local")).lower() == "spatial":
            from ._spatial import spatial_stencil
            return spatial_stencil("ambient_occlusion", dem_gpu, p)
        out, v = ambient_occlusion_plane(
            dem_gpu, num_samples=p.get("num_samples", 16), radius=p.get("radius", 10.0),
            intensity=p.get("intensity", 1.0), pixel_size=p.get("pixel_size", 1.0),
            pixel_scale_x=p.get("pixel_scale_x"), pixel_scale_y=p.get("pixel_scale_y"),
            stretch=p.get("global_stats"))
        return _arrays.wrap_result(out, v.origin)

    def get_default_params(self) -> dict:
        return {"num_samples": 16, "radius": 10.0, "intensity": 1.0, "pixel_size": 1.0, "mode": "local",
                "radii": None, "weights": None}


__all__ = ["compute_ambient_occlusion_block", "compute_ambient_occlusion_spatial_block",
           "AmbientOcclusionAlgorithm", "robust_unsigned_stretch_stat_func"]
