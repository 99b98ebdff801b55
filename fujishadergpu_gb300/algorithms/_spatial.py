"""Spatial (multi-radius) mode of the stencil products and openness."""
from __future__ import annotations


def spatial_stencil(name, dem_gpu, params):
    raise NotImplementedError("spatial mode for %s is not available yet" % name)


def spatial_openness(dem_gpu, params):
    raise NotImplementedError("spatial mode for openness is not available yet")
