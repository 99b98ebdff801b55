"""Tile algorithm module for openness (algorithms/tile/openness.py of the reference):
the class the tile loop finds by name, ``OpennessAlgorithm().process(dem_gpu, **params)``."""
from .._impl_openness import OpennessAlgorithm

__all__ = ["OpennessAlgorithm"]
