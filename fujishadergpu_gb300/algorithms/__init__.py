"""Drop-in algorithm layer: the reference's block functions and tile classes.

Block functions keep the reference names and keyword arguments
(``compute_hillshade_block`` ...) and take one halo window as a CUDA device
array; the classes keep the ``process(dem_gpu, **params)`` /
``get_default_params()`` interface of algorithms/tile_shared.py:19-44 and are
found by name through ``ALGORITHMS`` / ``load_algorithm`` (``registry.py``).
"""
from ._base import Constants, TileAlgorithm
from ._impl_ambient_occlusion import (AmbientOcclusionAlgorithm, compute_ambient_occlusion_block,
                                      compute_ambient_occlusion_spatial_block)
from ._impl_curvature import CurvatureAlgorithm, compute_curvature_block
from ._impl_hillshade import HillshadeAlgorithm, compute_hillshade_block
from ._impl_openness import OpennessAlgorithm, compute_openness_raw_degrees, compute_openness_vectorized
from ._impl_slope import SlopeAlgorithm, compute_slope_block
from ._impl_topousm_fast import (TopoUSMFastAlgorithm, compute_topousm_fast_efficient_block,
                                 compute_topousm_fast_large_coarse_field, split_radii_by_threshold,
                                 topousm_fast_default_large_radius_threshold)
from ._spatial import (compute_curvature_spatial_block, compute_hillshade_spatial_block,
                       compute_openness_spatial_block, compute_slope_spatial_block)
from ._stats import robust_unsigned_stretch_stat_func, topousm_fast_stat_func
from .registry import ALGORITHMS, DEFAULT_ALGORITHMS, load_algorithm

__all__ = [
    "Constants", "TileAlgorithm",
    "compute_hillshade_block", "HillshadeAlgorithm",
    "compute_slope_block", "SlopeAlgorithm",
    "compute_curvature_block", "CurvatureAlgorithm",
    "compute_openness_vectorized", "compute_openness_raw_degrees", "OpennessAlgorithm",
    "compute_openness_spatial_block",
    "compute_ambient_occlusion_block", "compute_ambient_occlusion_spatial_block", "AmbientOcclusionAlgorithm",
    "compute_topousm_fast_efficient_block", "compute_topousm_fast_large_coarse_field",
    "split_radii_by_threshold", "topousm_fast_default_large_radius_threshold", "TopoUSMFastAlgorithm",
    "topousm_fast_stat_func", "robust_unsigned_stretch_stat_func",
    "compute_hillshade_spatial_block", "compute_slope_spatial_block", "compute_curvature_spatial_block",
    "ALGORITHMS", "DEFAULT_ALGORITHMS", "load_algorithm",
]
