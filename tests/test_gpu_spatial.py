"""Spatial mode of the stencil products on the GPU: the smoothing and the spatial
block functions against the reference's golden fixtures, and the tile loop's
spatial mode (per-radius map_overlap windows, large radii from the overview,
weighted combination, NoData restore) against the oracle's restatement."""
import os

import numpy as np
import pytest

from oracle import restated as R
from tests._parity import (assert_close_range, assert_codes_close, assert_curvature_close,
                           assert_curvature_combined_close, assert_same_nan, to_np)

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SMOOTH_CASES = ((1.0, "hillshade"), (4.0, "hillshade"), (16.0, "slope"), (40.0, "curvature"), (100.0, "hillshade"))


@pytest.fixture(scope="module")
def sp():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300.algorithms import _spatial
    return _spatial


def _ulps(got, ref):
    g = to_np(got).astype(np.float32)
    r = np.asarray(ref, np.float32)
    assert_same_nan(g, r, "smooth")
    m = ~np.isnan(r)
    return np.abs(g[m].astype(np.float64) - r[m].astype(np.float64)) / np.spacing(np.abs(r[m])).astype(np.float64)


@pytest.mark.parametrize("variant", ["clean", "nan"])
def test_smoothing_matches_reference_to_the_last_bit(sp, golden_dir, variant):
    """Float-float Gaussian, NumPy-order block mean and float64 zoom: the reference's
    float32 results except where the exact value sits on a float32 rounding tie
    (at most 1 ulp there, in at most 0.1 % of the cells)."""
    g = np.load(os.path.join(golden_dir, "smooth.npz"))
    dem = g[f"{variant}/dem"]
    for r, algo in SMOOTH_CASES:
        got = sp.smooth_for_radius(torch.from_numpy(dem).cuda(), r, pixel_size=5.0, algorithm_name=algo)
        u = _ulps(got, g[f"{variant}/smooth_{algo}_{int(r)}"])
        assert u.max() <= 1.0, f"r={r} {algo}: {u.max()} ulp"
        assert (u > 0).mean() <= 1e-3, f"r={r} {algo}: {(u > 0).sum()} cells differ"


@pytest.mark.parametrize("variant", ["clean", "nan"])
def test_spatial_blocks_match_reference_golden(sp, golden_dir, variant):
    g = np.load(os.path.join(golden_dir, "spatial.npz"))
    dem = torch.from_numpy(g[f"{variant}/dem"]).cuda()
    kw = dict(pixel_size=5.0, pixel_scale_x=5.0, pixel_scale_y=-5.0)
    for r in (1.0, 3.0, 12.0, 40.0):
        hs = sp.compute_hillshade_spatial_block(dem, radius=r, azimuth=300.0, altitude=40.0, **kw)
        assert_close_range(hs, g[f"{variant}/hillshade_{int(r)}"], 1.0, f"hillshade r={r}")
        sl = sp.compute_slope_spatial_block(dem, radius=r, **kw)
        assert_close_range(sl, g[f"{variant}/slope_{int(r)}"], 90.0, f"slope r={r}")
        cv = sp.compute_curvature_spatial_block(dem, radius=r, curvature_type="profile", **kw)
        assert_curvature_close(cv, g[f"{variant}/curvature_profile_{int(r)}"], f"curvature r={r}")


@pytest.mark.parametrize("variant", ["clean", "nan"])
def test_local_multi_radius_hillshade_matches_reference_golden(sp, golden_dir, variant):
    from fujishadergpu_gb300.algorithms import HillshadeAlgorithm
    g = np.load(os.path.join(golden_dir, "spatial.npz"))
    dem = torch.from_numpy(g[f"{variant}/dem"]).cuda()
    got = HillshadeAlgorithm().process(dem, radii=[1, 4, 16], weights=[0.5, 0.3, 0.2], pixel_size=5.0,
                                       pixel_scale_x=5.0, pixel_scale_y=-5.0, mode="local")
    assert_close_range(got, g[f"{variant}/direct_hillshade_multiscale"], 1.0, "multi-radius hillshade")


def _dem(h, w, seed, sentinel=None):
    from fujishadergpu_gb300 import synth
    d = synth.fbm(h, w, hurst=0.75, seed=seed, lo=0.0, hi=2200.0)
    m = synth.nodata_disks(h, w, count=4, seed=seed + 1, rmin=4.0, rmax=25.0)
    d[m] = np.nan if sentinel is None else sentinel
    return d, m


def _oracle_loop(dem, mask, product, radii, weights, tile, pad, kw, *, ps=5.0, with_responses=False):
    H, W = dem.shape
    clean = np.where(mask, np.nan, dem).astype(np.float32)
    out = np.full((H, W), np.nan, np.float32)
    resp = [np.full((H, W), np.nan, np.float32) for _ in radii]
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in R.tile_grid(H, W, tile, pad):
        win = clean[wy:wy + wh, wx:wx + ww]
        res, parts = R.spatial_window(win, product, radii, weights, origin=(wy, wx), full_shape=(H, W),
                                      coarse_dem=clean, decimation=1.0, pixel_size=ps, psx=ps, psy=-ps,
                                      return_responses=True, **kw)
        sl = (slice(cy - wy, cy - wy + ch), slice(cx - wx, cx - wx + cw))
        out[cy:cy + ch, cx:cx + cw] = np.where(mask[cy:cy + ch, cx:cx + cw], np.float32(np.nan), res[sl])
        for k, prt in enumerate(parts):
            resp[k][cy:cy + ch, cx:cx + cw] = prt[sl]
    return (out, resp) if with_responses else out


@pytest.mark.parametrize("product", ["hillshade", "slope", "curvature"])
def test_tile_loop_spatial_mode_matches_oracle(sp, product):
    """Radii 2, 8, 32 through reflect-padded windows; 300 (> the 256 threshold) from the
    overview (a 600 x 640 raster is its own overview, decimation 1)."""
    from fujishadergpu_gb300.core import tile_loop
    H, W = 600, 640
    dem, mask = _dem(H, W, 131)
    radii, weights = [2, 8, 32, 300], [0.4, 0.3, 0.2, 0.1]
    kw = {"hillshade": {}, "slope": {"unit": "degree"}, "curvature": {"curvature_type": "planform"}}[product]
    res = tile_loop.process_dem_array(torch.from_numpy(dem).cuda(), product, tile_size=256, pixel_size=5.0,
                                      pixel_scale_x=5.0, pixel_scale_y=-5.0, mode="spatial", radii=radii,
                                      weights=weights, **kw)
    assert res.padding == 96
    got = to_np(res.output)
    ref, parts = _oracle_loop(dem, mask, product, radii, weights, 256, res.padding, kw, with_responses=True)
    if product == "curvature":
        # each response carries the curvature tail allowance into the weighted sum
        assert_curvature_combined_close(got, ref, parts, weights, "spatial curvature")
    else:
        assert_close_range(got, ref, 1.0 if product == "hillshade" else 90.0, f"spatial {product}")


def test_tile_loop_spatial_int16_with_sentinel(sp):
    from fujishadergpu_gb300.core import tile_loop
    H, W = 420, 380
    dem, mask = _dem(H, W, 137, sentinel=-9999.0)
    res = tile_loop.process_dem_array(torch.from_numpy(dem).cuda(), "slope", tile_size=200, pixel_size=5.0,
                                      pixel_scale_x=5.0, pixel_scale_y=-5.0, nodata=-9999.0, mode="spatial",
                                      radii=[3, 12], weights=None, output_dtype="int16")
    got = to_np(res.output)
    nd = R.nodata_mask(dem, -9999.0)
    radii, weights = R.resolve_spatial_radii_weights([3, 12], None, 5.0)
    ref = _oracle_loop(dem, nd, "slope", radii, weights, 200, res.padding, {"unit": "degree"})
    qp = R.quantize_params(0.0, 90.0, "int16")
    assert_codes_close(got, R.quantize_array(ref, qp, "int16"), "spatial slope int16")
