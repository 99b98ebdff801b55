"""The single-device tile loop against the reference's per-tile semantics:
every tile core equals the reference block function run on its clipped
window (process_single_tile, core/tile_processor.py:822-1024), including the
NoData sentinel, geographic per-tile scales, the topousm_fast overview split
and the int16/uint8 encoding."""
import math

import numpy as np
import pytest

from oracle import restated as R
from tests._parity import assert_close_range, assert_codes_close, assert_curvature_close, to_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def loop():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300.core import tile_loop
    return tile_loop


def _dem(h, w, seed, disks=4, sentinel=None):
    from fujishadergpu_gb300 import synth
    d = synth.fbm(h, w, hurst=0.7, seed=seed, lo=0.0, hi=2500.0)
    m = synth.nodata_disks(h, w, count=disks, seed=seed + 1, rmin=4.0, rmax=30.0)
    d[m] = np.nan if sentinel is None else sentinel
    return d


def test_padding_rule_matches_reference(loop):
    assert loop.required_padding("hillshade", {"mode": "local"}, 10.0, 1024) == 64
    assert loop.required_padding("topousm_fast", {"radii": [2, 8, 32, 128]}, 10.0, 4096) == 160
    assert loop.required_padding("slope", {"mode": "local"}, 1.0, 4096) == 32


def test_hillshade_uint8_with_nodata_sentinel(loop):
    dem = _dem(600, 700, 91, sentinel=-9999.0)
    res = loop.process_dem_array(torch.from_numpy(dem).cuda(), "hillshade", tile_size=256, pixel_size=5.0,
                                 pixel_scale_x=5.0, pixel_scale_y=-5.0, nodata=-9999.0, mode="local",
                                 output_dtype="uint8")
    assert res.padding == 64 and res.dtype == "uint8"
    got = to_np(res.output)
    mask = R.nodata_mask(dem, -9999.0)
    clean = np.where(mask, np.nan, dem).astype(np.float32)
    qp = R.quantize_params(0.0, 1.0, "uint8")
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in R.tile_grid(600, 700, 256, 64):
        win = clean[wy:wy + wh, wx:wx + ww]
        ref = R.hillshade(win, pixel_size=5.0, psx=5.0, psy=-5.0)[cy - wy:cy - wy + ch, cx - wx:cx - wx + cw]
        assert_codes_close(got[cy:cy + ch, cx:cx + cw], R.quantize_array(ref, qp, "uint8"), f"tile {ty},{tx}")
    assert np.array_equal(got == 0, mask)


def test_geographic_per_tile_scales(loop):
    from fujishadergpu_gb300.io.raster_info import tile_pixel_scales
    H, W = 520, 480
    dem = _dem(H, W, 93, disks=2)
    transform = (1.0 / 3600.0, 0.0, 135.0, 0.0, -(45.0 - 30.0) / H, 45.0)
    res = loop.process_dem_array(torch.from_numpy(dem).cuda(), "curvature", tile_size=128, pixel_size=25.0,
                                 transform=transform, geographic=True, mode="local", curvature_type="profile")
    got = to_np(res.output)
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in R.tile_grid(H, W, 128, res.padding):
        psx, psy = R.tile_pixel_scales(cy, ch, transform[0], transform[4], transform[5])
        assert (psx, psy) == tile_pixel_scales(cy, ch, transform)
        win = dem[wy:wy + wh, wx:wx + ww]
        ref = R.curvature(win, curvature_type="profile", pixel_size=25.0, psx=psx, psy=psy)
        assert_curvature_close(got[cy:cy + ch, cx:cx + cw], ref[cy - wy:cy - wy + ch, cx - wx:cx - wx + cw],
                               f"tile {ty},{tx}")


def test_topousm_overview_split_given_stats(loop):
    H, W = 640, 576
    dem = _dem(H, W, 95, disks=3)
    radii = [2, 8, 32, 128, 512]
    wts = [16 / 31, 8 / 31, 4 / 31, 2 / 31, 1 / 31]
    # threshold max(256, 256//16) = 256 -> 512 is a large radius; overview factor 1 (raster < 2048 px)
    field = R.coarse_field(dem, large_radii=[512], large_weights=[1 / 31], decimation=1.0)
    scale = R.topousm_scale(R.topousm_tile(dem, radii=None, weights=None, pixel_size=10.0, coarse=field,
                                           small_radii=radii[:4], small_weights=wts[:4], w_large=1 / 31,
                                           offset=(0, 0), full_shape=(H, W)))[0]
    res = loop.process_dem_array(torch.from_numpy(dem).cuda(), "topousm_fast", tile_size=256, pixel_size=10.0,
                                 radii=radii, weights=wts, global_stats=(scale,))
    pad = res.padding
    assert pad == 160
    got = to_np(res.output)
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in R.tile_grid(H, W, 256, pad):
        win = dem[wy:wy + wh, wx:wx + ww]
        raw = R.topousm_tile(win, radii=None, weights=None, pixel_size=10.0, coarse=field,
                             small_radii=radii[:4], small_weights=wts[:4], w_large=1 / 31, offset=(wy, wx),
                             full_shape=(H, W))
        ref = R.topousm_normalize(raw, (scale,))[cy - wy:cy - wy + ch, cx - wx:cx - wx + cw]
        assert_close_range(got[cy:cy + ch, cx:cx + cw], ref, 2 * 1.176, f"tile {ty},{tx}")


def test_topousm_stats_prepass_matches_oracle(loop):
    """Stratified full-res windows, full radii, trimmed interiors, p99(|x|) (_norm_stats.py:176-298)."""
    H, W = 700, 760
    dem = _dem(H, W, 97, disks=3)
    radii, wts = [2, 8, 32], [4 / 7, 2 / 7, 1 / 7]
    st = loop.global_stats_prepass(torch.from_numpy(dem).cuda(), "topousm_fast",
                                   {"radii": radii, "weights": wts, "pixel_size": 10.0})
    margin = max(radii) + 16
    tile = max(2048, 4 * margin)
    wins = loop.stratified_windows(W, H, 0, H, 0, W, grid=3, tile=min(tile, max(W, H)))
    pooled = []
    for wy0, wx0, tw, th in wins:
        raw = R.topousm_block(dem[wy0:wy0 + th, wx0:wx0 + tw], radii=radii, weights=wts, pixel_size=10.0)
        m = min(margin, raw.shape[0] // 3, raw.shape[1] // 3)
        pooled.append(raw[m:-m, m:-m].ravel())
    ref = R.topousm_scale(np.concatenate(pooled))
    assert st[0] == pytest.approx(ref[0], rel=2e-5)


def test_openness_loop_with_stretch_stats(loop):
    H, W = 300, 340
    dem = _dem(H, W, 99, disks=2)
    res = loop.process_dem_array(torch.from_numpy(dem).cuda(), "openness", tile_size=128, pixel_size=5.0,
                                 pixel_scale_x=5.0, pixel_scale_y=-5.0, mode="local", max_distance=20,
                                 global_stats=(0.6, 0.3))
    got = to_np(res.output)
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in R.tile_grid(H, W, 128, res.padding):
        win = dem[wy:wy + wh, wx:wx + ww]
        ref = R.apply_stretch(R.openness(win, max_distance=20, pixel_size=5.0, psx=5.0, psy=-5.0), (0.6, 0.3))
        assert_close_range(got[cy:cy + ch, cx:cx + cw], ref[cy - wy:cy - wy + ch, cx - wx:cx - wx + cw],
                           1.0 / 0.3, f"tile {ty},{tx}")
