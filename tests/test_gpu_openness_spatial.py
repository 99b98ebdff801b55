"""Spatial mode of openness on the GPU: the NaN-aware decimation and zoom entry
points and compute_openness_spatial_block against the reference's golden
fixtures, the combination modes, and the tile loop's spatial openness
(per-radius map_overlap windows, decimated rays, overview radii, display
stretch, NoData restore) against the oracle's restatement."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import restated as R
from tests._parity import assert_close_range, assert_codes_close, assert_same_nan, to_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def sp():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300.algorithms import _spatial
    return _spatial


def _golden(golden_dir):
    return np.load(os.path.join(golden_dir, "openness_spatial.npz"))


def _ulp_check(got, ref, what):
    """Bit-exact except on float32 rounding ties of the Gaussian void fill (<= 1 ulp, <= 0.1 %)."""
    g = to_np(got).astype(np.float32)
    r = np.asarray(ref, np.float32)
    assert g.shape == r.shape, what
    assert_same_nan(g, r, what)
    m = ~np.isnan(r)
    u = np.abs(g[m].astype(np.float64) - r[m].astype(np.float64)) / np.spacing(np.abs(r[m])).astype(np.float64)
    assert u.max(initial=0.0) <= 1.0, f"{what}: {u.max()} ulp"
    assert (u > 0).mean() <= 1e-3 if u.size else True, f"{what}: {(u > 0).sum()} cells differ"


@pytest.mark.parametrize("variant", ["clean", "nan"])
def test_downsample_and_zoom_match_reference(sp, golden_dir, variant):
    from fujishadergpu_gb300 import _native as N
    g = _golden(golden_dir)
    dem = torch.from_numpy(g[f"{variant}/dem"]).cuda()
    h, w = dem.shape
    lib = N.lib()
    for f in (2, 4, 8):
        hs, ws = (h + f - 1) // f, (w + f - 1) // f
        out = torch.full((hs, ws + 3), -7.0, device="cuda")
        N.check(lib.fsg_downsample_nan_aware(C.c_void_p(dem.data_ptr()), w, h, w, f, C.c_void_p(out.data_ptr()),
                                             ws + 3, None))
        torch.cuda.synchronize()
        _ulp_check(out[:, :ws], g[f"{variant}/down_{f}"], f"down {f}")
        assert bool((out[:, ws:] == -7.0).all()), "wrote past the row"
    small = torch.from_numpy(g[f"{variant}/down_4"]).cuda()
    sh, sw = small.shape
    for key, (th, tw) in (("up_4", (h, w)), ("up_4_odd", (131, 97))):
        ref = g[f"{variant}/{key}"]
        full = torch.empty((th, tw), device="cuda")
        N.check(lib.fsg_upsample_to_shape(C.c_void_p(small.data_ptr()), sw, sh, sw, th, tw, 0, 0, th, tw,
                                          C.c_void_p(full.data_ptr()), tw, None))
        # a region of the target only (the tile core)
        reg = torch.empty((th - 21, tw - 30), device="cuda")
        N.check(lib.fsg_upsample_to_shape(C.c_void_p(small.data_ptr()), sw, sh, sw, th, tw, 13, 17, th - 21,
                                          tw - 30, C.c_void_p(reg.data_ptr()), tw - 30, None))
        torch.cuda.synchronize()
        _ulp_check(full, ref, key)
        _ulp_check(reg, ref[13:th - 8, 17:tw - 13], key + " region")


@pytest.mark.parametrize("variant", ["clean", "nan"])
def test_openness_spatial_block_matches_reference(sp, golden_dir, variant):
    g = _golden(golden_dir)
    dem = torch.from_numpy(g[f"{variant}/dem"]).cuda()
    for md in (12, 40, 80, 150):
        for ot in ("positive", "negative"):
            got = sp.compute_openness_spatial_block(dem, openness_type=ot, num_directions=16, max_distance=md,
                                                    pixel_size=5.0, pixel_scale_x=5.0, pixel_scale_y=-5.0)
            assert_close_range(got, g[f"{variant}/openness_{ot}_{md}"], 1.0, f"{variant} {ot} md={md}")


def _dem(h, w, seed, sentinel=None):
    from fujishadergpu_gb300 import synth
    d = synth.fbm(h, w, hurst=0.75, seed=seed, lo=0.0, hi=2200.0)
    m = synth.nodata_disks(h, w, count=4, seed=seed + 1, rmin=4.0, rmax=25.0)
    d[m] = np.nan if sentinel is None else sentinel
    return d, m


@pytest.mark.parametrize("agg", ["mean", "max", "min", "sum"])
def test_window_spatial_openness_combination_modes(sp, agg):
    from fujishadergpu_gb300.algorithms import OpennessAlgorithm
    dem, _ = _dem(150, 170, 151)
    radii, weights = [3, 20, 45], [0.5, 0.3, 0.2]
    got = OpennessAlgorithm().process(torch.from_numpy(dem).cuda(), mode="spatial", radii=radii, weights=weights,
                                      agg=agg, pixel_size=5.0, pixel_scale_x=5.0, pixel_scale_y=-5.0,
                                      openness_type="negative", global_stats=(0.3, 0.4))
    rr, ww = R.resolve_spatial_radii_weights(radii, weights, 5.0)
    ref = R.spatial_window(dem, "openness", rr, ww, pixel_size=5.0, psx=5.0, psy=-5.0, agg=agg,
                           stretch=(0.3, 0.4), openness_type="negative", num_directions=16)
    assert_close_range(got, ref, 1.0 / 0.4 * (3.0 if agg == "sum" else 1.0), f"agg={agg}")


def test_window_spatial_hillshade_stack_and_plain_mean(sp):
    from fujishadergpu_gb300.algorithms import HillshadeAlgorithm, SlopeAlgorithm
    dem, _ = _dem(120, 130, 157)
    d = torch.from_numpy(dem).cuda()
    kw = dict(pixel_size=5.0, pixel_scale_x=5.0, pixel_scale_y=-5.0)
    st = HillshadeAlgorithm().process(d, mode="spatial", radii=[2, 6], weights=[1, 1], agg="stack", **kw)
    assert tuple(st.shape) == (2, 120, 130)
    for k, r in enumerate((2, 6)):
        ref = R.spatial_window(dem, "hillshade", [r], None, pixel_size=5.0, psx=5.0, psy=-5.0)
        assert_close_range(st[k], ref, 1.0, f"stack band {k}")
    # hillshade keeps the caller's weights; without a positive sum: the plain mean (float32 sum / n)
    got = HillshadeAlgorithm().process(d, mode="spatial", radii=[2, 6, 9], weights=[0, 0, 0], **kw)
    ref = R.spatial_window(dem, "hillshade", [2, 6, 9], [0, 0, 0], pixel_size=5.0, psx=5.0, psy=-5.0)
    assert_close_range(got, ref, 1.0, "plain mean")
    got = SlopeAlgorithm().process(d, mode="spatial", radii=[2, 6, 9], agg="max", **kw)
    rr, ww = R.resolve_spatial_radii_weights([2, 6, 9], None, 5.0)
    ref = R.spatial_window(dem, "slope", rr, ww, pixel_size=5.0, psx=5.0, psy=-5.0, agg="max")
    assert_close_range(got, ref, 90.0, "slope max")


def _oracle_loop(dem, mask, radii, weights, tile, pad, kw, stretch, *, ps=5.0):
    H, W = dem.shape
    clean = np.where(mask, np.nan, dem).astype(np.float32)
    out = np.full((H, W), np.nan, np.float32)
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in R.tile_grid(H, W, tile, pad):
        win = clean[wy:wy + wh, wx:wx + ww]
        res = R.spatial_window(win, "openness", radii, weights, origin=(wy, wx), full_shape=(H, W),
                               coarse_dem=clean, decimation=1.0, pixel_size=ps, psx=ps, psy=-ps, stretch=stretch,
                               **kw)
        sl = (slice(cy - wy, cy - wy + ch), slice(cx - wx, cx - wx + cw))
        out[cy:cy + ch, cx:cx + cw] = np.where(mask[cy:cy + ch, cx:cx + cw], np.float32(np.nan), res[sl])
    return out


@pytest.mark.parametrize("otype", ["positive", "negative"])
def test_tile_loop_spatial_openness_matches_oracle(sp, otype):
    """Distances 4 and 40 / 80 (decimated 2x, 4x) through reflect-padded windows; 300 (> the 256
    threshold) from the overview (a 600 x 640 raster is its own overview)."""
    from fujishadergpu_gb300.core import tile_loop
    H, W = 600, 640
    dem, mask = _dem(H, W, 163)
    radii, weights = [4, 40, 80, 300], [0.4, 0.3, 0.2, 0.1]
    stats = (0.25, 0.6)
    kw = {"openness_type": otype, "num_directions": 16}
    res = tile_loop.process_dem_array(torch.from_numpy(dem).cuda(), "openness", tile_size=256, pixel_size=5.0,
                                      pixel_scale_x=5.0, pixel_scale_y=-5.0, mode="spatial", radii=radii,
                                      weights=weights, global_stats=stats, **kw)
    assert res.padding == 96
    ref = _oracle_loop(dem, mask, radii, weights, 256, res.padding, kw, stats)
    assert_close_range(res.output, ref, 1.0 / stats[1], f"spatial openness {otype}")


def test_tile_loop_spatial_openness_u8_with_sentinel_and_prepass(sp):
    """Sentinel NoData, radii sanitised (1 -> 2, duplicates merged), the global-stats prepass
    of the local openness, uint8 codes."""
    from fujishadergpu_gb300.core import tile_loop
    H, W = 420, 380
    dem, mask = _dem(H, W, 167, sentinel=-9999.0)
    res = tile_loop.process_dem_array(torch.from_numpy(dem).cuda(), "openness", tile_size=200, pixel_size=5.0,
                                      pixel_scale_x=5.0, pixel_scale_y=-5.0, nodata=-9999.0, mode="spatial",
                                      radii=[1, 2, 30], weights=[0.2, 0.3, 0.5], output_dtype="uint8",
                                      max_distance=30)
    assert res.stats is not None
    nd = R.nodata_mask(dem, -9999.0)
    ref = _oracle_loop(dem, nd, [2, 30], [0.5, 0.5], 200, res.padding, {"openness_type": "positive",
                                                                           "num_directions": 16}, res.stats)
    qp = R.quantize_params(0.0, 1.0, "uint8")
    assert_codes_close(res.output, R.quantize_array(ref, qp, "uint8"), "spatial openness u8")
