"""GPU parity of the openness ray-march (reference and dense sampling)
against the reference's golden outputs and the CPU oracle."""
import json
import os

import numpy as np
import pytest

from oracle import restated as R
from tests._parity import assert_close_range, assert_codes_close, to_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

OPEN_CASES = ["o1_fbm_nan", "o2_peak", "o2_pit", "o2_flat", "o3_aniso_d5", "o4_r256"]


@pytest.fixture(scope="module")
def op():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300.algorithms import _impl_openness
    return _impl_openness


def _golden(golden_dir):
    g = np.load(os.path.join(golden_dir, "openness.npz"))
    with open(os.path.join(golden_dir, "openness.json")) as f:
        m = json.load(f)
    return g, m


@pytest.mark.parametrize("case", OPEN_CASES)
@pytest.mark.parametrize("otype", ["positive", "negative"])
def test_openness_matches_reference_golden(op, golden_dir, case, otype):
    g, meta = _golden(golden_dir)
    m = meta[case]
    dem = g[f"{case}/dem"]
    kw = dict(openness_type=otype, num_directions=m["num_directions"], max_distance=m["max_distance"],
              pixel_size=m["pixel_size"], pixel_scale_x=m["psx"], pixel_scale_y=m["psy"])
    out = op.compute_openness_vectorized(torch.from_numpy(dem).cuda(), **kw)
    assert_close_range(out, g[f"{case}/{otype}"], 1.0, f"{case} {otype}")
    raw = op.compute_openness_raw_degrees(torch.from_numpy(dem).cuda(), **kw)
    ref_raw = R.openness(dem, openness_type=otype, num_directions=m["num_directions"],
                         max_distance=m["max_distance"], pixel_size=m["pixel_size"], psx=m["psx"], psy=m["psy"],
                         raw_degrees=True)
    d = np.abs(to_np(raw).astype(np.float64) - ref_raw)
    assert float(np.nanmax(d)) <= 0.01, float(np.nanmax(d))


def test_reference_openness_known_answers_on_gpu(op):
    """reference tests/test_openness_yokoyama.py:1-47."""
    yy, xx = np.mgrid[0:101, 0:101]
    r = np.sqrt((xx - 50) ** 2 + (yy - 50) ** 2)

    def run(dem, ot):
        return float(to_np(op.compute_openness_vectorized(torch.from_numpy(dem.astype(np.float32)).cuda(),
                                                          openness_type=ot, num_directions=16,
                                                          max_distance=40))[50, 50])

    peak, pit, flat = 50 - r, r - 50, np.zeros((101, 101))
    assert run(peak, "positive") > run(pit, "positive")
    assert run(pit, "negative") > run(peak, "negative")
    assert run(flat, "positive") == pytest.approx(1.0, abs=1e-3)
    assert run(flat, "negative") == pytest.approx(1.0, abs=1e-3)


@pytest.mark.parametrize("otype", ["positive", "negative"])
def test_dense_ray_march_matches_oracle(op, otype):
    from fujishadergpu_gb300 import synth
    dem = synth.fbm(72, 80, hurst=0.7, seed=81, lo=0.0, hi=600.0)
    dem[synth.nodata_disks(72, 80, count=2, seed=82, rmin=3.0, rmax=6.0)] = np.nan
    kw = dict(openness_type=otype, num_directions=16, max_distance=24, pixel_size=5.0, pixel_scale_x=5.0,
              pixel_scale_y=-5.0)
    raw = to_np(op.compute_openness_raw_degrees(torch.from_numpy(dem).cuda(), sampling="dense", **kw))
    ref = R.openness(dem, openness_type=otype, num_directions=16, max_distance=24, pixel_size=5.0, psx=5.0,
                     psy=-5.0, raw_degrees=True, offsets=R.dense_offsets(16, 24))
    assert np.array_equal(np.isnan(raw), np.isnan(ref))
    assert float(np.nanmax(np.abs(raw.astype(np.float64) - ref))) <= 0.01
    disp = op.compute_openness_vectorized(torch.from_numpy(dem).cuda(), sampling="dense", **kw)
    ref_disp = R.openness(dem, openness_type=otype, num_directions=16, max_distance=24, pixel_size=5.0, psx=5.0,
                          psy=-5.0, offsets=R.dense_offsets(16, 24))
    assert_close_range(disp, ref_disp, 1.0, "dense display")


def test_display_stretch_and_quantisation(op):
    from fujishadergpu_gb300 import synth
    dem = synth.fbm(90, 110, hurst=0.7, seed=83, lo=0.0, hi=900.0)
    ref = R.openness(dem, max_distance=12, pixel_size=5.0)
    stats = R.stretch_stats(ref)
    out = op.OpennessAlgorithm().process(torch.from_numpy(dem).cuda(), max_distance=12, pixel_size=5.0,
                                         global_stats=stats)
    assert_close_range(out, R.apply_stretch(ref, stats), 1.0 / stats[1], "stretched")
    qp = R.quantize_params(0.0, 1.0, "uint8")
    disp, _, _ = op.openness_planes(torch.from_numpy(dem).cuda(), max_distance=12, pixel_size=5.0, stretch=stats,
                                    out_dtype="uint8", qp=qp)
    assert_codes_close(disp, R.quantize_array(R.apply_stretch(ref, stats), qp, "uint8"), "u8")


def test_tiled_openness_per_tile_pixel_scales(op):
    """Geographic tiles: each tile carries its own signed pixel scales."""
    from fujishadergpu_gb300 import _arrays, synth
    from fujishadergpu_gb300._native import Tile
    H, W = 200, 230
    dem = synth.fbm(H, W, hurst=0.7, seed=85, lo=0.0, hi=900.0)
    dem[synth.nodata_disks(H, W, count=3, seed=86, rmin=3.0, rmax=9.0)] = np.nan
    raw = torch.empty((H, W), device="cuda")
    tiles, meta = [], []
    for i, (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in enumerate(R.tile_grid(H, W, 64, 32)):
        t = Tile()
        t.win_y0, t.win_x0, t.win_h, t.win_w = wy, wx, wh, ww
        t.core_y0, t.core_x0, t.core_h, t.core_w = cy, cx, ch, cw
        t.out_y0, t.out_x0 = cy, cx
        psx, psy = 20.0 + ty, -30.8
        t.pixel_scale_x, t.pixel_scale_y = psx, psy
        tiles.append(t)
        meta.append((cx, cy, cw, ch, wx, wy, ww, wh, psx, psy))
    params = op.make_params(max_distance=20, pixel_size=25.0)
    op.run_openness(_arrays.as_device_f32_2d(torch.from_numpy(dem).cuda()), tiles, params, None, raw)
    got = to_np(raw)
    for cx, cy, cw, ch, wx, wy, ww, wh, psx, psy in meta:
        win = dem[wy:wy + wh, wx:wx + ww]
        ref = R.openness(win, max_distance=20, pixel_size=25.0, psx=psx, psy=psy, raw_degrees=True)
        ref = ref[cy - wy:cy - wy + ch, cx - wx:cx - wx + cw]
        g = got[cy:cy + ch, cx:cx + cw]
        assert np.array_equal(np.isnan(g), np.isnan(ref))
        assert float(np.nanmax(np.abs(g.astype(np.float64) - ref))) <= 0.01


@pytest.mark.parametrize("otype", ["positive", "negative"])
def test_interior_fast_path_with_numeric_nodata(op, otype):
    """A window much wider than the rays: most blocks take the interior path (no bounds
    checks); NoData given as a numeric sentinel on both sides of the comparison."""
    from fujishadergpu_gb300 import synth
    dem = synth.fbm(400, 420, hurst=0.7, seed=87, lo=0.0, hi=800.0)
    dem[synth.nodata_disks(400, 420, count=6, seed=88, rmin=3.0, rmax=12.0)] = -9999.0
    kw = dict(openness_type=otype, num_directions=16, max_distance=16, pixel_size=5.0, pixel_scale_x=5.0,
              pixel_scale_y=-5.0)
    raw = to_np(op.compute_openness_raw_degrees(torch.from_numpy(dem).cuda(), nodata=-9999.0, **kw))
    clean = np.where(R.nodata_mask(dem, -9999.0), np.nan, dem).astype(np.float32)
    ref = R.openness(clean, openness_type=otype, num_directions=16, max_distance=16, pixel_size=5.0, psx=5.0,
                     psy=-5.0, raw_degrees=True)
    assert np.array_equal(np.isnan(raw), np.isnan(ref))
    assert float(np.nanmax(np.abs(raw.astype(np.float64) - ref))) <= 0.01
