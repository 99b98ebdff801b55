"""GPU parity of topousm_fast, its coarse large-radius field, the FP64
percentile statistics and the normalisation/encoding kernels, against the
reference's golden outputs and the CPU oracle (through the C ABI)."""
import json
import os

import numpy as np
import pytest

from oracle import restated as R
from tests._parity import assert_close_range, assert_codes_close, assert_same_nan, to_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

NORM_RANGE = 2 * 1.176  # topousm output range (io/output_encoding.py:39-42)


@pytest.fixture(scope="module")
def tu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300.algorithms import _impl_topousm_fast
    return _impl_topousm_fast


def _golden(golden_dir):
    g = np.load(os.path.join(golden_dir, "topousm.npz"))
    with open(os.path.join(golden_dir, "topousm.json")) as f:
        m = json.load(f)
    return g, m


def assert_topousm_close(got, ref, what):
    """Raw topousm: 1e-5 of the normalised output range, i.e. 2.352e-5 x p99(|ref|)."""
    scale = R.topousm_scale(np.asarray(ref))[0]
    return assert_close_range(got, ref, NORM_RANGE * scale, what)


@pytest.mark.parametrize("case", ["t1_clean", "t2_nan", "t3_halfmetre", "t4_nan_r2"])
def test_topousm_block_matches_reference_golden(tu, golden_dir, case):
    g, meta = _golden(golden_dir)
    out = tu.compute_topousm_fast_efficient_block(
        torch.from_numpy(g[f"{case}/dem"]).cuda(), radii=[int(r) for r in g[f"{case}/radii"]],
        weights=[float(w) for w in g[f"{case}/weights"]], pixel_size=meta[case]["pixel_size"])
    assert_topousm_close(out, g[f"{case}/out"], case)


def test_topousm_block_vs_fp64_oracle(tu):
    """Error statement against the FP64 restatement of the same algorithm."""
    from fujishadergpu_gb300 import synth
    dem = synth.fbm_ridged(300, 340, hurst=0.8, seed_fbm=61, seed_ridged=62, lo=0.0, hi=3500.0)
    dem[synth.nodata_disks(300, 340, count=4, seed=63, rmin=5.0, rmax=30.0)] = np.nan
    radii, w = [2, 8, 32, 128], [32 / 60, 16 / 60, 8 / 60, 4 / 60]
    got = to_np(tu.compute_topousm_fast_efficient_block(torch.from_numpy(dem).cuda(), radii=radii, weights=w,
                                                          pixel_size=10.0)).astype(np.float64)
    ref64 = R.topousm_block(dem.astype(np.float64), radii=radii, weights=w, pixel_size=10.0)
    scale = R.topousm_scale(ref64)[0]
    assert_same_nan(got, ref64, "fp64")
    m = ~np.isnan(ref64)
    rel = float(np.abs(got[m] - ref64[m]).max()) / scale
    assert rel <= 1e-5, rel


def test_coarse_field_matches_reference_golden(tu, golden_dir):
    g, _ = _golden(golden_dir)
    field = tu.compute_topousm_fast_large_coarse_field(torch.from_numpy(g["coarse/dem"]).cuda(),
                                                       large_radii=[512, 2048],
                                                       large_weights=[2.0 / 63.0, 1.0 / 63.0], decimation=16.0)
    ref = g["coarse/field"]
    assert_close_range(field, ref, float(np.nanmax(np.abs(ref))), "coarse field", rel=2e-6)


def _tiles(H, W, tile, pad):
    """The product's tile descriptors (core.tile_loop), checked against the oracle's grid."""
    from fujishadergpu_gb300.core import tile_loop
    infos = tile_loop.tile_grid(H, W, tile, pad)
    assert [(i.ty, i.tx, i.core_x, i.core_y, i.core_w, i.core_h, i.win_x, i.win_y, i.win_w, i.win_h)
            for i in infos] == [tuple(t) for t in R.tile_grid(H, W, tile, pad)]
    return tile_loop.make_tiles(infos, pixel_scale_x=10.0, pixel_scale_y=-10.0)


@pytest.mark.parametrize("dtype", ["float32", "int16"])
def test_tiled_topousm_with_coarse_field_and_normalisation(tu, dtype):
    """Tile loop semantics of dask_bridge._direct_topousm_fast: small radii per window,
    large radii from a global coarse field sampled at global coords, / p99 scale."""
    from fujishadergpu_gb300 import _arrays, synth
    from fujishadergpu_gb300.algorithms._stencil import make_plane
    H, W = 520, 608
    dem = synth.fbm_ridged(H, W, hurst=0.8, seed_fbm=71, seed_ridged=72, lo=0.0, hi=3500.0)
    dem[synth.nodata_disks(H, W, count=5, seed=73, rmin=5.0, rmax=25.0)] = np.nan
    small_r, small_w = [2, 8, 32], [32 / 63, 16 / 63, 8 / 63]
    large_r, large_w = [512, 2048], [2 / 63, 1 / 63]
    # overview grid: decimate by 4 (the oracle uses the same block mean as the GPU overview kernel)
    dec = 4
    d = torch.from_numpy(dem).cuda()
    oh, ow = H // dec, W // dec
    cdem = tu.overview(d, (oh, ow))
    cells = dem[:oh * dec, :ow * dec].reshape(oh, dec, ow, dec).astype(np.float64)
    with np.errstate(invalid="ignore"):
        ref_cdem = np.nanmean(cells, axis=(1, 3)).astype(np.float32)
    cd = to_np(cdem)
    assert_close_range(cd, ref_cdem, 3500.0, "overview block mean", rel=1e-7)
    field = tu.compute_topousm_fast_large_coarse_field(cdem, large_radii=large_r, large_weights=large_w,
                                                       decimation=float(dec))
    ref_field = R.coarse_field(cd.copy(), large_radii=large_r, large_weights=large_w, decimation=float(dec))
    assert_close_range(field, ref_field, float(np.nanmax(np.abs(ref_field))), "field", rel=2e-6)
    pad = max(32, ((max(small_r) + 16 + 31) // 32) * 32)
    tiles = _tiles(H, W, 192, pad)
    # a realistic normalisation scale: p99(|raw|) of the untiled oracle result
    raw_all = R.topousm_tile(dem, radii=None, weights=None, pixel_size=10.0, coarse=to_np(field),
                             small_radii=small_r, small_weights=small_w, w_large=sum(large_w), offset=(0, 0),
                             full_shape=(H, W))
    scale = R.topousm_scale(raw_all)[0]
    qp = R.quantize_params(-1.176, 1.176, "int16") if dtype == "int16" else None
    out = _arrays.empty(H, W, dtype)
    params, keep = tu.make_params(small_r, small_w, 10.0, coarse=field, w_large=sum(large_w), full_shape=(H, W),
                                  scale=scale)
    tu.run_topousm(_arrays.as_device_f32_2d(d), tiles, params, make_plane(out, dtype, qp))
    got = to_np(out)
    F = to_np(field)
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in R.tile_grid(H, W, 192, pad):
        win = dem[wy:wy + wh, wx:wx + ww]
        raw = R.topousm_tile(win, radii=None, weights=None, pixel_size=10.0, coarse=F, small_radii=small_r,
                             small_weights=small_w, w_large=sum(large_w), offset=(wy, wx), full_shape=(H, W))
        ref = R.topousm_normalize(raw, (scale,))[cy - wy:cy - wy + ch, cx - wx:cx - wx + cw]
        g = got[cy:cy + ch, cx:cx + cw]
        if dtype == "float32":
            assert_close_range(g, ref, NORM_RANGE, f"tile {ty},{tx}")
        else:
            assert_codes_close(g, R.quantize_array(ref, qp, "int16"), f"tile {ty},{tx} int16")


def test_percentiles_exact_against_numpy():
    from fujishadergpu_gb300.algorithms import _stats
    rng = np.random.default_rng(5)
    for n in (1, 2, 7, 1000, 123457):
        x = (rng.standard_normal(n) * 10).astype(np.float32)
        if n > 10:
            x[rng.integers(0, n, n // 10)] = np.nan
        v = x[~np.isnan(x)]
        qs = [0.0, 1.0, 37.5, 50.0, 99.0, 100.0]
        got, nv = _stats.percentile(torch.from_numpy(x).cuda(), qs)
        assert nv == v.size
        v64 = v.astype(np.float64)  # FP64 interpolation between the exact float32 order statistics
        ref = [float(np.percentile(v64, q)) for q in qs]
        assert got == pytest.approx(ref, rel=1e-12, abs=1e-12), (n, got, ref)
        ref32 = [float(np.percentile(v, q)) for q in qs]  # NumPy's float32 interpolation (scalar q)
        assert got == pytest.approx(ref32, rel=2.5e-7, abs=1e-30)
        ga, _ = _stats.percentile(torch.from_numpy(x).cuda(), [99.0], absolute=True)
        assert ga[0] == pytest.approx(float(np.percentile(np.abs(v64), 99.0)), rel=1e-12)


def test_stat_funcs_match_reference_golden(golden_dir):
    from fujishadergpu_gb300.algorithms import _stats
    g, _ = _golden(golden_dir)
    for k in ("outliers", "ridge"):
        got = _stats.topousm_fast_stat_func(torch.from_numpy(g[f"stats/{k}"]).cuda())
        assert got[0] == pytest.approx(float(g[f"stats/{k}_scale"][0]), rel=1e-7)
    got = _stats.topousm_fast_stat_func(torch.from_numpy(g["t2_nan/out"]).cuda())
    assert got[0] == pytest.approx(float(g["stats/t2_scale"][0]), rel=1e-7)
    st = _stats.robust_unsigned_stretch_stat_func(torch.from_numpy(g["stats/stretch_in"]).cuda())
    ref = tuple(float(x) for x in g["stats/stretch"])
    assert st == pytest.approx(ref, rel=1e-7)
    # near-constant data falls back to std, then 1.0 (_normalization.py:29-31)
    const = torch.full((100,), 3.0, device="cuda")
    assert _stats.topousm_fast_stat_func(const)[0] == pytest.approx(3.0)
    assert _stats.topousm_fast_stat_func(torch.zeros(50, device="cuda"))[0] == 1.0
    assert _stats.topousm_fast_stat_func(torch.full((5,), float("nan"), device="cuda"))[0] == 1.0


def test_normalisation_matches_reference_golden(tu, golden_dir):
    g, _ = _golden(golden_dir)
    raw = torch.from_numpy(g["t2_nan/out"]).cuda()
    out = tu.normalize(raw, (float(g["stats/t2_scale"][0]),))
    ref = g["stats/t2_norm"]
    assert_same_nan(to_np(out), ref, "norm")
    assert np.array_equal(to_np(out)[~np.isnan(ref)], ref[~np.isnan(ref)])


def test_topousm_algorithm_class_tile_estimated_stats(tu, golden_dir):
    """TopoUSMFastAlgorithm.process without global_stats: per-tile p99 normalisation."""
    g, meta = _golden(golden_dir)
    dem = g["t1_clean/dem"]
    radii = [int(r) for r in g["t1_clean/radii"]]
    w = [float(x) for x in g["t1_clean/weights"]]
    out = tu.TopoUSMFastAlgorithm().process(torch.from_numpy(dem).cuda(), radii=radii, weights=w, pixel_size=10.0)
    raw = g["t1_clean/out"]
    ref = R.topousm_normalize(raw, R.topousm_scale(raw))
    assert_close_range(out, ref, NORM_RANGE, "class normalised")


def test_weights_length_mismatch_raises(tu):
    with pytest.raises(ValueError):
        tu.compute_topousm_fast_efficient_block(torch.zeros((16, 16), device="cuda"), radii=[2, 4], weights=[1.0])
