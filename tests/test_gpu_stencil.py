"""GPU parity of the fused stencil kernel against the reference (golden
fixtures) and the CPU oracle, through the C ABI (ctypes)."""
import json
import os

import numpy as np
import pytest

from oracle import restated as R
from tests._parity import (assert_close_range, assert_codes_close,
                           assert_curvature_close, assert_same_nan, to_np)

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

STENCIL_CASES = ["s1_fbm_10m", "s2_fbm_5m_nan", "s3_geo_edges_nan", "s4_tiny_3x5", "s5_single_valid",
                 "s6_all_nan", "s7_parabolic_cylinder", "s8_dome", "s9_big_void"]


@pytest.fixture(scope="module")
def fsg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300 import algorithms
    return algorithms


def _golden(golden_dir):
    g = np.load(os.path.join(golden_dir, "stencil.npz"))
    with open(os.path.join(golden_dir, "stencil.json")) as f:
        m = json.load(f)
    return g, m


@pytest.mark.parametrize("case", STENCIL_CASES)
def test_stencil_matches_reference_golden(fsg, golden_dir, case):
    g, meta = _golden(golden_dir)
    m = meta[case]
    dem = g[f"{case}/dem"]
    d = torch.from_numpy(dem).cuda()
    kw = dict(pixel_size=m["pixel_size"], pixel_scale_x=m["psx"], pixel_scale_y=m["psy"])
    hs = fsg.compute_hillshade_block(d, azimuth=m["azimuth"], altitude=m["altitude"],
                                     z_factor=m["z_factor"], **kw)
    assert_close_range(hs, g[f"{case}/hillshade"], 1.0, f"{case} hillshade")
    for unit, rng in (("degree", 90.0), ("radian", np.pi / 2)):
        assert_close_range(fsg.compute_slope_block(d, unit=unit, **kw), g[f"{case}/slope_{unit}"], rng,
                           f"{case} slope {unit}")
    # percent = tan(atan(|grad|)) * 100 is ill-conditioned near 90 degrees (the reference
    # rounds atan to float32 first), so it is compared in the angle domain.
    pct = to_np(fsg.compute_slope_block(d, unit="percent", **kw))
    ref_pct = g[f"{case}/slope_percent"]
    assert_close_range(np.arctan(pct.astype(np.float64) / 100.0), np.arctan(ref_pct.astype(np.float64) / 100.0),
                       np.pi / 2, f"{case} slope percent (as angle)")
    for ct in ("mean", "gaussian", "planform", "profile"):
        assert_curvature_close(fsg.compute_curvature_block(d, curvature_type=ct, **kw),
                               g[f"{case}/curvature_{ct}"], f"{case} curvature {ct}")


@pytest.mark.parametrize("case", ["s1_fbm_10m", "s2_fbm_5m_nan", "s3_geo_edges_nan", "s9_big_void", "s4_tiny_3x5"])
def test_gradient_and_nan_fill_bit_exact(fsg, golden_dir, case):
    """dy, dx of handle_nan_for_gradient: bit-exact np.gradient incl. edge rules and the NaN fill."""
    from fujishadergpu_gb300.algorithms._stencil import stencil_block
    g, meta = _golden(golden_dir)
    m = meta[case]
    dem = g[f"{case}/dem"]
    out = stencil_block(torch.from_numpy(dem).cuda(), ["dx", "dy"], pixel_size=m["pixel_size"],
                        pixel_scale_x=m["psx"], pixel_scale_y=m["psy"])
    dy, dx, nan = R.nan_aware_gradient(dem, pixel_size=m["pixel_size"], psx=m["psx"], psy=m["psy"])
    for name, ref in (("dx", dx), ("dy", dy)):
        got = to_np(out[name])
        ref = np.where(nan, np.nan, ref).astype(np.float32)
        assert_same_nan(got, ref, name)
        v = ~nan
        assert np.array_equal(got[v], ref[v]), (
            f"{case} {name}: {int((got[v] != ref[v]).sum())} of {int(v.sum())} differ; "
            f"max {float(np.abs(got[v] - ref[v]).max()):.3e}")


def test_reference_curvature_known_answers_on_gpu(fsg):
    """reference tests/test_curvature_analytic.py:26-54."""
    zero = 0.5 ** (1.0 / 2.2)
    x = torch.arange(64, dtype=torch.float32, device="cuda")[None, :].repeat(64, 1)
    y = torch.arange(64, dtype=torch.float32, device="cuda")[:, None].repeat(1, 64)
    cyl = 0.01 * (x - 32.0) ** 2
    plan = to_np(fsg.compute_curvature_block(cyl, curvature_type="planform"))
    prof = to_np(fsg.compute_curvature_block(cyl, curvature_type="profile"))
    assert float(np.abs(plan[20:44, 20:44] - zero).max()) < 0.02
    assert float(np.abs(prof[20:44, 20:44] - zero).max()) > 0.05
    dome = -0.01 * ((x - 32.0) ** 2 + (y - 32.0) ** 2)
    for ct in ("planform", "profile"):
        assert float(np.abs(to_np(fsg.compute_curvature_block(dome, curvature_type=ct))[20:44, 20:44]
                            - zero).max()) > 0.05


def _fbm_nan(h, w, seed, disks, lo=0.0, hi=3000.0):
    from fujishadergpu_gb300 import synth
    d = synth.fbm(h, w, hurst=0.7, seed=seed, lo=lo, hi=hi)
    if disks:
        d[synth.nodata_disks(h, w, count=disks, seed=seed + 1, rmin=3.0, rmax=30.0)] = np.nan
    return d


def test_fused_products_match_oracle_large(fsg):
    from fujishadergpu_gb300.algorithms._stencil import stencil_block
    dem = _fbm_nan(700, 900, 41, 12)
    names = ["hillshade", "slope", "curvature_mean", "curvature_gaussian", "curvature_planform",
             "curvature_profile"]
    out = stencil_block(torch.from_numpy(dem).cuda(), names, azimuth=300.0, altitude=40.0,
                        pixel_size=5.0, pixel_scale_x=5.0, pixel_scale_y=-5.0)
    kw = dict(pixel_size=5.0, psx=5.0, psy=-5.0)
    assert_close_range(out["hillshade"], R.hillshade(dem, azimuth=300.0, altitude=40.0, **kw), 1.0, "hs")
    assert_close_range(out["slope"], R.slope(dem, **kw), 90.0, "slope")
    for ct in ("mean", "gaussian", "planform", "profile"):
        assert_curvature_close(out["curvature_" + ct], R.curvature(dem, curvature_type=ct, **kw), ct)


def test_nodata_sentinel_is_masked(fsg):
    from fujishadergpu_gb300.algorithms._stencil import stencil_block
    dem = _fbm_nan(200, 260, 43, 0)
    mask = np.zeros(dem.shape, bool)
    mask[50:80, 100:140] = True
    mask[0:5, :] = True
    raw = dem.copy()
    raw[mask] = -9999.0
    out = stencil_block(torch.from_numpy(raw).cuda(), ["hillshade", "slope"], pixel_size=10.0,
                        pixel_scale_x=10.0, pixel_scale_y=-10.0, nodata=-9999.0)
    ref_mask = R.nodata_mask(raw, -9999.0)
    clean = np.where(ref_mask, np.nan, raw).astype(np.float32)
    kw = dict(pixel_size=10.0, psx=10.0, psy=-10.0)
    assert_close_range(out["hillshade"], R.hillshade(clean, **kw), 1.0, "hs nodata")
    assert_close_range(out["slope"], R.slope(clean, **kw), 90.0, "slope nodata")
    assert np.array_equal(np.isnan(to_np(out["slope"])), ref_mask)


def _tile_descs(H, W, tile, pad, psx, psy):
    """The product's tile descriptors (core.tile_loop), checked against the oracle's grid."""
    from fujishadergpu_gb300.core import tile_loop
    infos = tile_loop.tile_grid(H, W, tile, pad)
    assert [(i.ty, i.tx, i.core_x, i.core_y, i.core_w, i.core_h, i.win_x, i.win_y, i.win_w, i.win_h)
            for i in infos] == [tuple(t) for t in R.tile_grid(H, W, tile, pad)]
    return tile_loop.make_tiles(infos, pixel_scale_x=psx, pixel_scale_y=psy)


@pytest.mark.parametrize("tile,pad", [(128, 8), (100, 2), (256, 64)])
def test_tiled_launch_matches_per_window_oracle(fsg, tile, pad):
    """Many tiles in one launch: each core equals the reference run on its clipped window."""
    from fujishadergpu_gb300 import _arrays
    from fujishadergpu_gb300.algorithms import _stencil as S
    H, W = 300, 517
    dem = _fbm_nan(H, W, 47, 8)
    v = _arrays.as_device_f32_2d(torch.from_numpy(dem).cuda())
    hs = torch.empty((H, W), device="cuda")
    cp = torch.empty((H, W), device="cuda")
    qp = R.quantize_params(0.0, 1.0, "uint8")
    hs8 = torch.empty((H, W), device="cuda", dtype=torch.uint8)
    params = S.make_params(pixel_size=5.0)
    planes = {S.OUTPUT_INDEX["hillshade"]: S.make_plane(hs),
              S.OUTPUT_INDEX["curvature_profile"]: S.make_plane(cp)}
    tiles = _tile_descs(H, W, tile, pad, 5.0, -5.0)
    S.launch(v, tiles, params, planes)
    S.launch(v, tiles, params, {S.OUTPUT_INDEX["hillshade"]: S.make_plane(hs8, "uint8", qp)})
    hs, cp, hs8 = to_np(hs), to_np(cp), to_np(hs8)
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in R.tile_grid(H, W, tile, pad):
        win = dem[wy:wy + wh, wx:wx + ww]
        sl = (slice(cy - wy, cy - wy + ch), slice(cx - wx, cx - wx + cw))
        core = (slice(cy, cy + ch), slice(cx, cx + cw))
        ref_hs = R.hillshade(win, pixel_size=5.0, psx=5.0, psy=-5.0)[sl]
        assert_close_range(hs[core], ref_hs, 1.0, f"tile {ty},{tx} hs")
        assert_curvature_close(cp[core], R.curvature(win, curvature_type="profile", pixel_size=5.0,
                                                     psx=5.0, psy=-5.0)[sl], f"tile {ty},{tx} profile")
        assert_codes_close(hs8[core], R.quantize_array(ref_hs, qp, "uint8"), f"tile {ty},{tx} u8")


def test_quantized_planes_within_one_lsb(fsg):
    from fujishadergpu_gb300.algorithms._stencil import stencil_block
    dem = _fbm_nan(257, 333, 53, 5)
    qs = R.quantize_params(0.0, 90.0, "int16")
    qh = R.quantize_params(0.0, 1.0, "uint8")
    d = torch.from_numpy(dem).cuda()
    s16 = stencil_block(d, ["slope"], pixel_size=5.0, out_dtype="int16", quantize={"slope": qs})["slope"]
    h8 = stencil_block(d, ["hillshade"], pixel_size=5.0, out_dtype="uint8", quantize={"hillshade": qh})["hillshade"]
    assert s16.dtype == torch.int16 and h8.dtype == torch.uint8
    assert_codes_close(s16, R.quantize_array(R.slope(dem, pixel_size=5.0), qs, "int16"), "slope i16")
    assert_codes_close(h8, R.quantize_array(R.hillshade(dem, pixel_size=5.0), qh, "uint8"), "hs u8")
    assert np.array_equal(to_np(h8) == 0, np.isnan(dem))


def test_window_too_small_raises_value_error(fsg):
    with pytest.raises(ValueError):
        fsg.compute_hillshade_block(torch.zeros((2, 5), device="cuda"))
    with pytest.raises(ValueError):
        fsg.compute_slope_block(torch.zeros((7, 1), device="cuda"))


def test_z_factor_and_azimuth(fsg):
    dem = _fbm_nan(120, 140, 59, 3)
    for z, az, alt in ((2.5, 10.0, 20.0), (0.5, 200.0, 70.0)):
        got = fsg.compute_hillshade_block(torch.from_numpy(dem).cuda(), azimuth=az, altitude=alt, z_factor=z,
                                          pixel_size=2.0, pixel_scale_x=-2.0, pixel_scale_y=3.0)
        ref = R.hillshade(dem, azimuth=az, altitude=alt, z_factor=z, pixel_size=2.0, psx=-2.0, psy=3.0)
        assert_close_range(got, ref, 1.0, f"hs z={z}")


@pytest.mark.parametrize("dtype", ["float32", "uint8"])
def test_host_buffer_tile_loop_equals_device_path(fsg, dtype):
    """fsg_stencil_host (pinned host raster and planes, overlapped copies) == fsg_stencil."""
    from fujishadergpu_gb300 import _arrays
    from fujishadergpu_gb300.algorithms import _stencil as S
    H, W = 700, 910
    dem = _fbm_nan(H, W, 101, 6)
    names = ["hillshade", "slope", "curvature_profile", "curvature_planform"]
    qp = R.quantize_params(0.0, 1.0, "uint8") if dtype == "uint8" else None
    tdt = torch.float32 if dtype == "float32" else torch.uint8
    tiles = _tile_descs(H, W, 256, 8, 5.0, -5.0)
    params = S.make_params(pixel_size=5.0)
    dev = {n: torch.empty((H, W), device="cuda", dtype=tdt) for n in names}
    S.launch(_arrays.as_device_f32_2d(torch.from_numpy(dem).cuda()), tiles, params,
             {S.OUTPUT_INDEX[n]: S.make_plane(dev[n], dtype, qp) for n in names})
    host_in = torch.from_numpy(dem).pin_memory()
    host = {n: torch.full((H, W), 7, dtype=tdt).pin_memory() for n in names}
    S.launch_host(host_in, tiles, params, {S.OUTPUT_INDEX[n]: S.host_plane(host[n], dtype, qp) for n in names})
    torch.cuda.synchronize()
    for n in names:
        a, b = to_np(dev[n]), host[n].numpy()
        assert np.array_equal(a, b, equal_nan=True), n


def test_back_to_back_host_buffer_calls_keep_their_own_tables(fsg):
    """Calls queued without a synchronisation in between (their tile tables staged in turn
    through the library's pinned ring, more calls than the ring has slots, different tile
    grids and rasters) each equal the device path of their own inputs."""
    from fujishadergpu_gb300 import _arrays
    from fujishadergpu_gb300.algorithms import _stencil as S
    params = S.make_params(pixel_size=5.0)
    runs = []
    for k in range(40):
        H, W = 300 + 7 * (k % 5), 410 - 5 * (k % 3)
        tile = (96, 128, 200)[k % 3]
        dem = _fbm_nan(H, W, 500 + k, 3)
        tiles = _tile_descs(H, W, tile, 8, 5.0, -5.0)
        host_in = torch.from_numpy(dem).pin_memory()
        host = torch.full((H, W), 7.0).pin_memory()
        S.launch_host(host_in, tiles, params, {S.OUTPUT_INDEX["curvature_profile"]: S.host_plane(host)})
        runs.append((dem, tiles, host))
    torch.cuda.synchronize()
    for dem, tiles, host in runs:
        dev = torch.empty(dem.shape, device="cuda")
        S.launch(_arrays.as_device_f32_2d(torch.from_numpy(dem).cuda()), tiles, params,
                 {S.OUTPUT_INDEX["curvature_profile"]: S.make_plane(dev)})
        assert np.array_equal(to_np(dev), host.numpy(), equal_nan=True)


@pytest.mark.parametrize("offset", [0, 1])
def test_tensor_copy_ring_equals_cp_async_ring(fsg, offset):
    """The streaming pass fills its row ring with one tensor-memory copy per row when the raster
    and the unit columns are 16-byte aligned, else with cp.async; both give identical planes,
    and no wait on a tensor copy runs out (fsg_kernel_errors)."""
    from fujishadergpu_gb300 import _native as N
    from fujishadergpu_gb300.algorithms import _stencil as S
    from fujishadergpu_gb300.core import tile_loop as loop
    H, W = 900, 1100
    base = torch.from_numpy(_fbm_nan(H, W + 4, 77, 10)).cuda()
    d = base[:, offset:offset + W]  # offset 1: unaligned columns, the cp.async ring everywhere
    v = __import__("fujishadergpu_gb300._arrays", fromlist=["x"]).as_device_f32_2d(d)
    tiles = loop.make_tiles(loop.tile_grid(H, W, 512, 8), pixel_scale_x=5.0, pixel_scale_y=-5.0)
    names = ["hillshade", "slope", "curvature_profile", "curvature_planform"]
    sp = S.make_params(pixel_size=5.0)
    outs = {}
    for mode in ("tma", "cp_async"):
        if mode == "cp_async":
            os.environ["FSG_NO_TMA"] = "1"
        try:
            o = {n: torch.full((H, W), 3.0, device="cuda") for n in names}
            S.launch(v, tiles, sp, {S.OUTPUT_INDEX[n]: S.make_plane(o[n]) for n in names})
            torch.cuda.synchronize()
            outs[mode] = o
        finally:
            os.environ.pop("FSG_NO_TMA", None)
    assert N.kernel_errors() == 0
    for n in names:
        a, b = outs["tma"][n], outs["cp_async"][n]
        assert torch.equal(a.nan_to_num(-9.0), b.nan_to_num(-9.0)), n
    kw = dict(pixel_size=5.0, psx=5.0, psy=-5.0)
    dem = to_np(d)
    assert_close_range(outs["tma"]["hillshade"][8:-8, 8:-8], R.hillshade(dem, **kw)[8:-8, 8:-8], 1.0, "hs")
