"""GPU parity of ambient occlusion (fsg_ambient_occlusion) against the reference's
golden outputs and the CPU oracle: local and spatial block functions, the display
stretch and output codes, per-tile pixel scales and window edges, the direct-load
path for reaches beyond shared memory, numeric NoData, plans and the tile loop.
Tolerance: 1e-5 on the [0, 1] output (tests/_parity.py)."""
import json
import os

import numpy as np
import pytest

from oracle import restated as R
from tests._parity import assert_close_range, assert_codes_close, to_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

AO_CASES = ["a1_fbm_nan", "a2_aniso", "a3_r1", "a4_peak_pit", "a5_wide_radius", "a6_flat"]


@pytest.fixture(scope="module")
def ao():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300.algorithms import _impl_ambient_occlusion
    return _impl_ambient_occlusion


def _golden(golden_dir):
    g = np.load(os.path.join(golden_dir, "ambient_occlusion.npz"))
    with open(os.path.join(golden_dir, "ambient_occlusion.json")) as f:
        m = json.load(f)
    return g, m


@pytest.mark.parametrize("case", AO_CASES)
def test_ambient_occlusion_matches_reference_golden(ao, golden_dir, case):
    g, meta = _golden(golden_dir)
    m = meta[case]
    out = ao.compute_ambient_occlusion_block(torch.from_numpy(g[f"{case}/dem"]).cuda(),
                                             num_samples=m["num_samples"], radius=m["radius"],
                                             intensity=m["intensity"], pixel_size=m["pixel_size"],
                                             pixel_scale_x=m["psx"], pixel_scale_y=m["psy"])
    assert_close_range(out, g[f"{case}/ao"], 1.0, case)


def test_stretch_and_spatial_blocks_match_reference_golden(ao, golden_dir):
    g, _ = _golden(golden_dir)
    out = ao.AmbientOcclusionAlgorithm().process(torch.from_numpy(g["a1_fbm_nan/dem"]).cuda(), num_samples=16,
                                                 radius=10.0, pixel_size=5.0, pixel_scale_x=5.0,
                                                 pixel_scale_y=-5.0, global_stats=(0.55, 0.4))
    assert_close_range(out, g["a1_fbm_nan/direct_stretch"], 1.0 / 0.4, "stretched")
    for dn in ("clean", "nan"):
        dem = torch.from_numpy(g[f"spatial_{dn}/dem"]).cuda()
        for r in (8, 40, 100):
            out = ao.compute_ambient_occlusion_spatial_block(dem, num_samples=16, radius=float(r), pixel_size=5.0,
                                                             pixel_scale_x=5.0, pixel_scale_y=-5.0)
            assert_close_range(out, g[f"spatial_{dn}/ao_{r}"], 1.0, f"spatial {dn} r={r}")


@pytest.mark.parametrize("radius,ns", [(10.0, 16), (3.3, 24), (0.0, 16)])
def test_block_matches_oracle(ao, radius, ns):
    from fujishadergpu_gb300 import synth
    dem = synth.fbm(330, 410, hurst=0.7, seed=91, lo=0.0, hi=1500.0)
    dem[synth.nodata_disks(330, 410, count=5, seed=92, rmin=3.0, rmax=14.0)] = np.nan
    out = ao.compute_ambient_occlusion_block(torch.from_numpy(dem).cuda(), num_samples=ns, radius=radius,
                                             intensity=0.8, pixel_size=5.0, pixel_scale_x=4.0, pixel_scale_y=-6.0)
    ref = R.ambient_occlusion(dem, num_samples=ns, radius=radius, intensity=0.8, pixel_size=5.0, psx=4.0,
                              psy=-6.0)
    assert_close_range(out, ref, 1.0, f"r={radius}")


def test_reach_beyond_shared_memory_reads_the_raster(ao):
    """radius 120: the staged block would exceed shared memory, so the samples are
    clamped loads from the raster (the same results)."""
    from fujishadergpu_gb300 import synth
    dem = synth.fbm(260, 300, hurst=0.8, seed=93, lo=0.0, hi=2500.0)
    dem[synth.nodata_disks(260, 300, count=3, seed=94, rmin=4.0, rmax=10.0)] = np.nan
    out = ao.compute_ambient_occlusion_block(torch.from_numpy(dem).cuda(), num_samples=8, radius=120.0,
                                             pixel_size=10.0)
    ref = R.ambient_occlusion(dem, num_samples=8, radius=120.0, pixel_size=10.0)
    assert_close_range(out, ref, 1.0, "r=120")


def test_numeric_nodata_and_codes(ao):
    from fujishadergpu_gb300 import synth
    dem = synth.fbm(150, 170, hurst=0.7, seed=95, lo=0.0, hi=900.0)
    dem[synth.nodata_disks(150, 170, count=4, seed=96, rmin=3.0, rmax=9.0)] = -9999.0
    clean = np.where(R.nodata_mask(dem, -9999.0), np.nan, dem).astype(np.float32)
    ref = R.ambient_occlusion(clean, radius=8.0, pixel_size=5.0)
    stats = R.stretch_stats(ref)
    qp = R.quantize_params(0.0, 1.0, "uint8")
    out, _ = ao.ambient_occlusion_plane(torch.from_numpy(dem).cuda(), radius=8.0, pixel_size=5.0, stretch=stats,
                                        out_dtype="uint8", qp=qp, nodata=-9999.0)
    assert_codes_close(out, R.quantize_array(R.apply_stretch(ref, stats), qp, "uint8"), "u8")
    f32, _ = ao.ambient_occlusion_plane(torch.from_numpy(dem).cuda(), radius=8.0, pixel_size=5.0, nodata=-9999.0)
    assert_close_range(f32, ref, 1.0, "f32")


def test_tiles_with_their_own_scales_and_window_edges(ao):
    """Each tile is its own block: samples clamp to its window, the Gaussian is
    'nearest' at the window edge, and each tile carries its own pixel scales."""
    from fujishadergpu_gb300 import _arrays, synth
    from fujishadergpu_gb300._native import Tile
    from fujishadergpu_gb300.algorithms._stencil import make_plane
    H, W = 210, 240
    dem = synth.fbm(H, W, hurst=0.7, seed=97, lo=0.0, hi=900.0)
    dem[synth.nodata_disks(H, W, count=3, seed=98, rmin=3.0, rmax=9.0)] = np.nan
    out = torch.full((H, W), 5.0, device="cuda")
    tiles, meta = [], []
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in R.tile_grid(H, W, 64, 12):
        t = Tile()
        t.win_y0, t.win_x0, t.win_h, t.win_w = wy, wx, wh, ww
        t.core_y0, t.core_x0, t.core_h, t.core_w = cy, cx, ch, cw
        t.out_y0, t.out_x0 = cy, cx
        psx, psy = 20.0 + 2 * ty, -30.8
        t.pixel_scale_x, t.pixel_scale_y = psx, psy
        tiles.append(t)
        meta.append((cx, cy, cw, ch, wx, wy, ww, wh, psx, psy))
    ao.run_ambient_occlusion(_arrays.as_device_f32_2d(torch.from_numpy(dem).cuda()), tiles,
                             ao.make_params(radius=9.0, pixel_size=25.0), make_plane(out))
    got = to_np(out)
    for cx, cy, cw, ch, wx, wy, ww, wh, psx, psy in meta:
        ref = R.ambient_occlusion(dem[wy:wy + wh, wx:wx + ww], radius=9.0, pixel_size=25.0, psx=psx, psy=psy)
        assert_close_range(got[cy:cy + ch, cx:cx + cw], ref[cy - wy:cy - wy + ch, cx - wx:cx - wx + cw], 1.0,
                           f"tile {cy},{cx}")


def test_plan_matches_the_eager_call(ao):
    import ctypes as C
    from fujishadergpu_gb300 import _arrays, synth
    from fujishadergpu_gb300 import _native as N
    from fujishadergpu_gb300.algorithms._stencil import make_plane
    from fujishadergpu_gb300.core import plans
    H, W = 300, 280
    dem = torch.from_numpy(synth.fbm(H, W, hurst=0.7, seed=99, lo=0.0, hi=700.0)).cuda()
    v = _arrays.as_device_f32_2d(dem)
    tiles = [ao.whole_tile(H, W, 5.0, 5.0)]
    p = ao.make_params(radius=10.0, pixel_size=5.0)
    eager = torch.empty((H, W), device="cuda")
    ao.run_ambient_occlusion(v, tiles, p, make_plane(eager))
    out = torch.empty((H, W), device="cuda")
    tarr = (N.Tile * 1)(*tiles)
    h = C.c_void_p()
    N.check(N.lib().fsg_ambient_occlusion_plan(C.c_void_p(v.ptr), v.ld, v.h, v.w, tarr, 1, C.byref(p),
                                               C.byref(make_plane(out)), C.byref(h)))
    plan = plans.Plan(h, [v])
    plan.launch()
    torch.cuda.synchronize()
    assert torch.equal(out, eager)
    plan.close()


def test_tile_loop_local_with_stats_prepass(ao):
    from fujishadergpu_gb300 import synth
    from fujishadergpu_gb300.core import tile_loop as loop
    H, W = 300, 340
    dem = synth.fbm(H, W, hurst=0.7, seed=101, lo=0.0, hi=900.0)
    dem[synth.nodata_disks(H, W, count=2, seed=102, rmin=3.0, rmax=8.0)] = np.nan
    res = loop.process_dem_array(torch.from_numpy(dem).cuda(), "ambient_occlusion", tile_size=128, pixel_size=5.0,
                                 pixel_scale_x=5.0, pixel_scale_y=-5.0, mode="local", radius=10.0)
    assert res.stats is not None and res.stats[1] > 0
    got = to_np(res.output)
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww, wh) in R.tile_grid(H, W, 128, res.padding):
        ref = R.apply_stretch(R.ambient_occlusion(dem[wy:wy + wh, wx:wx + ww], radius=10.0, pixel_size=5.0,
                                                  psx=5.0, psy=-5.0), res.stats)
        assert_close_range(got[cy:cy + ch, cx:cx + cw], ref[cy - wy:cy - wy + ch, cx - wx:cx - wx + cw],
                           1.0 / res.stats[1], f"tile {ty},{tx}")


@pytest.mark.parametrize("agg", ["mean", "max"])
def test_window_spatial_mode_matches_oracle(ao, agg):
    """process(mode='spatial') on one window: per radius the reflect-padded spatial block
    (decimated 2x for radius 40), combined, stretched."""
    from fujishadergpu_gb300 import synth
    dem = synth.fbm(150, 170, hurst=0.8, seed=105, lo=0.0, hi=2000.0)
    dem[synth.nodata_disks(150, 170, count=2, seed=106, rmin=3.0, rmax=8.0)] = np.nan
    radii, weights = [3, 12, 40], [0.5, 0.3, 0.2]
    got = ao.AmbientOcclusionAlgorithm().process(torch.from_numpy(dem).cuda(), mode="spatial", radii=radii,
                                                 weights=weights, agg=agg, pixel_size=5.0, pixel_scale_x=5.0,
                                                 pixel_scale_y=-5.0, global_stats=(0.3, 0.6))
    rr, ww = R.resolve_spatial_radii_weights(radii, weights, 5.0)
    ref = R.spatial_window(dem, "ambient_occlusion", rr, ww, pixel_size=5.0, psx=5.0, psy=-5.0, agg=agg,
                           stretch=(0.3, 0.6), num_samples=16, intensity=1.0)
    assert_close_range(got, ref, 1.0 / 0.6, f"agg={agg}")


def test_tile_loop_spatial_mode(ao):
    """The tile loop in spatial mode: radii 4 and 40 through reflect-padded windows, 300
    (> the 256 threshold) from the overview (the raster is its own overview)."""
    from fujishadergpu_gb300 import synth
    from fujishadergpu_gb300.core import tile_loop as loop
    H, W = 600, 640
    dem = synth.fbm(H, W, hurst=0.8, seed=107, lo=0.0, hi=2000.0)
    mask = synth.nodata_disks(H, W, count=3, seed=108, rmin=3.0, rmax=8.0)
    dem[mask] = np.nan
    radii, weights = [4, 40, 300], [0.5, 0.3, 0.2]
    stats = (0.4, 0.55)
    res = loop.process_dem_array(torch.from_numpy(dem).cuda(), "ambient_occlusion", tile_size=256, pixel_size=5.0,
                                 pixel_scale_x=5.0, pixel_scale_y=-5.0, mode="spatial", radii=radii,
                                 weights=weights, global_stats=stats)
    got = to_np(res.output)
    rr, ww = loop.sanitize_spatial_radii_weights("ambient_occlusion", radii, weights)
    rr, ww = R.resolve_spatial_radii_weights(rr, ww, 5.0)
    for (ty, tx, cx, cy, cw, ch, wx, wy, ww_, wh) in R.tile_grid(H, W, 256, res.padding):
        win = dem[wy:wy + wh, wx:wx + ww_]
        comb = R.spatial_window(win, "ambient_occlusion", rr, ww, origin=(wy, wx), full_shape=(H, W),
                                coarse_dem=dem, decimation=1.0, pixel_size=5.0, psx=5.0, psy=-5.0,
                                stretch=stats, num_samples=16, intensity=1.0)
        ref = np.where(np.isnan(win), np.float32(np.nan), comb)[cy - wy:cy - wy + ch, cx - wx:cx - wx + cw]
        assert_close_range(got[cy:cy + ch, cx:cx + cw], ref, 1.0 / stats[1], f"tile {ty},{tx}")
