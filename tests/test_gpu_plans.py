"""Prepared launches (fsg_plan), their capture into a CUDA graph, and the
batched uneven-tile workload over an overview pyramid: every output equals
the eager entry point / the per-level tile loop on the same inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def mods():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300 import _arrays, _native, synth
    from fujishadergpu_gb300.algorithms import _impl_openness as OP
    from fujishadergpu_gb300.algorithms import _impl_topousm_fast as TU
    from fujishadergpu_gb300.algorithms import _stencil as S
    from fujishadergpu_gb300.core import plans as PL
    from fujishadergpu_gb300.core import tile_loop
    return dict(A=_arrays, N=_native, synth=synth, OP=OP, TU=TU, S=S, PL=PL, loop=tile_loop)


def _dem(m, h, w, seed):
    d = m["synth"].fbm(h, w, hurst=0.75, seed=seed, lo=0.0, hi=3000.0)
    d[m["synth"].nodata_disks(h, w, count=6, seed=seed + 1, rmin=5.0, rmax=40.0)] = np.nan
    return torch.from_numpy(d).cuda()


def _eq(a, b):
    return torch.equal(a.nan_to_num(-12345.0), b.nan_to_num(-12345.0))


def test_stencil_plan_and_graph_match_the_eager_call(mods):
    m = mods
    S, PL, loop = m["S"], m["PL"], m["loop"]
    d = _dem(m, 700, 900, 11)
    v = m["A"].as_device_f32_2d(d)
    tiles = loop.make_tiles(loop.tile_grid(700, 900, 256, 8), pixel_scale_x=5.0, pixel_scale_y=-5.0)
    names = ["hillshade", "slope", "curvature_profile", "curvature_planform"]
    sp = S.make_params(pixel_size=5.0)
    eager = {n: torch.empty_like(d) for n in names}
    S.launch(v, tiles, sp, {S.OUTPUT_INDEX[n]: S.make_plane(eager[n]) for n in names})
    got = {n: torch.full_like(d, 7.0) for n in names}
    plan = PL.stencil_plan(v, tiles, sp, {S.OUTPUT_INDEX[n]: S.make_plane(got[n]) for n in names})
    plan.launch()
    torch.cuda.synchronize()
    for n in names:
        assert _eq(got[n], eager[n]), n
    for n in names:
        got[n].fill_(3.0)
    g = PL.GraphStep(plan.launch, warmup=0)
    for n in names:
        got[n].fill_(5.0)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    for n in names:
        assert _eq(got[n], eager[n]), n
    plan.close()


def test_openness_plan_matches_the_eager_call(mods):
    m = mods
    OP, PL, loop = m["OP"], m["PL"], m["loop"]
    d = _dem(m, 520, 610, 21)
    v = m["A"].as_device_f32_2d(d)
    tiles = loop.make_tiles(loop.tile_grid(520, 610, 256, 64), pixel_scale_x=5.0, pixel_scale_y=-5.0)
    op = OP.make_params(max_distance=48, pixel_size=5.0)
    eager = torch.empty_like(d)
    OP.run_openness(v, tiles, op, None, eager)
    got = torch.full_like(d, 1.0)
    plan = PL.openness_plan(v, tiles, op, None, got)
    g = PL.GraphStep(plan.launch)
    got.fill_(2.0)
    g.replay()
    torch.cuda.synchronize()
    assert _eq(got, eager)


def test_topousm_plan_and_graph_match_the_eager_call(mods):
    m = mods
    TU, S, PL, loop = m["TU"], m["S"], m["PL"], m["loop"]
    H, W = 600, 700
    d = _dem(m, H, W, 31)
    v = m["A"].as_device_f32_2d(d)
    radii, weights = [2, 8, 32, 128], [8 / 15, 4 / 15, 2 / 15, 1 / 15]
    tiles = loop.make_tiles(loop.tile_grid(H, W, 256, 160), pixel_scale_x=10.0, pixel_scale_y=-10.0)
    cd = TU.overview(d, (H // 4, W // 4))
    field = TU.compute_topousm_fast_large_coarse_field(cd, large_radii=[512], large_weights=[0.1], decimation=4.0)
    tp, keep = TU.make_params(radii, weights, 10.0, coarse=field, w_large=0.1, full_shape=(H, W), scale=37.0)
    eager = torch.empty_like(d)
    TU.run_topousm(v, tiles, tp, S.make_plane(eager))
    got = torch.full_like(d, 9.0)
    plan = PL.topousm_plan(v, tiles, tp, S.make_plane(got), keep=keep)
    plan.launch()
    torch.cuda.synchronize()
    assert _eq(got, eager)
    g = PL.GraphStep(plan.launch, warmup=0)
    got.fill_(4.0)
    g.replay()
    torch.cuda.synchronize()
    assert _eq(got, eager)


def test_batched_pyramid_matches_the_per_level_tile_loop(mods, tmp_path):
    m = mods
    loop = m["loop"]
    from fujishadergpu_gb300.core.autotune import Autotuner
    from fujishadergpu_gb300.core.batch import BatchConfig, BatchedTiles
    H, W = 1024, 1536
    d = _dem(m, H, W, 41)
    T6 = (1.0 / 3600.0, 0.0, 135.0, 0.0, -(45.0 - 30.0) / H, 45.0)
    sizes = {"hillshade": [512, 256, 256], "topousm_fast": [1024, 512, 256], "openness": [512, 256, 256]}
    cfg = BatchConfig(levels=3, topousm_radii=(2, 8, 32, 128, 512), openness_distance=40, tile_sizes=sizes)
    b = BatchedTiles(d, T6, config=cfg, tuner=Autotuner(path=str(tmp_path / "t.json")))
    b.step()
    torch.cuda.synchronize()
    eager = {k: v.clone() for k, v in b.outputs.items()}
    for v in b.outputs.values():
        v.fill_(0.5)
    b.capture()
    for v in b.outputs.values():
        v.fill_(0.25)
    b.replay()
    torch.cuda.synchronize()
    for k in eager:  # the atlas columns right of levels 1 and 2 belong to no level
        for L in b.pyr.levels:
            sl = (slice(L.row0, L.row0 + L.h), slice(0, L.w))
            assert _eq(b.outputs[k][sl], eager[k][sl]), (k, L.index)
    w = b._topousm_weights()
    for L in b.pyr.levels:
        lv = b.pyr.level_view(L).contiguous()
        T = L.transform
        ref = loop.process_dem_array(lv, "hillshade", tile_size=sizes["hillshade"][L.index], pixel_size=L.pixel_size_m(),
                                     transform=T, geographic=True, mode="local").output
        got = b.outputs["hillshade"][L.row0:L.row0 + L.h, :L.w]
        assert torch.allclose(got.nan_to_num(-9.0), ref.nan_to_num(-9.0), atol=1e-6, rtol=0), ("hillshade", L.index)
        ref = loop.process_dem_array(lv, "topousm_fast", tile_size=sizes["topousm_fast"][L.index],
                                     pixel_size=L.pixel_size_m(), radii=list(cfg.topousm_radii), weights=w).output
        got = b.outputs["topousm_fast"][L.row0:L.row0 + L.h, :L.w]
        assert _eq(got, ref), ("topousm_fast", L.index)
        # openness raw degrees of the same tiles, eager
        _, tiles = __import__("fujishadergpu_gb300.core.batch", fromlist=["level_tiles"]).level_tiles(
            type(L)(L.index, L.factor, 0, L.h, L.w, L.transform), sizes["openness"][L.index], 40 + 32)
        raw = torch.empty_like(lv)
        op = m["OP"].make_params(max_distance=40, pixel_size=L.pixel_size_m())
        m["OP"].run_openness(m["A"].as_device_f32_2d(lv), tiles, op, None, raw)
        got = b.outputs["openness"][L.row0:L.row0 + L.h, :L.w]
        assert _eq(got, raw), ("openness", L.index)
    b.close()


def test_autotuned_batch_picks_candidate_sizes(mods, tmp_path):
    m = mods
    from fujishadergpu_gb300.core.autotune import Autotuner
    from fujishadergpu_gb300.core.batch import BatchConfig, BatchedTiles
    H, W = 768, 1024
    d = _dem(m, H, W, 51)
    T6 = (1.0 / 3600.0, 0.0, 135.0, 0.0, -(15.0) / H, 45.0)
    path = str(tmp_path / "tune.json")
    cfg = BatchConfig(levels=2, products=("hillshade", "openness"), openness_distance=24, candidates=(256, 512),
                      sample=512)
    b = BatchedTiles(d, T6, config=cfg, tuner=Autotuner(path=path, enabled=True))
    for prod, sizes in b.tile_sizes.items():
        assert len(sizes) == 2 and all(s in (256, 512) for s in sizes), (prod, sizes)
    b.step()
    torch.cuda.synchronize()
    import json
    data = json.load(open(path))
    assert len(data) == 4 and all(set(v["costs"]) <= {"256", "512"} for v in data.values())
    b.close()
