"""Name-based lookup at the boundary: ``ALGORITHMS[name]`` (algorithms/dask_registry.py:27-49)
and ``_load_algorithm(name)`` over ``algorithms/tile/<name>.py``
(core/tile_processor.py:807-820).  The CPU tests check the lookup only; the GPU
test runs every hot-path name through ``process`` and compares it with the
block function the name stands for."""
import numpy as np
import pytest

HOT = ("hillshade", "slope", "curvature", "topousm_fast", "openness", "ambient_occlusion")


def test_every_hot_path_name_resolves():
    from fujishadergpu_gb300.algorithms import ALGORITHMS, DEFAULT_ALGORITHMS, TileAlgorithm
    from fujishadergpu_gb300.core.tile_loop import HOT_PATH_ALGORITHMS, _load_algorithm
    assert set(ALGORITHMS) == set(HOT) == set(HOT_PATH_ALGORITHMS) == set(DEFAULT_ALGORITHMS)
    for name in HOT:
        a = _load_algorithm(name)
        assert isinstance(a, TileAlgorithm)
        assert type(a) is type(ALGORITHMS[name])
        assert type(a).__name__ == DEFAULT_ALGORITHMS[name]
        assert isinstance(a.get_default_params(), dict)
        assert a is not _load_algorithm(name), "the loader returns a new instance per call"


@pytest.mark.parametrize("name", ["specular", "frangi", "no_such_algorithm", ""])
def test_unknown_names_raise_value_error(name):
    from fujishadergpu_gb300.core.tile_loop import _load_algorithm
    with pytest.raises(ValueError, match="not found or not available"):
        _load_algorithm(name)


def test_tile_modules_expose_the_classes():
    import importlib
    from fujishadergpu_gb300.algorithms import DEFAULT_ALGORITHMS
    for name, cls in DEFAULT_ALGORITHMS.items():
        mod = importlib.import_module(f"fujishadergpu_gb300.algorithms.tile.{name}")
        assert hasattr(mod, cls), (name, cls)


@pytest.mark.gpu
def test_every_name_runs_and_matches_its_block_function():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fujishadergpu_gb300 import algorithms as A
    from fujishadergpu_gb300 import synth
    from tests._parity import to_np
    dem = synth.fbm(160, 176, hurst=0.7, seed=21, lo=0.0, hi=1500.0)
    dem[synth.nodata_disks(160, 176, count=2, seed=22, rmin=3.0, rmax=8.0)] = np.nan
    d = torch.from_numpy(dem).cuda()
    kw = dict(pixel_size=5.0, pixel_scale_x=5.0, pixel_scale_y=-5.0)
    expected = {
        "hillshade": lambda: A.compute_hillshade_block(d, **kw),
        "slope": lambda: A.compute_slope_block(d, **kw),
        "curvature": lambda: A.compute_curvature_block(d, curvature_type="mean", **kw),
        "openness": lambda: A.compute_openness_vectorized(d, max_distance=20, **kw),
        "ambient_occlusion": lambda: A.compute_ambient_occlusion_block(d, radius=6.0, **kw),
    }
    params = {"openness": dict(max_distance=20), "ambient_occlusion": dict(radius=6.0),
              "curvature": dict(curvature_type="mean")}
    for name in HOT:
        p = dict(kw, mode="local", **params.get(name, {}))
        if name == "topousm_fast":
            p = dict(kw, radii=[2, 8], weights=[0.5, 0.5], global_stats=(7.0,))
        got = to_np(A.ALGORITHMS[name].process(d, **p))
        assert got.shape == dem.shape, name
        if name == "topousm_fast":
            ref = to_np(A.compute_topousm_fast_efficient_block(d, radii=[2, 8], weights=[0.5, 0.5],
                                                               pixel_size=5.0)) / np.float32(7.0)
            assert np.allclose(got, ref, rtol=0, atol=1e-5, equal_nan=True), name
        else:
            ref = to_np(expected[name]())
            assert np.array_equal(got, ref, equal_nan=True), name
