"""Batched rendering (cr_batch_*): many scenes of uneven size from captured
CUDA graphs, on the persistent megakernel or the many-scene wavefront.
Each scene's film must equal what cr_render adds for the same sample
indices (float-atomic summation order aside), successive replays must
advance the sample indices, and the autotuner must time every tuning and
leave the films cleared."""
import numpy as np
import pytest

from craystal_gb300 import scenes
from craystal_gb300.api import BatchRenderer, PathTraceIntegrator, Scene

pytestmark = pytest.mark.gpu


def make_batch(n=5):
    params = [{"seed": 10 + i, "tris": [2000, 30000, 500, 9000, 60000][i % 5], "res": [64, 96, 40, 128, 72][i % 5],
               "spp": [3, 8, 1, 5, 2][i % 5], "depth": [8, 12, 16, 9, 10][i % 5]} for i in range(n)]
    scs, integs = [], []
    for p in params:
        data, cam = scenes.box_clutter(p["seed"], p["tris"], p["res"], p["res"])
        sc = Scene(data)
        sc.setCamera(cam)
        scs.append(sc)
        integs.append(PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=p["depth"], rrThreshold=0.05),
                                          compat=False, spectral=(p["seed"] % 3 == 0)))
    return params, scs, integs


@pytest.mark.parametrize("tile,run,wave", [(16, 4, 0), (8, 1, 0), (8, 16, 0), (16, 4, 16), (16, 4, 20)])
def test_batch_equals_per_scene_renders(gpu_lib, tile, run, wave):
    params, scs, integs = make_batch()
    b = BatchRenderer(scs, integs, [p["spp"] for p in params], first_sample=[7] * len(params))
    b.set_tuning(tile, run, wave_log2=wave)
    b.render()
    batch = [sc.film_read() for sc in scs]
    rays = [sc.render_ray_count() for sc in scs]
    for sc, integ, p, (rgb, w), r in zip(scs, integs, params, batch, rays):
        sc.film_clear()
        integ.dispatch(sc, p["spp"], first_sample=7, readback=False)
        rgb2, w2 = sc.film_read()
        np.testing.assert_allclose(w, w2, rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(rgb, rgb2, rtol=1e-4, atol=1e-5)
        assert sc.render_ray_count() == r


def test_batch_large_shared_wave(gpu_lib):
    """Three 512x512 scenes at 4 spp share one wave of 3.1M paths (wave_log2
    22): a wave that large finishes its tail in one launch once few paths
    are live; each film still equals the scene's own render (1M paths, a
    wave that keeps its bounce-by-bounce tail), and so do the ray counts."""
    params, scs, integs = [], [], []
    for i, depth in enumerate((8, 12, 16)):
        data, cam = scenes.box_clutter(40 + i, 20000, 512, 512)
        sc = Scene(data)
        sc.setCamera(cam)
        scs.append(sc)
        integs.append(PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=depth, rrThreshold=0.05), compat=False))
    b = BatchRenderer(scs, integs, [4] * 3, first_sample=[5] * 3)
    b.set_tuning(16, 4, wave_log2=22)
    b.render()
    batch = [sc.film_read() for sc in scs]
    rays = [sc.render_ray_count() for sc in scs]
    for sc, integ, (rgb, w), r in zip(scs, integs, batch, rays):
        sc.film_clear()
        integ.dispatch(sc, 4, first_sample=5, readback=False)
        rgb2, w2 = sc.film_read()
        np.testing.assert_allclose(w, w2, rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(rgb, rgb2, rtol=1e-4, atol=1e-5)
        assert sc.render_ray_count() == r


@pytest.mark.parametrize("wave", [0, 17])
def test_batch_replays_advance_samples(gpu_lib, wave):
    params, scs, integs = make_batch(3)
    b = BatchRenderer(scs, integs, [p["spp"] for p in params])
    b.set_tuning(8, 2, wave_log2=wave)
    b.render()
    w1 = [sc.film_read()[1].copy() for sc in scs]
    b.render()  # sample indices spp .. 2*spp - 1
    for sc, integ, p, a in zip(scs, integs, params, w1):
        w2 = sc.film_read()[1]
        sc.film_clear()
        integ.dispatch(sc, 2 * p["spp"], readback=False)
        np.testing.assert_allclose(w2, sc.film_read()[1], rtol=1e-5, atol=1e-6)


def test_autotune_times_every_tuning_and_clears(gpu_lib, tmp_path):
    params, scs, integs = make_batch(4)
    b = BatchRenderer(scs, integs, [p["spp"] for p in params])
    out = b.autotune(json_path=str(tmp_path / "tuning.json"))
    assert len(out["timings_ms"]) == 15
    best = min(out["timings_ms"], key=lambda r: r["ms"])
    assert out["best"] == {"tile": best["tile"], "spp_per_item": best["spp_per_item"], "wave_log2": best["wave_log2"]}
    assert b.tuning()["wave_log2"] == best["wave_log2"]
    for sc in scs:
        rgb, w = sc.film_read()
        assert not w.any() and sc.render_ray_count() == 0
    assert (tmp_path / "tuning.json").exists()


def make_cached_batch(n=4):
    """RGB scenes (the cache learns RGB) of uneven size, depth and spp."""
    params, scs, integs = make_batch(n)
    integs = [PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=p["depth"], rrThreshold=0.05), compat=False)
              for p in params]
    return params, scs, integs


@pytest.mark.parametrize("freeze", [True, False])
def test_batch_cached_equals_per_scene_cached(gpu_lib, freeze):
    """cr_batch_render_cached against cr_render_cached scene by scene, each
    scene with its own network of the same seed: frozen networks give the
    same films, queries and records (float-atomic order aside); trained ones
    the same training sequence, so films agree to the float-order noise the
    updates pick up (relMSE < 1e-3)."""
    from craystal_gb300.api import CachedPathTraceIntegrator, RadianceCache
    params, scs, integs = make_cached_batch()
    spp = [p["spp"] + 2 for p in params]
    b = BatchRenderer(scs, integs, spp, first_sample=[7] * len(params))
    stats = b.render_cached([RadianceCache(seed=40 + i) for i in range(len(scs))], train_every=4, freeze=freeze)
    batch = [sc.film_read() for sc in scs]
    for i, (sc, integ, (rgb, w)) in enumerate(zip(scs, integs, batch)):
        sc.film_clear()
        single = CachedPathTraceIntegrator(integ.configs, train_every=4, cache=RadianceCache(seed=40 + i))
        single.dispatch(sc, spp[i], first_sample=7, readback=False, freeze=freeze)
        rgb2, w2 = sc.film_read()
        np.testing.assert_allclose(w, w2, rtol=1e-5, atol=1e-6)
        assert stats[i]["frames"] == spp[i] == single.stats.frames
        assert stats[i]["queries"] == single.stats.queries and stats[i]["train_records"] == single.stats.train_records
        if freeze:
            np.testing.assert_allclose(rgb, rgb2, rtol=1e-4, atol=1e-5)
        else:
            a = np.nan_to_num(rgb / w[..., None])
            c = np.nan_to_num(rgb2 / w2[..., None])
            assert float(np.mean((a - c) ** 2 / (c ** 2 + 1e-2))) < 1e-3


def test_batch_cached_training_paths_equal_plain(gpu_lib):
    """With every pixel a training path, each scene's cached film is its own
    plain render (cr_render, the same sample indices)."""
    from craystal_gb300.api import RadianceCache
    params, scs, integs = make_cached_batch(3)
    b = BatchRenderer(scs, integs, [p["spp"] for p in params], first_sample=[3] * len(params))
    stats = b.render_cached([RadianceCache(seed=i) for i in range(len(scs))], train_every=1)
    batch = [sc.film_read() for sc in scs]
    for sc, integ, p, (rgb, w), st in zip(scs, integs, params, batch, stats):
        sc.film_clear()
        integ.dispatch(sc, p["spp"], first_sample=3, readback=False)
        rgb2, w2 = sc.film_read()
        np.testing.assert_allclose(w, w2, rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(rgb, rgb2, rtol=1e-4, atol=1e-5)
        assert st["queries"] == 0 and st["train_records"] > 0
