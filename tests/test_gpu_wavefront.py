"""The wavefront integrator (CR_RENDER_WAVEFRONT: extend, counting sort by
material, shade per bounce) traces the same paths as the megakernel
(CR_RENDER_MEGAKERNEL) with the same arithmetic and sampler sequence: films
equal up to the order of the float atomics, ray counts exactly equal.
Covered: MIS on and off, spectral mode, spheres + textures + an
environment, a wave large enough for the large-wave grids, max depth 0,
the automatic choice, and a wavefront render captured in a CUDA graph."""
import numpy as np
import pytest

from craystal_gb300 import scenes
from craystal_gb300.api import MaterialData, PathTraceIntegrator, Scene, SphereData

pytestmark = pytest.mark.gpu


def film_of(sc, integ, spp, first=0):
    sc.film_clear()
    integ.dispatch(sc, spp, first_sample=first, readback=False)
    rgb, w = sc.film_read()
    return rgb.copy(), w.copy(), sc.render_ray_count()


def compare(sc, depth=8, mis=True, spectral=False, spp=16, first=3):
    cfg = PathTraceIntegrator.Configs(maxDepth=depth, rrThreshold=0.05, useMIS=mis)
    mega = film_of(sc, PathTraceIntegrator(cfg, compat=False, spectral=spectral, wavefront=False), spp, first)
    wave = film_of(sc, PathTraceIntegrator(cfg, compat=False, spectral=spectral, wavefront=True), spp, first)
    np.testing.assert_allclose(wave[1], mega[1], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(wave[0], mega[0], rtol=2e-4, atol=2e-4)
    assert wave[2] == mega[2]
    return mega


@pytest.mark.parametrize("mis,spectral", [(True, False), (False, False), (True, True)])
def test_wavefront_equals_megakernel_cornell(gpu_lib, mis, spectral):
    data, cam = scenes.cornell_box(seed=5, width=64, height=48)
    sc = Scene(data)
    sc.setCamera(cam)
    compare(sc, mis=mis, spectral=spectral)


def test_wavefront_spheres_textures_environment(gpu_lib):
    data, cam = scenes.textured_cornell_box(seed=6, width=48, height=48)
    m = MaterialData(diffuseRefl=(0.3, 0.6, 0.9))
    m.finalize()
    data.materials.append(m)
    data.spheres = [SphereData((0.3, -0.6, 0.2), 0.35, len(data.materials) - 1)]
    sc = Scene(data)
    sc.setCamera(cam)
    sc.set_environment((0.2, 0.25, 0.3))
    compare(sc, depth=12)


def test_wavefront_several_waves_and_depth_zero(gpu_lib):
    data, cam = scenes.cornell_box(seed=7, width=2048, height=2048)
    sc = Scene(data)
    sc.setCamera(cam)
    # 37.7 M paths in one wave: its bounces run the large-wave grids (the shade
    # stage's blocks take chunks from a counter, the sort kernels stride)
    compare(sc, spp=9)
    rgb, w, rays = compare(sc, depth=0, spp=2)
    assert rays == 0 and w.sum() > 0 and not rgb.any()


def test_auto_schedule_and_graph_capture(gpu_lib):
    import ctypes

    import torch

    from craystal_gb300._lib import CrIntegratorConfig, check, load
    data, cam = scenes.cornell_box(seed=8, width=128, height=128)
    sc = Scene(data)
    sc.setCamera(cam)
    cfg = PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05)
    ref = film_of(sc, PathTraceIntegrator(cfg, compat=False, wavefront=False), 8)
    auto = film_of(sc, PathTraceIntegrator(cfg, compat=False), 8)  # 131,072 paths: the wavefront
    np.testing.assert_allclose(auto[0], ref[0], rtol=2e-4, atol=2e-4)
    # the wavefront schedule records into a CUDA graph and replays the same samples
    lib = load()
    c = CrIntegratorConfig(8, 0.05, 1, 2)
    s = torch.cuda.Stream()
    sc.film_clear()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        check(lib.cr_render(sc.handle, ctypes.byref(c), 8, 0, ctypes.c_void_p(s.cuda_stream)))
    sc.film_clear()
    torch.cuda.synchronize()
    g.replay()
    torch.cuda.synchronize()
    rgb, w = sc.film_read()
    np.testing.assert_allclose(w, ref[1], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(rgb, ref[0], rtol=2e-4, atol=2e-4)
    with pytest.raises(Exception):
        check(lib.cr_render(sc.handle, ctypes.byref(CrIntegratorConfig(8, 0.05, 1, 6)), 1, 0, None))


def test_wavefront_two_waves(gpu_lib):
    """More paths than one wave holds (2048^2 x 17 spp = 71.3M > 2^26): the
    render runs as two waves, and its film equals the sum of two renders of
    9 and 8 spp (one wave each) over the same sample indices."""
    data, cam = scenes.cornell_box(seed=8, width=2048, height=2048)
    sc = Scene(data)
    sc.setCamera(cam)
    cfg = PathTraceIntegrator.Configs(maxDepth=6, rrThreshold=0.05, useMIS=True)
    integ = PathTraceIntegrator(cfg, compat=False, wavefront=True)
    whole = film_of(sc, integ, 17, first=11)
    a = film_of(sc, integ, 9, first=11)
    b = film_of(sc, integ, 8, first=20)
    np.testing.assert_allclose(whole[1], a[1] + b[1], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(whole[0], a[0] + b[0], rtol=2e-4, atol=2e-4)
    assert whole[2] == a[2] + b[2]
