"""Hero-wavelength spectral rendering (CR_RENDER_SPECTRAL, an extension of
the RGB reference) on the GPU against the oracle's spectral mode and against
the RGB integrator, which it must equal in expectation on the grey-albedo,
flat-emission Cornell box.  relMSE = mean((I - R)^2 / (R^2 + 1e-2))."""
import numpy as np
import pytest

import oracle
from craystal_gb300 import scenes
from craystal_gb300._lib import CrIntegratorConfig, check, load
from craystal_gb300.api import Scene, flatten_scene

pytestmark = pytest.mark.gpu


def rel_mse(a, b):
    a = np.nan_to_num(np.asarray(a, np.float64))
    b = np.nan_to_num(np.asarray(b, np.float64))
    return float(np.mean((a - b) ** 2 / (b ** 2 + 1e-2)))


def render(sc, spp, first, spectral, depth=8):
    import ctypes
    sc.film_clear()
    cfg = CrIntegratorConfig(depth, 0.05, 1, 1 if spectral else 0)
    check(load().cr_render(sc.handle, ctypes.byref(cfg), spp, first, None))
    rgb, w = sc.film_read()
    return rgb / w[..., None]


def test_spectral_equal_seed_vs_oracle(gpu_lib):
    data, cam = scenes.cornell_box(seed=0, width=48, height=48)
    sc = Scene(data)
    sc.setCamera(cam)
    img = render(sc, 16, 0, True)
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, 48, 48)
    (rgb, w), _ = oracle.OracleScene(flatten_scene(data)).render(oc, 8, 0.05, True, spp=16, spectral=True)
    assert rel_mse(img, rgb / w[..., None]) < 2e-3


def test_spectral_grey_scene_equals_rgb_in_expectation(gpu_lib):
    data, cam = scenes.cornell_box(seed=0, width=64, height=64)
    sc = Scene(data)
    sc.setCamera(cam)
    ref = render(sc, 8192, 500_000, False)
    e_rgb = rel_mse(render(sc, 256, 0, False), ref)
    spec = render(sc, 256, 0, True)
    e_spec = rel_mse(spec, ref)
    # spectral adds colour noise from the wavelength choice, no bias
    assert e_spec < 3.0 * e_rgb, (e_spec, e_rgb)
    # per-channel means within 3 % (colour noise of 256 spp; a wrong white
    # balance or wavelength weight shows as a shift of 10 % or more)
    for ch in range(3):
        assert abs(np.nanmean(spec[..., ch]) / np.nanmean(ref[..., ch]) - 1.0) < 0.03, ch


def test_spectral_colored_differs_from_rgb_but_is_sane(gpu_lib):
    data, cam = scenes.cornell_box(seed=1, width=32, height=32)
    data.materials[3].diffuseRefl = (0.8, 0.1, 0.1)  # a red wall
    data.materials[4].diffuseRefl = (0.1, 0.8, 0.1)  # a green wall
    sc = Scene(data)
    sc.setCamera(cam)
    spec = render(sc, 512, 0, True)
    rgb = render(sc, 512, 0, False)
    assert np.isfinite(spec).all()
    # both keep the red wall red and the green wall green on average
    assert spec[..., 0].mean() > 0 and abs(spec.mean() / rgb.mean() - 1.0) < 0.1
