"""Diffuse textures on the GPU: TextureView::sample (Core/Texture.cu:15-35)
bit-exact against the oracle at coordinates inside, on and beyond the edges;
and a render of the textured Cornell box against the oracle at equal seeds
(relMSE = mean((I - R)^2 / (R^2 + 1e-2)))."""
import numpy as np
import pytest

import oracle
from craystal_gb300 import scenes
from craystal_gb300.api import PathTraceIntegrator, Scene, flatten_scene

pytestmark = pytest.mark.gpu


def rel_mse(a, b):
    a = np.nan_to_num(np.asarray(a, np.float64))
    b = np.nan_to_num(np.asarray(b, np.float64))
    return float(np.mean((a - b) ** 2 / (b ** 2 + 1e-2)))


def test_texture_sample_bit_exact(gpu_lib):
    data, _ = scenes.textured_cornell_box(width=8, height=8, tex_res=37)
    sc = Scene(data)
    osc = oracle.OracleScene(flatten_scene(data))
    rng = np.random.default_rng(5)
    uv = np.concatenate([rng.uniform(-0.5, 1.5, (20000, 2)), rng.uniform(0, 1, (20000, 2)),
                         [[0, 0], [1, 1], [1, 0], [0, 1], [np.nan, 0.5], [1e30, -1e30]]]).astype(np.float32)
    for t in range(2):
        np.testing.assert_array_equal(sc.texture_sample(t, uv), osc.texture_sample(t, uv))


def test_textured_render_vs_oracle(gpu_lib):
    data, cam = scenes.textured_cornell_box(seed=2, width=48, height=48)
    sc = Scene(data)
    sc.setCamera(cam)
    integ = PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05), compat=False)
    integ.dispatch(sc, 32)
    img = cam.sensor.createImage()
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, 48, 48)
    (rgb, w), _ = oracle.OracleScene(flatten_scene(data)).render(oc, 8, 0.05, True, spp=32)
    ref = rgb / w[..., None]
    assert rel_mse(img, ref) < 2e-3
    # the textures show: the grey box turns coloured (channel means differ)
    plain, pcam = scenes.cornell_box(seed=2, width=48, height=48)
    ps = Scene(plain)
    ps.setCamera(pcam)
    integ.dispatch(ps, 32)
    tm = np.nanmean(img, axis=(0, 1))
    pm = np.nanmean(pcam.sensor.createImage(), axis=(0, 1))
    assert tm.max() / tm.min() > 1.1 and pm.max() / pm.min() < 1.02


def test_texture_errors(gpu_lib):
    from craystal_gb300._lib import CrayError
    data, _ = scenes.textured_cornell_box(width=8, height=8)
    sc = Scene(data)
    with pytest.raises(CrayError):
        sc.texture_sample(5, np.zeros((1, 2), np.float32))
    with pytest.raises(CrayError):
        sc.set_diffuse_textures([np.zeros((0, 4, 4), np.float32)], [0] * len(data.materials))
    with pytest.raises(CrayError):
        sc.set_diffuse_textures([np.zeros((2, 2, 4), np.float32)], [3] * len(data.materials))
