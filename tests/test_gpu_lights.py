"""The lights beyond the reference (constant environment, sphere lights) on
the GPU against the oracle's restatement of the same extension, at equal
seed, on a small version of the radiance-cache scene (displaced icospheres,
Principled materials, no emissive triangles).  relMSE tolerance as for the
reference path's renders."""
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


@pytest.mark.parametrize("spectral", [False, True])
def test_environment_and_sphere_light_equal_seed(gpu_lib, spectral):
    data, cam, env, spheres = scenes.cache_scene(seed=0, width=64, height=36, level=2)
    sc = Scene(data)
    sc.setCamera(cam)
    sc.set_environment(env)
    sc.set_sphere_lights(spheres)
    PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=16, rrThreshold=0.05), compat=False,
                        spectral=spectral).dispatch(sc, 16)
    img = cam.sensor.createImage()
    osc = oracle.OracleScene(flatten_scene(data))
    osc.set_lights(env, spheres)
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, 64, 36)
    (rgb, w), _ = osc.render(oc, 16, 0.05, True, spp=16, spectral=spectral)
    ref = rgb / w[..., None]
    assert np.nanmean(ref) > 0.05  # the lights reach the film
    assert rel_mse(img, ref) < 2e-3


def test_sphere_light_hit_and_occlusion(gpu_lib):
    """A sphere light seen directly has its emission in the image, and it
    casts a shadow on the ground (it occludes the environment)."""
    data, cam, env, spheres = scenes.cache_scene(seed=0, width=48, height=27, level=1)
    cam.setTarget(spheres[0][0])  # look at the light
    sc = Scene(data)
    sc.setCamera(cam)
    sc.set_sphere_lights(spheres)
    PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=2), compat=False).dispatch(sc, 4)
    img = cam.sensor.createImage()
    assert np.nanmax(img) > 10.0  # emission (40, 38, 34) at the image centre
