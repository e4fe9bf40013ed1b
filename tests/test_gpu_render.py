"""GPU parity of the integrator's stages and of whole renders against the
CPU oracle.

Tolerances.  Camera rays and the Lambertian BSDF use only +,-,*,/ and sqrt
and are compared bit for bit.  Phong and Principled call pow / acos /
sin / cos, whose CUDA and glibc results may differ in the last ulp, so
they are compared with rtol 2e-5.  Renders at equal seed follow the same
paths until such an ulp difference changes a branch, so images are
compared by relMSE = mean((I - R)^2 / (R^2 + 1e-2)) with the tolerance
written at each check."""
import ctypes

import numpy as np
import pytest

import oracle
from craystal_gb300 import scenes
from craystal_gb300._lib import MATERIAL_DTYPE, RAY_DTYPE, CrCamera, check, load, ptr
from craystal_gb300.api import PathTraceIntegrator, Scene, flatten_scene

pytestmark = pytest.mark.gpu


def rel_mse(img, ref):
    img = np.nan_to_num(np.asarray(img, np.float64))
    ref = np.nan_to_num(np.asarray(ref, np.float64))
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def gpu_camera_rays(pos, target, up, fov, w, h, sp):
    c = CrCamera()
    c.pos[:], c.target[:], c.up[:] = pos, target, up
    c.fov_y, c.width, c.height = fov, w, h
    sp = np.ascontiguousarray(sp, np.float32)
    out = np.empty(len(sp), RAY_DTYPE)
    check(load().cr_camera_generate_rays(ctypes.byref(c), ptr(sp), len(sp), ptr(out)))
    return out


def test_camera_known_answers_on_gpu(gpu_lib):
    r = gpu_camera_rays((0, 0, 0), (0, 0, -1), (0, 1, 0), 60.0, 512, 512, [(256, 256), (0, 0), (511, 511)])
    np.testing.assert_allclose(r["d"][0], (0, 0, -1), atol=1e-5)                                  # CameraTest.cpp:16-24
    np.testing.assert_allclose(r["d"][1], (-0.44721359, 0.44721359, -0.774596691), atol=1e-4)     # :26-37
    np.testing.assert_allclose(r["d"][2], (0.446162969, -0.446162969, -0.77580744), atol=1e-4)    # :39-50


def test_camera_rays_bit_exact(gpu_lib):
    rng = np.random.default_rng(0)
    sp = (rng.random((100000, 2)) * [640, 480]).astype(np.float32)
    args = ((0.5, 1.0, 4.0), (0.1, -0.2, 0.0), (0.0, 1.0, 0.0), 40.0, 640, 480)
    g = gpu_camera_rays(*args, sp)
    o = oracle.camera_rays(oracle.make_camera(*args), sp)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def _material(kind):
    m = np.zeros(1, MATERIAL_DTYPE)
    m["diffuse"] = (0.6, 0.4, 0.3)
    if kind == "phong":
        m["type"], m["specular"], m["shininess"] = 2, (0.2, 0.2, 0.2), 32.0
    elif kind == "principled":
        m["type"], m["specular"], m["shininess"] = 1, (0.3, 0.3, 0.3), 12.0
    return m


def _dirs(rng, n):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def _gpu_bsdf_eval(m, n, wo, wi):
    f = np.empty((len(n), 3), np.float32)
    pdf = np.empty(len(n), np.float32)
    check(load().cr_bsdf_evaluate(ptr(m), ptr(n), ptr(wo), ptr(wi), len(n), ptr(f), ptr(pdf)))
    return f, pdf


def _gpu_bsdf_sample(m, n, wo, u):
    wi = np.empty((len(n), 3), np.float32)
    f = np.empty((len(n), 3), np.float32)
    pdf = np.empty(len(n), np.float32)
    check(load().cr_bsdf_sample(ptr(m), ptr(n), ptr(wo), ptr(u), len(n), ptr(wi), ptr(f), ptr(pdf)))
    return wi, f, pdf


@pytest.mark.parametrize("kind", ["lambert", "phong", "principled"])
def test_bsdf_evaluate(gpu_lib, kind):
    rng = np.random.default_rng(1)
    n, wo, wi = _dirs(rng, 50000), _dirs(rng, 50000), _dirs(rng, 50000)
    m = _material(kind)
    gf, gp = _gpu_bsdf_eval(m, n, wo, wi)
    of, op = oracle.bsdf_eval(m, n, wo, wi)
    if kind == "lambert":
        assert np.array_equal(gf.view(np.uint32), of.view(np.uint32))
        assert np.array_equal(gp.view(np.uint32), op.view(np.uint32))
    else:
        np.testing.assert_allclose(gf, of, rtol=2e-5, atol=1e-7)
        np.testing.assert_allclose(gp, op, rtol=2e-5, atol=1e-7)
    assert (of > 0).any()


@pytest.mark.parametrize("kind", ["lambert", "phong", "principled"])
def test_bsdf_sample(gpu_lib, kind):
    rng = np.random.default_rng(2)
    n, wo = _dirs(rng, 50000), _dirs(rng, 50000)
    u = rng.random((50000, 2)).astype(np.float32)
    m = _material(kind)
    gw, gf, gp = _gpu_bsdf_sample(m, n, wo, u)
    ow, of, op = oracle.bsdf_sample(m, n, wo, u)
    # near the horizon z = sqrt(1 - x^2 - y^2) turns ulp differences of sin / cos
    # into absolute errors of ~1e-6 in z, hence pdf and f (both <= 1/pi * max albedo)
    np.testing.assert_allclose(gw, ow, rtol=0, atol=2e-5)
    np.testing.assert_allclose(gp, op, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(gf, of, rtol=1e-4, atol=1e-5)


def _cornell(w=64, h=64, seed=0):
    data, cam = scenes.cornell_box(seed=seed, width=w, height=h)
    g = Scene(data)
    g.setCamera(cam)
    o = oracle.OracleScene(flatten_scene(data))
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, w, h)
    return g, o, oc, cam


@pytest.mark.parametrize("use_mis", [True, False])
def test_cornell_equal_seed(gpu_lib, use_mis):
    g, o, oc, cam = _cornell()
    integ = PathTraceIntegrator(PathTraceIntegrator.Configs(useMIS=use_mis))  # reference-effective: depth 10, rr 0.05
    integ.dispatch(g, 16)
    img = cam.sensor.createImage()
    (rgb, w), orays = o.render(oc, 10, 0.05, use_mis, spp=16)
    ref = rgb / w[..., None]
    err = rel_mse(img, ref)
    assert err < 1e-3, err  # equal seed: paths agree except after ulp-level divergence
    grays = g.render_ray_count()
    assert abs(grays - orays) <= 0.02 * orays, (grays, orays)
    # film weights: the same jittered positions, so equal up to float summation order
    np.testing.assert_allclose(cam.sensor.weight, w, rtol=1e-5)


def test_cornell_converges_to_fp64_reference(gpu_lib):
    """GPU image at 64 spp vs a 4096-spp oracle image with an FP64 film
    (independent sample indices): its error must be that of the oracle's own
    64-spp image, within 30 %."""
    g, o, oc, cam = _cornell(48, 48)
    (rgb, w), _ = o.render(oc, 10, 0.05, True, spp=4096, first_sample=100000)
    ref = rgb / w[..., None]
    PathTraceIntegrator().dispatch(g, 64)
    e_gpu = rel_mse(cam.sensor.createImage(), ref)
    (rgb2, w2), _ = o.render(oc, 10, 0.05, True, spp=64)
    e_orc = rel_mse(rgb2 / w2[..., None], ref)
    assert e_gpu < 1.3 * e_orc + 1e-5, (e_gpu, e_orc)


def test_principled_scene_equal_seed(gpu_lib):
    data, cam = scenes.cornell_box(seed=3, width=48, height=48)
    from craystal_gb300.api import MaterialType
    for m in data.materials:
        if not m.isEmissive():
            m.type = MaterialType.Principled
            m.specularRefl = (0.3, 0.3, 0.3)
            m.shininess = 20.0
            m.flags = 0
            m.finalize()
    g = Scene(data)
    g.setCamera(cam)
    o = oracle.OracleScene(flatten_scene(data))
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, 48, 48)
    PathTraceIntegrator().dispatch(g, 16)
    (rgb, w), _ = o.render(oc, 10, 0.05, True, spp=16)
    assert rel_mse(cam.sensor.createImage(), rgb / w[..., None]) < 2e-3


def test_film_accumulates_and_clears(gpu_lib):
    g, o, oc, cam = _cornell(32, 32)
    integ = PathTraceIntegrator()
    integ.dispatch(g, 4)
    w1 = cam.sensor.weight.copy()
    # the reference never clears the film and restarts at sample index 0 on
    # every dispatch: a second dispatch adds the same samples again
    integ.dispatch(g, 4)
    assert np.allclose(cam.sensor.weight, 2 * w1, rtol=1e-5)
    integ.dispatch(g, 4, first_sample=4)  # new sample indices: new jitter, more weight
    assert (cam.sensor.weight > 2 * w1).mean() > 0.3
    g.film_clear()
    rgb, w = g.film_read()
    assert not rgb.any() and not w.any()
    resolved = g.film_resolve()
    assert np.isnan(resolved).all()  # 0 / 0, as Sensor::createImage without a guard


@pytest.mark.parametrize("spectral", [False, True])
@pytest.mark.parametrize("wavefront", [True, False])
def test_c1_config_equal_seed(gpu_lib, spectral, wavefront):
    """The plain-method configuration the benchmark renders, exactly: the
    procedural Cornell box (seed 0), 256 x 256, 16 spp, max depth 8, rr 0.05,
    NEE + MIS, RGB and hero-wavelength spectral, on both schedules, against
    the oracle at the same seed.  Equal seeds give the same paths until an
    ulp difference of a transcendental flips a branch, so relMSE stays near
    zero (bars as the smaller equal-seed tests: 1e-3 RGB, 2e-3 spectral);
    ray counts agree within 2 % and film weights (the same jittered filter
    positions) within float summation order."""
    g, o, oc, cam = _cornell(256, 256, seed=0)
    integ = PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05, useMIS=True),
                                compat=False, spectral=spectral, wavefront=wavefront)
    integ.dispatch(g, 16)
    img = cam.sensor.createImage()
    (rgb, w), orays = o.render(oc, 8, 0.05, True, spp=16, spectral=spectral)
    err = rel_mse(img, rgb / w[..., None])
    assert err < (2e-3 if spectral else 1e-3), err
    grays = g.render_ray_count()
    assert abs(grays - orays) <= 0.02 * orays, (grays, orays)
    np.testing.assert_allclose(cam.sensor.weight, w, rtol=1e-5)
