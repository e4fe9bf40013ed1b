"""Analytic spheres on the GPU (SphereSOA::intersect, Scene/Sphere.cu:6-52,
in a BVH of their own) against the oracle's linear sphere loop: closest
hits (prim and t bit-exact; u, v from acosf / atan2f within 1e-6), any-hit
occlusion, and renders of the Cornell box with diffuse, textured Phong and
emissive spheres at equal seeds (relMSE = mean((I - R)^2 / (R^2 + 1e-2)))."""
import numpy as np
import pytest

import oracle
from craystal_gb300 import scenes
from craystal_gb300._lib import CR_SPHERE_BIT, CrayError
from craystal_gb300.api import (MaterialData, MaterialFlags, MaterialType, PathTraceIntegrator, Scene, SphereData,
                                flatten_scene)

pytestmark = pytest.mark.gpu


def rel_mse(a, b):
    a = np.nan_to_num(np.asarray(a, np.float64))
    b = np.nan_to_num(np.asarray(b, np.float64))
    return float(np.mean((a - b) ** 2 / (b ** 2 + 1e-2)))


def sphere_soup(n_tris=20000, n_sph=20000, seed=9):
    data = scenes.random_triangle_scene(n_tris, seed)
    rng = np.random.default_rng(seed)
    c = rng.random((n_sph, 3))
    r = rng.uniform(0.001, 0.02, n_sph)
    r[:50] = 0.005  # some identical spheres: ties broken by index
    c[25:50] = c[:25]
    data.spheres = [SphereData(tuple(ci), float(ri), 0) for ci, ri in zip(c, r)]
    return data


def test_sphere_queries_match_oracle(gpu_lib):
    data = sphere_soup()
    sc = Scene(data)
    osc = oracle.OracleScene(flatten_scene(data))
    rays = scenes.random_rays(200000, seed=10)
    gh = sc.trace_closest(rays)
    oh, ties = osc.trace_closest(rays)
    same = (gh["prim"] == oh["prim"]) & (gh["t"].view(np.uint32) == oh["t"].view(np.uint32))
    assert (same | ties).all(), int((~(same | ties)).sum())
    sph = (oh["prim"] & CR_SPHERE_BIT).astype(bool) & (oh["prim"] != 0xFFFFFFFF) & ~ties
    assert sph.sum() > 1000
    np.testing.assert_allclose(gh["u"][sph], oh["u"][sph], atol=1e-6)
    np.testing.assert_allclose(gh["v"][sph], oh["v"][sph], atol=1e-6)
    tri = ~sph & (oh["prim"] != 0xFFFFFFFF) & ~ties
    assert (gh["u"][tri].view(np.uint32) == oh["u"][tri].view(np.uint32)).all()
    r2 = rays.copy()
    r2["tmax"] = np.random.default_rng(11).uniform(0.01, 1.5, len(r2)).astype(np.float32)
    np.testing.assert_array_equal(sc.trace_occluded(r2), osc.trace_occluded(r2))
    # the persistent kernel's per-block ray ranges (the form of the entry point
    # that allocates nothing) give the same hits on a sphere scene
    from craystal_gb300 import _lib
    few = rays[: _lib.CR_NOALLOC_MAX_RAYS]
    na = np.zeros(len(few), gh.dtype)
    assert _lib.load().cr_trace_closest_noalloc(sc.handle, _lib.ptr(few), len(few), _lib.ptr(na), None) == 0
    assert np.array_equal(na.view(np.uint32), gh[: len(few)].view(np.uint32))


def cornell_with_spheres(res=48):
    data, cam = scenes.textured_cornell_box(seed=4, width=res, height=res)
    red = MaterialData(diffuseRefl=(0.8, 0.2, 0.2), type=MaterialType.FullDiffuse)
    tex = MaterialData(diffuseRefl=(1, 1, 1), specularRefl=(0.2, 0.2, 0.2), shininess=30.0, type=MaterialType.Phong,
                       flags=int(MaterialFlags.hasDiffuseTexture), diffuseHandle=0)
    lamp = MaterialData(emission=(4.0, 3.0, 2.0))
    for m in (red, tex, lamp):
        m.finalize()
    base = len(data.materials)
    data.materials += [red, tex, lamp]
    data.spheres = [SphereData((-0.45, -0.65, 0.35), 0.3, base), SphereData((0.45, -0.7, 0.5), 0.28, base + 1),
                    SphereData((0.0, 0.55, -0.4), 0.12, base + 2)]
    return data, cam


def test_render_with_spheres_vs_oracle(gpu_lib):
    data, cam = cornell_with_spheres()
    sc = Scene(data)
    sc.setCamera(cam)
    PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05), compat=False).dispatch(sc, 32)
    img = cam.sensor.createImage()
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, 48, 48)
    (rgb, w), _ = oracle.OracleScene(flatten_scene(data)).render(oc, 8, 0.05, True, spp=32)
    ref = rgb / w[..., None]
    assert rel_mse(img, ref) < 2e-3
    # the spheres show: the image differs from the box without them
    plain, pcam = scenes.textured_cornell_box(seed=4, width=48, height=48)
    ps = Scene(plain)
    ps.setCamera(pcam)
    PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05), compat=False).dispatch(ps, 32)
    assert rel_mse(img, pcam.sensor.createImage()) > 10 * rel_mse(img, ref)


def test_sphere_errors(gpu_lib):
    data, _ = cornell_with_spheres(8)
    sc = Scene(data)
    with pytest.raises(CrayError):
        sc.set_spheres([[0, 0, 0, -1.0]], [0])
    with pytest.raises(CrayError):
        sc.set_spheres([[0, 0, 0, 1.0]], [len(data.materials)])
    sc.set_spheres(np.zeros((0, 4)), [])  # removing all spheres is allowed
