"""The oracle's spheres: SphereSOA::intersect (Scene/Sphere.cu:6-52) known
answers (entry and exit roots, the tMin / tMax window, the (u, v) of the
hit normal) and the order of SceneView::intersect (Scene/Scene.cu:5-14):
spheres first, so a triangle at exactly the same distance does not replace
a sphere, and of equal spheres the lower index wins."""
import numpy as np

import oracle
from craystal_gb300 import scenes
from craystal_gb300._lib import CR_MISS, CR_SPHERE_BIT, RAY_DTYPE
from craystal_gb300.api import MaterialData, MeshData, SceneData, SphereData, flatten_scene


def rays(o, d, tmin=0.0, tmax=np.inf):
    r = np.zeros(len(o), RAY_DTYPE)
    r["o"], r["d"], r["tmin"], r["tmax"] = o, d, tmin, tmax
    return r


def scene(spheres, tris=None):
    m = MaterialData(diffuseRefl=(0.5, 0.5, 0.5))
    m.finalize()
    meshes = []
    if tris is not None:
        pos = np.asarray(tris, np.float32).reshape(-1, 3)
        meshes.append(MeshData(position=pos, index=np.arange(len(pos), dtype=np.uint32)))
    return oracle.OracleScene(flatten_scene(SceneData(meshes=meshes, materials=[m], spheres=spheres)))


def test_sphere_roots_window_and_uv():
    o = scene([SphereData((0, 0, 0), 1.0, 0)])
    r = rays([[0, 0, 5], [0, 0, 0], [0, 0, 5], [0, 0, 5], [3, 0, 5]],
             [[0, 0, -1], [0, 0, -1], [0, 0, -1], [0, 0, -1], [0, 0, -1]],
             tmin=[0, 0, 4.5, 0, 0], tmax=[np.inf, np.inf, np.inf, 3.9, np.inf])
    h, _ = o.trace_closest(r)
    assert h["prim"].tolist() == [CR_SPHERE_BIT, CR_SPHERE_BIT, CR_SPHERE_BIT, CR_MISS, CR_MISS]
    # entry at 4, from inside the exit at 1, tMin past the entry gives the exit 6
    assert h["t"][:3].tolist() == [4.0, 1.0, 6.0]
    # normal (0, 0, 1): theta = pi/2, phi = atan2(-1, 0) + pi = pi/2 -> (0.25, 0.5)
    np.testing.assert_allclose([h["u"][0], h["v"][0]], [0.25, 0.5], atol=1e-7)
    # exit point normal (0, 0, -1): phi = atan2(1, 0) + pi = 3pi/2 -> u = 0.75
    np.testing.assert_allclose([h["u"][1], h["v"][1]], [0.75, 0.5], atol=1e-7)
    occ = o.trace_occluded(r)
    assert occ.tolist() == [1, 1, 1, 0, 0]


def test_spheres_before_triangles_and_lower_index_first():
    # a triangle in the plane z = 1 touching the front of the sphere at the ray's hit point
    tri = [[-1, -1, 1], [1, -1, 1], [0, 1, 1]]
    o = scene([SphereData((0, 0, 0), 1.0, 0), SphereData((0, 0, 0), 1.0, 0)], tris=tri)
    h, ties = o.trace_closest(rays([[0, 0, 5]], [[0, 0, -1]]))
    assert h["prim"][0] == CR_SPHERE_BIT and h["t"][0] == 4.0 and ties[0]
