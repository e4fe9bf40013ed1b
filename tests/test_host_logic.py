"""Host-side logic of the facade: scene flattening (TriangleMeshManager,
Scene/Triangle.cu:98-131), MaterialData::finalize, the integrator's
effective configuration, and the synthetic workloads."""
import numpy as np

from craystal_gb300 import scenes
from craystal_gb300.api import (MaterialData, MaterialType, MeshData, PathTraceIntegrator, SceneData,
                                flatten_scene)


def test_flatten_rebases_indices_and_fills_mesh_descs():
    a = MeshData(position=np.zeros((4, 3)), index=np.array([0, 1, 2, 0, 2, 3]), materialID=1)
    b = MeshData(position=np.ones((3, 3)), index=np.array([0, 1, 2]), materialID=0)
    f = flatten_scene(SceneData(meshes=[a, b], materials=[MaterialData(), MaterialData()]))
    assert f["pos"].shape == (7, 3) and f["idx"].dtype == np.uint32
    assert list(f["idx"]) == [0, 1, 2, 0, 2, 3, 4, 5, 6]
    assert list(f["meshes"]["index_offset"]) == [0, 6]
    assert list(f["meshes"]["index_count"]) == [6, 3]
    assert list(f["meshes"]["vertex_offset"]) == [0, 4]
    assert list(f["meshes"]["material_id"]) == [1, 0]
    assert f["nrm"].shape == (7, 3) and f["uv"].shape == (7, 2)


def test_material_finalize_flags():
    m = MaterialData(emission=(0.0, 2.0, 0.0))
    m.finalize()
    assert m.flags == 3  # emissive, and no specular -> diffuse
    m = MaterialData(specularRefl=(0.1, 0, 0), type=MaterialType.Phong)
    m.finalize()
    assert m.flags == 0


def test_integrator_compat_config():
    cfg = PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.15, useMIS=False)
    c = PathTraceIntegrator(cfg).device_config()
    # the reference's device view keeps its defaults (Core/Integrator.h:20-23)
    assert (c.max_depth, round(c.rr_threshold, 6), c.use_mis) == (10, 0.05, 0)
    c = PathTraceIntegrator(cfg, compat=False).device_config()
    assert (c.max_depth, round(c.rr_threshold, 6), c.use_mis) == (8, 0.15, 0)


def test_cornell_box_shape():
    data, cam = scenes.cornell_box(seed=0)
    f = flatten_scene(data)
    assert len(f["idx"]) // 3 == 36
    assert list(data.emissiveIndex) == [34, 35]
    assert sum(1 for m in data.materials if m.isEmissive()) == 1
    assert cam.fovY == 40.0 and cam.sensor.size == (256, 256)
    f2 = flatten_scene(scenes.cornell_box(seed=0)[0])
    assert np.array_equal(f["pos"], f2["pos"])
    # every wall and box triangle faces the inside / outside consistently
    p = f["pos"][f["idx"].reshape(-1, 3)]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    assert (np.linalg.norm(n, axis=1) > 0).all()


def test_random_workloads_are_seeded():
    p1, i1 = scenes.random_triangles(1000, seed=3)
    p2, _ = scenes.random_triangles(1000, seed=3)
    assert np.array_equal(p1, p2) and len(i1) == 3000
    r = scenes.random_rays(1000, seed=4)
    assert np.allclose(np.linalg.norm(r["o"], axis=1), 2.0, atol=1e-5)
    assert np.allclose(np.linalg.norm(r["d"], axis=1), 1.0, atol=1e-5)
    assert (r["tmin"] == np.float32(1e-4)).all() and np.isinf(r["tmax"]).all()
