"""The C++ facade (include/craystal.hpp) drives the library the way the
reference's CRayli does: a C++ program is compiled against the header,
linked with libcraystal_gb300.so and run; its image must equal the same
render made through the Python binding of the same C ABI."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_crayli_demo_matches_python_binding(gpu_lib, tmp_path):
    from craystal_gb300 import _lib
    exe = tmp_path / "crayli_demo"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "craystal_gb300", "cpp", "crayli_demo.cpp"), "-L", libdir,
                    "-lcraystal_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = tmp_path / "img.f32"
    r = subprocess.run([str(exe), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    img_cpp = np.fromfile(out, np.float32).reshape(48, 64, 3)

    import craystal_gb300 as cg
    floor = cg.MeshData(position=np.array([[-1, -1, -1], [1, -1, -1], [1, -1, 1], [-1, -1, 1]], np.float32),
                        normal=np.tile(np.float32([0, 1, 0]), (4, 1)), index=np.array([0, 2, 1, 0, 3, 2]),
                        materialID=0)
    light = cg.MeshData(position=np.array([[-0.3, 0.9, -0.3], [0.3, 0.9, -0.3], [0.3, 0.9, 0.3], [-0.3, 0.9, 0.3]],
                                          np.float32),
                        normal=np.tile(np.float32([0, -1, 0]), (4, 1)), index=np.array([0, 1, 2, 0, 2, 3]),
                        materialID=1)
    m0 = cg.MaterialData(diffuseRefl=(0.7, 0.5, 0.3), specularRefl=(0.1, 0.1, 0.1), shininess=16.0,
                         type=cg.MaterialType.Phong)
    m1 = cg.MaterialData(emission=(10.0, 10.0, 10.0))
    m0.finalize()
    m1.finalize()
    sc = cg.Scene(cg.SceneData(meshes=[floor, light], materials=[m0, m1], emissiveIndex=[2, 3]))
    cam = cg.Camera()
    cam.setWorldPosition((0, 0.2, 3))
    cam.setTarget((0, -0.5, 0))
    cam.setUp((0, 1, 0))
    cam.setFovY(45)
    cam.setSensor(cg.Sensor((64, 48)))
    sc.setCamera(cam)
    cg.PathTraceIntegrator().dispatch(sc, 8)
    img_py = cam.sensor.createImage()
    both = np.isfinite(img_py) & np.isfinite(img_cpp)
    assert both.mean() > 0.99
    # identical paths; the film sums may differ in the last bits (float atomics)
    np.testing.assert_allclose(img_cpp[both], img_py[both], rtol=1e-5, atol=1e-6)
