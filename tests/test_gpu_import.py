"""Imported scenes on the GPU.  The textured Cornell box is exported as XML
+ OBJ + MTL + PNG and imported again (Importer::import); its render must
match the oracle's render of the imported SceneData at equal seeds.  The
CRayli-style command-line renderer (craystal_gb300/cpp/crayli.cpp, built
against include/craystal.hpp) must write the EXR film that the Python
binding of the same C ABI produces.  relMSE = mean((I - R)^2 / (R^2 + 1e-2))."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from craystal_gb300 import scenes
from craystal_gb300.api import Image, Importer, PathTraceIntegrator, flatten_scene

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def rel_mse(a, b):
    a = np.nan_to_num(np.asarray(a, np.float64))
    b = np.nan_to_num(np.asarray(b, np.float64))
    return float(np.mean((a - b) ** 2 / (b ** 2 + 1e-2)))


def exported(tmp_path, res=40):
    data, cam = scenes.textured_cornell_box(seed=3, width=res, height=res)
    return scenes.export_obj_scene(data, cam, str(tmp_path / "cornell.xml"))


def test_imported_scene_renders_like_the_oracle(gpu_lib, tmp_path):
    xml = exported(tmp_path)
    sc = Importer().import_(xml)
    data, cam = Importer().load(xml)
    integ = PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05), compat=False)
    integ.dispatch(sc, 32)
    img = sc.getCamera().sensor.createImage()
    oc = oracle.make_camera(cam.posW, cam.target, cam.up, cam.fovY, 40, 40)
    (rgb, w), _ = oracle.OracleScene(flatten_scene(data)).render(oc, 8, 0.05, True, spp=32)
    assert rel_mse(img, rgb / w[..., None]) < 2e-3
    assert sc.n_tris == 36


def test_crayli_cli_writes_the_film(gpu_lib, tmp_path):
    from craystal_gb300 import _lib
    xml = exported(tmp_path, res=32)
    exe = tmp_path / "crayli"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "craystal_gb300", "cpp", "crayli.cpp"), "-L", libdir, "-lcraystal_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = tmp_path / "craystal.exr"
    r = subprocess.run([str(exe), xml, "--spp", "8", "--out", str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    cli = Image.load(str(out)).data
    sc = Importer().import_(xml)
    PathTraceIntegrator().dispatch(sc, 8)  # the reference's effective configuration, as the CLI uses
    ref_path = str(tmp_path / "py.exr")
    Image(data=np.nan_to_num(sc.getCamera().sensor.createImage())).writeEXR(ref_path)
    py = Image.load(ref_path).data
    assert cli.shape == (32, 32, 3)
    # same samples; float atomics may order the film sums differently
    np.testing.assert_allclose(cli, py, rtol=4e-3, atol=1e-4)
    bad = subprocess.run([str(exe), str(tmp_path / "missing.xml")], capture_output=True, text=True, timeout=60)
    assert bad.returncode == 1 and "cannot read" in bad.stderr or "Invalid XML" in bad.stderr
