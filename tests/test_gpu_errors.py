"""The scene's device error word: a kernel that detects an error (a traversal
stack that would overflow) sets a bit instead of failing, and the host
reports it as CR_ERR_DEVICE, where the reference would throw
(Core/Error.h:113-124).  Each error must be reported exactly once: the word
is cleared when a call reports it, so later calls on the scene succeed.

The error is raised from the host (cr_scene_set_error_flags), as a kernel
would raise it: no kernel is made to fail."""
import ctypes

import numpy as np
import pytest

import craystal_gb300 as cg
from craystal_gb300 import _lib, scenes
from craystal_gb300.api import PathTraceIntegrator, Scene

pytestmark = pytest.mark.gpu


def _raise(sc, flags=_lib.CR_DEVICE_ERROR_STACK_OVERFLOW):
    _lib.check(_lib.load().cr_scene_set_error_flags(sc.handle, flags))


def test_host_query_reports_once(gpu_lib):
    sc = Scene(scenes.random_triangle_scene(5000, seed=41))
    rays = scenes.random_rays(20000, seed=42)
    ref = sc.trace_closest(rays)
    _raise(sc)
    with pytest.raises(cg.CrayError) as e:
        sc.trace_closest(rays)
    assert e.value.code == _lib.CR_ERR_DEVICE and "stack overflow" in str(e.value)
    # reported once: the next calls succeed with the same hits
    for _ in range(2):
        assert np.array_equal(sc.trace_closest(rays).view(np.uint32), ref.view(np.uint32))
    assert sc.check_errors() == 0


def test_check_errors_reports_device_entry_points(gpu_lib):
    import torch
    sc = Scene(scenes.random_triangle_scene(5000, seed=43))
    rays = scenes.random_rays(4096, seed=44)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.empty(len(rays) * 16, dtype=torch.uint8, device="cuda")
    _raise(sc)
    # a device-buffer query returns before its kernel runs and reports nothing
    sc.trace_closest_device(d_rays.data_ptr(), len(rays), d_hits.data_ptr(), 0)
    flags = ctypes.c_uint32()
    lib = _lib.load()
    assert lib.cr_scene_check_errors(sc.handle, ctypes.byref(flags)) == _lib.CR_ERR_DEVICE
    assert flags.value == _lib.CR_DEVICE_ERROR_STACK_OVERFLOW
    assert lib.cr_scene_check_errors(sc.handle, ctypes.byref(flags)) == _lib.CR_OK
    assert flags.value == 0
    hits = d_hits.cpu().numpy().view(cg.HIT_DTYPE)
    assert np.array_equal(hits.view(np.uint32), sc.trace_closest(rays).view(np.uint32))


def test_film_read_reports_once(gpu_lib):
    data, cam = scenes.cornell_box(width=32, height=32)
    sc = Scene(data)
    sc.setCamera(cam)
    PathTraceIntegrator().dispatch(sc, 2, readback=False)
    _raise(sc, 0x10)
    with pytest.raises(cg.CrayError) as e:
        sc.film_read()
    assert e.value.code == _lib.CR_ERR_DEVICE and "0x10" in str(e.value)
    rgb, w = sc.film_read()
    assert w.sum() > 0


def test_noalloc_reports_once(gpu_lib):
    lib = _lib.load()
    sc = Scene(scenes.random_triangle_scene(5000, seed=45))
    rays = scenes.random_rays(1000, seed=46)
    hits = np.zeros(len(rays), cg.HIT_DTYPE)
    _raise(sc)
    assert lib.cr_trace_closest_noalloc(sc.handle, _lib.ptr(rays), len(rays), _lib.ptr(hits), None) == \
        _lib.CR_ERR_DEVICE
    assert lib.cr_trace_closest_noalloc(sc.handle, _lib.ptr(rays), len(rays), _lib.ptr(hits), None) == _lib.CR_OK
    assert np.array_equal(hits.view(np.uint32), sc.trace_closest(rays).view(np.uint32))
