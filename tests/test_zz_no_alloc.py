"""cr_trace_closest_noalloc: the closest-hit query for callers that cannot let
a library allocate GPU memory (a host whose GPU memory is already committed
to its own pool, a thread that must not stall on the synchronisation
cudaMalloc / cudaFree imply).  It stages rays and hits in a fixed area of the
library's device image instead of allocating.

Checked through the C ABI against cr_trace_closest, bit for bit (the
tolerance every hit comparison in this suite uses), on two calls in a row
with different rays; batches above CR_NOALLOC_MAX_RAYS are refused with a
message.  Each no-allocation call is bracketed on its own: the device's
stream-ordered pool must see no allocation (its used-memory high-water mark,
reset before the call, stays 0), and after the first call, which may make the
driver load the staging area, free device memory must not move.  Collected
last (zz) so that a failure here cannot hide the other tests; it also passes
alone in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CU_MEMPOOL_ATTR_USED_MEM_HIGH = 8  # cuda.h, CUmemPool_attribute


class _CurrentPool:
    """The device's current memory pool (where cudaMallocAsync allocates),
    through the driver API."""

    def __init__(self, ordinal=0):
        self.cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int()
        assert self.cu.cuDeviceGet(ctypes.byref(dev), ordinal) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetMemPool(ctypes.byref(self.pool), dev) == 0

    def reset_high(self):
        zero = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, ctypes.byref(zero)) == 0

    def used_high(self):
        v = ctypes.c_uint64()
        assert self.cu.cuMemPoolGetAttribute(self.pool, CU_MEMPOOL_ATTR_USED_MEM_HIGH, ctypes.byref(v)) == 0
        return v.value


def test_noalloc_matches_allocating_entry_point(gpu_lib):
    import torch

    import craystal_gb300 as cg
    from craystal_gb300 import _lib, scenes

    lib = _lib.load()
    sc = cg.Scene(scenes.random_triangle_scene(100000, seed=31))
    pool = _CurrentPool(0)
    for call, seed in enumerate((32, 33)):
        rays = scenes.random_rays(50000, seed=seed)
        ref = sc.trace_closest(rays)  # existing, allocating entry point
        hits = np.zeros(len(rays), cg.HIT_DTYPE)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        pool.reset_high()
        rc = lib.cr_trace_closest_noalloc(sc.handle, _lib.ptr(rays), len(rays), _lib.ptr(hits), None)
        torch.cuda.synchronize()
        assert rc == 0, lib.cr_last_error().decode()
        assert pool.used_high() == 0, "the no-allocation call made a stream-ordered allocation"
        if call > 0:
            assert torch.cuda.mem_get_info()[0] == free_before, "the no-allocation call allocated device memory"
        assert np.array_equal(hits.view(np.uint32), ref.view(np.uint32)), f"call {call} differs"
        assert (hits["prim"] != cg.CR_MISS).mean() > 0.5


def test_noalloc_rejects_oversized_batches(gpu_lib):
    import craystal_gb300 as cg
    from craystal_gb300 import _lib, scenes

    lib = _lib.load()
    sc = cg.Scene(scenes.random_triangle_scene(1000, seed=34))
    n = _lib.CR_NOALLOC_MAX_RAYS + 1
    rays = scenes.random_rays(n, seed=35)
    hits = np.zeros(n, cg.HIT_DTYPE)
    rc = lib.cr_trace_closest_noalloc(sc.handle, _lib.ptr(rays), n, _lib.ptr(hits), None)
    assert rc == _lib.CR_ERR_INVALID_ARGUMENT
    assert b"at most 65536 rays" in lib.cr_last_error()
    assert not hits.view(np.uint32).any()
    # an empty batch is accepted
    assert lib.cr_trace_closest_noalloc(sc.handle, _lib.ptr(rays), 0, _lib.ptr(hits), None) == 0
