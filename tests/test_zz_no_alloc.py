"""cr_trace_closest_noalloc: the closest-hit query for callers that cannot let
a library allocate GPU memory (a host whose GPU memory is already committed
to its own pool, a thread that must not stall on the synchronisation
cudaMalloc / cudaFree imply).  It stages rays and hits in a fixed area of the
library's device image instead of allocating.

Checked through the C ABI against cr_trace_closest, bit for bit (the
tolerance every hit comparison in this suite uses), on two calls in a row
with different rays; batches above CR_NOALLOC_MAX_RAYS are refused with a
message.  Collected last (zz) so that a failure here cannot hide the other
tests; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point(gpu_lib):
    import torch

    import craystal_gb300 as cg
    from craystal_gb300 import _lib, scenes

    lib = _lib.load()
    sc = cg.Scene(scenes.random_triangle_scene(100000, seed=31))
    free_after_first = None
    for call, seed in enumerate((32, 33)):
        rays = scenes.random_rays(50000, seed=seed)
        ref = sc.trace_closest(rays)  # existing, allocating entry point
        hits = np.zeros(len(rays), cg.HIT_DTYPE)
        rc = lib.cr_trace_closest_noalloc(sc.handle, _lib.ptr(rays), len(rays), _lib.ptr(hits), None)
        assert rc == 0, lib.cr_last_error().decode()
        assert np.array_equal(hits.view(np.uint32), ref.view(np.uint32)), f"call {call} differs"
        assert (hits["prim"] != cg.CR_MISS).mean() > 0.5
        torch.cuda.synchronize()
        free_now = torch.cuda.mem_get_info()[0]
        if free_after_first is None:
            free_after_first = free_now
        else:
            assert free_now == free_after_first  # the second call allocated nothing


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
