"""The restated reference kernels (the comparators bench.py times) must do
the reference's work: on the reference-layout tree the product exports, the
restated traversal's closest hits equal the oracle's up to the last bits
that FMA contraction changes (the reference's CUDA build contracts; the
oracle does not), and the restated path tracer renders the product's image
(same estimator and sample indices; FMA contraction makes paths diverge
now and then, so the films agree statistically) with about the same rays."""
import numpy as np
import pytest

import oracle
from craystal_gb300 import scenes
from craystal_gb300._lib import HIT_DTYPE, RAY_DTYPE
from craystal_gb300.api import Scene, flatten_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_tris", [1, 5000, 200000])
def test_restated_reference_matches_oracle(gpu_lib, n_tris):
    import torch
    from baseline.restated import RestatedTraversal
    data = scenes.random_triangle_scene(n_tris, seed=21)
    flat = flatten_scene(data)
    sc = Scene(data)
    rays = scenes.random_rays(100000, seed=22)
    ref = RestatedTraversal(sc, flat)
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.empty(len(rays) * 16, dtype=torch.uint8, device="cuda")
    ref.trace_closest_device(d_rays.data_ptr(), len(rays), d_hits.data_ptr())
    torch.cuda.synchronize()
    got = d_hits.cpu().numpy().view(HIT_DTYPE)
    want, ties = oracle.OracleScene(flat).trace_closest(rays)
    same_prim = (got["prim"] == want["prim"]) | ties
    assert same_prim.mean() > 0.9995, same_prim.mean()
    both = (got["prim"] == want["prim"]) & (want["prim"] != 0xFFFFFFFF)
    np.testing.assert_allclose(got["t"][both], want["t"][both], rtol=1e-4)
    assert RAY_DTYPE.itemsize == 32


def test_restated_path_tracer_renders_the_same_image(gpu_lib):
    from baseline.restated import RestatedPathTracer
    from craystal_gb300.api import PathTraceIntegrator
    data, cam = scenes.cornell_box(seed=3, width=48, height=48)
    sc = Scene(data)
    sc.setCamera(cam)
    (rgb, w), rays = RestatedPathTracer(sc, flatten_scene(data)).render(cam, 64, max_depth=8, rr_threshold=0.05)
    sc.film_clear()
    PathTraceIntegrator(PathTraceIntegrator.Configs(maxDepth=8, rrThreshold=0.05), compat=False).dispatch(sc, 64)
    ours = cam.sensor.createImage()
    ref = rgb / w[..., None]
    err = float(np.mean((np.nan_to_num(ref) - np.nan_to_num(ours)) ** 2 / (np.nan_to_num(ours) ** 2 + 1e-2)))
    assert err < 2e-3, err
    assert abs(rays / sc.render_ray_count() - 1.0) < 0.02
