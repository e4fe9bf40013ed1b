"""GPU parity of the BVH build and the ray queries against the CPU oracle.

Contract: the GPU builder produces the reference's tree (same topology and
boxes, bit for bit), and closest hits (prim, t, u, v) equal the
reference's on identical FP32 rays bit for bit.  The one allowed
difference is which of two triangles hit at exactly the same t in the same
leaf is reported; the oracle flags those rays ("ties") and they are counted
and bounded, not ignored silently."""
import numpy as np
import pytest

import oracle
from craystal_gb300 import scenes
from craystal_gb300.api import Scene, flatten_scene

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF


def both(data):
    return Scene(data), oracle.OracleScene(flatten_scene(data))


def assert_same_tree(gpu: Scene, orc):
    gn, gmap = gpu.bvh_export()
    on, omap = orc.bvh_export()
    assert len(gn) == len(on)
    assert np.array_equal(gn["is_leaf"], on["is_leaf"])
    assert np.array_equal(gn["bmin"].view(np.uint32), on["bmin"].view(np.uint32))
    assert np.array_equal(gn["bmax"].view(np.uint32), on["bmax"].view(np.uint32))
    assert np.array_equal(gn["a"], on["a"]) and np.array_equal(gn["b"], on["b"])
    for nd in gn[gn["is_leaf"] == 1]:
        s, c = nd["a"], nd["b"]
        assert sorted(gmap[s:s + c]) == sorted(omap[s:s + c])
    gs, os_ = gpu.bvh_stats(), orc.bvh_stats()
    for k in ("node_count", "leaf_count", "max_depth", "max_leaf_size"):
        assert gs[k] == os_[k], k


def assert_same_hits(gh, oh, ties, max_tie_frac=1e-4):
    ok = (gh["prim"] == oh["prim"])
    hit = oh["prim"] != MISS
    ok &= ~hit | (gh["t"].view(np.uint32) == oh["t"].view(np.uint32))
    ok &= ~hit | (gh["u"].view(np.uint32) == oh["u"].view(np.uint32))
    ok &= ~hit | (gh["v"].view(np.uint32) == oh["v"].view(np.uint32))
    bad = ~ok & ~ties
    assert not bad.any(), f"{bad.sum()} rays differ, first {np.flatnonzero(bad)[:5]}"
    assert ties.mean() <= max_tie_frac
    # tie rays still agree on t
    assert np.array_equal(gh["t"][ties].view(np.uint32), oh["t"][ties].view(np.uint32))


@pytest.mark.parametrize("n", [1, 4, 5, 37, 2048, 2049, 30000, 200000])
def test_bvh_matches_reference_build(gpu_lib, n):
    g, o = both(scenes.random_triangle_scene(n, seed=n))
    assert_same_tree(g, o)


def test_bvh_cornell_flat_boxes(gpu_lib):
    g, o = both(scenes.cornell_box()[0])
    assert_same_tree(g, o)


def test_bvh_coincident_centroids(gpu_lib):
    """Every triangle with the same centroid: the split fails (one side
    empty) and the node becomes a leaf holding everything."""
    pos = np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), (50, 1))
    from craystal_gb300.api import MaterialData, MeshData, SceneData
    data = SceneData(meshes=[MeshData(position=pos, index=np.arange(150, dtype=np.uint32))],
                     materials=[MaterialData()])
    g, o = both(data)
    assert_same_tree(g, o)
    assert g.bvh_stats()["leaf_count"] == 1


def test_closest_hits_bit_exact(gpu_lib):
    g, o = both(scenes.random_triangle_scene(200000, seed=21))
    rays = scenes.random_rays(1 << 20, seed=22)
    gh = g.trace_closest(rays)
    oh, ties = o.trace_closest(rays)
    assert (oh["prim"] != MISS).mean() > 0.5
    assert_same_hits(gh, oh, ties)


def _star_cluster(n, centre, rng):
    """n triangles of random orientations and sizes that share one centroid:
    no split separates them, so the builder makes one leaf of n.  Vertex
    offsets are multiples of 2^-7, so ((v0 + v1) + v2) / 3 is the same float
    for every triangle."""
    a = rng.integers(-12, 13, (n, 3)).astype(np.float32) / 128.0
    b = rng.integers(-12, 13, (n, 3)).astype(np.float32) / 128.0
    c = np.asarray(centre, np.float32)
    tri = np.stack([c + a, c + b, c - a - b], axis=1)
    return tri.reshape(-1, 3).astype(np.float32)


@pytest.mark.parametrize("size", [7, 8, 150])
@pytest.mark.parametrize("with_others", [False, True])
def test_closest_hits_large_leaves(gpu_lib, with_others, size):
    """A leaf of up to 7 slots carries its range in the child ref; a larger one
    keeps it in the leaf table.  Leaves of 7, 8 and 150 coincident-centroid
    triangles, as the root and below interior nodes among 3000 other
    triangles, hit bit-exactly."""
    from craystal_gb300.api import MaterialData, MeshData, SceneData
    rng = np.random.default_rng(31)
    pos = _star_cluster(size, (0.5, 0.5, 0.5), rng)
    if with_others:
        pos = np.concatenate([pos, scenes.random_triangles(3000, seed=32)[0]]).astype(np.float32)
    data = SceneData(meshes=[MeshData(position=pos, index=np.arange(len(pos), dtype=np.uint32))],
                     materials=[MaterialData()])
    g, o = both(data)
    assert_same_tree(g, o)
    st = g.bvh_stats()
    assert st["max_leaf_size"] == size
    assert (st["leaf_count"] == 1) == (not with_others)
    rays = scenes.random_rays(200000, seed=33)
    gh = g.trace_closest(rays)
    oh, ties = o.trace_closest(rays)
    cluster = (oh["prim"] != MISS) & (oh["prim"] < size)
    assert cluster.sum() > 100
    assert_same_hits(gh, oh, ties, max_tie_frac=1e-3)
    assert np.array_equal(g.trace_occluded(rays), o.trace_occluded(rays))


def test_device_and_host_entry_points_agree(gpu_lib):
    import torch
    g, _ = both(scenes.random_triangle_scene(20000, seed=23))
    rays = scenes.random_rays(100000, seed=24)
    host = g.trace_closest(rays)
    dr = torch.from_numpy(rays.view(np.uint8)).cuda()
    dh = torch.empty(len(rays) * 16, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    g.trace_closest_device(dr.data_ptr(), len(rays), dh.data_ptr(), s.cuda_stream)
    s.synchronize()
    dev = dh.cpu().numpy().view(host.dtype)
    assert np.array_equal(dev.view(np.uint32), host.view(np.uint32))


def test_pinned_host_buffers_used_in_place(gpu_lib):
    """Page-locked host buffers (a pinned torch tensor) are read and written
    by the GPU in place; pageable ones go through staging copies.  Both give
    the device path's hits and occlusion flags, also for a range that starts
    inside its allocation and for a ray count that spans several chunks."""
    import ctypes
    import torch
    from craystal_gb300._lib import check, load
    lib = load()
    g, o = both(scenes.random_triangle_scene(20000, seed=41))
    n = (1 << 21) + 1000  # more than one 2^21-ray staging chunk
    rays = scenes.random_rays(n, seed=42)
    rays["tmax"][::3] = np.float32(1.5)
    host = g.trace_closest(rays)  # pageable: staged
    occ_host = g.trace_occluded(rays)
    pin_r = torch.empty(n * 32 + 64, dtype=torch.uint8).pin_memory()
    pin_h = torch.empty(n * 16 + 64, dtype=torch.uint8).pin_memory()
    pin_o = torch.empty(n + 64, dtype=torch.uint8).pin_memory()
    for off in (0, 32):  # 16-byte aligned starts inside the allocation
        pin_r.numpy()[off:off + n * 32] = rays.view(np.uint8)
        pin_h.zero_()
        rp = ctypes.c_void_p(pin_r.data_ptr() + off)
        check(lib.cr_trace_closest(g.handle, rp, n, ctypes.c_void_p(pin_h.data_ptr() + off)))
        got = pin_h.numpy()[off:off + n * 16].copy().view(host.dtype)
        assert np.array_equal(got.view(np.uint32), host.view(np.uint32))
        pin_o.fill_(7)
        check(lib.cr_trace_occluded(g.handle, rp, n, ctypes.c_void_p(pin_o.data_ptr() + off)))
        assert np.array_equal(pin_o.numpy()[off:off + n], occ_host)
    oh, ties = o.trace_closest(rays[:200000])
    assert_same_hits(host[:200000], oh, ties)


def test_occlusion_exact(gpu_lib):
    g, o = both(scenes.random_triangle_scene(50000, seed=25))
    rays = scenes.random_rays(300000, seed=26)
    rays["tmax"] = np.random.default_rng(1).uniform(0.2, 3.5, len(rays)).astype(np.float32)
    assert np.array_equal(g.trace_occluded(rays), o.trace_occluded(rays))


def test_edge_cases(gpu_lib):
    # empty scene: everything misses
    from craystal_gb300.api import MaterialData, SceneData
    g = Scene(SceneData(materials=[MaterialData()]))
    h = g.trace_closest(scenes.random_rays(1000))
    assert (h["prim"] == MISS).all() and np.isinf(h["t"]).all()
    assert g.trace_closest(scenes.random_rays(0)).shape == (0,)
    # single triangle (the root is a leaf), rays aimed at it
    pos = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    from craystal_gb300.api import MeshData
    data = SceneData(meshes=[MeshData(position=pos, index=np.arange(3, dtype=np.uint32))], materials=[MaterialData()])
    g, o = both(data)
    rays = scenes.random_rays(5000, seed=27)
    aim = np.random.default_rng(2).random((5000, 3)).astype(np.float32) * np.float32([0.7, 0.7, 0])
    d = aim - rays["o"]
    rays["d"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    gh = g.trace_closest(rays)
    oh, ties = o.trace_closest(rays)
    assert (oh["prim"] == 0).mean() > 0.5
    assert_same_hits(gh, oh, ties, 0.0)


def test_cornell_axis_parallel_rays(gpu_lib):
    """Flat boxes (degenerate slabs), axis-parallel directions (zero
    components, infinite inverse direction), ray windows [tmin, tmax]."""
    g, o = both(scenes.cornell_box()[0])
    rng = np.random.default_rng(3)
    rays = scenes.random_rays(200000, seed=28)
    rays["o"] *= np.float32(0.45)
    d = rays["d"].copy()
    d[rng.random((len(d), 3)) < 0.3] = 0.0
    d[(d == 0).all(1), 1] = -1.0
    rays["d"] = d
    rays["tmin"] = rng.choice(np.float32([0, 1e-4, 0.5]), len(rays))
    rays["tmax"] = rng.choice(np.float32([np.inf, 1.0, 2.0]), len(rays))
    gh = g.trace_closest(rays)
    oh, ties = o.trace_closest(rays)
    assert_same_hits(gh, oh, ties, 1e-2)
    assert np.array_equal(g.trace_occluded(rays), o.trace_occluded(rays))


def test_full_size_ray_cast(gpu_lib):
    """The ray-cast benchmark at its full size: 1M triangles, 16M rays, every
    hit compared with the oracle."""
    g, o = both(scenes.random_triangle_scene(1 << 20, seed=0))
    assert_same_tree(g, o)
    rays = scenes.random_rays(1 << 24, seed=1)
    gh = g.trace_closest(rays)
    oh, ties = o.trace_closest(rays)
    assert_same_hits(gh, oh, ties)


def _set_two_level(g):
    g.set_traversal("two_level")
    return g


@pytest.mark.parametrize("case", ["random", "large_leaves", "cornell", "spheres"])
def test_two_level_traversal_same_hits(gpu_lib, case):
    """The two-level step (the near child's pair of a group tested in the
    same step) visits the reference's nodes in the reference's order: its
    closest hits equal the one-level step's bit for bit and the oracle's,
    and its occlusion answers are the oracle's, on a random soup, on leaves
    too large for the child ref, on the Cornell box with flat boxes and
    axis-parallel rays, and with analytic spheres in their own tree."""
    rng = np.random.default_rng(7)
    if case == "random":
        data = scenes.random_triangle_scene(100000, seed=50)
        rays = scenes.random_rays(400000, seed=51)
    elif case == "large_leaves":
        from craystal_gb300.api import MaterialData, MeshData, SceneData
        pos = np.concatenate([_star_cluster(150, (0.5, 0.5, 0.5), rng),
                              scenes.random_triangles(3000, seed=52)[0]]).astype(np.float32)
        data = SceneData(meshes=[MeshData(position=pos, index=np.arange(len(pos), dtype=np.uint32))],
                         materials=[MaterialData()])
        rays = scenes.random_rays(200000, seed=53)
    elif case == "cornell":
        data = scenes.cornell_box()[0]
        rays = scenes.random_rays(200000, seed=54)
        rays["o"] *= np.float32(0.45)
        d = rays["d"].copy()
        d[rng.random((len(d), 3)) < 0.3] = 0.0
        d[(d == 0).all(1), 1] = -1.0
        rays["d"] = d
    else:
        from craystal_gb300.api import SphereData
        data = scenes.random_triangle_scene(20000, seed=55)
        c, r = rng.random((300, 3)), rng.uniform(0.005, 0.03, 300)
        data.spheres = [SphereData(tuple(ci), float(ri), 0) for ci, ri in zip(c, r)]
        rays = scenes.random_rays(200000, seed=56)
    g, o = both(data)
    one = g.trace_closest(rays)
    _set_two_level(g)
    two = g.trace_closest(rays)
    assert np.array_equal(one.view(np.uint32), two.view(np.uint32))
    oh, ties = o.trace_closest(rays)
    if case == "spheres":  # sphere (u, v) come from acosf / atan2f: prim and t only
        assert ((two["prim"] == oh["prim"]) | ties).all()
        assert np.array_equal(two["t"].view(np.uint32), oh["t"].view(np.uint32))
        assert (two["prim"] >= 0x80000000).sum() > 1000
    else:
        assert_same_hits(two, oh, ties, 1e-2)
    if case == "random":  # an imported tree gets its grouped copy too
        g.bvh_import(*o.bvh_export())
        assert np.array_equal(g.trace_closest(rays).view(np.uint32), one.view(np.uint32))
    rays["tmax"] = np.float32(1.0)
    occ = o.trace_occluded(rays)
    assert np.array_equal(g.trace_occluded(rays), occ)
    g.set_traversal("one_level")  # frees the grouped copy
    assert np.array_equal(g.trace_occluded(rays), occ)
    with pytest.raises(Exception):
        g.set_traversal("four_level")


@pytest.mark.parametrize("n", [1, 31, 33, 1000, 123457])
def test_dynamic_fetch_sizes(gpu_lib, n):
    """The persistent ray cast hands rays to lanes as they free up; every
    batch size (partial warps, fewer rays than lanes, many rays per block)
    gives the oracle's hits, and the occlusion answers too."""
    g, o = both(scenes.random_triangle_scene(30000, seed=40))
    rays = scenes.random_rays(n, seed=41)
    gh = g.trace_closest(rays)
    oh, ties = o.trace_closest(rays)
    assert_same_hits(gh, oh, ties)
    rays["tmax"] = np.float32(1.5)
    assert np.array_equal(g.trace_occluded(rays), o.trace_occluded(rays))


def test_concurrent_streams_and_graph_capture(gpu_lib):
    """Device-buffer queries on two streams at once (each call has its own
    stream-ordered ray counter), and one captured in a CUDA graph and
    replayed, give the host entry point's hits."""
    import torch
    g, _ = both(scenes.random_triangle_scene(50000, seed=42))
    ra, rb = scenes.random_rays(300000, seed=43), scenes.random_rays(200000, seed=44)
    ha, hb = g.trace_closest(ra), g.trace_closest(rb)
    dra = torch.from_numpy(ra.view(np.uint8)).cuda()
    drb = torch.from_numpy(rb.view(np.uint8)).cuda()
    dha = torch.zeros(len(ra) * 16, dtype=torch.uint8, device="cuda")
    dhb = torch.zeros(len(rb) * 16, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    for _ in range(3):
        g.trace_closest_device(dra.data_ptr(), len(ra), dha.data_ptr(), s1.cuda_stream)
        g.trace_closest_device(drb.data_ptr(), len(rb), dhb.data_ptr(), s2.cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(dha.cpu().numpy().view(np.uint32), ha.view(np.uint32))
    assert np.array_equal(dhb.cpu().numpy().view(np.uint32), hb.view(np.uint32))
    dha.zero_()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        g.trace_closest_device(dra.data_ptr(), len(ra), dha.data_ptr(), torch.cuda.current_stream().cuda_stream)
    graph.replay()
    torch.cuda.synchronize()
    assert np.array_equal(dha.cpu().numpy().view(np.uint32), ha.view(np.uint32))
