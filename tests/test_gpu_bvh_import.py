"""cr_scene_bvh_import: a tree in the reference's BVHData layout
(Core/BVH.h:17-30, as BVH::createFinalBVH fills it, Core/BVH.cu:303-338)
replaces the scene's own, and queries traverse it in the reference's order.

- The oracle's tree (the reference's host build, its leaves in the order
  std::partition leaves them): hits equal the oracle's bit for bit, exact-t
  ties included, since the same tree is visited in the same order.
- A median-split tree the SAH builder would not make: closest t equals brute
  force, and export returns the imported tree.
- A chain tree at the stack's depth limit traverses without overflow; one
  level deeper is refused, as are malformed trees, and a refused import
  leaves the scene's tree in place."""
import numpy as np
import pytest

import craystal_gb300 as cg
import oracle
from craystal_gb300 import _lib, scenes
from craystal_gb300._lib import BVH_NODE_DTYPE
from craystal_gb300.api import MaterialData, MeshData, Scene, SceneData, flatten_scene

pytestmark = pytest.mark.gpu

MISS = 0xFFFFFFFF


def test_import_oracle_tree_bit_exact_with_ties(gpu_lib):
    data = scenes.random_triangle_scene(200000, seed=51)
    g = Scene(data)
    o = oracle.OracleScene(flatten_scene(data))
    nodes, pmap = o.bvh_export()
    g.bvh_import(nodes, pmap)
    st, ost = g.bvh_stats(), o.bvh_stats()
    for k in ("node_count", "leaf_count", "max_depth", "max_leaf_size"):
        assert st[k] == ost[k], k
    # export gives back the imported tree, node for node
    gn, gmap = g.bvh_export()
    assert np.array_equal(gn.view(np.uint8), nodes.view(np.uint8))
    assert np.array_equal(gmap, pmap)
    rays = scenes.random_rays(1 << 19, seed=52)
    gh = g.trace_closest(rays)
    oh, ties = o.trace_closest(rays)
    assert (oh["prim"] != MISS).mean() > 0.5
    # the same tree in the same order: every ray equal, tie rays included
    assert np.array_equal(gh["prim"], oh["prim"])
    hit = oh["prim"] != MISS
    for k in ("t", "u", "v"):
        assert np.array_equal(gh[k][hit].view(np.uint32), oh[k][hit].view(np.uint32)), k
    assert np.array_equal(g.trace_occluded(rays), o.trace_occluded(rays))


def _median_tree(tri):
    """Nodes (post-order, root last) and slot map of a median-split tree over
    the triangles tri (n x 3 x 3): split the centroids at the median of the
    widest axis, leaves of at most 3."""
    cen = tri.mean(axis=1)
    nodes, pmap = [], []

    def rec(ids):
        lo = tri[ids].reshape(-1, 3).min(axis=0)
        hi = tri[ids].reshape(-1, 3).max(axis=0)
        if len(ids) <= 3:
            nodes.append((lo, hi, 1, len(pmap), len(ids)))
            pmap.extend(ids.tolist())
            return len(nodes) - 1
        c = cen[ids]
        ax = int(np.argmax(c.max(axis=0) - c.min(axis=0)))
        srt = ids[np.argsort(c[:, ax], kind="stable")]
        a = rec(srt[: len(srt) // 2])
        b = rec(srt[len(srt) // 2:])
        nodes.append((lo, hi, 0, a, b))
        return len(nodes) - 1

    rec(np.arange(len(tri)))
    out = np.zeros(len(nodes), BVH_NODE_DTYPE)
    for i, (lo, hi, leaf, a, b) in enumerate(nodes):
        out[i] = (lo, hi, leaf, a, b)
    return out, np.asarray(pmap, np.uint32)


def test_import_median_split_tree_vs_brute_force(gpu_lib):
    data = scenes.random_triangle_scene(20000, seed=53)
    flat = flatten_scene(data)
    tri = flat["pos"][flat["idx"].reshape(-1, 3)]
    nodes, pmap = _median_tree(tri)
    g = Scene(data)
    g.bvh_import(nodes, pmap)
    gn, gmap = g.bvh_export()
    assert np.array_equal(gn.view(np.uint8), nodes.view(np.uint8)) and np.array_equal(gmap, pmap)
    rays = scenes.random_rays(100000, seed=54)
    gh = g.trace_closest(rays)
    brute = oracle.OracleScene(flat).trace_brute(rays)
    hit = brute["prim"] != MISS
    assert hit.mean() > 0.5
    assert np.array_equal(gh["prim"] != MISS, hit)
    # closest t bit for bit; where two triangles share that t either may be reported
    same_t = gh["t"].view(np.uint32) == brute["t"].view(np.uint32)
    assert same_t.all(), np.flatnonzero(~same_t)[:5]
    assert (gh["prim"] == brute["prim"]).mean() > 0.9999


def _chain_scene(n):
    """n unit triangles in the planes x = 0 .. n-1 and a chain tree over them:
    interior node k (depth k) has triangle k as its left leaf and the rest
    as its right subtree, so its deepest interior node has depth n - 2."""
    pos = []
    for i in range(n):
        pos += [[i, -1, -1], [i, 1, -1], [i, 0, 1]]
    pos = np.asarray(pos, np.float32)
    data = SceneData(meshes=[MeshData(position=pos, index=np.arange(len(pos), dtype=np.uint32))],
                     materials=[MaterialData()])
    nodes = []

    def leaf(i):
        nodes.append(((i, -1, -1), (i, 1, 1), 1, i, 1))
        return len(nodes) - 1

    def rec(i):
        if i == n - 2:
            a, b = leaf(i), leaf(i + 1)
        else:
            a, b = leaf(i), rec(i + 1)
        nodes.append(((i, -1, -1), (n - 1, 1, 1), 0, a, b))
        return len(nodes) - 1

    rec(0)
    out = np.zeros(len(nodes), BVH_NODE_DTYPE)
    for k, (lo, hi, lf, a, b) in enumerate(nodes):
        out[k] = (lo, hi, lf, a, b)
    return data, out, np.arange(n, dtype=np.uint32)


def test_chain_tree_at_stack_limit(gpu_lib):
    """Rays from +x visit the right (nearer) subtree first and push every
    left leaf: the deepest interior node (depth 31) makes the 32nd push."""
    data, nodes, pmap = _chain_scene(33)
    g = Scene(data)
    g.bvh_import(nodes, pmap)
    assert g.bvh_stats()["max_depth"] == 31
    rays = np.zeros(64, _lib.RAY_DTYPE)
    rng = np.random.default_rng(55)
    rays["o"] = np.c_[np.full(64, 100.0), rng.uniform(-0.3, 0.3, (64, 2))]
    rays["d"] = (-1.0, 0.0, 0.0)
    rays["tmax"] = np.inf
    h = g.trace_closest(rays)  # raises CR_ERR_DEVICE if the stack overflowed
    assert (h["prim"] == 32).all()
    assert np.array_equal(h["t"], np.full(64, 68.0, np.float32))
    # from -x the near leaf comes first and nothing deep is pushed
    rays["o"][:, 0], rays["d"] = -100.0, (1.0, 0.0, 0.0)
    assert (g.trace_closest(rays)["prim"] == 0).all()


def test_refused_imports_keep_the_tree(gpu_lib):
    data, nodes, pmap = _chain_scene(34)  # deepest interior node at depth 32
    g = Scene(data)
    rays = scenes.random_rays(1000, seed=56)
    before = g.trace_closest(rays)
    lib = _lib.load()

    def attempt(nd, pm, code):
        nd = np.ascontiguousarray(nd, BVH_NODE_DTYPE)
        pm = np.ascontiguousarray(pm, np.uint32)
        assert lib.cr_scene_bvh_import(g.handle, _lib.ptr(nd), len(nd), _lib.ptr(pm)) == code
        return lib.cr_last_error().decode()

    assert "depth 32" in attempt(nodes, pmap, _lib.CR_ERR_UNSUPPORTED)
    bad = nodes.copy()
    bad[-1]["b"] = len(bad)  # child out of range
    assert "child" in attempt(bad, pmap, _lib.CR_ERR_INVALID_ARGUMENT)
    bad = nodes.copy()
    bad[-1]["b"] = bad[-1]["a"]  # a node reached twice
    assert "twice" in attempt(bad, pmap, _lib.CR_ERR_INVALID_ARGUMENT)
    bad = nodes.copy()
    bad[0]["b"] = 40  # a leaf past the slots
    attempt(bad, pmap, _lib.CR_ERR_INVALID_ARGUMENT)
    assert "not a triangle" in attempt(nodes, np.full(34, 99, np.uint32), _lib.CR_ERR_INVALID_ARGUMENT)
    _, shallow, _ = _chain_scene(33)
    unreached = np.concatenate([shallow[:1], shallow])  # node 0 is nobody's child
    unreached["a"][unreached["is_leaf"] == 0] += 1
    unreached["b"][unreached["is_leaf"] == 0] += 1
    assert "not reached" in attempt(unreached, pmap, _lib.CR_ERR_INVALID_ARGUMENT)
    after = g.trace_closest(rays)
    assert np.array_equal(before.view(np.uint32), after.view(np.uint32))
    st = g.bvh_stats()
    assert st["build_ms"] > 0  # still the built tree
    with pytest.raises(ValueError):
        g.bvh_import(nodes, pmap[:10])
    with pytest.raises(cg.CrayError):
        g.bvh_import(nodes, pmap)
