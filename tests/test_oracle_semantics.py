"""Checks the oracle's arithmetic against an independent numpy float32
restatement (each operation rounded separately, glm's order), and its BVH
build and traversal against brute force and structural invariants."""
import numpy as np
import pytest

import oracle
from craystal_gb300 import scenes
from craystal_gb300.api import flatten_scene

f32 = np.float32


def np_dot(a, b):
    return (a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1]) + a[..., 2] * b[..., 2]


def np_cross(a, b):
    return np.stack([a[..., 1] * b[..., 2] - b[..., 1] * a[..., 2],
                     a[..., 2] * b[..., 0] - b[..., 2] * a[..., 0],
                     a[..., 0] * b[..., 1] - b[..., 0] * a[..., 1]], -1)


def np_mt(v0, v1, v2, o, d, tmin, tmax):
    """Scene/Triangle.cu:40-75 + Scene/Shape.h:26-31 in numpy float32."""
    with np.errstate(all="ignore"):
        e1, e2 = v1 - v0, v2 - v0
        p = np_cross(d, e2)
        det = np_dot(e1, p)
        ok = ~(np.abs(det) < f32(1e-6))
        inv = f32(1.0) / det
        tv = o - v0
        u = np_dot(tv, p) * inv
        ok &= ~((u < 0) | (u > 1))
        q = np_cross(tv, e1)
        v = np_dot(d, q) * inv
        ok &= ~((v < 0) | (u + v > 1))
        t = np_dot(e2, q) * inv
        ok &= ~(t <= 0)
        ok &= ~((t < tmin) | (t > tmax))
    return ok, t, u, v


def test_moller_trumbore_bits():
    rng = np.random.default_rng(5)
    n = 200000
    c = rng.random((n, 3)).astype(f32)
    v0, v1, v2 = (c + rng.normal(0, 0.05, (n, 3)).astype(f32) for _ in range(3))
    rays = scenes.random_rays(n, seed=6)
    aim = (v0 + v1 + v2) / f32(3) + rng.normal(0, 0.02, (n, 3)).astype(f32)  # about half of the rays hit
    d = aim.astype(np.float64) - rays["o"]
    rays["d"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(f32)
    hit, t, u, v = oracle.triangle_intersect(v0, v1, v2, rays)
    ok, tt, uu, vv = np_mt(v0, v1, v2, rays["o"], rays["d"], rays["tmin"], rays["tmax"])
    # the oracle entry point reports the raw Moller-Trumbore result (no range check)
    ok_raw, _, _, _ = np_mt(v0, v1, v2, rays["o"], rays["d"], np.full(n, -np.inf, f32), np.full(n, np.inf, f32))
    assert hit.sum() > 1000
    assert np.array_equal(hit, ok_raw)
    assert np.array_equal(t[hit].view(np.uint32), tt[hit].view(np.uint32))
    assert np.array_equal(u[hit].view(np.uint32), uu[hit].view(np.uint32))
    assert np.array_equal(v[hit].view(np.uint32), vv[hit].view(np.uint32))


def np_aabb(bmin, bmax, o, d, tmin, tmax):
    """Math/AABB.cu:6-46 in numpy float32 (vectorised over rays)."""
    eps = f32(np.finfo(np.float32).eps)
    lo, hi = tmin.copy(), tmax.copy()
    alive = np.ones(len(o), bool)
    with np.errstate(all="ignore"):
        for i in range(3):
            deg = np.abs(bmax[:, i] - bmin[:, i]) < eps
            dz = np.abs(d[:, i]) < eps
            out = deg & dz & (np.abs(o[:, i] - bmin[:, i]) > eps)
            alive &= ~out
            tdeg = (bmin[:, i] - o[:, i]) / d[:, i]
            inv = f32(1) / d[:, i]
            t0 = (bmin[:, i] - o[:, i]) * inv
            t1 = (bmax[:, i] - o[:, i]) * inv
            sw = inv < 0
            t0, t1 = np.where(sw, t1, t0), np.where(sw, t0, t1)
            a = np.where(deg, tdeg, t0)
            b = np.where(deg, tdeg, t1)
            use = ~(deg & dz)
            lo = np.where(use & (lo < a), a, lo)
            hi = np.where(use & (b < hi), b, hi)
    hit = alive & ~(lo > hi) & ~((lo > tmax) | (hi < tmin))
    return hit, lo


def test_aabb_bits():
    rng = np.random.default_rng(7)
    n = 100000
    a = rng.random((n, 3)).astype(f32)
    b = a + rng.random((n, 3)).astype(f32) * f32(0.3)
    flat = rng.random((n, 3)) < 0.2  # degenerate slabs
    b = np.where(flat, a, b).astype(f32)
    rays = scenes.random_rays(n, seed=8)
    zero = rng.random((n, 3)) < 0.05  # axis-parallel rays
    rays["d"] = np.where(zero, f32(0), rays["d"])
    hit, t = oracle.aabb_intersect(a, b, rays)
    h2, t2 = np_aabb(a, b, rays["o"], rays["d"], rays["tmin"], rays["tmax"])
    assert hit.sum() > 1000
    assert np.array_equal(hit, h2)
    assert np.array_equal(t[hit].view(np.uint32), t2[hit].view(np.uint32))


def test_offset_ray_origin():
    """Math/Ray.cu:11-22 in numpy: integer ulp nudge, or p + n/65535 near 0."""
    rng = np.random.default_rng(9)
    p = (rng.normal(size=(50000, 3)) * rng.choice([1e-3, 1.0, 100.0], size=(50000, 1))).astype(f32)
    nrm = rng.normal(size=(50000, 3)).astype(f32)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True).astype(f32)
    out = oracle.offset_ray_origin(p, nrm)
    of = np.trunc(f32(256.0) * nrm).astype(np.int32)
    pi = (p.view(np.int32) + np.where(p < 0, -of, of)).view(f32)
    ref = np.where(np.abs(p) < f32(1 / 32), p + f32(1.0 / 65535.0) * nrm, pi)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))


def _check_tree(nodes, pmap, n_tris):
    root = len(nodes) - 1
    seen = np.zeros(n_tris, int)
    stack = [(root, 0)]
    while stack:
        i, depth = stack.pop()
        nd = nodes[i]
        if nd["is_leaf"]:
            assert depth <= 20 and nd["b"] >= 1
            seen[pmap[nd["a"]:nd["a"] + nd["b"]]] += 1
        else:
            assert depth < 20
            for c in (nd["a"], nd["b"]):
                assert c < i  # post-order: children before parent
                assert (nodes[c]["bmin"] >= nd["bmin"]).all() and (nodes[c]["bmax"] <= nd["bmax"]).all()
                stack.append((c, depth + 1))
    assert (seen == 1).all()


@pytest.mark.parametrize("n", [1, 3, 5, 100, 20000])
def test_bvh_structure(n):
    sd = scenes.random_triangle_scene(n, seed=n)
    osc = oracle.OracleScene(flatten_scene(sd))
    nodes, pmap = osc.bvh_export()
    st = osc.bvh_stats()
    assert st["node_count"] == 2 * st["leaf_count"] - 1
    _check_tree(nodes, pmap, n)


def test_traversal_matches_brute_force():
    sd = scenes.random_triangle_scene(20000, seed=11)
    osc = oracle.OracleScene(flatten_scene(sd))
    rays = scenes.random_rays(20000, seed=12)
    hits, ties = osc.trace_closest(rays)
    brute = osc.trace_brute(rays)
    same = (hits["prim"] == brute["prim"]) | ties
    assert same.all()
    m = hits["prim"] != 0xFFFFFFFF
    assert m.sum() > 15000
    assert np.array_equal(hits["t"][m].view(np.uint32), brute["t"][m].view(np.uint32))


def test_occlusion_matches_any_hit():
    sd = scenes.random_triangle_scene(5000, seed=13)
    osc = oracle.OracleScene(flatten_scene(sd))
    rays = scenes.random_rays(20000, seed=14)
    rays["tmax"] = np.random.default_rng(0).uniform(0.5, 3.0, len(rays)).astype(f32)
    occ = osc.trace_occluded(rays)
    brute = osc.trace_brute(rays)  # closest hit within [tmin, tmax]
    assert np.array_equal(occ.astype(bool), brute["prim"] != 0xFFFFFFFF)


def test_degenerate_and_flat_geometry():
    """Axis-aligned quads (flat boxes take the degenerate-slab branch) and
    zero-area triangles (culled by |det| < 1e-6)."""
    data, _ = scenes.cornell_box()
    flat = flatten_scene(data)
    pos = np.concatenate([flat["pos"], np.array([[0, 0, 0], [0.5, 0.5, 0.5], [1, 1, 1]], f32)])
    idx = np.concatenate([flat["idx"], np.array([len(flat["pos"]), len(flat["pos"]) + 1, len(flat["pos"]) + 2],
                                                np.uint32)])
    flat2 = dict(flat, pos=pos, nrm=np.zeros_like(pos), uv=np.zeros((len(pos), 2), f32), idx=idx)
    flat2["meshes"] = flat["meshes"].copy()
    flat2["meshes"][-1]["index_count"] += 3
    osc = oracle.OracleScene(flat2)
    rays = scenes.random_rays(20000, seed=15)
    rays["o"] *= f32(0.4)  # origins inside the box
    hits, ties = osc.trace_closest(rays)
    brute = osc.trace_brute(rays)
    assert ((hits["prim"] == brute["prim"]) | ties).all()
    assert (hits["prim"] != 0xFFFFFFFF).mean() > 0.6  # the box is open towards +z
    assert not (hits["prim"] == len(idx) // 3 - 1).any()
