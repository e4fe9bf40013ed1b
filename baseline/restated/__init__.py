"""The reference's closest-hit traversal restated as a CUDA comparator.

The reference's own CUDA build cannot be compiled in this image (it needs
glm, fmt and cmake), so its BVH traversal -- BVHData::intersect
(Core/BVH.cu:13-84), AABB::intersect (Math/AABB.cu:6-46),
TriangleMeshSOA::intersect (Scene/Triangle.cu:40-75) and intersectShape
(Scene/Shape.h:16-37) -- is restated here as written (36-byte variant nodes,
a per-box division, a 64-entry local stack, indexed float3 vertex fetches,
separately compiled device functions) and launched one thread per ray over
the reference-layout BVH that the product exports.  It is a measurement
comparator for the ray-cast workload, never part of the product path.
"""
import ctypes

import numpy as np

from . import build as _build

NODE_DTYPE = np.dtype([("a", "<u4"), ("b", "<u4"), ("index", "u1"), ("pad", "u1", 3),
                       ("bmin", "<f4", 3), ("bmax", "<f4", 3)])
assert NODE_DTYPE.itemsize == 36

_lib = None


def load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build())
        f = _lib.refk_trace_closest
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float),
                      ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                      ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    return _lib


def reference_nodes(exported):
    """Reference BVHNode array from the exported tree (post-order, root last):
    variant index 0 holds LeafProp {leafOffset, leafCount}, 1 holds
    InternalProp {left, right}."""
    out = np.zeros(len(exported), NODE_DTYPE)
    out["a"] = exported["a"]
    out["b"] = exported["b"]
    out["index"] = np.where(exported["is_leaf"] != 0, 0, 1)
    out["bmin"] = exported["bmin"]
    out["bmax"] = exported["bmax"]
    return out


class RestatedTraversal:
    """Device-resident reference-layout BVH + mesh for one scene."""

    def __init__(self, scene, flat):
        import torch
        nodes, pmap = scene.bvh_export()
        st = scene.bvh_stats()
        dev = torch.device("cuda")
        ref = reference_nodes(nodes)
        self.nodes = torch.from_numpy(ref.view(np.uint8).copy()).to(dev)
        self.pmap = torch.from_numpy(pmap.view(np.int32).copy()).to(dev)
        self.pos = torch.from_numpy(np.ascontiguousarray(flat["pos"], np.float32)).to(dev)
        self.idx = torch.from_numpy(np.ascontiguousarray(flat["idx"], np.uint32).view(np.int32)).to(dev)
        self.root = len(ref) - 1
        self.rmin = (ctypes.c_float * 3)(*st["root_min"])
        self.rmax = (ctypes.c_float * 3)(*st["root_max"])

    def trace_closest_device(self, rays_ptr, n, hits_ptr, stream=0):
        rc = load().refk_trace_closest(self.nodes.data_ptr(), self.root, self.rmin, self.rmax,
                                       self.pmap.data_ptr(), self.pos.data_ptr(), self.idx.data_ptr(),
                                       rays_ptr, n, hits_ptr, stream or None)
        if rc != 0:
            raise RuntimeError("restated reference traversal launch failed")
