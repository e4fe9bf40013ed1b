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


MATERIAL_GPU_DTYPE = np.dtype([("kd", "<f4", 3), ("ks", "<f4", 3), ("em", "<f4", 3), ("shininess", "<f4"),
                               ("type", "<u4"), ("flags", "<u4"), ("dProb", "<f4"), ("sProb", "<f4"),
                               ("rough", "<f4"), ("metal", "<f4"), ("tex", "<u4")])


def derived_materials(mats):
    """Per-material records as MaterialData::finalize and the BSDF
    constructors derive them (Core/Material.h:57-65, Material/PhongBRDF.cu:10-19,
    Material/PrincipledBRDF.cu:35-55), in float32 operation order."""
    f = np.float32
    out = np.zeros(len(mats), MATERIAL_GPU_DTYPE)
    for i, m in enumerate(mats):
        kd, ks, em = (np.asarray(m[k], np.float32) for k in ("diffuse", "specular", "emission"))
        out[i]["kd"], out[i]["ks"], out[i]["em"] = kd, ks, em
        out[i]["shininess"], out[i]["type"] = m["shininess"], m["type"]
        flags = int(m["flags"])
        if em.max() != 0:
            flags |= 1
        if ks.max() == 0:
            flags |= 2
        out[i]["flags"] = flags
        avg = lambda v: f(f(f(f(0) + v[0]) + v[1]) + v[2]) / f(3)
        if m["type"] == 2:
            d, s = max(avg(kd), f(0)), max(avg(ks), f(0))
            tot = max(f(d + s), f(1e-6))
            out[i]["dProb"], out[i]["sProb"] = d / tot, s / tot
        elif m["type"] == 1:
            r = np.sqrt(f(2) / f(f(m["shininess"]) + f(1)))
            met = min(max(avg(ks), f(0)), f(1))
            spr = f(f(f(0.1) * f(f(1) - met)) + f(f(1) * met))
            d = f(1) / f(f(1) + spr)
            s = spr / f(d + spr)
            out[i]["rough"], out[i]["metal"] = min(max(r, f(0)), f(1)), met
            out[i]["dProb"], out[i]["sProb"] = d, s
        else:
            out[i]["dProb"], out[i]["sProb"] = 1.0, 0.0
        out[i]["tex"] = 0xFFFFFFFF
    return out


class RestatedPathTracer:
    """The reference's pathTraceKernel + dispatch restated (ref_path.cu) on a
    product scene's reference-layout BVH and the flattened scene arrays."""

    def __init__(self, scene, flat):
        import torch
        self.bvh = RestatedTraversal(scene, flat)
        dev = torch.device("cuda")
        nv_mesh = flat["meshes"]
        prim_to_mesh = np.zeros(len(flat["idx"]) // 3, np.uint32)
        for k, d in enumerate(nv_mesh):
            prim_to_mesh[d["index_offset"] // 3:(d["index_offset"] + d["index_count"]) // 3] = k
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).to(dev)
        self.nrm = t(np.asarray(flat["nrm"], np.float32))
        self.p2m = t(prim_to_mesh)
        self.mmat = t(np.asarray(nv_mesh["material_id"], np.uint32))
        self.mats = t(derived_materials(flat["mats"]))
        self.emissive = t(np.asarray(flat["emissive"], np.uint32))
        self.n_emissive = len(flat["emissive"])
        lib = load()
        f = lib.refk_render
        f.restype = ctypes.c_int
        f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                      ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                      ctypes.c_uint32, ctypes.c_float, ctypes.c_int, ctypes.c_uint32, ctypes.c_void_p,
                      ctypes.c_void_p, ctypes.c_void_p]

    def render(self, cam, spp, max_depth=10, rr_threshold=0.05, use_mis=True):
        """Film (rgb sum, weight) and ray count of spp samples (indices 0..spp-1)."""
        import torch

        from craystal_gb300._lib import CrCamera
        c = cam._c()
        w, h = c.width, c.height
        rgb = torch.zeros(h * w * 3, dtype=torch.float32, device="cuda")
        wt = torch.zeros(h * w, dtype=torch.float32, device="cuda")
        rays = torch.zeros(1, dtype=torch.int64, device="cuda")
        b = self.bvh
        rc = load().refk_render(b.nodes.data_ptr(), b.root, b.rmin, b.rmax, b.pmap.data_ptr(), b.pos.data_ptr(),
                                self.nrm.data_ptr(), b.idx.data_ptr(), self.p2m.data_ptr(), self.mmat.data_ptr(),
                                self.mats.data_ptr(), self.emissive.data_ptr(), self.n_emissive, ctypes.byref(c),
                                max_depth, rr_threshold, 1 if use_mis else 0, spp, rgb.data_ptr(), wt.data_ptr(),
                                rays.data_ptr())
        if rc != 0:
            raise RuntimeError("restated reference path tracer failed")
        return (rgb.cpu().numpy().reshape(h, w, 3), wt.cpu().numpy().reshape(h, w)), int(rays.item())
