"""ctypes wrapper of the CPU oracle (oracle/craystal_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product never imports it.
The oracle restates the reference (Hyiker/CRaystal) on the CPU; it is a port
because the reference cannot be built here (its dependencies are fetched
from the network).  Pins: the reference's camera-ray and spectrum
known-answer tests and sampler statistics (Tests/CameraTest.cpp:16-50,
Tests/CoreTest.cpp:14-280), reproduced in tests/test_oracle_pins.py.
"""
import ctypes
import os

import numpy as np

from . import build as _build

RAY_DTYPE = np.dtype([("o", "<f4", 3), ("tmin", "<f4"), ("d", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("prim", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4")])
MATERIAL_DTYPE = np.dtype([("diffuse", "<f4", 3), ("specular", "<f4", 3), ("emission", "<f4", 3),
                           ("shininess", "<f4"), ("type", "<u4"), ("flags", "<u4")])
MESH_DTYPE = np.dtype([("index_offset", "<u4"), ("index_count", "<u4"), ("vertex_offset", "<u4"),
                       ("material_id", "<u4")])
NODE_DTYPE = np.dtype([("bmin", "<f4", 3), ("bmax", "<f4", 3), ("is_leaf", "<u4"), ("a", "<u4"), ("b", "<u4")])


class OrcCamera(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_float * 3), ("target", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("fov_y", ctypes.c_float), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]


class OrcConfig(ctypes.Structure):
    _fields_ = [("max_depth", ctypes.c_uint32), ("rr_threshold", ctypes.c_float), ("use_mis", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


class OrcStats(ctypes.Structure):
    _fields_ = [("node_count", ctypes.c_uint32), ("leaf_count", ctypes.c_uint32), ("root_index", ctypes.c_uint32),
                ("max_depth", ctypes.c_uint32), ("max_leaf_size", ctypes.c_uint32),
                ("max_leaf_depth", ctypes.c_uint32), ("root_min", ctypes.c_float * 3),
                ("root_max", ctypes.c_float * 3)]


class OrcCounters(ctypes.Structure):
    _fields_ = [("rays", ctypes.c_uint64), ("boxes", ctypes.c_uint64), ("tris", ctypes.c_uint64),
                ("map_reads", ctypes.c_uint64), ("ties", ctypes.c_uint64)]


_P = ctypes.c_void_p
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        U32, U64, I = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
        sig = {
            "orc_sampler_draws": (None, [U32, U32, U32, U32, _P]),
            "orc_sampler_raw": (None, [U32, U32, U32, U32, _P]),
            "orc_camera_basis": (None, [ctypes.POINTER(OrcCamera), _P]),
            "orc_camera_rays": (None, [ctypes.POINTER(OrcCamera), _P, U64, _P]),
            "orc_offset_ray_origin": (None, [_P, _P, U64, _P]),
            "orc_aabb_intersect": (None, [_P, _P, _P, U64, _P, _P]),
            "orc_triangle_intersect": (None, [_P, _P, _P, _P, U64, _P, _P, _P, _P]),
            "orc_scene_create": (_P, [_P, _P, _P, U64, _P, U64, _P, U32, _P, U32, _P, U32]),
            "orc_scene_destroy": (None, [_P]),
            "orc_scene_set_lights": (None, [_P, _P, _P, U32]),
            "orc_scene_set_textures": (None, [_P, _P, _P, U32, _P, U32]),
            "orc_scene_set_spheres": (None, [_P, _P, _P, U32]),
            "orc_texture_sample": (None, [_P, U32, _P, U64, _P]),
            "orc_scene_bvh_stats": (None, [_P, ctypes.POINTER(OrcStats)]),
            "orc_scene_bvh_export": (None, [_P, _P, _P]),
            "orc_trace_closest": (None, [_P, _P, U64, _P, _P, I, ctypes.POINTER(OrcCounters)]),
            "orc_trace_occluded": (None, [_P, _P, U64, _P, I]),
            "orc_trace_brute": (None, [_P, _P, U64, _P, I]),
            "orc_bsdf_eval": (None, [_P, _P, _P, _P, U64, _P, _P]),
            "orc_bsdf_sample": (None, [_P, _P, _P, _P, U64, _P, _P, _P]),
            "orc_render": (None, [_P, ctypes.POINTER(OrcCamera), ctypes.POINTER(OrcConfig), U32, U32, U32, U32,
                                  _P, _P, I, ctypes.POINTER(ctypes.c_uint64)]),
            "orc_spectral_cmf": (None, [_P, U64, _P]),
            "orc_spectral_white_balance": (None, [_P]),
            "orc_spectral_upsample": (None, [_P, _P, U64, _P]),
            "orc_hardware_threads": (I, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def sampler_draws(px, py, sample_index, n):
    out = np.empty(n, np.float32)
    lib().orc_sampler_draws(px, py, sample_index, n, _p(out))
    return out


def sampler_raw(px, py, sample_index, n):
    out = np.empty(n, np.uint32)
    lib().orc_sampler_raw(px, py, sample_index, n, _p(out))
    return out


def make_camera(pos, target, up, fov_y, width, height):
    c = OrcCamera()
    c.pos[:] = pos
    c.target[:] = target
    c.up[:] = up
    c.fov_y = fov_y
    c.width, c.height = width, height
    return c


def camera_rays(cam: OrcCamera, sensor_pos):
    sp = np.ascontiguousarray(sensor_pos, np.float32).reshape(-1, 2)
    out = np.empty(len(sp), RAY_DTYPE)
    lib().orc_camera_rays(ctypes.byref(cam), _p(sp), len(sp), _p(out))
    return out


def offset_ray_origin(p, n):
    p = np.ascontiguousarray(p, np.float32).reshape(-1, 3)
    n = np.ascontiguousarray(n, np.float32).reshape(-1, 3)
    out = np.empty_like(p)
    lib().orc_offset_ray_origin(_p(p), _p(n), len(p), _p(out))
    return out


def aabb_intersect(bmin, bmax, rays):
    bmin = np.ascontiguousarray(bmin, np.float32).reshape(-1, 3)
    bmax = np.ascontiguousarray(bmax, np.float32).reshape(-1, 3)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    hit = np.empty(len(rays), np.uint8)
    t = np.empty(len(rays), np.float32)
    lib().orc_aabb_intersect(_p(bmin), _p(bmax), _p(rays), len(rays), _p(hit), _p(t))
    return hit.astype(bool), t


def triangle_intersect(v0, v1, v2, rays):
    v0, v1, v2 = (np.ascontiguousarray(v, np.float32).reshape(-1, 3) for v in (v0, v1, v2))
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    n = len(rays)
    hit = np.empty(n, np.uint8)
    t, u, v = (np.empty(n, np.float32) for _ in range(3))
    lib().orc_triangle_intersect(_p(v0), _p(v1), _p(v2), _p(rays), n, _p(hit), _p(t), _p(u), _p(v))
    return hit.astype(bool), t, u, v


class OracleScene:
    """A scene in the oracle: the flattened arrays of craystal_gb300.api.flatten_scene."""

    def __init__(self, flat: dict):
        self.flat = flat
        L = lib()
        mats = np.ascontiguousarray(flat["mats"]).view(MATERIAL_DTYPE)
        meshes = np.ascontiguousarray(flat["meshes"]).view(MESH_DTYPE)
        self.n_tris = len(flat["idx"]) // 3
        self._keep = (flat["pos"], flat["nrm"], flat["uv"], flat["idx"], meshes, mats, flat["emissive"])
        self.h = L.orc_scene_create(_p(flat["pos"]), _p(flat["nrm"]), _p(flat["uv"]), len(flat["pos"]),
                                    _p(flat["idx"]), self.n_tris, _p(meshes), len(meshes), _p(mats), len(mats),
                                    _p(flat["emissive"]), len(flat["emissive"]))
        if flat.get("textures"):
            self.set_textures(flat["textures"], flat["mat_tex"])
        if len(flat.get("sph_mat", ())):
            self.set_spheres(flat["sph_geom"], flat["sph_mat"])

    def set_spheres(self, geom, mats):
        """Spheres: geom n x 4 (centre, radius), mats n material ids."""
        g = np.ascontiguousarray(geom, np.float32).reshape(-1, 4)
        m = np.ascontiguousarray(mats, np.uint32)
        self._sph = (g, m)
        lib().orc_scene_set_spheres(self.h, _p(g), _p(m), len(m))

    def set_textures(self, textures, material_texture):
        """RGBA texel arrays (HxWx4) and the texture of each material (0xFFFFFFFF = none)."""
        texels = np.concatenate([np.ascontiguousarray(t, np.float32).reshape(-1) for t in textures])
        descs, first = [], 0
        for t in textures:
            descs += [first, t.shape[1], t.shape[0]]
            first += t.shape[0] * t.shape[1]
        descs = np.asarray(descs, np.uint32)
        mt = np.ascontiguousarray(material_texture, np.uint32)
        self._tex = (texels, descs, mt)
        lib().orc_scene_set_textures(self.h, _p(texels), _p(descs), len(textures), _p(mt), len(mt))

    def texture_sample(self, texture, uv):
        """TextureView::sample at n coordinates -> n x 4."""
        uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        out = np.empty((len(uv), 4), np.float32)
        lib().orc_texture_sample(self.h, texture, _p(uv), len(uv), _p(out))
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_scene_destroy(self.h)
            self.h = None

    def set_lights(self, env=(0.0, 0.0, 0.0), spheres=()):
        """Environment radiance and sphere lights [(center, radius, emission)] (extensions)."""
        e = np.asarray(env, np.float32)
        sp = np.asarray([[*c, r, *em] for c, r, em in spheres], np.float32).reshape(-1, 7)
        self._lights = (e, sp)
        lib().orc_scene_set_lights(self.h, _p(e), _p(sp) if len(sp) else None, len(sp))

    def bvh_stats(self):
        st = OrcStats()
        lib().orc_scene_bvh_stats(self.h, ctypes.byref(st))
        return {k: (list(getattr(st, k)) if k in ("root_min", "root_max") else getattr(st, k))
                for k, _ in OrcStats._fields_}

    def bvh_export(self):
        st = self.bvh_stats()
        nodes = np.zeros(st["node_count"], NODE_DTYPE)
        pmap = np.zeros(self.n_tris, np.uint32)
        lib().orc_scene_bvh_export(self.h, _p(nodes), _p(pmap))
        return nodes, pmap

    def trace_closest(self, rays, threads=0, counters=False):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        hits = np.empty(len(rays), HIT_DTYPE)
        ties = np.empty(len(rays), np.uint8)
        c = OrcCounters()
        lib().orc_trace_closest(self.h, _p(rays), len(rays), _p(hits), _p(ties), threads, ctypes.byref(c))
        if counters:
            return hits, ties.astype(bool), {k: getattr(c, k) for k, _ in OrcCounters._fields_}
        return hits, ties.astype(bool)

    def trace_occluded(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        occ = np.empty(len(rays), np.uint8)
        lib().orc_trace_occluded(self.h, _p(rays), len(rays), _p(occ), threads)
        return occ

    def trace_brute(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        hits = np.empty(len(rays), HIT_DTYPE)
        lib().orc_trace_brute(self.h, _p(rays), len(rays), _p(hits), threads)
        return hits

    def render(self, cam: OrcCamera, max_depth=10, rr_threshold=0.05, use_mis=True, spp=1, first_sample=0,
               rows=None, threads=0, film=None, spectral=False):
        """FP64 film (rgb sum HxWx3, weight HxW) of spp samples; accumulates into film if given."""
        W, H = cam.width, cam.height
        if film is None:
            film = (np.zeros((H, W, 3), np.float64), np.zeros((H, W), np.float64))
        cfg = OrcConfig(max_depth, rr_threshold, 1 if use_mis else 0, 1 if spectral else 0)
        rays = ctypes.c_uint64()
        r0, r1 = rows if rows else (0, 0)
        lib().orc_render(self.h, ctypes.byref(cam), ctypes.byref(cfg), spp, first_sample, r0, r1, _p(film[0]),
                         _p(film[1]), threads, ctypes.byref(rays))
        return film, rays.value


def bsdf_eval(mat, n, wo, wi):
    mat = np.ascontiguousarray(mat, MATERIAL_DTYPE).reshape(1)
    n, wo, wi = (np.ascontiguousarray(x, np.float32).reshape(-1, 3) for x in (n, wo, wi))
    f = np.empty((len(n), 3), np.float32)
    pdf = np.empty(len(n), np.float32)
    lib().orc_bsdf_eval(_p(mat), _p(n), _p(wo), _p(wi), len(n), _p(f), _p(pdf))
    return f, pdf


def bsdf_sample(mat, n, wo, u):
    mat = np.ascontiguousarray(mat, MATERIAL_DTYPE).reshape(1)
    n, wo = (np.ascontiguousarray(x, np.float32).reshape(-1, 3) for x in (n, wo))
    u = np.ascontiguousarray(u, np.float32).reshape(-1, 2)
    wi = np.empty((len(n), 3), np.float32)
    f = np.empty((len(n), 3), np.float32)
    pdf = np.empty(len(n), np.float32)
    lib().orc_bsdf_sample(_p(mat), _p(n), _p(wo), _p(u), len(n), _p(wi), _p(f), _p(pdf))
    return wi, f, pdf


def hardware_threads() -> int:
    return int(lib().orc_hardware_threads())


def spectral_cmf(lam):
    lam = np.ascontiguousarray(lam, np.float32)
    out = np.empty((len(lam), 3), np.float32)
    lib().orc_spectral_cmf(_p(lam), len(lam), _p(out))
    return out


def spectral_white_balance():
    out = np.empty(3, np.float32)
    lib().orc_spectral_white_balance(_p(out))
    return out


def spectral_upsample(rgb, lam):
    rgb = np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
    lam = np.ascontiguousarray(lam, np.float32)
    out = np.empty(len(lam), np.float32)
    lib().orc_spectral_upsample(_p(rgb), _p(lam), len(lam), _p(out))
    return out
