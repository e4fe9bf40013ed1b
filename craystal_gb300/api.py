"""Host-side mirror of the reference's hot-path API (Source/CRaystal):
Scene / SceneData / MeshData / MaterialData (Scene/Scene.h:40-58,
Scene/Triangle.h:36-42, Core/Material.h:34-66), Camera (Core/Camera.h),
Sensor (Core/Sensor.h) and PathTraceIntegrator (Core/Integrator.h).

Everything runs through the C ABI of libcraystal_gb300.so; there is no CPU
path.  Errors raise CrayError (the reference raises RuntimeError).
"""
import ctypes
import enum
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _lib
from ._lib import (BVH_NODE_DTYPE, HIT_DTYPE, MATERIAL_DTYPE, MESH_DTYPE, RAY_DTYPE, CrBvhStats, CrCamera,
                   CrIntegratorConfig, check, load, ptr)


class MaterialType(enum.IntEnum):
    """Core/Material.h:12-16."""
    FullDiffuse = 0
    Principled = 1
    Phong = 2


class MaterialFlags(enum.IntFlag):
    """Core/Material.h:26-30."""
    IsEmissive = 1
    IsDiffuse = 2
    hasDiffuseTexture = 4


@dataclass
class MaterialData:
    """Core/Material.h:34-66 (the fields the path reads)."""
    diffuseRefl: tuple = (0.0, 0.0, 0.0)
    specularRefl: tuple = (0.0, 0.0, 0.0)
    emission: tuple = (0.0, 0.0, 0.0)
    shininess: float = 0.0
    type: MaterialType = MaterialType.FullDiffuse
    flags: int = 0
    diffuseHandle: int = 0  # index into SceneData.textureImages when hasDiffuseTexture
    name: str = ""          # the material's name in its source file (imported scenes)

    def finalize(self):
        """MaterialData::finalize, Core/Material.h:57-65."""
        if max(self.emission) != 0.0:
            self.flags |= int(MaterialFlags.IsEmissive)
        if max(self.specularRefl) == 0.0:
            self.flags |= int(MaterialFlags.IsDiffuse)

    def isEmissive(self) -> bool:
        return bool(self.flags & MaterialFlags.IsEmissive)

    def hasDiffuseTexture(self) -> bool:
        return bool(self.flags & MaterialFlags.hasDiffuseTexture)


@dataclass
class MeshData:
    """Scene/Triangle.h:36-42: per-mesh vertex arrays and local indices."""
    position: np.ndarray
    index: np.ndarray
    materialID: int = 0
    normal: Optional[np.ndarray] = None
    texCrd: Optional[np.ndarray] = None


@dataclass
class SphereData:
    """Scene/Sphere.h:9-12, with the material the reference's spheres lack."""
    center: tuple = (0.0, 0.0, 0.0)
    radius: float = 1.0
    materialID: int = 0


@dataclass
class SceneData:
    """Scene/Scene.h:40-47.  textureImages: images as HxWxC float arrays
    (C = 1..4, row 0 first, as Image holds them after loading); spheres:
    analytic spheres with materials (emitting spheres without a material
    are Scene.set_sphere_lights)."""
    meshes: List[MeshData] = field(default_factory=list)
    materials: List[MaterialData] = field(default_factory=list)
    emissiveIndex: List[int] = field(default_factory=list)
    textureImages: List[np.ndarray] = field(default_factory=list)
    spheres: List[SphereData] = field(default_factory=list)


def texture_texels(image) -> np.ndarray:
    """Texture(const Image&), Core/Texture.cu:45-60: row-major RGBA float4
    texels, channels beyond the image's left at 0."""
    a = np.asarray(image, np.float32)
    if a.ndim == 2:
        a = a[..., None]
    if a.ndim != 3 or not 1 <= a.shape[2] <= 4 or a.shape[0] == 0 or a.shape[1] == 0:
        raise ValueError(f"texture image of shape {a.shape}")
    out = np.zeros((a.shape[0], a.shape[1], 4), np.float32)
    out[..., : a.shape[2]] = a
    return out


def flatten_scene(data: SceneData):
    """TriangleMeshManager's concatenation (Scene/Triangle.cu:98-131): global
    vertex arrays, indices rebased by each mesh's vertex offset, MeshDesc."""
    pos, nrm, uv, idx = [], [], [], []
    descs = np.zeros(len(data.meshes), MESH_DTYPE)
    nv = ni = 0
    for m, mesh in enumerate(data.meshes):
        p = np.ascontiguousarray(mesh.position, np.float32).reshape(-1, 3)
        n = (np.zeros_like(p) if mesh.normal is None else np.ascontiguousarray(mesh.normal, np.float32).reshape(-1, 3))
        t = (np.zeros((len(p), 2), np.float32) if mesh.texCrd is None
             else np.ascontiguousarray(mesh.texCrd, np.float32).reshape(-1, 2))
        i = np.ascontiguousarray(mesh.index, np.uint32).reshape(-1)
        descs[m] = (ni, len(i), nv, mesh.materialID)
        pos.append(p)
        nrm.append(n)
        uv.append(t)
        idx.append(i + np.uint32(nv))
        nv += len(p)
        ni += len(i)
    cat = lambda xs, shape, dt: np.concatenate(xs) if xs else np.zeros(shape, dt)
    mats = np.zeros(len(data.materials), MATERIAL_DTYPE)
    mat_tex = np.full(len(data.materials), _lib.CR_NO_TEXTURE, np.uint32)
    for k, md in enumerate(data.materials):
        mats[k] = (md.diffuseRefl, md.specularRefl, md.emission, md.shininess, int(md.type),
                   md.flags & int(MaterialFlags.IsEmissive | MaterialFlags.IsDiffuse))
        if md.flags & MaterialFlags.hasDiffuseTexture:
            if not 0 <= md.diffuseHandle < len(data.textureImages):
                raise ValueError(f"material {k}: texture {md.diffuseHandle} of {len(data.textureImages)}")
            mat_tex[k] = md.diffuseHandle
    return dict(pos=cat(pos, (0, 3), np.float32), nrm=cat(nrm, (0, 3), np.float32), uv=cat(uv, (0, 2), np.float32),
                idx=cat(idx, (0,), np.uint32), meshes=descs, mats=mats,
                emissive=np.asarray(data.emissiveIndex, np.uint32),
                textures=[texture_texels(t) for t in data.textureImages], mat_tex=mat_tex,
                sph_geom=np.array([[*sd.center, sd.radius] for sd in data.spheres], np.float32).reshape(-1, 4),
                sph_mat=np.array([sd.materialID for sd in data.spheres], np.uint32))


class Sensor:
    """Core/Sensor.h:35-61: film size, spp and the host copy of the film."""

    def __init__(self, size=(512, 512), spp: int = 1):
        self.size = (int(size[0]), int(size[1]))
        self.spp = int(spp)
        self.data = np.zeros((self.size[1], self.size[0], 3), np.float32)
        self.weight = np.zeros((self.size[1], self.size[0]), np.float32)

    def setSPP(self, value: int):
        self.spp = int(value)

    def getSPP(self) -> int:
        return self.spp

    def getSize(self):
        return self.size

    def createImage(self) -> np.ndarray:
        """Sensor::createImage (Core/Sensor.cu:93-112): sum / weight, HxWx3."""
        with np.errstate(divide="ignore", invalid="ignore"):
            return self.data / self.weight[..., None]


class Camera:
    """Core/Camera.h:18-46 with the defaults of CameraProxy (Core/CameraProxy.h:12-23)."""

    def __init__(self):
        self.posW = (0.0, 0.0, 0.0)
        self.fovY = 60.0
        self.target = (0.0, 0.0, -1.0)
        self.up = (0.0, 1.0, 0.0)
        self.sensor: Optional[Sensor] = None

    def setFovY(self, v):
        self.fovY = float(v)

    def setWorldPosition(self, p):
        self.posW = tuple(float(x) for x in p)

    def setTarget(self, t):
        self.target = tuple(float(x) for x in t)

    def setUp(self, u):
        self.up = tuple(float(x) for x in u)

    def setSensor(self, s: Sensor):
        self.sensor = s

    def getSensor(self) -> Optional[Sensor]:
        return self.sensor

    def calculateCameraData(self):
        """The basis is computed in the library when the camera is set on a scene."""

    def _c(self) -> CrCamera:
        c = CrCamera()
        c.pos[:] = self.posW
        c.target[:] = self.target
        c.up[:] = self.up
        c.fov_y = self.fovY
        w, h = self.sensor.size if self.sensor else (512, 512)
        c.width, c.height = w, h
        return c


class Scene:
    """Scene/Scene.h:50-82.  Construction uploads the geometry and builds the
    BVH on the GPU."""

    def __init__(self, data: SceneData):
        lib = load()
        f = flatten_scene(data)
        self._flat = f
        self.n_tris = len(f["idx"]) // 3
        h = ctypes.c_void_p()
        check(lib.cr_scene_create(ptr(f["pos"]), ptr(f["nrm"]), ptr(f["uv"]), len(f["pos"]), ptr(f["idx"]),
                                  self.n_tris, ptr(f["meshes"]), len(f["meshes"]), ptr(f["mats"]), len(f["mats"]),
                                  ptr(f["emissive"]), len(f["emissive"]), ctypes.byref(h)))
        self._h = h
        self._camera: Optional[Camera] = None
        if f["textures"]:
            self.set_diffuse_textures(f["textures"], f["mat_tex"])
        if len(f["sph_mat"]):
            self.set_spheres(f["sph_geom"], f["sph_mat"])

    def set_spheres(self, geom, materials):
        """Analytic spheres: geom n x 4 (centre, radius), a material each;
        builds their BVH on the GPU."""
        g = np.asarray(geom, np.float32).reshape(-1, 4)
        arr = np.zeros(len(g), _lib.SPHERE_DTYPE)
        arr["center"] = g[:, :3]
        arr["radius"] = g[:, 3]
        arr["material"] = np.asarray(materials, np.uint32)
        check(load().cr_scene_set_spheres(self._h, ptr(arr) if len(arr) else None, len(arr)))

    def set_diffuse_textures(self, textures, material_texture):
        """Uploads RGBA texel arrays (HxWx4) and the texture of each material
        (CR_NO_TEXTURE for none)."""
        keep = [np.ascontiguousarray(t, np.float32) for t in textures]
        descs = (_lib.CrTexture * max(1, len(keep)))()
        for i, t in enumerate(keep):
            descs[i].width, descs[i].height = t.shape[1], t.shape[0]
            descs[i].texels = t.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        mt = np.ascontiguousarray(material_texture, np.uint32)
        check(load().cr_scene_set_diffuse_textures(self._h, descs, len(keep), ptr(mt), len(mt)))

    def texture_sample(self, texture: int, uv: np.ndarray) -> np.ndarray:
        """TextureView::sample on the device at n texture coordinates -> n x 4."""
        uv = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        out = np.empty((len(uv), 4), np.float32)
        check(load().cr_texture_sample(self._h, texture, ptr(uv), len(uv), ptr(out)))
        return out

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().cr_scene_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def setCamera(self, cam: Camera):
        self._camera = cam
        check(load().cr_scene_set_camera(self._h, ctypes.byref(cam._c())))

    def getCamera(self) -> Optional[Camera]:
        return self._camera

    # --- lights beyond the reference (extensions) ---
    def set_environment(self, radiance):
        e = np.asarray(radiance, np.float32).reshape(3)
        check(load().cr_scene_set_environment(self._h, ptr(e)))

    def set_sphere_lights(self, lights):
        """lights: iterable of (center xyz, radius, emission rgb)."""
        arr = np.zeros(len(lights), _lib.SPHERE_LIGHT_DTYPE)
        for i, (c, r, em) in enumerate(lights):
            arr[i] = (c, r, em, 0.0)
        check(load().cr_scene_set_sphere_lights(self._h, ptr(arr) if len(arr) else None, len(arr)))

    # --- BVH introspection (Core/BVH.cu:111-115 logs the same figures) ---
    def bvh_stats(self) -> dict:
        st = CrBvhStats()
        check(load().cr_scene_bvh_stats(self._h, ctypes.byref(st)))
        return {k: (list(getattr(st, k)) if k in ("root_min", "root_max") else getattr(st, k))
                for k, _ in CrBvhStats._fields_}

    def bvh_export(self):
        """Nodes in the reference layout (post-order, root last) and the
        leaf-slot -> primitive map."""
        st = self.bvh_stats()
        nodes = np.zeros(st["node_count"], BVH_NODE_DTYPE)
        pmap = np.zeros(self.n_tris, np.uint32)
        check(load().cr_scene_bvh_export(self._h, ptr(nodes), ptr(pmap)))
        return nodes, pmap

    def bvh_import(self, nodes: np.ndarray, prim_map: np.ndarray):
        """Replaces the tree with one in the reference layout (nodes with the
        root last, leaf (first slot, count) into prim_map), e.g. the tree the
        reference's host builder makes (Core/BVH.cu:303-338)."""
        nodes = np.ascontiguousarray(nodes, BVH_NODE_DTYPE)
        prim_map = np.ascontiguousarray(prim_map, np.uint32)
        if len(prim_map) != self.n_tris:
            raise ValueError(f"prim_map has {len(prim_map)} entries; the scene has {self.n_tris} triangles")
        check(load().cr_scene_bvh_import(self._h, ptr(nodes), len(nodes), ptr(prim_map)))

    def set_traversal(self, mode: str):
        """"one_level" (default) or "two_level": how the ray-cast queries step
        through the BVH (cr_scene_set_traversal).  The hits are the same."""
        modes = {"one_level": _lib.CR_TRAVERSAL_ONE_LEVEL, "two_level": _lib.CR_TRAVERSAL_TWO_LEVEL}
        if mode not in modes:
            raise ValueError(f"traversal mode {mode!r}; one of {sorted(modes)}")
        check(load().cr_scene_set_traversal(self._h, modes[mode]))

    def check_errors(self) -> int:
        """Waits for the device, then reports (CrayError, code CR_ERR_DEVICE)
        and clears the errors kernels raised on this scene; returns 0."""
        flags = ctypes.c_uint32()
        check(load().cr_scene_check_errors(self._h, ctypes.byref(flags)))
        return flags.value

    # --- ray queries (SceneView::intersect / intersectOcclusion) ---
    def trace_closest(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        hits = np.empty(len(rays), HIT_DTYPE)
        check(load().cr_trace_closest(self._h, ptr(rays), len(rays), ptr(hits)))
        return hits

    def trace_occluded(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, RAY_DTYPE)
        occ = np.empty(len(rays), np.uint8)
        check(load().cr_trace_occluded(self._h, ptr(rays), len(rays), ptr(occ)))
        return occ

    def trace_closest_device(self, rays_ptr: int, n: int, hits_ptr: int, stream: int = 0):
        check(load().cr_trace_closest_device(self._h, rays_ptr, n, hits_ptr, stream or None))

    def trace_occluded_device(self, rays_ptr: int, n: int, occ_ptr: int, stream: int = 0):
        check(load().cr_trace_occluded_device(self._h, rays_ptr, n, occ_ptr, stream or None))

    # --- film ---
    def film_clear(self):
        check(load().cr_film_clear(self._h))

    def film_read(self):
        w, h = self._camera.sensor.size
        rgb = np.zeros((h, w, 3), np.float32)
        wt = np.zeros((h, w), np.float32)
        check(load().cr_film_read(self._h, ptr(rgb), ptr(wt)))
        return rgb, wt

    def film_resolve(self) -> np.ndarray:
        w, h = self._camera.sensor.size
        out = np.zeros((h, w, 3), np.float32)
        check(load().cr_film_resolve(self._h, ptr(out)))
        return out

    def render_ray_count(self) -> int:
        v = ctypes.c_uint64()
        check(load().cr_render_ray_count(self._h, ctypes.byref(v)))
        return v.value


class PathTraceIntegrator:
    """Core/Integrator.h:10-38.

    The reference never copies Configs into its device view, so its kernel
    always runs with maxDepth 10 and rrThreshold 0.05 and only useMIS takes
    effect (Core/Integrator.cu:8-11, 234, 247).  compat=True (default)
    reproduces that; compat=False hands Configs to the kernel.
    """

    class Configs:
        def __init__(self, maxDepth: int = 10, rrThreshold: float = 0.15, useMIS: bool = True):
            self.maxDepth = maxDepth
            self.rrThreshold = rrThreshold
            self.useMIS = useMIS

    def __init__(self, configs: "PathTraceIntegrator.Configs" = None, compat: bool = True, spectral: bool = False,
                 wavefront: Optional[bool] = None):
        self.configs = configs or PathTraceIntegrator.Configs()
        self.compat = compat
        self.spectral = spectral  # hero-wavelength spectral rendering (an extension)
        # schedule: True = wavefront (material sort per bounce), False = megakernel, None = the library's choice
        self.wavefront = wavefront

    def device_config(self) -> CrIntegratorConfig:
        c = CrIntegratorConfig()
        if self.compat:
            c.max_depth, c.rr_threshold = 10, 0.05
        else:
            c.max_depth, c.rr_threshold = self.configs.maxDepth, self.configs.rrThreshold
        c.use_mis = 1 if self.configs.useMIS else 0
        c.flags = (1 if self.spectral else 0) | {None: 0, True: 2, False: 4}[self.wavefront]
        return c

    def dispatch(self, scene: Scene, spp: int, first_sample: int = 0, stream: int = 0, readback: bool = True):
        """PathTraceIntegrator::dispatch (Core/Integrator.cu:233-262): spp
        samples per pixel with sample indices first_sample.. (the reference
        always starts at 0), then the film is read back into the sensor."""
        cam = scene.getCamera()
        if cam is None or cam.sensor is None:
            raise _lib.CrayError(_lib.CR_ERR_INVALID_ARGUMENT, "scene has no camera with a sensor")
        cam.sensor.setSPP(spp)
        scene.setCamera(cam)
        cfg = self.device_config()
        check(load().cr_render(scene.handle, ctypes.byref(cfg), int(spp), int(first_sample), stream or None))
        if readback:
            rgb, wt = scene.film_read()
            cam.sensor.data[...] = rgb
            cam.sensor.weight[...] = wt


def kernel_launch_count() -> int:
    return int(load().cr_kernel_launch_count())


def version() -> str:
    return load().cr_version().decode()


class RadianceCache:
    """The online-trained MLP radiance cache (no counterpart in the
    reference): cr_mlp_* plus cr_render_cached."""

    def __init__(self, lr=1e-2, beta1=0.9, beta2=0.99, eps=1e-8, seed=0):
        from ._lib import CrMlpConfig
        h = ctypes.c_void_p()
        cfg = CrMlpConfig(lr, beta1, beta2, eps, seed)
        check(load().cr_mlp_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().cr_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def params(self) -> np.ndarray:
        p = np.zeros(load().cr_mlp_param_count(), np.float32)
        check(load().cr_mlp_get_params(self._h, ptr(p)))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        check(load().cr_mlp_set_params(self._h, ptr(p)))

    def infer(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32)
        out = np.zeros((len(x), 3), np.float32)
        check(load().cr_mlp_infer(self._h, ptr(x), len(x), ptr(out)))
        return out

    def infer_device(self, inputs: int, n: int, outputs: int, stream: int = 0):
        """Inference on device pointers (n x 7 in, n x 3 out), ordered on
        `stream` without waiting."""
        check(load().cr_mlp_infer_device(self._h, inputs, n, outputs, stream))

    def train_step_device(self, inputs: int, targets: int, n: int, stream: int = 0):
        """One Adam step on device pointers (n x 7 inputs, n x 3 targets),
        ordered on `stream` without waiting."""
        check(load().cr_mlp_train_step_device(self._h, inputs, targets, n, stream))


class CachedPathTraceIntegrator(PathTraceIntegrator):
    """Path tracing with the radiance cache: one frame = one sample per pixel
    (cr_render_cached)."""

    def __init__(self, configs=None, compat=False, query_vertex=1, train_every=0, train_samples=8192,
                 train_steps=1, cache: "RadianceCache" = None, wavefront: Optional[bool] = None):
        # schedule: the wavefront unless wavefront=False (the megakernel form)
        super().__init__(configs or PathTraceIntegrator.Configs(), compat, wavefront=wavefront)
        from ._lib import CrCacheConfig, CrCacheStats
        self.cache = cache or RadianceCache()
        self.cc = CrCacheConfig(query_vertex, train_every, train_samples, train_steps, 0)
        self.stats = CrCacheStats()

    def dispatch(self, scene: "Scene", frames: int, first_sample: int = 0, stream: int = 0, readback: bool = True,
                 freeze: bool = False):
        cam = scene.getCamera()
        if cam is None or cam.sensor is None:
            raise _lib.CrayError(_lib.CR_ERR_INVALID_ARGUMENT, "scene has no camera with a sensor")
        scene.setCamera(cam)
        cfg = self.device_config()
        self.cc.freeze = 1 if freeze else 0
        check(load().cr_render_cached(scene.handle, ctypes.byref(cfg), ctypes.byref(self.cc), self.cache.handle,
                                      int(frames), int(first_sample), stream or None, ctypes.byref(self.stats)))
        if readback:
            rgb, wt = scene.film_read()
            cam.sensor.data[...] = rgb
            cam.sensor.weight[...] = wt


class BatchRenderer:
    """Many scenes in one persistent launch replayed from a CUDA graph
    (cr_batch_*); items: one (PathTraceIntegrator, spp, first_sample) per scene."""

    def __init__(self, scenes, integrators, spp, first_sample=None):
        from ._lib import CrBatchItem
        n = len(scenes)
        self.scenes = list(scenes)
        items = (CrBatchItem * n)()
        for i in range(n):
            items[i].config = integrators[i].device_config()
            items[i].spp = int(spp[i])
            items[i].first_sample = int(first_sample[i]) if first_sample is not None else 0
        for sc in self.scenes:
            if sc.getCamera() is None:
                raise _lib.CrayError(_lib.CR_ERR_INVALID_ARGUMENT, "every scene needs a camera")
        handles = (ctypes.c_void_p * n)(*[sc.handle.value for sc in self.scenes])
        h = ctypes.c_void_p()
        check(load().cr_batch_create(handles, items, n, ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            load().cr_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self, stream: int = 0):
        check(load().cr_batch_render(self._h, stream or None))

    def render_cached(self, caches, query_vertex=1, train_every=0, train_samples=8192, train_steps=1,
                      freeze=False):
        """The batch with the radiance cache: scene i renders its spp cached
        frames with its own network caches[i] (RadianceCache); returns one
        stats dict per scene (cr_batch_render_cached)."""
        from ._lib import CrCacheConfig, CrCacheStats
        n = len(self.scenes)
        if len(caches) != n:
            raise ValueError(f"{len(caches)} networks for {n} scenes")
        nets = (ctypes.c_void_p * n)(*[c.handle.value for c in caches])
        cc = CrCacheConfig(query_vertex, train_every, train_samples, train_steps, 1 if freeze else 0)
        stats = (CrCacheStats * n)()
        check(load().cr_batch_render_cached(self._h, nets, ctypes.byref(cc), stats))
        return [{"frames": st.frames, "queries": st.queries, "train_records": st.train_records,
                 "last_loss": st.last_loss, "last_train_every": st.last_train_every} for st in stats]

    def set_tuning(self, tile=16, spp_per_item=4, blocks_per_sm=0, wave_log2=0):
        """wave_log2 = 0: the persistent megakernel with (tile, spp_per_item,
        blocks_per_sm); 16..25: the wavefront in waves of 2^wave_log2 paths."""
        from ._lib import CrBatchTuning
        t = CrBatchTuning(tile, spp_per_item, blocks_per_sm, wave_log2)
        check(load().cr_batch_set_tuning(self._h, ctypes.byref(t)))

    def tuning(self) -> dict:
        from ._lib import CrBatchTuning
        t = CrBatchTuning()
        check(load().cr_batch_get_tuning(self._h, ctypes.byref(t)))
        return {"tile": t.tile, "spp_per_item": t.spp_per_item, "blocks_per_sm": t.blocks_per_sm,
                "wave_log2": t.wave_log2}

    def autotune(self, json_path: str = None) -> dict:
        """Times every tuning on this batch, keeps the fastest (films are
        cleared afterwards); optionally writes the table as JSON."""
        from ._lib import CrBatchTuning, CrBatchTuningResult
        best = CrBatchTuning()
        res = (CrBatchTuningResult * 32)()
        n = ctypes.c_uint32()
        check(load().cr_batch_autotune(self._h, ctypes.byref(best), res, 32, ctypes.byref(n)))
        out = {"best": {"tile": best.tile, "spp_per_item": best.spp_per_item, "wave_log2": best.wave_log2},
               "timings_ms": [{"tile": res[i].tuning.tile, "spp_per_item": res[i].tuning.spp_per_item,
                               "wave_log2": res[i].tuning.wave_log2, "ms": round(res[i].ms, 4)}
                              for i in range(n.value)]}
        if json_path:
            import json
            with open(json_path, "w") as f:
                json.dump(out, f, indent=1)
        return out


class Image:
    """Utils/Image.h: an image of float pixels, held as an HxWxC array (the
    reference keeps one plane per channel; the pixel values are the same)."""

    def __init__(self, width: int = 0, height: int = 0, channels: int = 3, data: Optional[np.ndarray] = None):
        if data is None:
            data = np.zeros((int(height), int(width), int(channels)), np.float32)
        data = np.asarray(data, np.float32)
        if data.ndim == 2:
            data = data[..., None]
        self.data = np.ascontiguousarray(data)

    def getWidth(self) -> int:
        return self.data.shape[1]

    def getHeight(self) -> int:
        return self.data.shape[0]

    def getChannels(self) -> int:
        return self.data.shape[2]

    def getPixel(self, x: int, y: int, c: int) -> float:
        return float(self.data[y, x, c])

    def setPixel(self, x: int, y: int, c: int, value: float):
        self.data[y, x, c] = value

    def writeEXR(self, path: str):
        """Image::writeEXR, Utils/Image.cpp:49-106."""
        check(load().cr_image_write_exr(path.encode(), self.getWidth(), self.getHeight(), self.getChannels(),
                                        ptr(self.data)))

    def writePNG(self, path: str, gammaCorrect: bool):
        """Image::writePNG, Utils/Image.cpp:182-217."""
        check(load().cr_image_write_png(path.encode(), self.getWidth(), self.getHeight(), self.getChannels(),
                                        ptr(self.data), 1 if gammaCorrect else 0))

    @staticmethod
    def load(path: str, toLinear: bool = True) -> "Image":
        """Image::load, Utils/Image.cpp:262-270."""
        img = _lib.CrImage()
        check(load().cr_image_load(path.encode(), 1 if toLinear else 0, ctypes.byref(img)))
        try:
            n = img.width * img.height * img.channels
            arr = np.ctypeslib.as_array(img.pixels, shape=(n,)).copy() if n else np.zeros(0, np.float32)
        finally:
            load().cr_image_free(ctypes.byref(img))
        return Image(data=arr.reshape(img.height, img.width, img.channels))


def sensor_image(sensor: Sensor) -> Image:
    """Sensor::createImage as an Image (rgb / weight)."""
    return Image(data=np.nan_to_num(sensor.createImage()).astype(np.float32))


class Importer:
    """Utils/Importer.h: an XML file (camera, emissive materials) beside an
    OBJ/MTL file of the same name."""

    def load(self, path: str):
        """The imported SceneData and Camera (host arrays, nothing uploaded)."""
        lib = load()
        h = ctypes.c_void_p()
        check(lib.cr_import_xml(str(path).encode(), ctypes.byref(h)))
        try:
            v = _lib.CrImportView()
            check(lib.cr_import_get(h, ctypes.byref(v)))
            nv, nt = v.n_vertices, v.n_tris

            def arr(p, n, dt):
                return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True) if n else np.zeros(0, dt)

            pos = arr(v.pos, 3 * nv, np.float32).reshape(-1, 3)
            nrm = arr(v.nrm, 3 * nv, np.float32).reshape(-1, 3)
            uv = arr(v.uv, 2 * nv, np.float32).reshape(-1, 2)
            idx = arr(v.idx, 3 * nt, np.uint32)
            descs = (np.frombuffer(ctypes.string_at(v.meshes, v.n_meshes * MESH_DTYPE.itemsize), MESH_DTYPE).copy()
                     if v.n_meshes else np.zeros(0, MESH_DTYPE))
            mats = (np.frombuffer(ctypes.string_at(v.mats, v.n_mats * MATERIAL_DTYPE.itemsize), MATERIAL_DTYPE).copy()
                    if v.n_mats else np.zeros(0, MATERIAL_DTYPE))
            mat_tex = arr(v.material_texture, v.n_mats, np.uint32)
            textures = []
            for t in range(v.n_textures):
                tx = v.textures[t]
                textures.append(np.ctypeslib.as_array(tx.texels, shape=(tx.height * tx.width * 4,))
                                .astype(np.float32, copy=True).reshape(tx.height, tx.width, 4))
            data = SceneData()
            for k, d in enumerate(descs):
                vo = int(d["vertex_offset"])
                ve = int(descs[k + 1]["vertex_offset"]) if k + 1 < len(descs) else nv
                io0, ic = int(d["index_offset"]), int(d["index_count"])
                data.meshes.append(MeshData(position=pos[vo:ve], normal=nrm[vo:ve], texCrd=uv[vo:ve],
                                            index=idx[io0:io0 + ic] - np.uint32(vo), materialID=int(d["material_id"])))
            for k, m in enumerate(mats):
                md = MaterialData(diffuseRefl=tuple(float(x) for x in m["diffuse"]),
                                  specularRefl=tuple(float(x) for x in m["specular"]),
                                  emission=tuple(float(x) for x in m["emission"]), shininess=float(m["shininess"]),
                                  type=MaterialType(int(m["type"])))
                md.name = lib.cr_import_material_name(h, k).decode()
                md.finalize()
                if mat_tex[k] != _lib.CR_NO_TEXTURE:
                    md.flags |= int(MaterialFlags.hasDiffuseTexture)
                    md.diffuseHandle = int(mat_tex[k])
                data.materials.append(md)
            data.emissiveIndex = arr(v.emissive, v.n_emissive, np.uint32).tolist()
            data.textureImages = textures
            c = v.camera
            cam = Camera()
            cam.setWorldPosition(tuple(c.pos))
            cam.setTarget(tuple(c.target))
            cam.setUp(tuple(c.up))
            cam.setFovY(c.fov_y)
            cam.setSensor(Sensor((c.width, c.height)))
            return data, cam
        finally:
            lib.cr_import_destroy(h)

    def import_(self, path: str) -> Scene:
        """Importer::import (Utils/Importer.cpp:203-236): the scene, with its
        camera set."""
        data, cam = self.load(path)
        sc = Scene(data)
        sc.setCamera(cam)
        return sc
