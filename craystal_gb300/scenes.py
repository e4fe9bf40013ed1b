"""Seeded synthetic workloads (the reference ships no scene assets).

cornell_box  -- procedural Cornell box: 5 wall quads in [-1,1]^3 open towards
                +z, two boxes (half heights 0.6 and 0.3) rotated about y by
                U(0, 45 deg), a 0.25 x 0.25 ceiling light of emission 15;
                34 + 2 triangles; grey albedos U(0.2, 0.8) per object,
                Lambertian walls, Phong boxes (exponent 32); fov 40 deg.
random_triangles -- N triangles, centroids U[0,1]^3, vertices c + e_k with
                e_k ~ N(0, 0.01^2) per component.
random_rays  -- origins on the sphere of radius 2 about the origin,
                directions towards U[0,1]^3, tmin 1e-4, tmax +inf.
"""
import math

import numpy as np

from ._lib import RAY_DTYPE
from .api import Camera, MaterialData, MaterialFlags, MaterialType, MeshData, SceneData, Sensor


def _quad(p0, p1, p2, p3, normal):
    pos = np.array([p0, p1, p2, p3], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3], np.uint32)
    nrm = np.repeat(np.asarray(normal, np.float32)[None], 4, 0)
    return pos, nrm, idx


def _oriented(pos, idx, inward_point):
    """Flips triangles whose geometric normal points away from inward_point,
    and returns per-vertex face normals (flat shading)."""
    idx = idx.copy().reshape(-1, 3)
    out_pos, out_nrm, out_idx = [], [], []
    for t in idx:
        v = pos[t]
        n = np.cross(v[1] - v[0], v[2] - v[0])
        c = v.mean(0)
        if np.dot(n, np.asarray(inward_point) - c) < 0:
            t = t[[0, 2, 1]]
            v = pos[t]
            n = -n
        n = n / np.linalg.norm(n)
        base = len(out_pos) * 3
        out_pos.append(v)
        out_nrm.append(np.repeat(n[None], 3, 0))
        out_idx.append(np.arange(base, base + 3))
    return (np.concatenate(out_pos).astype(np.float32), np.concatenate(out_nrm).astype(np.float32),
            np.concatenate(out_idx).astype(np.uint32))


def _box(center, half, angle):
    cx, cy, cz = center
    hx, hy, hz = half
    corners = []
    for sx in (-1, 1):
        for sy in (-1, 1):
            for sz in (-1, 1):
                x, z = sx * hx, sz * hz
                ca, sa = math.cos(angle), math.sin(angle)
                corners.append((cx + ca * x + sa * z, cy + sy * hy, cz - sa * x + ca * z))
    c = np.array(corners, np.float64)
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    tris = []
    for a, b, cc, d in faces:
        tris += [(a, b, cc), (a, cc, d)]
    idx = np.array(tris, np.uint32).reshape(-1)
    # orient outward: flip so that normals point away from the center
    idx3 = idx.reshape(-1, 3).copy()
    pos, nrm, out = [], [], []
    for t in idx3:
        v = c[t]
        n = np.cross(v[1] - v[0], v[2] - v[0])
        if np.dot(n, v.mean(0) - np.array(center)) < 0:
            t = t[[0, 2, 1]]
            v = c[t]
            n = -n
        n /= np.linalg.norm(n)
        base = len(pos) * 3
        pos.append(v)
        nrm.append(np.repeat(n[None], 3, 0))
        out.append(np.arange(base, base + 3))
    return (np.concatenate(pos).astype(np.float32), np.concatenate(nrm).astype(np.float32),
            np.concatenate(out).astype(np.uint32))


def cornell_box(seed: int = 0, width: int = 256, height: int = 256):
    """Returns (SceneData, Camera) of the procedural Cornell box."""
    rng = np.random.default_rng(seed)
    meshes, mats = [], []
    walls = [
        ((-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1)),   # floor
        ((-1, 1, -1), (-1, 1, 1), (1, 1, 1), (1, 1, -1)),       # ceiling
        ((-1, -1, -1), (-1, 1, -1), (1, 1, -1), (1, -1, -1)),   # back
        ((-1, -1, -1), (-1, -1, 1), (-1, 1, 1), (-1, 1, -1)),   # left
        ((1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1)),       # right
    ]
    for quad in walls:
        pos = np.array(quad, np.float32)
        p, n, i = _oriented(pos, np.array([0, 1, 2, 0, 2, 3], np.uint32), (0.0, 0.0, 0.0))
        a = float(rng.uniform(0.2, 0.8))
        mats.append(MaterialData(diffuseRefl=(a, a, a), type=MaterialType.FullDiffuse))
        meshes.append(MeshData(position=p, normal=n, index=i, materialID=len(mats) - 1))
    for center, half in (((-0.35, -1.0 + 0.6 + 1e-4, -0.3), (0.3, 0.6, 0.3)),
                         ((0.4, -1.0 + 0.3 + 1e-4, 0.3), (0.3, 0.3, 0.3))):
        ang = float(rng.uniform(0.0, math.pi / 4))
        p, n, i = _box(center, half, ang)
        a = float(rng.uniform(0.2, 0.8))
        mats.append(MaterialData(diffuseRefl=(a, a, a), specularRefl=(0.1, 0.1, 0.1), shininess=32.0,
                                 type=MaterialType.Phong))
        meshes.append(MeshData(position=p, normal=n, index=i, materialID=len(mats) - 1))
    y = 1.0 - 1e-3
    lp = np.array([(-0.125, y, -0.125), (0.125, y, -0.125), (0.125, y, 0.125), (-0.125, y, 0.125)], np.float32)
    p, n, i = _oriented(lp, np.array([0, 1, 2, 0, 2, 3], np.uint32), (0.0, -1.0, 0.0))
    mats.append(MaterialData(emission=(15.0, 15.0, 15.0), type=MaterialType.FullDiffuse))
    meshes.append(MeshData(position=p, normal=n, index=i, materialID=len(mats) - 1))
    for m in mats:
        m.finalize()
    n_tris = sum(len(m.index) // 3 for m in meshes)
    data = SceneData(meshes=meshes, materials=mats, emissiveIndex=[n_tris - 2, n_tris - 1])
    cam = Camera()
    cam.setWorldPosition((0.0, 0.0, 3.9))
    cam.setTarget((0.0, 0.0, 0.0))
    cam.setUp((0.0, 1.0, 0.0))
    cam.setFovY(40.0)
    cam.setSensor(Sensor((width, height)))
    return data, cam


def textured_cornell_box(seed: int = 0, width: int = 256, height: int = 256, tex_res: int = 64):
    """The Cornell box with two diffuse textures: a checkerboard on the floor
    (Phong, so its lobe probabilities follow the texel) and a colour ramp on
    the back wall (Lambertian).  The planar texture coordinates run over
    [-0.1, 1.1], so the edge clamp and the extrapolation below 0 are used."""
    data, cam = cornell_box(seed, width, height)
    rng = np.random.default_rng(seed + 1000)
    k = np.arange(tex_res)
    checker = ((k[:, None] // 8 + k[None, :] // 8) % 2).astype(np.float32)
    floor_tex = np.stack([0.15 + 0.7 * checker, 0.15 + 0.6 * checker, 0.1 + 0.5 * (1 - checker)], -1)
    ramp = np.stack(np.meshgrid(np.linspace(0.1, 0.9, tex_res), np.linspace(0.9, 0.1, tex_res // 2)), -1)
    wall_tex = np.concatenate([ramp, rng.uniform(0.2, 0.6, (tex_res // 2, tex_res, 1))], -1).astype(np.float32)
    data.textureImages = [floor_tex, wall_tex]
    for mesh_id, axes, tex in ((0, (0, 2), 0), (2, (0, 1), 1)):
        mesh = data.meshes[mesh_id]
        p = np.asarray(mesh.position, np.float32)
        mesh.texCrd = (-0.1 + 1.2 * (p[:, list(axes)] + 1.0) / 2.0).astype(np.float32)
        m = data.materials[mesh.materialID]
        m.diffuseHandle = tex
        m.flags |= int(MaterialFlags.hasDiffuseTexture)
        if tex == 0:
            m.type = MaterialType.Phong
            m.specularRefl = (0.3, 0.3, 0.3)
            m.shininess = 20.0
            m.flags &= ~int(MaterialFlags.IsDiffuse)
    return data, cam


def random_triangles(n: int, seed: int = 0):
    """Positions (3n x 3 float32) and indices (3n uint32) of n random triangles."""
    rng = np.random.default_rng(seed)
    c = rng.random((n, 1, 3), dtype=np.float64)
    e = rng.normal(0.0, 0.01, size=(n, 3, 3))
    pos = (c + e).astype(np.float32).reshape(-1, 3)
    idx = np.arange(3 * n, dtype=np.uint32)
    return pos, idx


def random_triangle_scene(n: int, seed: int = 0) -> SceneData:
    pos, idx = random_triangles(n, seed)
    mat = MaterialData(diffuseRefl=(0.5, 0.5, 0.5), type=MaterialType.FullDiffuse)
    mat.finalize()
    return SceneData(meshes=[MeshData(position=pos, index=idx, materialID=0)], materials=[mat], emissiveIndex=[])


def random_rays(n: int, seed: int = 1, tmin: float = 1e-4) -> np.ndarray:
    rng = np.random.default_rng(seed)
    rays = np.empty(n, RAY_DTYPE)
    chunk = 1 << 22
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        o = rng.normal(size=(m, 3))
        o *= 2.0 / np.linalg.norm(o, axis=1, keepdims=True)
        p = rng.random((m, 3))
        d = p - o
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rays["o"][s:s + m] = o.astype(np.float32)
        rays["d"][s:s + m] = d.astype(np.float32)
    rays["tmin"] = np.float32(tmin)
    rays["tmax"] = np.float32(np.inf)
    return rays


# ---------------------------------------------------------------------------
# radiance-cache scene: displaced icospheres on a ground plane
# ---------------------------------------------------------------------------
def icosphere(level: int):
    """Unit icosphere: vertices (float64) and faces after `level` 4:1 subdivisions."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    for _ in range(level):
        n = len(v)
        e = np.stack([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], 1).reshape(-1, 2)
        es = np.sort(e, 1)
        key = es[:, 0] * n + es[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        i, j = np.divmod(uniq, n)
        mid = v[i] + v[j]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid])
        m = (n + inv).reshape(-1, 3)  # ab, bc, ca
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1), np.stack([c, ca, bc], 1),
                            np.stack([ab, bc, ca], 1)])
    return v, f


def _hash3(ix, iy, iz, seed):
    h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ (iy.astype(np.uint32) * np.uint32(0xD8163841)) ^ \
        (iz.astype(np.uint32) * np.uint32(0xCB1AB31F)) ^ np.uint32(seed * 0x9E3779B1 & 0xFFFFFFFF)
    h ^= h >> np.uint32(16)
    h *= np.uint32(0x7FEB352D)
    h ^= h >> np.uint32(15)
    h *= np.uint32(0x846CA68B)
    h ^= h >> np.uint32(16)
    return (h >> np.uint32(8)).astype(np.float64) / 16777216.0


def value_noise(p, seed=0):
    """3D value noise in [0, 1]: hashed lattice values, smoothstep-trilinear."""
    fl = np.floor(p)
    fr = p - fl
    w = fr * fr * (3.0 - 2.0 * fr)
    i = fl.astype(np.int64)
    out = 0.0
    with np.errstate(over="ignore"):
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    val = _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
                    wx = w[:, 0] if dx else 1.0 - w[:, 0]
                    wy = w[:, 1] if dy else 1.0 - w[:, 1]
                    wz = w[:, 2] if dz else 1.0 - w[:, 2]
                    out = out + val * wx * wy * wz
    return out


def vertex_normals(pos, faces):
    fn = np.cross(pos[faces[:, 1]] - pos[faces[:, 0]], pos[faces[:, 2]] - pos[faces[:, 0]])
    vn = np.zeros_like(pos)
    for k in range(3):
        np.add.at(vn, faces[:, k], fn)
    return vn / np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-20)


def cache_scene(seed: int = 0, width: int = 1920, height: int = 1080, level: int = 7):
    """Returns (SceneData, Camera, environment, sphere_lights) of the radiance-cache
    workload: 8 displaced icospheres (20 * 4^level triangles each; level 7 gives
    2,621,440 in all) with Principled materials on a 2-triangle ground plane,
    a constant environment of 0.5 and one sphere light."""
    rng = np.random.default_rng(seed)
    base_v, base_f = icosphere(level)
    meshes, mats = [], []
    centers = [(x, z) for z in (-1.2, 1.2) for x in (-3.6, -1.2, 1.2, 3.6)]
    for k, (cx, cz) in enumerate(centers):
        disp = 1.0 + 0.05 * value_noise(base_v * 4.0 + 17.0 * k, seed)
        r = 0.9
        pos = base_v * (r * disp)[:, None] + np.array([cx, r, cz])
        mats.append(MaterialData(diffuseRefl=tuple(float(c) for c in rng.uniform(0.0, 1.0, 3)),
                                 specularRefl=(1.0, 1.0, 1.0) if rng.random() < 0.3 else (0.0, 0.0, 0.0),
                                 type=MaterialType.Principled))
        rough = float(rng.uniform(0.05, 1.0))
        mats[-1].shininess = 2.0 / (rough * rough) - 1.0  # PrincipledBRDF.cu:51-55: r = sqrt(2 / (s + 1))
        meshes.append(MeshData(position=pos.astype(np.float32), normal=vertex_normals(pos, base_f).astype(np.float32),
                               index=base_f.astype(np.uint32).reshape(-1), materialID=len(mats) - 1))
    g = 20.0
    gp = np.array([[-g, 0, -g], [g, 0, -g], [g, 0, g], [-g, 0, g]], np.float32)
    mats.append(MaterialData(diffuseRefl=(0.5, 0.5, 0.5), type=MaterialType.FullDiffuse))
    meshes.append(MeshData(position=gp, normal=np.tile(np.float32([0, 1, 0]), (4, 1)),
                           index=np.array([0, 2, 1, 0, 3, 2], np.uint32), materialID=len(mats) - 1))
    for m in mats:
        m.finalize()
    data = SceneData(meshes=meshes, materials=mats, emissiveIndex=[])
    cam = Camera()
    cam.setWorldPosition((0.0, 3.2, 8.5))
    cam.setTarget((0.0, 0.6, 0.0))
    cam.setUp((0.0, 1.0, 0.0))
    cam.setFovY(40.0)
    cam.setSensor(Sensor((width, height)))
    env = (0.5, 0.5, 0.5)
    spheres = [((2.5, 6.0, 3.0), 1.0, (40.0, 38.0, 34.0))]
    return data, cam, env, spheres


# ---------------------------------------------------------------------------
# batched workload: random-box clutter scenes of uneven size
# ---------------------------------------------------------------------------
_FACE_AXES = [(0, 1, 2, 1.0), (0, 1, 2, -1.0), (1, 2, 0, 1.0), (1, 2, 0, -1.0), (2, 0, 1, 1.0), (2, 0, 1, -1.0)]


def _boxes(centers, half, angles):
    """24 vertices (4 per face, flat normals) and 12 triangles per box."""
    nb = len(centers)
    pos = np.empty((nb, 24, 3))
    nrm = np.empty((nb, 24, 3))
    quad = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], np.float64)
    for f, (u, v, w, sgn) in enumerate(_FACE_AXES):
        local = np.zeros((4, 3))
        local[:, u] = quad[:, 0]
        local[:, v] = quad[:, 1] * sgn
        local[:, w] = sgn
        n = np.zeros(3)
        n[w] = sgn
        pos[:, 4 * f:4 * f + 4] = local[None] * half[:, None, :]
        nrm[:, 4 * f:4 * f + 4] = n
    ca, sa = np.cos(angles)[:, None], np.sin(angles)[:, None]
    x, z = pos[..., 0].copy(), pos[..., 2].copy()
    pos[..., 0], pos[..., 2] = ca * x + sa * z, -sa * x + ca * z
    nx, nz = nrm[..., 0].copy(), nrm[..., 2].copy()
    nrm[..., 0], nrm[..., 2] = ca * nx + sa * nz, -sa * nx + ca * nz
    pos += centers[:, None, :]
    tri = np.array([[0, 1, 2], [0, 2, 3]])
    idx = (np.arange(6)[:, None, None] * 4 + tri[None]).reshape(-1, 3)  # 12 x 3 per box
    idx = (np.arange(nb)[:, None, None] * 24 + idx[None]).reshape(-1)
    return pos.reshape(-1, 3), nrm.reshape(-1, 3), idx


def box_clutter(seed: int = 0, n_tris: int = 100000, width: int = 256, height: int = 256, n_materials: int = 6):
    """Returns (SceneData, Camera): about n_tris / 12 boxes (scale log-uniform
    0.05 - 0.6, rotated about y) on a ground quad, lit by a 3 x 3 emissive
    ceiling quad; materials drawn from Lambertian / Phong / Principled."""
    rng = np.random.default_rng(seed)
    nb = max(1, n_tris // 12)
    centers = np.stack([rng.uniform(-5, 5, nb), np.zeros(nb), rng.uniform(-5, 5, nb)], 1)
    half = np.exp(rng.uniform(np.log(0.05), np.log(0.6), (nb, 1))) * rng.uniform(0.6, 1.4, (nb, 3))
    centers[:, 1] = half[:, 1] + rng.uniform(0, 2.5, nb) * (rng.random(nb) < 0.3)
    pos, nrm, idx = _boxes(centers, half, rng.uniform(0, np.pi / 2, nb))
    mat_of_box = rng.integers(0, n_materials, nb)
    meshes, mats = [], []
    for m in range(n_materials):
        sel = np.flatnonzero(mat_of_box == m)
        if len(sel) == 0:
            continue
        vsel = (sel[:, None] * 24 + np.arange(24)[None]).reshape(-1)
        remap = np.full(len(pos), -1, np.int64)
        remap[vsel] = np.arange(len(vsel))
        isel = (sel[:, None] * 36 + np.arange(36)[None]).reshape(-1)
        kind = m % 3
        kd = tuple(float(c) for c in rng.uniform(0.1, 0.9, 3))
        if kind == 0:
            md = MaterialData(diffuseRefl=kd, type=MaterialType.FullDiffuse)
        elif kind == 1:
            md = MaterialData(diffuseRefl=kd, specularRefl=(0.15, 0.15, 0.15), shininess=float(rng.uniform(8, 64)),
                              type=MaterialType.Phong)
        else:
            md = MaterialData(diffuseRefl=kd, specularRefl=(0.5, 0.5, 0.5) if rng.random() < 0.3 else (0.0, 0.0, 0.0),
                              shininess=float(rng.uniform(1, 100)), type=MaterialType.Principled)
        mats.append(md)
        meshes.append(MeshData(position=pos[vsel].astype(np.float32), normal=nrm[vsel].astype(np.float32),
                               index=remap[idx[isel]].astype(np.uint32), materialID=len(mats) - 1))
    g = 8.0
    mats.append(MaterialData(diffuseRefl=(0.5, 0.5, 0.5), type=MaterialType.FullDiffuse))
    meshes.append(MeshData(position=np.array([[-g, 0, -g], [g, 0, -g], [g, 0, g], [-g, 0, g]], np.float32),
                           normal=np.tile(np.float32([0, 1, 0]), (4, 1)), index=np.array([0, 2, 1, 0, 3, 2], np.uint32),
                           materialID=len(mats) - 1))
    y = 6.0
    mats.append(MaterialData(emission=(8.0, 8.0, 8.0), type=MaterialType.FullDiffuse))
    meshes.append(MeshData(position=np.array([[-1.5, y, -1.5], [1.5, y, -1.5], [1.5, y, 1.5], [-1.5, y, 1.5]],
                                             np.float32),
                           normal=np.tile(np.float32([0, -1, 0]), (4, 1)), index=np.array([0, 1, 2, 0, 2, 3], np.uint32),
                           materialID=len(mats) - 1))
    for m in mats:
        m.finalize()
    n_total = sum(len(m.index) // 3 for m in meshes)
    data = SceneData(meshes=meshes, materials=mats, emissiveIndex=[n_total - 2, n_total - 1])
    cam = Camera()
    cam.setWorldPosition((0.0, 4.0, 12.0))
    cam.setTarget((0.0, 0.5, 0.0))
    cam.setUp((0.0, 1.0, 0.0))
    cam.setFovY(50.0)
    cam.setSensor(Sensor((width, height)))
    return data, cam


def batch_workload(n_scenes: int = 64, seed: int = 0):
    """Per-scene parameters of the batched workload: triangles log-uniform in
    [10k, 500k], square resolution from {128, 256, 512, 1024}, spp
    log-uniform in [4, 256], max depth uniform in {8..16}; scene i uses seed i."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_scenes):
        out.append({"seed": i, "tris": int(np.exp(rng.uniform(np.log(10e3), np.log(500e3)))),
                    "res": int(rng.choice([128, 256, 512, 1024])),
                    "spp": int(round(np.exp(rng.uniform(np.log(4), np.log(256))))),
                    "depth": int(rng.integers(8, 17))})
    return out


def export_obj_scene(data: SceneData, cam: Camera, xml_path: str) -> str:
    """Writes a scene as the importer reads it: <name>.xml (camera, one
    <light> per emissive material), <name>.obj (one object per mesh) and
    <name>.mtl (Kd, Ks, Ns; map_Kd to an 8-bit PNG per texture).  Emission
    goes through the XML, as the reference's scene files carry it."""
    import os

    from .api import Image
    base = os.path.splitext(str(xml_path))[0]
    stem = os.path.basename(base)
    folder = os.path.dirname(base)
    tex_names = []
    for t, img in enumerate(data.textureImages):
        name = f"{stem}_tex{t}.png"
        a = np.asarray(img, np.float32)
        # rows are stored bottom-up after loading, so write them top-down
        Image(data=a[::-1, :, :3] if a.ndim == 3 else a[::-1]).writePNG(os.path.join(folder, name), False)
        tex_names.append(name)
    with open(base + ".mtl", "w") as f:
        for k, m in enumerate(data.materials):
            f.write(f"newmtl mat{k}\n")
            f.write("Kd {:.9g} {:.9g} {:.9g}\n".format(*m.diffuseRefl))
            f.write("Ks {:.9g} {:.9g} {:.9g}\n".format(*m.specularRefl))
            f.write(f"Ns {m.shininess:.9g}\n")
            if m.flags & MaterialFlags.hasDiffuseTexture:
                f.write(f"map_Kd {tex_names[m.diffuseHandle]}\n")
    with open(base + ".obj", "w") as f:
        f.write(f"mtllib {stem}.mtl\n")
        nv = 0
        for k, mesh in enumerate(data.meshes):
            p = np.asarray(mesh.position, np.float32).reshape(-1, 3)
            n = None if mesh.normal is None else np.asarray(mesh.normal, np.float32).reshape(-1, 3)
            t = None if mesh.texCrd is None else np.asarray(mesh.texCrd, np.float32).reshape(-1, 2)
            f.write(f"o mesh{k}\nusemtl mat{mesh.materialID}\n")
            for v in p:
                f.write("v {:.9g} {:.9g} {:.9g}\n".format(*v))
            if n is not None:
                for v in n:
                    f.write("vn {:.9g} {:.9g} {:.9g}\n".format(*v))
            if t is not None:
                for v in t:
                    f.write("vt {:.9g} {:.9g}\n".format(*v))
            for tri in np.asarray(mesh.index, np.int64).reshape(-1, 3) + 1 + nv:
                if n is not None and t is not None:
                    f.write("f " + " ".join(f"{i}/{i}/{i}" for i in tri) + "\n")
                elif n is not None:
                    f.write("f " + " ".join(f"{i}//{i}" for i in tri) + "\n")
                elif t is not None:
                    f.write("f " + " ".join(f"{i}/{i}" for i in tri) + "\n")
                else:
                    f.write("f " + " ".join(str(i) for i in tri) + "\n")
            nv += len(p)
    w, h = cam.sensor.size if cam.sensor else (512, 512)
    with open(base + ".xml", "w") as f:
        f.write('<?xml version="1.0" encoding="utf-8"?>\n')
        f.write(f'<camera type="perspective" width="{w}" height="{h}" fovy="{cam.fovY:.9g}">\n')
        for tag, v in (("eye", cam.posW), ("lookat", cam.target), ("up", cam.up)):
            f.write(f'  <{tag} x="{v[0]:.9g}" y="{v[1]:.9g}" z="{v[2]:.9g}"/>\n')
        f.write("</camera>\n")
        for k, m in enumerate(data.materials):
            if max(m.emission) != 0.0:
                f.write(f'<light mtlname="mat{k}" radiance="{m.emission[0]:.9g},{m.emission[1]:.9g},'
                        f'{m.emission[2]:.9g}"/>\n')
    return base + ".xml"


def _fbm_grid(n: int, octaves: int, seed: int, base_res: int = 8) -> np.ndarray:
    """fBm of 2D value noise sampled on an n x n grid over the unit square:
    octave o has a (base_res 2^o + 1)^2 lattice of uniform values, smoothstep-
    bilinear interpolation, amplitude 2^-o; result normalised to [0, 1]."""
    rng = np.random.default_rng(seed)
    t = np.linspace(0.0, 1.0, n, dtype=np.float64)
    h = np.zeros((n, n), np.float32)
    for o in range(octaves):
        res = base_res << o
        lat = rng.random((res + 1, res + 1)).astype(np.float32)
        x = t * res
        i0 = np.minimum(np.floor(x).astype(np.int64), res - 1)
        f = (x - i0).astype(np.float32)
        w1 = f * f * (3.0 - 2.0 * f)
        w0 = 1.0 - w1
        amp = np.float32(0.5 ** o)
        h += amp * (lat[np.ix_(i0, i0)] * (w0[:, None] * w0[None, :]) +
                    lat[np.ix_(i0 + 1, i0)] * (w1[:, None] * w0[None, :]) +
                    lat[np.ix_(i0, i0 + 1)] * (w0[:, None] * w1[None, :]) +
                    lat[np.ix_(i0 + 1, i0 + 1)] * (w1[:, None] * w1[None, :]))
    h -= h.min()
    h /= max(float(h.max()), 1e-6)
    return h


def _box_soup(centers, halves, angles):
    """Vectorised boxes: 12 outward-facing triangles per box with flat normals
    (positions, normals: (36 n) x 3; indices 0 .. 36 n - 1)."""
    corners = np.array([[sx, sy, sz] for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)], np.float64)
    quads = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    tri = []
    for a, b, c, d in quads:
        tri += [(a, b, c), (a, c, d)]
    tri = np.array(tri)
    local = corners[tri]                                    # 12 x 3 x 3 (unit cube corners)
    n0 = np.cross(local[:, 1] - local[:, 0], local[:, 2] - local[:, 0])
    flip = (n0 * local.mean(1)).sum(1) < 0                  # orient outward
    local[flip] = local[flip][:, [0, 2, 1]]
    p = local[None] * halves[:, None, None, :]              # n x 12 x 3 x 3
    ca, sa = np.cos(angles)[:, None, None], np.sin(angles)[:, None, None]
    x, z = p[..., 0].copy(), p[..., 2].copy()
    p[..., 0] = ca * x + sa * z
    p[..., 2] = -sa * x + ca * z
    p += centers[:, None, None, :]
    nrm = np.cross(p[:, :, 1] - p[:, :, 0], p[:, :, 2] - p[:, :, 0])
    nrm /= np.linalg.norm(nrm, axis=-1, keepdims=True)
    pos = p.reshape(-1, 3).astype(np.float32)
    nrm = np.repeat(nrm[:, :, None, :], 3, axis=2).reshape(-1, 3).astype(np.float32)
    return pos, nrm, np.arange(len(pos), dtype=np.uint32)


def large_terrain_scene(width: int = 3840, height: int = 2160, grid: int = 4096, n_boxes: int = 10000,
                        seed: int = 7, extent: float = 200.0, relief: float = 25.0):
    """Returns (SceneData, Camera, environment, sphere_lights) of the large
    workload: a grid x grid heightfield (2 (grid - 1)^2 triangles; 33.5M for
    4096) of 6-octave fBm heights over [-extent/2, extent/2]^2, 10k boxes of
    scale log-uniform 0.5-20 standing on it, Principled materials, a sun
    sphere light and a constant sky."""
    rng = np.random.default_rng(seed)
    h = _fbm_grid(grid, 6, seed) * np.float32(relief)
    t = np.linspace(-extent / 2, extent / 2, grid, dtype=np.float32)
    xx, zz = np.meshgrid(t, t, indexing="ij")
    pos = np.stack([xx, h, zz], -1).reshape(-1, 3)
    dh_x = np.gradient(h, t, axis=0)
    dh_z = np.gradient(h, t, axis=1)
    nrm = np.stack([-dh_x, np.ones_like(h), -dh_z], -1).reshape(-1, 3)
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    i = np.arange(grid - 1, dtype=np.uint32)
    v00 = (i[:, None] * grid + i[None, :]).reshape(-1)
    v10, v01, v11 = v00 + grid, v00 + 1, v00 + grid + 1
    idx = np.empty((len(v00), 2, 3), np.uint32)
    idx[:, 0] = np.stack([v00, v01, v11], -1)  # normals point up (+y)
    idx[:, 1] = np.stack([v00, v11, v10], -1)
    mats = [MaterialData(diffuseRefl=(0.42, 0.38, 0.30), specularRefl=(0.04, 0.04, 0.04), shininess=3.0,
                         type=MaterialType.Principled)]
    meshes = [MeshData(position=pos.astype(np.float32), normal=nrm.astype(np.float32), index=idx.reshape(-1),
                       materialID=0)]
    # boxes on the terrain, in 4 material groups
    cx = rng.uniform(-extent * 0.45, extent * 0.45, n_boxes)
    cz = rng.uniform(-extent * 0.45, extent * 0.45, n_boxes)
    scale = np.exp(rng.uniform(np.log(0.5), np.log(20.0), n_boxes))
    halves = scale[:, None] * rng.uniform(0.3, 1.0, (n_boxes, 3)) * 0.5
    gi = np.clip(((cx + extent / 2) / extent * (grid - 1)).astype(np.int64), 0, grid - 1)
    gj = np.clip(((cz + extent / 2) / extent * (grid - 1)).astype(np.int64), 0, grid - 1)
    centers = np.stack([cx, h[gi, gj] + halves[:, 1] * 0.9, cz], -1)
    angles = rng.uniform(0.0, np.pi / 2, n_boxes)
    group = rng.integers(0, 4, n_boxes)
    for g in range(4):
        base = rng.uniform(0.2, 0.9, 3)
        metal = g == 3
        mats.append(MaterialData(diffuseRefl=tuple(base), specularRefl=(0.9, 0.9, 0.9) if metal else (0.04,) * 3,
                                 shininess=float(rng.uniform(5, 200)), type=MaterialType.Principled))
        sel = group == g
        p, n, ix = _box_soup(centers[sel], halves[sel], angles[sel])
        meshes.append(MeshData(position=p, normal=n, index=ix, materialID=len(mats) - 1))
    for m in mats:
        m.finalize()
    cam = Camera()
    cam.setWorldPosition((-extent * 0.42, relief * 2.2, -extent * 0.42))
    cam.setTarget((0.0, relief * 0.3, 0.0))
    cam.setUp((0.0, 1.0, 0.0))
    cam.setFovY(50.0)
    cam.setSensor(Sensor((width, height)))
    env = (0.35, 0.45, 0.65)
    sun = [((extent * 2.0, extent * 3.0, extent * 1.0), extent * 0.12, (60.0, 55.0, 45.0))]
    return SceneData(meshes=meshes, materials=mats, emissiveIndex=[]), cam, env, sun
