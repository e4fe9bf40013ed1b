// cr_core.cu -- C ABI plumbing: errors, scene lifetime, camera, film.

#include <cstdarg>
#include <cstring>

#include "cr_internal.cuh"
#include "cr_math.cuh"
#include "cr_traverse.cuh"

namespace cr {
namespace {
thread_local std::string gError;
std::atomic<uint64_t> gLaunches{0};
}  // namespace

void setError(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    gError = buf;
}

void clearError() { gError.clear(); }

int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    gError = buf;
    return code;
}

void countLaunch(uint64_t n) { gLaunches.fetch_add(n, std::memory_order_relaxed); }

// Reads the scene's device error word and, when a bit is set, clears it and
// returns CR_ERR_DEVICE: each error a kernel raises is reported by exactly
// one call.  The caller has waited for the work whose errors it reports.
int takeDeviceErrors(cr_scene* s, const char* what) {
    uint32_t err = 0;
    CR_CUDA(cudaMemcpy(&err, s->errFlags, sizeof(err), cudaMemcpyDeviceToHost));
    if (!err) return CR_OK;
    CR_CUDA(cudaMemset(s->errFlags, 0, sizeof(err)));
    return fail(CR_ERR_DEVICE, "%s: device error flags 0x%x%s", what, err,
                (err & kErrStackOverflow) ? " (traversal stack overflow)" : "");
}

namespace {

// MaterialData::finalize (Core/Material.h:57-65) and the per-material part
// of the BSDF constructors (Material/PhongBRDF.cu:10-18,
// Material/PrincipledBRDF.cu:35-55).
MaterialGpu deriveMaterial(const cr_material& m) {
    MaterialGpu g;
    std::memset(&g, 0, sizeof(g));
    for (int k = 0; k < 3; k++) {
        g.kd[k] = m.diffuse[k];
        g.ks[k] = m.specular[k];
        g.em[k] = m.emission[k];
    }
    g.shininess = m.shininess;
    g.type = m.type;
    g.flags = m.flags;
    const Spec kd = sp(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
    const Spec ks = sp(m.specular[0], m.specular[1], m.specular[2]);
    const Spec em = sp(m.emission[0], m.emission[1], m.emission[2]);
    if (maxValue(em) != 0.0f) g.flags |= CR_MATERIAL_EMISSIVE;
    if (maxValue(ks) == 0.0f) g.flags |= CR_MATERIAL_DIFFUSE_ONLY;
    g.tex = CR_NO_TEXTURE;
    if (m.type == CR_MATERIAL_PHONG) {
        phongLobeProbs(kd, ks, kEps, g.dProb, g.sProb);
    } else if (m.type == CR_MATERIAL_PRINCIPLED) {
        float r = sqrtf(2.0f / (m.shininess + 1.0f));
        float met = averageValue(ks);
        g.rough = r < 0.0f ? 0.0f : (1.0f < r ? 1.0f : r);
        g.metal = met < 0.0f ? 0.0f : (1.0f < met ? 1.0f : met);
        float spr = 0.1f * (1.0f - g.metal) + 1.0f * g.metal;
        float d = 1.0f, s = spr;
        d /= (d + s);
        s /= (d + s);  // uses the updated d, as PrincipledBRDF.cu:47-48 does
        g.dProb = d;
        g.sProb = s;
    } else {
        g.dProb = 1.0f;
        g.sProb = 0.0f;
    }
    return g;
}

template <class T>
int upload(T** dst, const T* src, size_t n) {
    CR_CUDA(cudaMalloc(dst, std::max<size_t>(n, 1) * sizeof(T)));
    if (n) CR_CUDA(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return CR_OK;
}

void freeScene(cr_scene* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    void* ptrs[] = {s->pos,  s->nrm,      s->uv,         s->idx,        s->primToMesh, s->meshes,
                    s->mats, s->emissive, s->pairs,      s->leaves,     s->tris,       s->slotToPrim,
                    s->buildNodes, s->errFlags, s->filmRgb, s->filmW, s->rayCounter, s->spheres, s->sphereEm,
                    s->texels, s->texDescs, s->sphGeom, s->sphMat, s->sphPairs, s->sphLeaves, s->sphBlocks,
                    s->groupPairs};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    freeCacheBuffers(s->cacheBuffers);
    freeWavefrontBuffers(s->wfBuffers);
    for (int k = 0; k < 2; k++) {
        if (s->stageRays[k]) cudaFree(s->stageRays[k]);
        if (s->stageHits[k]) cudaFree(s->stageHits[k]);
        if (s->stageOcc[k]) cudaFree(s->stageOcc[k]);
        if (s->streams[k]) cudaStreamDestroy(s->streams[k]);
    }
    delete s;
}

int createScene(const float* pos, const float* nrm, const float* uv, uint64_t nv, const uint32_t* idx, uint64_t nt,
                const cr_mesh_desc* meshes, uint32_t nMeshes, const cr_material* mats, uint32_t nMats,
                const uint32_t* emissive, uint32_t nEmissive, cr_scene* s) {
    if (nv && !pos) return fail(CR_ERR_INVALID_ARGUMENT, "positions are NULL");
    if (nt && !idx) return fail(CR_ERR_INVALID_ARGUMENT, "indices are NULL");
    if (nt && (!meshes || nMeshes == 0)) return fail(CR_ERR_INVALID_ARGUMENT, "triangles need at least one mesh");
    if (nMeshes && (!mats || nMats == 0)) return fail(CR_ERR_INVALID_ARGUMENT, "meshes need materials");
    if (nEmissive && !emissive) return fail(CR_ERR_INVALID_ARGUMENT, "emissive list is NULL");
    if (nv >= 0xffffffffull) return fail(CR_ERR_UNSUPPORTED, "too many vertices (%llu)", (unsigned long long)nv);
    for (uint64_t i = 0; i < 3 * nv; i++)
        if (!std::isfinite(pos[i])) return fail(CR_ERR_INVALID_ARGUMENT, "vertex position %llu is not finite",
                                                (unsigned long long)(i / 3));
    for (uint64_t i = 0; i < 3 * nt; i++)
        if (idx[i] >= nv) return fail(CR_ERR_INVALID_ARGUMENT, "index %llu = %u is out of range (%llu vertices)",
                                      (unsigned long long)i, idx[i], (unsigned long long)nv);
    // primitive -> mesh, Scene/Triangle.cu:121-131
    std::vector<uint32_t> primToMesh(nt, 0);
    for (uint32_t m = 0; m < nMeshes; m++) {
        if (meshes[m].material_id >= nMats)
            return fail(CR_ERR_INVALID_ARGUMENT, "mesh %u uses material %u of %u", m, meshes[m].material_id, nMats);
        if (meshes[m].index_offset % 3 || meshes[m].index_count % 3 ||
            (uint64_t)meshes[m].index_offset + meshes[m].index_count > 3 * nt)
            return fail(CR_ERR_INVALID_ARGUMENT, "mesh %u index range is invalid", m);
        const uint32_t start = meshes[m].index_offset / 3u, count = meshes[m].index_count / 3u;
        for (uint32_t k = 0; k < count; k++) primToMesh[start + k] = m;
    }
    for (uint32_t e = 0; e < nEmissive; e++)
        if (emissive[e] >= nt) return fail(CR_ERR_INVALID_ARGUMENT, "emitter %u = %u is not a triangle", e, emissive[e]);
    std::vector<MaterialGpu> gm(nMats);
    for (uint32_t m = 0; m < nMats; m++) {
        if (mats[m].type > CR_MATERIAL_PHONG) return fail(CR_ERR_INVALID_ARGUMENT, "material %u type %u", m, mats[m].type);
        gm[m] = deriveMaterial(mats[m]);
        if (mats[m].type == CR_MATERIAL_PRINCIPLED) s->hasPrincipled = true;
    }
    std::vector<float> zeros;
    s->nv = nv;
    s->nt = nt;
    s->nMeshes = nMeshes;
    s->nMats = nMats;
    s->nEmissive = nEmissive;
    int rc;
    if ((rc = upload(&s->pos, reinterpret_cast<const float3*>(pos), nv))) return rc;
    if (!nrm || !uv) zeros.assign(3 * std::max<uint64_t>(nv, 1), 0.0f);
    if ((rc = upload(&s->nrm, reinterpret_cast<const float3*>(nrm ? nrm : zeros.data()), nv))) return rc;
    if ((rc = upload(&s->uv, reinterpret_cast<const float2*>(uv ? uv : zeros.data()), nv))) return rc;
    if ((rc = upload(&s->idx, idx, 3 * nt))) return rc;
    if ((rc = upload(&s->primToMesh, primToMesh.data(), nt))) return rc;
    if ((rc = upload(&s->meshes, meshes, nMeshes))) return rc;
    if ((rc = upload(&s->mats, gm.data(), nMats))) return rc;
    if ((rc = upload(&s->emissive, emissive, nEmissive))) return rc;
    CR_CUDA(cudaMalloc(&s->errFlags, 4));
    CR_CUDA(cudaMemset(s->errFlags, 0, 4));
    CR_CUDA(cudaMalloc(&s->rayCounter, sizeof(unsigned long long)));
    CR_CUDA(cudaMemset(s->rayCounter, 0, sizeof(unsigned long long)));
    return buildBvh(s);
}

}  // namespace

MaterialGpu deriveMaterialPublic(const cr_material& m) { return deriveMaterial(m); }

}  // namespace cr

using namespace cr;

extern "C" {

const char* cr_last_error(void) { return gError.c_str(); }

const char* cr_version(void) { return "craystal_gb300 0.1 (sm_103a)"; }

uint64_t cr_kernel_launch_count(void) { return gLaunches.load(); }

int cr_set_device(int device) {
    clearError();
    CR_CUDA(cudaSetDevice(device));
    return CR_OK;
}

int cr_scene_create(const float* pos, const float* nrm, const float* uv, uint64_t n_vertices, const uint32_t* idx,
                    uint64_t n_tris, const cr_mesh_desc* meshes, uint32_t n_meshes, const cr_material* mats,
                    uint32_t n_mats, const uint32_t* emissive, uint32_t n_emissive, cr_scene** out) {
    clearError();
    if (!out) return fail(CR_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    cr_scene* s = new cr_scene();
    CR_CUDA(cudaGetDevice(&s->device));
    int rc = createScene(pos, nrm, uv, n_vertices, idx, n_tris, meshes, n_meshes, mats, n_mats, emissive, n_emissive, s);
    if (rc) {
        std::string msg = gError;
        freeScene(s);
        gError = msg;
        return rc;
    }
    *out = s;
    return CR_OK;
}

int cr_scene_destroy(cr_scene* scene) {
    clearError();
    freeScene(scene);
    return CR_OK;
}

int cr_scene_bvh_stats(const cr_scene* scene, cr_bvh_stats* out) {
    clearError();
    if (!scene || !out) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = scene->stats;
    return CR_OK;
}

int cr_scene_bvh_export(const cr_scene* scene, cr_bvh_node* nodes, uint32_t* prim_map) {
    clearError();
    if (!scene) return fail(CR_ERR_INVALID_ARGUMENT, "scene is NULL");
    CR_CUDA(cudaSetDevice(scene->device));
    return exportBvh(scene, nodes, prim_map);
}

int cr_scene_bvh_import(cr_scene* scene, const cr_bvh_node* nodes, uint32_t node_count, const uint32_t* prim_map) {
    clearError();
    if (!scene) return fail(CR_ERR_INVALID_ARGUMENT, "scene is NULL");
    CR_CUDA(cudaSetDevice(scene->device));
    return importBvh(scene, nodes, node_count, prim_map);
}

int cr_scene_set_camera(cr_scene* scene, const cr_camera* cam) {
    clearError();
    if (!scene || !cam) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (cam->width == 0 || cam->height == 0 || cam->width > 65536 || cam->height > 65536)
        return fail(CR_ERR_INVALID_ARGUMENT, "sensor size %ux%u", cam->width, cam->height);
    CR_CUDA(cudaSetDevice(scene->device));
    // Camera::calculateCameraData, Core/Camera.cu:35-39
    const float3 pos = mk3(cam->pos[0], cam->pos[1], cam->pos[2]);
    const float3 tgt = mk3(cam->target[0], cam->target[1], cam->target[2]);
    const float3 up = mk3(cam->up[0], cam->up[1], cam->up[2]);
    CameraGpu c;
    c.pos = pos;
    c.W = normalize(sub(tgt, pos));
    c.U = normalize(cross(c.W, up));
    c.V = normalize(cross(c.U, c.W));
    // CameraProxy::generateRay, Core/CameraProxy.h:32-35: the tangent is
    // evaluated in double (fovY * 0.5 promotes) and stored as float
    c.halfH = (float)std::tan(((double)cam->fov_y * 0.5) * 0.01745329251994329576923690768489);
    const float aspect = (float)cam->width / (float)cam->height;
    c.halfW = aspect * c.halfH;
    c.width = cam->width;
    c.height = cam->height;
    const bool resize = !scene->hasCamera || scene->cam.width != c.width || scene->cam.height != c.height;
    if (resize) {
        if (scene->filmRgb) cudaFree(scene->filmRgb);
        if (scene->filmW) cudaFree(scene->filmW);
        scene->filmRgb = nullptr;
        scene->filmW = nullptr;
        const size_t px = (size_t)c.width * c.height;
        CR_CUDA(cudaMalloc(&scene->filmRgb, px * 3 * sizeof(float)));
        CR_CUDA(cudaMalloc(&scene->filmW, px * sizeof(float)));
        CR_CUDA(cudaMemset(scene->filmRgb, 0, px * 3 * sizeof(float)));
        CR_CUDA(cudaMemset(scene->filmW, 0, px * sizeof(float)));
        CR_CUDA(cudaMemset(scene->rayCounter, 0, sizeof(unsigned long long)));
    }
    scene->cam = c;
    scene->hasCamera = true;
    return CR_OK;
}

int cr_scene_set_environment(cr_scene* scene, const float radiance[3]) {
    clearError();
    if (!scene || !radiance) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    for (int k = 0; k < 3; k++)
        if (!std::isfinite(radiance[k]) || radiance[k] < 0.0f)
            return fail(CR_ERR_INVALID_ARGUMENT, "environment radiance must be finite and non-negative");
    scene->env = mk3(radiance[0], radiance[1], radiance[2]);
    return CR_OK;
}

int cr_scene_set_sphere_lights(cr_scene* scene, const cr_sphere_light* lights, uint32_t n) {
    clearError();
    if (!scene || (n && !lights)) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n > kMaxSphereLights) return fail(CR_ERR_INVALID_ARGUMENT, "at most %u sphere lights", kMaxSphereLights);
    std::vector<float4> sp(n), em(n);
    for (uint32_t i = 0; i < n; i++) {
        const cr_sphere_light& l = lights[i];
        if (!(l.radius > 0.0f) || !std::isfinite(l.radius))
            return fail(CR_ERR_INVALID_ARGUMENT, "sphere light %u radius %g", i, l.radius);
        sp[i] = make_float4(l.center[0], l.center[1], l.center[2], l.radius);
        em[i] = make_float4(l.emission[0], l.emission[1], l.emission[2], 0.0f);
    }
    CR_CUDA(cudaSetDevice(scene->device));
    CR_CUDA(cudaDeviceSynchronize());
    if (scene->spheres) cudaFree(scene->spheres);
    if (scene->sphereEm) cudaFree(scene->sphereEm);
    scene->spheres = scene->sphereEm = nullptr;
    scene->nSpheres = 0;
    if (n) {
        CR_CUDA(cudaMalloc(&scene->spheres, n * sizeof(float4)));
        CR_CUDA(cudaMalloc(&scene->sphereEm, n * sizeof(float4)));
        CR_CUDA(cudaMemcpy(scene->spheres, sp.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
        CR_CUDA(cudaMemcpy(scene->sphereEm, em.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    }
    scene->nSpheres = n;
    return CR_OK;
}

int cr_scene_set_diffuse_textures(cr_scene* scene, const cr_texture* textures, uint32_t nTex,
                                  const uint32_t* matTex, uint32_t nMats) {
    clearError();
    if (!scene || (nTex && !textures) || (nMats && !matTex)) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (nMats != scene->nMats)
        return fail(CR_ERR_INVALID_ARGUMENT, "%u material textures for %u materials", nMats, scene->nMats);
    std::vector<uint4> descs(nTex);
    uint64_t total = 0;
    for (uint32_t t = 0; t < nTex; t++) {
        const cr_texture& x = textures[t];
        if (x.width == 0 || x.height == 0 || !x.texels)
            return fail(CR_ERR_INVALID_ARGUMENT, "texture %u is empty (%u x %u)", t, x.width, x.height);
        const uint64_t texels = (uint64_t)x.width * x.height;
        if (texels > 0xFFFFFFFFull || total + texels > 0xFFFFFFFFull)
            return fail(CR_ERR_INVALID_ARGUMENT, "textures exceed 2^32 texels");
        descs[t] = make_uint4((uint32_t)total, x.width, x.height, 0u);
        total += texels;
    }
    for (uint32_t m = 0; m < nMats; m++)
        if (matTex[m] != CR_NO_TEXTURE && matTex[m] >= nTex)
            return fail(CR_ERR_INVALID_ARGUMENT, "material %u names texture %u of %u", m, matTex[m], nTex);
    CR_CUDA(cudaSetDevice(scene->device));
    CR_CUDA(cudaDeviceSynchronize());
    std::vector<MaterialGpu> mats(nMats);
    if (nMats) CR_CUDA(cudaMemcpy(mats.data(), scene->mats, nMats * sizeof(MaterialGpu), cudaMemcpyDeviceToHost));
    bool textured = false;
    for (uint32_t m = 0; m < nMats; m++) {
        mats[m].tex = matTex[m];
        textured |= matTex[m] != CR_NO_TEXTURE;
    }
    if (scene->texels) cudaFree(scene->texels);
    if (scene->texDescs) cudaFree(scene->texDescs);
    scene->texels = nullptr;
    scene->texDescs = nullptr;
    scene->nTex = 0;
    if (nTex) {
        CR_CUDA(cudaMalloc(&scene->texels, total * sizeof(float4)));
        CR_CUDA(cudaMalloc(&scene->texDescs, nTex * sizeof(uint4)));
        for (uint32_t t = 0; t < nTex; t++)
            CR_CUDA(cudaMemcpy(scene->texels + descs[t].x, textures[t].texels,
                               (size_t)descs[t].y * descs[t].z * sizeof(float4), cudaMemcpyHostToDevice));
        CR_CUDA(cudaMemcpy(scene->texDescs, descs.data(), nTex * sizeof(uint4), cudaMemcpyHostToDevice));
    }
    scene->nTex = nTex;
    if (nMats) CR_CUDA(cudaMemcpy(scene->mats, mats.data(), nMats * sizeof(MaterialGpu), cudaMemcpyHostToDevice));
    scene->hasTextures = textured && nTex > 0;
    return CR_OK;
}

int cr_scene_set_spheres(cr_scene* scene, const cr_sphere* spheres, uint32_t n) {
    clearError();
    if (!scene || (n && !spheres)) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (n > kMaxSpheres) return fail(CR_ERR_INVALID_ARGUMENT, "%u spheres; the limit is %u", n, kMaxSpheres);
    std::vector<float4> geom(n);
    std::vector<uint32_t> mat(n);
    for (uint32_t i = 0; i < n; i++) {
        const cr_sphere& x = spheres[i];
        if (!(x.radius > 0.0f) || !std::isfinite(x.radius) || !std::isfinite(x.center[0]) ||
            !std::isfinite(x.center[1]) || !std::isfinite(x.center[2]))
            return fail(CR_ERR_INVALID_ARGUMENT, "sphere %u: centre or radius %g is not finite and positive", i,
                        x.radius);
        if (x.material >= scene->nMats)
            return fail(CR_ERR_INVALID_ARGUMENT, "sphere %u: material %u of %u", i, x.material, scene->nMats);
        geom[i] = make_float4(x.center[0], x.center[1], x.center[2], x.radius);
        mat[i] = x.material;
    }
    CR_CUDA(cudaSetDevice(scene->device));
    CR_CUDA(cudaDeviceSynchronize());
    if (scene->sphGeom) cudaFree(scene->sphGeom);
    if (scene->sphMat) cudaFree(scene->sphMat);
    scene->sphGeom = nullptr;
    scene->sphMat = nullptr;
    scene->nSph = 0;
    int rc;
    if ((rc = upload(&scene->sphGeom, geom.data(), n))) return rc;
    if ((rc = upload(&scene->sphMat, mat.data(), n))) return rc;
    scene->nSph = n;
    return buildSphereBvh(scene);
}

int cr_film_clear(cr_scene* scene) {
    clearError();
    if (!scene || !scene->hasCamera) return fail(CR_ERR_INVALID_ARGUMENT, "scene has no camera / film");
    CR_CUDA(cudaSetDevice(scene->device));
    CR_CUDA(cudaDeviceSynchronize());
    const size_t px = (size_t)scene->cam.width * scene->cam.height;
    CR_CUDA(cudaMemset(scene->filmRgb, 0, px * 3 * sizeof(float)));
    CR_CUDA(cudaMemset(scene->filmW, 0, px * sizeof(float)));
    CR_CUDA(cudaMemset(scene->rayCounter, 0, sizeof(unsigned long long)));
    CR_CUDA(cudaDeviceSynchronize());
    return CR_OK;
}

int cr_film_read(cr_scene* scene, float* rgb, float* weight) {
    clearError();
    if (!scene || !scene->hasCamera) return fail(CR_ERR_INVALID_ARGUMENT, "scene has no camera / film");
    CR_CUDA(cudaSetDevice(scene->device));
    CR_CUDA(cudaDeviceSynchronize());
    const size_t px = (size_t)scene->cam.width * scene->cam.height;
    if (rgb) CR_CUDA(cudaMemcpy(rgb, scene->filmRgb, px * 3 * sizeof(float), cudaMemcpyDeviceToHost));
    if (weight) CR_CUDA(cudaMemcpy(weight, scene->filmW, px * sizeof(float), cudaMemcpyDeviceToHost));
    return takeDeviceErrors(scene, "render");
}

int cr_scene_check_errors(cr_scene* scene, uint32_t* flags) {
    clearError();
    if (flags) *flags = 0;
    if (!scene) return fail(CR_ERR_INVALID_ARGUMENT, "scene is NULL");
    CR_CUDA(cudaSetDevice(scene->device));
    CR_CUDA(cudaDeviceSynchronize());
    uint32_t err = 0;
    CR_CUDA(cudaMemcpy(&err, scene->errFlags, sizeof(err), cudaMemcpyDeviceToHost));
    if (flags) *flags = err;
    return takeDeviceErrors(scene, "scene");
}

int cr_scene_set_error_flags(cr_scene* scene, uint32_t flags) {
    clearError();
    if (!scene) return fail(CR_ERR_INVALID_ARGUMENT, "scene is NULL");
    CR_CUDA(cudaSetDevice(scene->device));
    CR_CUDA(cudaDeviceSynchronize());
    uint32_t err = 0;
    CR_CUDA(cudaMemcpy(&err, scene->errFlags, sizeof(err), cudaMemcpyDeviceToHost));
    err |= flags;
    CR_CUDA(cudaMemcpy(scene->errFlags, &err, sizeof(err), cudaMemcpyHostToDevice));
    return CR_OK;
}

int cr_scene_set_traversal(cr_scene* scene, uint32_t mode) {
    clearError();
    if (!scene) return fail(CR_ERR_INVALID_ARGUMENT, "scene is NULL");
    if (mode != CR_TRAVERSAL_ONE_LEVEL && mode != CR_TRAVERSAL_TWO_LEVEL)
        return fail(CR_ERR_INVALID_ARGUMENT, "traversal mode %u (CR_TRAVERSAL_ONE_LEVEL or CR_TRAVERSAL_TWO_LEVEL)",
                    mode);
    CR_CUDA(cudaSetDevice(scene->device));
    if (mode == CR_TRAVERSAL_TWO_LEVEL && !scene->groupPairs) {
        int rc = buildGroupedPairs(scene);
        if (rc) return rc;
    } else if (mode == CR_TRAVERSAL_ONE_LEVEL && scene->groupPairs) {
        CR_CUDA(cudaDeviceSynchronize());  // queries still in flight may read the copy
        cudaFree(scene->groupPairs);
        scene->groupPairs = nullptr;
    }
    scene->traversal = mode;
    return CR_OK;
}

int cr_film_resolve(cr_scene* scene, float* rgb) {
    clearError();
    if (!scene || !scene->hasCamera || !rgb) return fail(CR_ERR_INVALID_ARGUMENT, "scene has no film / rgb is NULL");
    CR_CUDA(cudaSetDevice(scene->device));
    return resolveFilm(scene, rgb);
}

int cr_render(cr_scene* scene, const cr_integrator_config* cfg, uint32_t spp, uint32_t first_sample, void* stream) {
    clearError();
    if (!scene || !cfg) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    if (!scene->hasCamera) return fail(CR_ERR_INVALID_ARGUMENT, "scene has no camera; call cr_scene_set_camera");
    if (cfg->max_depth > 1024) return fail(CR_ERR_INVALID_ARGUMENT, "max_depth %u", cfg->max_depth);
    if (cfg->flags & ~(CR_RENDER_SPECTRAL | CR_RENDER_WAVEFRONT | CR_RENDER_MEGAKERNEL))
        return fail(CR_ERR_INVALID_ARGUMENT, "unknown render flags 0x%x", cfg->flags);
    if ((cfg->flags & CR_RENDER_WAVEFRONT) && (cfg->flags & CR_RENDER_MEGAKERNEL))
        return fail(CR_ERR_INVALID_ARGUMENT, "CR_RENDER_WAVEFRONT and CR_RENDER_MEGAKERNEL exclude each other");
    CR_CUDA(cudaSetDevice(scene->device));
    const uint64_t paths = (uint64_t)scene->cam.width * scene->cam.height * spp;
    const bool wavefront =
        (cfg->flags & CR_RENDER_WAVEFRONT) || (!(cfg->flags & CR_RENDER_MEGAKERNEL) && paths >= (1u << 16));
    if (wavefront) return renderWavefront(scene, cfg, spp, first_sample, static_cast<cudaStream_t>(stream));
    return renderDevice(scene, cfg, spp, first_sample, static_cast<cudaStream_t>(stream));
}

int cr_render_ray_count(cr_scene* scene, uint64_t* rays) {
    clearError();
    if (!scene || !rays) return fail(CR_ERR_INVALID_ARGUMENT, "NULL argument");
    CR_CUDA(cudaSetDevice(scene->device));
    CR_CUDA(cudaDeviceSynchronize());
    unsigned long long v = 0;
    CR_CUDA(cudaMemcpy(&v, scene->rayCounter, sizeof(v), cudaMemcpyDeviceToHost));
    *rays = v;
    return CR_OK;
}

}  // extern "C"
