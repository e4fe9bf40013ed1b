/*
 * craystal_oracle.h -- C ABI of the CPU oracle for the CRaystal path-tracing
 * hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain-C++ restatement of the
 * reference algorithms (Hyiker/CRaystal, Source/CRaystal/...), used by the
 * test-suite, the smoke check and the CPU-baseline leg of the benchmark as the
 * checker.  The product (craystal_gb300) never links, loads or calls it.
 *
 * Parity status: the reference cannot be compiled in this environment (its
 * glm / fmt / Catch2 dependencies are fetched from the network at configure
 * time), so the oracle is a port.  It is pinned against every known-answer
 * vector the reference's own tests hold for this path (Tests/CameraTest.cpp
 * ray directions, Tests/CoreTest.cpp spectrum arithmetic and sampler
 * statistics).  Nothing in the reference pins BVH, Moller-Trumbore, BSDF or
 * image values; for those the oracle's arithmetic is the source-level
 * semantics of the reference (no FMA contraction, glm's evaluation order).
 */
#ifndef CRAYSTAL_ORACLE_H
#define CRAYSTAL_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Ray record, same layout as Math/Ray.h:8-13 (origin, tMin, direction, tMax). */
typedef struct {
    float o[3];
    float tmin;
    float d[3];
    float tmax;
} orc_ray;

/* Closest-hit record: primitive id (0xFFFFFFFF on miss), t, barycentric u, v. */
typedef struct {
    uint32_t prim;
    float t;
    float u;
    float v;
} orc_hit;

/* Material record, the fields of MaterialData (Core/Material.h:34-43) that the
 * hot path reads. type: 0 FullDiffuse, 1 Principled, 2 Phong. flags as
 * MaterialFlags (1 IsEmissive, 2 IsDiffuse). */
typedef struct {
    float diffuse[3];
    float specular[3];
    float emission[3];
    float shininess;
    uint32_t type;
    uint32_t flags;
} orc_material;

/* MeshDesc, Scene/Triangle.h:27-32. */
typedef struct {
    uint32_t index_offset;
    uint32_t index_count;
    uint32_t vertex_offset;
    uint32_t material_id;
} orc_mesh_desc;

/* Binary BVH node in the reference layout (Core/BVH.h:17-30): post-order,
 * root last.  is_leaf selects (a,b) = (leafOffset, leafCount) or (left,right). */
typedef struct {
    float bmin[3];
    float bmax[3];
    uint32_t is_leaf;
    uint32_t a;
    uint32_t b;
} orc_bvh_node;

typedef struct {
    uint32_t node_count;
    uint32_t leaf_count;
    uint32_t root_index;
    uint32_t max_depth;      /* deepest interior node depth (BVH.cu:210) */
    uint32_t max_leaf_size;  /* BVH.cu:167 */
    uint32_t max_leaf_depth;
    float root_min[3];
    float root_max[3];
} orc_bvh_stats;

/* Camera inputs (Core/Camera.h setters + sensor size). */
typedef struct {
    float pos[3];
    float target[3];
    float up[3];
    float fov_y;
    uint32_t width;
    uint32_t height;
} orc_camera;

typedef struct {
    uint32_t max_depth;     /* PathTraceIntegrator::DeviceView::maxDepth */
    float rr_threshold;     /* DeviceView::rrThreshold */
    uint32_t use_mis;       /* Configs::useMIS */
    uint32_t flags;         /* 1 = hero-wavelength spectral rendering */
} orc_integrator_config;

/* Per-ray traversal counters, for the algorithmic byte count of the
 * ray-cast roofline: child boxes tested, triangles tested, leaf map reads. */
typedef struct {
    uint64_t rays;
    uint64_t boxes;
    uint64_t tris;
    uint64_t map_reads;
    uint64_t ties;
} orc_trace_counters;

typedef struct orc_scene orc_scene;

/* ---- sampler (Core/Sampler.cu) ---- */
void orc_sampler_draws(uint32_t px, uint32_t py, uint32_t sample_index,
                       uint32_t n, float* out);
void orc_sampler_raw(uint32_t px, uint32_t py, uint32_t sample_index,
                     uint32_t n, uint32_t* out);

/* ---- camera (Core/Camera.cu:35-39, Core/CameraProxy.h:25-40) ---- */
void orc_camera_basis(const orc_camera* cam, float out_uvw[9]);
void orc_camera_rays(const orc_camera* cam, const float* sensor_pos,
                     uint64_t n, orc_ray* out);

/* ---- geometry helpers ---- */
void orc_offset_ray_origin(const float* p, const float* n, uint64_t count,
                           float* out);
void orc_aabb_intersect(const float* bmin, const float* bmax,
                        const orc_ray* rays, uint64_t n, uint8_t* hit,
                        float* t_entry);
void orc_triangle_intersect(const float* v0, const float* v1, const float* v2,
                            const orc_ray* rays, uint64_t n, uint8_t* hit,
                            float* t, float* u, float* v);

/* ---- scene + BVH (Scene/Scene.cu:61-78, Core/BVH.cu:88-338) ---- */
orc_scene* orc_scene_create(const float* pos, const float* nrm,
                            const float* uv, uint64_t n_vertices,
                            const uint32_t* idx, uint64_t n_tris,
                            const orc_mesh_desc* meshes, uint32_t n_meshes,
                            const orc_material* mats, uint32_t n_mats,
                            const uint32_t* emissive, uint32_t n_emissive);
void orc_scene_destroy(orc_scene* s);
/* Lights beyond the reference (extensions): constant environment radiance
 * and sphere lights (center xyz, radius, emission rgb per light). */
void orc_scene_set_lights(orc_scene* s, const float* env3,
                          const float* spheres7, uint32_t n_spheres);
/* Analytic spheres (centre xyz, radius per sphere; a material each),
 * intersected before the triangles (Scene/Scene.cu:5-14); hits report
 * prim = 0x80000000 | index. */
void orc_scene_set_spheres(orc_scene* s, const float* geom4,
                           const uint32_t* mats, uint32_t n);
/* Diffuse textures: texels = RGBA floats of all textures, descs = (first
 * texel, width, height) per texture, mat_tex = texture per material or
 * 0xFFFFFFFF (Core/Texture.cu, Core/Material.h:29-36). */
void orc_scene_set_textures(orc_scene* s, const float* texels,
                            const uint32_t* descs, uint32_t n_tex,
                            const uint32_t* mat_tex, uint32_t n_mats);
/* TextureView::sample (Core/Texture.cu:15-35) at n coordinates. */
void orc_texture_sample(const orc_scene* s, uint32_t tex, const float* uv,
                        uint64_t n, float* rgba);
void orc_scene_bvh_stats(const orc_scene* s, orc_bvh_stats* out);
/* Exports nodes (post-order, root last) and the leaf-slot -> primitive map. */
void orc_scene_bvh_export(const orc_scene* s, orc_bvh_node* nodes,
                          uint32_t* prim_map);

/* ---- traversal (Core/BVH.cu:13-84, Scene/Scene.cu:5-29) ---- */
void orc_trace_closest(const orc_scene* s, const orc_ray* rays, uint64_t n,
                       orc_hit* hits, uint8_t* ties, int threads,
                       orc_trace_counters* counters);
void orc_trace_occluded(const orc_scene* s, const orc_ray* rays, uint64_t n,
                        uint8_t* occluded, int threads);
/* Brute force over all triangles, closest-hit rule of Scene/Shape.h:16-37 in
 * primitive order; for checking the BVH build and traversal. */
void orc_trace_brute(const orc_scene* s, const orc_ray* rays, uint64_t n,
                     orc_hit* hits, int threads);

/* ---- BSDF (Material/PhongBRDF.cu, PrincipledBRDF.cu, LambertianBRDF.cu)
 * in a shading frame built from normal n ---- */
void orc_bsdf_eval(const orc_material* m, const float* n, const float* wo,
                   const float* wi, uint64_t count, float* f, float* pdf);
void orc_bsdf_sample(const orc_material* m, const float* n, const float* wo,
                     const float* u, uint64_t count, float* wi, float* f,
                     float* pdf);

/* ---- integrator (Core/Integrator.cu:13-262) + film (Core/Sensor.cu) ----
 * Renders spp samples starting at sample index first_sample into an FP64
 * film (rgb sum, weight sum), accumulated on top of what the arrays hold.
 * Pixels [y0, y1) only when row_end > row_begin (a crop); else all rows. */
void orc_render(const orc_scene* s, const orc_camera* cam,
                const orc_integrator_config* cfg, uint32_t spp,
                uint32_t first_sample, uint32_t row_begin, uint32_t row_end,
                double* film_rgb, double* film_w, int threads,
                uint64_t* rays_traced);

/* ---- hero-wavelength spectral mode (an extension) ---- */
void orc_spectral_cmf(const float* lambda, uint64_t n, float* xyz);
void orc_spectral_white_balance(float* out3);
void orc_spectral_upsample(const float* rgb, const float* lambda, uint64_t n, float* out);

int orc_hardware_threads(void);

#ifdef __cplusplus
}
#endif
#endif
