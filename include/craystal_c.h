/*
 * craystal_c.h -- C ABI of craystal_gb300, a GB300-native (sm_103a)
 * implementation of the CRaystal path-tracing hot path.
 *
 * The entry points replace the C++ classes of the reference library
 * (Hyiker/CRaystal, Source/CRaystal) one for one; each declaration cites
 * the reference interface it stands for.  Conventions:
 *   - every function returns CR_OK (0) or an error code; cr_last_error()
 *     returns a message for the calling thread's last failure (no exceptions
 *     cross the ABI, where the reference throws RuntimeError,
 *     Core/Error.h:113-124 and Utils/CudaUtils.h:3-12);
 *   - host arrays passed to cr_scene_create are copied; the caller keeps them;
 *   - "_device" entry points take device pointers and a cudaStream_t (passed
 *     as void*, NULL = legacy default stream) and return without waiting;
 *     the others take host pointers and return when the results are in them;
 *   - a scene handle is not thread-safe; distinct handles are independent.
 */
#ifndef CRAYSTAL_C_H
#define CRAYSTAL_C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CR_OK 0
#define CR_ERR_INVALID_ARGUMENT 1
#define CR_ERR_CUDA 2
#define CR_ERR_OUT_OF_MEMORY 3
#define CR_ERR_DEVICE 4       /* a kernel reported an error (stack overflow, timeout) */
#define CR_ERR_UNSUPPORTED 5
#define CR_ERR_IO 6           /* a file could not be read, written or parsed */

#define CR_MISS 0xFFFFFFFFu

/* Material types, Core/Material.h:12-16. */
#define CR_MATERIAL_DIFFUSE 0u
#define CR_MATERIAL_PRINCIPLED 1u
#define CR_MATERIAL_PHONG 2u
/* Material flags, Core/Material.h:26-30 (set by MaterialData::finalize). */
#define CR_MATERIAL_EMISSIVE 1u
#define CR_MATERIAL_DIFFUSE_ONLY 2u

/* Ray, Math/Ray.h:8-13: origin, tMin, direction, tMax (32 bytes). */
typedef struct {
    float o[3];
    float tmin;
    float d[3];
    float tmax;
} cr_ray;

/* Closest hit: primitive index (CR_MISS when nothing is hit), t and the
 * barycentrics (u, v) of Scene/Triangle.cu:68-69; RayHit, Core/Hit.h:26-30. */
typedef struct {
    uint32_t prim;
    float t;
    float u;
    float v;
} cr_hit;

/* MaterialData, Core/Material.h:34-66, the fields the path reads. */
typedef struct {
    float diffuse[3];   /* Kd */
    float specular[3];  /* Ks */
    float emission[3];
    float shininess;    /* Phong exponent; Principled roughness = sqrt(2/(s+1)) */
    uint32_t type;      /* CR_MATERIAL_* */
    uint32_t flags;     /* CR_MATERIAL_EMISSIVE | CR_MATERIAL_DIFFUSE_ONLY; 0 = derive */
} cr_material;

/* MeshDesc, Scene/Triangle.h:27-32 (indices already rebased to the global
 * vertex array, as TriangleMeshManager does at Scene/Triangle.cu:98-120). */
typedef struct {
    uint32_t index_offset;
    uint32_t index_count;
    uint32_t vertex_offset;
    uint32_t material_id;
} cr_mesh_desc;

/* Camera + sensor size: Camera::setWorldPosition/setTarget/setUp/setFovY
 * (Core/Camera.h:24-31) and Sensor(UInt2 size) (Core/Sensor.h:35). */
typedef struct {
    float pos[3];
    float target[3];
    float up[3];
    float fov_y;        /* degrees */
    uint32_t width;
    uint32_t height;
} cr_camera;

/* PathTraceIntegrator::Configs / DeviceView, Core/Integrator.h:14-23.
 * The reference never copies Configs into the device view, so its kernels
 * always run with max_depth 10 and rr_threshold 0.05; pass those for the
 * reference's effective behaviour. */
typedef struct {
    uint32_t max_depth;
    float rr_threshold;
    uint32_t use_mis;
    uint32_t flags;     /* CR_RENDER_* bits */
} cr_integrator_config;

/* Hero-wavelength spectral rendering (an extension; the reference renders
 * RGB): every path carries three wavelengths over 360-830 nm, material RGB
 * is upsampled to spectra, the film receives linear sRGB white-balanced so
 * that a flat spectrum renders as in RGB. */
#define CR_RENDER_SPECTRAL 1u
/* Schedules of the same paths.  The megakernel keeps each path in one
 * thread's registers for all its bounces (the reference's structure); the
 * wavefront keeps live paths in HBM between bounces and runs each bounce as
 * a traversal launch, a counting sort of the hits by material and a shading
 * launch.  Per path the arithmetic and the sampler sequence are the same,
 * so the film is the same up to the order of its float additions.  Without
 * either flag cr_render takes the wavefront for 65,536 paths (pixels x spp)
 * or more and the megakernel below.  Neither waits on the host; the
 * wavefront's path state is allocated with the scene on first use (render
 * once before capturing cr_render into a CUDA graph). */
#define CR_RENDER_WAVEFRONT 2u
#define CR_RENDER_MEGAKERNEL 4u

/* Binary BVH node in the reference's layout (Core/BVH.h:17-30): nodes in
 * post-order with the root last; leaf: (a, b) = (first leaf slot, count),
 * interior: (a, b) = (left child, right child). */
typedef struct {
    float bmin[3];
    float bmax[3];
    uint32_t is_leaf;
    uint32_t a;
    uint32_t b;
} cr_bvh_node;

typedef struct {
    uint32_t node_count;
    uint32_t leaf_count;
    uint32_t max_depth;        /* deepest interior node */
    uint32_t max_leaf_size;
    uint32_t max_leaf_depth;
    uint32_t levels;           /* breadth-first build levels executed */
    float root_min[3];
    float root_max[3];
    double build_ms;           /* device time of the GPU build */
    uint64_t device_bytes;     /* BVH + triangle blocks resident in HBM */
} cr_bvh_stats;

typedef struct cr_scene cr_scene;

/* Thread-local message of the last failed call ("" after success). */
const char* cr_last_error(void);

/* Library version string. */
const char* cr_version(void);

/* Selects the CUDA device used by subsequent calls of this thread. */
int cr_set_device(int device);

/* Scene(SceneData&&), Scene/Scene.cu:61-78: uploads the global vertex and
 * index arrays (TriangleMeshManager, Scene/Triangle.cu:98-165), the
 * materials and emitter list (MaterialManager, Core/Material.cu:15-31) and
 * builds the BVH on the GPU (replacing the host build of Core/BVH.cu:88-116;
 * same binned-SAH decisions, see cr_scene_bvh_export).  nrm and uv may be
 * NULL (zeros).  Material flags of 0 are derived as MaterialData::finalize
 * does (Core/Material.h:57-65). */
int cr_scene_create(const float* pos, const float* nrm, const float* uv,
                    uint64_t n_vertices, const uint32_t* idx, uint64_t n_tris,
                    const cr_mesh_desc* meshes, uint32_t n_meshes,
                    const cr_material* mats, uint32_t n_mats,
                    const uint32_t* emissive, uint32_t n_emissive,
                    cr_scene** out);

int cr_scene_destroy(cr_scene* scene);

/* BVH statistics, the figures BVH::build logs (Core/BVH.cu:111-115). */
int cr_scene_bvh_stats(const cr_scene* scene, cr_bvh_stats* out);

/* Copies the BVH out in the reference's node layout: nodes (node_count
 * entries, post-order, root last, as BVH::buildRecursive numbers them,
 * Core/BVH.cu:150-212) and prim_map (n_tris entries: leaf slot -> primitive,
 * bvhToMeshPrimitiveIndex of Core/BVH.cu:322-338).  Either may be NULL. */
int cr_scene_bvh_export(const cr_scene* scene, cr_bvh_node* nodes,
                        uint32_t* prim_map);

/* Replaces the scene's triangle BVH with a tree in the same layout, e.g. one
 * built by the reference's host builder (BVH::build + createFinalBVH,
 * Core/BVH.cu:88-116 and :303-338; BVHData, Core/BVH.h:17-30): node_count
 * nodes with the root last, interior (a, b) = child indices, leaf (a, b) =
 * (first slot, count) into prim_map, which has n_tris entries, each a
 * triangle index.  Node order need not be post-order, but every node must be
 * reached exactly once from the root.  Queries and renders then traverse this
 * tree in the reference's order, so hits equal the reference's on the same
 * tree bit for bit, ties included.  Rejected: indices out of range, a node
 * reached twice or not at all (CR_ERR_INVALID_ARGUMENT), an interior node
 * deeper than 31 levels, which the 32-entry traversal stack cannot hold
 * (CR_ERR_UNSUPPORTED; the reference builder stops at depth 20).  The
 * scene's statistics describe the imported tree (build_ms 0).  Waits for
 * work that uses the old tree. */
int cr_scene_bvh_import(cr_scene* scene, const cr_bvh_node* nodes,
                        uint32_t node_count, const uint32_t* prim_map);

/* How the ray-cast queries (cr_trace_closest, cr_trace_occluded, their
 * "_device" forms and cr_trace_closest_noalloc) step through the BVH.  No
 * counterpart in the reference, whose traversal (Core/BVH.cu:13-84) visits
 * one binary level per loop iteration.  CR_TRAVERSAL_ONE_LEVEL (the
 * default) tests one node pair per step.  CR_TRAVERSAL_TWO_LEVEL builds a
 * second copy of the scene's node pairs laid out in two-level groups (each
 * interior node at even depth followed by its interior children's pairs; 64
 * bytes per interior node, at most 2^28 interior nodes) and also tests the
 * near child's pair of a group in the same step, from the adjacent record;
 * switching back frees the copy.  Both modes visit nodes and leaves in the
 * reference's order with its culling, so the hits are the same bit for bit;
 * on GB300 the one-level step is the faster of the two at every tree size
 * measured.  Returns CR_ERR_INVALID_ARGUMENT for another mode.  The path
 * tracers always use the one-level step.  Not thread-safe with queries in
 * flight on the scene from other threads. */
#define CR_TRAVERSAL_ONE_LEVEL 0u
#define CR_TRAVERSAL_TWO_LEVEL 1u
int cr_scene_set_traversal(cr_scene* scene, uint32_t mode);

/* Errors that kernels detect (a traversal stack that would overflow) set
 * bits of the scene's device error word.  cr_trace_closest,
 * cr_trace_occluded, cr_trace_closest_noalloc and cr_film_read read it when
 * they finish and return CR_ERR_DEVICE when a bit is set; the "_device" entry
 * points and cr_render return before their kernels run, so their errors are
 * reported by the next of those calls or by cr_scene_check_errors.  The word
 * is cleared when it is reported: each error is reported once.
 * cr_scene_check_errors waits for the device, stores the word in *flags (may
 * be NULL), clears it and returns CR_ERR_DEVICE when it was set.
 * cr_scene_set_error_flags ORs bits into the word from the host, as a kernel
 * that detected an error does, so that callers can test their handling of
 * CR_ERR_DEVICE without a failing kernel. */
#define CR_DEVICE_ERROR_STACK_OVERFLOW 1u
int cr_scene_check_errors(cr_scene* scene, uint32_t* flags);
int cr_scene_set_error_flags(cr_scene* scene, uint32_t flags);

/* Scene::setCamera + Camera::calculateCameraData + Sensor(size)
 * (Scene/Scene.h:56-58, Core/Camera.cu:35-39, Core/Sensor.cu:46-60).  A
 * sensor of a new size gets a new film, cleared to zero. */
int cr_scene_set_camera(cr_scene* scene, const cr_camera* cam);

/* ---- lights beyond the reference (extensions) ----
 * The reference has neither: its paths end with 0 on a miss
 * (Core/Integrator.cu:205-207), and its spheres (Scene/Sphere.cu:6-52)
 * are shaded through the triangle-mesh tables, which is wrong for them.
 * Environment: constant radiance collected by every ray that leaves the
 * scene.  Sphere lights: analytic emitting spheres, intersected in a linear
 * loop after the BVH (as SceneView::intersect does for spheres,
 * Scene/Scene.cu:5-14), occluding shadow rays, reached by BSDF sampling (not
 * by next-event estimation, whose emitter list stays the triangle list). */
typedef struct {
    float center[3];
    float radius;
    float emission[3];
    float pad;
} cr_sphere_light;
int cr_scene_set_environment(cr_scene* scene, const float radiance[3]);
int cr_scene_set_sphere_lights(cr_scene* scene, const cr_sphere_light* lights,
                               uint32_t n);

/* ---- analytic spheres ----
 * SceneData::spheres (Scene/Scene.h:41, Scene/Sphere.h:9-12) with a
 * material each (the reference's spheres have none and are shaded through
 * the triangle-mesh tables).  Intersection is SphereSOA::intersect
 * (Scene/Sphere.cu:6-52): the nearer root inside [tMin, tMax], else the
 * farther one; (u, v) = (phi / 2pi, theta / pi) of the hit normal, which
 * is also the texture coordinate.  Spheres are tested before the triangles
 * (SceneView::intersect, Scene/Scene.cu:5-14), through a BVH of their own
 * built on the GPU; a sphere hit reports prim = CR_SPHERE_BIT | index.
 * Emissive spheres are reached by BSDF sampling only (next-event estimation
 * samples the emissive triangles).  A new call replaces all spheres. */
#define CR_SPHERE_BIT 0x80000000u
typedef struct {
    float center[3];
    float radius;
    uint32_t material;
    uint32_t pad[3];
} cr_sphere;
int cr_scene_set_spheres(cr_scene* scene, const cr_sphere* spheres,
                         uint32_t n);

/* ---- diffuse textures ----
 * SceneData::textureImages + MaterialData::diffuseHandle and the
 * hasDiffuseTexture flag (Scene/Scene.h:45, Core/Material.h:29-36): a
 * texture is width x height texels, row-major RGBA float4, row 0 first
 * (Texture(const Image&), Core/Texture.cu:45-60).  A textured material's
 * diffuse reflectance is the texture's bilinear sample at the hit's
 * interpolated texture coordinates (getBSDF, Material/BSDF.cu:11-15;
 * TextureView::sample, Core/Texture.cu:15-35), and a Phong material's lobe
 * probabilities follow from that per-hit reflectance
 * (Material/PhongBRDF.cu:10-19).  material_texture[m] is the texture of
 * material m or CR_NO_TEXTURE; n_mats must equal the scene's material
 * count.  A new call replaces all textures. */
#define CR_NO_TEXTURE 0xFFFFFFFFu
typedef struct {
    uint32_t width;
    uint32_t height;
    const float* texels; /* width * height * 4 floats */
} cr_texture;
int cr_scene_set_diffuse_textures(cr_scene* scene, const cr_texture* textures,
                                  uint32_t n_textures,
                                  const uint32_t* material_texture,
                                  uint32_t n_mats);

/* TextureView::sample (Core/Texture.cu:15-35) on the device for n texture
 * coordinates (uv: 2n floats, host) into rgba (4n floats, host). */
int cr_texture_sample(const cr_scene* scene, uint32_t texture, const float* uv,
                      uint64_t n, float* rgba);

/* ---- scene import ----
 * Importer::import (Utils/Importer.cpp:203-236): path names an XML file
 * with the camera and the emissive materials; the geometry is the OBJ file
 * of the same name beside it, with its MTL library.  All materials are
 * Phong; a material listed in a <light> element gets that radiance; a
 * map_Kd texture is loaded (PNG or EXR) and linearised as Image::load does.
 * The result stays on the host until cr_import_create_scene uploads it:
 * cr_import_get exposes its arrays (valid until cr_import_destroy) in the
 * layout cr_scene_create takes. */
typedef struct cr_import cr_import;
typedef struct {
    const float* pos;             /* n_vertices * 3 */
    const float* nrm;             /* n_vertices * 3 */
    const float* uv;              /* n_vertices * 2 */
    uint64_t n_vertices;
    const uint32_t* idx;          /* n_tris * 3, global vertex indices */
    uint64_t n_tris;
    const cr_mesh_desc* meshes;
    uint32_t n_meshes;
    const cr_material* mats;
    const uint32_t* material_texture;  /* per material: texture or CR_NO_TEXTURE */
    uint32_t n_mats;
    const uint32_t* emissive;     /* SceneData::emissiveIndex */
    uint32_t n_emissive;
    const cr_texture* textures;
    uint32_t n_textures;
    cr_camera camera;             /* fovy, eye, lookat, up, width, height */
} cr_import_view;
int cr_import_xml(const char* path, cr_import** out);
int cr_import_get(const cr_import* imp, cr_import_view* out);
/* The OBJ material name of a material ("" when out of range). */
const char* cr_import_material_name(const cr_import* imp, uint32_t material);
/* Scene(SceneData&&) + Scene::setCamera of the imported scene. */
int cr_import_create_scene(const cr_import* imp, cr_scene** out);
int cr_import_destroy(cr_import* imp);

/* ---- image files (Utils/Image.cpp) ----
 * Pixels are interleaved: (y * width + x) * channels + c, row 0 first. */
typedef struct {
    uint32_t width;
    uint32_t height;
    uint32_t channels;
    float* pixels;                /* owned by the library: cr_image_free */
} cr_image;
/* Image::load (:262-270): ".exr" files by readEXR (R, G, B found by channel
 * name; other channels read as 0), otherwise PNG by readMisc (rows flipped
 * to bottom-up; values / 255, raised to 2.2 when to_linear). */
int cr_image_load(const char* path, int to_linear, cr_image* out);
int cr_image_free(cr_image* img);
/* Image::writeEXR (:49-106): channels 0, 1, 2 as R, G, B in half floats. */
int cr_image_write_exr(const char* path, uint32_t width, uint32_t height,
                       uint32_t channels, const float* pixels);
/* Image::writePNG (:182-217): 8-bit; gamma_correct encodes linear values
 * with pow(v, 1/2.2) and clamps to [0, 1]; values are truncated. */
int cr_image_write_png(const char* path, uint32_t width, uint32_t height,
                       uint32_t channels, const float* pixels,
                       int gamma_correct);

/* Zeroes the film (the reference never clears its film, Core/Sensor.cu:55-59). */
int cr_film_clear(cr_scene* scene);

/* Sensor::readbackDeviceData (Core/Sensor.cu:82-86): rgb = width*height*3
 * floats (sum of weighted radiance), weight = width*height floats.  Either
 * may be NULL.  Waits for all work on the scene's film. */
int cr_film_read(cr_scene* scene, float* rgb, float* weight);

/* Sensor::createImage (Core/Sensor.cu:93-112): rgb = sum / weight per pixel,
 * resolved on the GPU; width*height*3 floats. */
int cr_film_resolve(cr_scene* scene, float* rgb);

/* PathTraceIntegrator::dispatch(scene, spp), Core/Integrator.cu:233-262:
 * renders spp samples per pixel with sample indices first_sample ..
 * first_sample+spp-1 into the film, on the given stream, without waiting.
 * rays_out (host, may be NULL) receives the number of closest-hit and
 * occlusion traversals after the next cr_film_read / stream sync. */
int cr_render(cr_scene* scene, const cr_integrator_config* cfg, uint32_t spp,
              uint32_t first_sample, void* stream);

/* Number of traversals (camera/continuation, shadow, MIS-BSDF rays) the
 * renders since the last cr_film_clear performed; synchronises the film. */
int cr_render_ray_count(cr_scene* scene, uint64_t* rays);

/* SceneView::intersect (Scene/Scene.cu:5-14) on a batch of rays: closest
 * hit with the reference's traversal order (Core/BVH.cu:13-84) and
 * intersection arithmetic (Scene/Triangle.cu:40-75), so that prim, t, u and
 * v equal the reference's bit for bit.  Host arrays.  When both arrays lie
 * in page-locked host memory of the scene's device (cudaHostAlloc,
 * cudaHostRegister, a pinned torch tensor), each inside one mapped
 * allocation and 16-byte aligned, the GPU reads the rays and writes the hits
 * there in place (over NVLink-C2C on GB300); otherwise copies in and out go
 * through device staging buffers, pipelined with the traversal.  The call
 * returns when the hits are written.  cr_trace_occluded does the same. */
int cr_trace_closest(cr_scene* scene, const cr_ray* rays, uint64_t n,
                     cr_hit* hits);
/* The same on device buffers, ordered on `stream` (NULL = the default
 * stream) and returning without waiting.  Each call takes an 8-byte
 * stream-ordered allocation (cudaMallocAsync / cudaFreeAsync on `stream`)
 * for its ray counter, so concurrent calls on different streams are
 * independent and the call can be captured in a CUDA graph. */
int cr_trace_closest_device(cr_scene* scene, const cr_ray* rays, uint64_t n,
                            cr_hit* hits, void* stream);

/* SceneView::intersectOcclusion (Scene/Scene.cu:16-29): 1 when any
 * triangle is hit with t in [tmin, tmax].  The reference finds this with a
 * full closest-hit traversal; an any-hit traversal with early exit gives the
 * same answer. */
int cr_trace_occluded(cr_scene* scene, const cr_ray* rays, uint64_t n,
                      uint8_t* occluded);
int cr_trace_occluded_device(cr_scene* scene, const cr_ray* rays, uint64_t n,
                             uint8_t* occluded, void* stream);

/* CameraProxy::generateRay (Core/CameraProxy.h:25-40) on the GPU for a
 * batch of film positions (sensor_pos: n pairs x, y in pixels). */
int cr_camera_generate_rays(const cr_camera* cam, const float* sensor_pos,
                            uint64_t n, cr_ray* rays);

/* BSDF::evaluate and BSDF::evaluatePdf (Material/BSDF.cu:36-70) on the GPU
 * for a batch: the shading frame is Frame(n) (Core/Frame.cu:6-23), wo / wi
 * world directions; f = n*3 floats (BSDF value times |cos|), pdf = n. */
int cr_bsdf_evaluate(const cr_material* mat, const float* n, const float* wo,
                     const float* wi, uint64_t count, float* f, float* pdf);

/* BSDF::sampleEvaluate (Material/BSDF.cu:87-103) with the two uniform
 * numbers given (u = count*2 floats) instead of drawn: wi = count*3,
 * f = count*3, pdf = count. */
int cr_bsdf_sample(const cr_material* mat, const float* n, const float* wo,
                   const float* u, uint64_t count, float* wi, float* f,
                   float* pdf);

/* Closest-hit query on host buffers that allocates no GPU memory.  This
 * entry point has no counterpart in the reference.  It is for callers that
 * cannot let a library allocate device memory: a host that has already
 * committed its GPU memory budget to its own pool, a render thread that must
 * not stall on the device synchronisation cudaMalloc / cudaFree imply, or a
 * plugin whose host forbids allocation after start-up.  Rays and hits pass
 * through a fixed staging area inside the library's device image
 * (CR_NOALLOC_MAX_RAYS rays and hits, 3 MiB); n above CR_NOALLOC_MAX_RAYS is
 * rejected with CR_ERR_INVALID_ARGUMENT.  The staging area is shared by all
 * calls on a device: calls whose work overlaps on the GPU race on it, so
 * callers serialise them.
 * First call on a device: under CUDA's default lazy module loading it makes
 * the driver load the staging area (3 MiB of device memory, which then stays
 * resident on that device until the process exits) and the traversal
 * kernel's code; make that call at start-up, before the caller commits its
 * memory budget (or set CUDA_MODULE_LOADING=EAGER), and before any stream
 * capture begins.  It also looks up the staging area's device address, again
 * whenever the device's context has changed (after cudaDeviceReset).
 * Results equal cr_trace_closest's.  The scene's device error word is shared
 * by all its queries: a call reports (and clears) every error set when it
 * finishes, including errors of earlier "_device" queries on the scene.
 * Returns when the hits are in the host array; the copies and the traversal
 * run on `stream` (NULL = legacy default stream). */
#define CR_NOALLOC_MAX_RAYS 65536u
int cr_trace_closest_noalloc(cr_scene* scene, const cr_ray* rays, uint64_t n,
                             cr_hit* hits, void* stream);

/* ---- radiance-cache network (no counterpart in the reference) ----
 * MLP with 7 inputs (position and direction mapped to [0,1]^3, roughness in
 * [0,1]), a 12-frequency sin / cos encoding of each input (168 features), five
 * hidden layers of 64 ReLU units and 3 linear outputs (RGB radiance); FP16
 * weights and activations with FP32 accumulation on the tensor cores; Adam on
 * FP32 master weights; loss = mean over samples and channels of
 * (y - t)^2 / (sg(y)^2 + 0.01).  Parameters are a flat FP32 vector, layer
 * after layer, each layer k-major (W[k][n] at k * N + n; layer shapes
 * 176x64, 64x64 four times, 64x3; rows 168..175 of the first layer meet
 * zero features). */
typedef struct {
    float lr;       /* Adam step size (1e-2) */
    float beta1;    /* 0.9 */
    float beta2;    /* 0.99 */
    float eps;      /* 1e-8 */
    uint32_t seed;  /* initialisation */
} cr_mlp_config;
typedef struct cr_mlp cr_mlp;
uint64_t cr_mlp_param_count(void);
int cr_mlp_create(const cr_mlp_config* cfg, cr_mlp** out);
int cr_mlp_destroy(cr_mlp* mlp);
int cr_mlp_get_params(cr_mlp* mlp, float* params);
int cr_mlp_set_params(cr_mlp* mlp, const float* params);
/* inputs: n x 7 host floats; outputs: n x 3 host floats (not clamped) */
int cr_mlp_infer(cr_mlp* mlp, const float* inputs, uint64_t n, float* outputs);
/* gradient of the loss over n samples (no update); grads = param_count floats */
int cr_mlp_gradients(cr_mlp* mlp, const float* inputs, const float* targets,
                     uint64_t n, float* grads, float* loss);
/* one Adam step on n samples; loss (may be NULL) before the step.  The
 * gradients and the step are reproducible: the per-CTA gradient partials
 * are summed in a fixed order (no atomics), so the same weights, inputs and
 * n give the same new weights bit for bit, here and through
 * cr_mlp_train_step_device.  (The reported loss is summed with atomics and
 * may differ in its last bits.) */
int cr_mlp_train_step(cr_mlp* mlp, const float* inputs, const float* targets,
                      uint64_t n, float* loss);
/* The same two operations on device-resident buffers, ordered on `stream`
 * (NULL = the default stream) and returning without waiting: inputs n x 7,
 * outputs / targets n x 3 device floats.  These are the calls the cached
 * integrator makes each frame. */
int cr_mlp_infer_device(cr_mlp* mlp, const float* inputs, uint64_t n, float* outputs, void* stream);
int cr_mlp_train_step_device(cr_mlp* mlp, const float* inputs, const float* targets,
                             uint64_t n, void* stream);

/* ---- path tracing with the radiance cache (no counterpart in the
 * reference) ----
 * Each frame renders one sample per pixel.  Most paths stop at
 * query_vertex (1 = the hit of the first bounce) and take the network's
 * radiance there, weighted by the path throughput; one pixel in train_every
 * (a hash of pixel and sample index) traces its whole path with the plain
 * estimator, adds that unbiased sample to the film, and turns every vertex
 * v >= 1 into a training record (inputs at v, target = radiance gathered from
 * v on / throughput at v).  For each frame the network takes train_steps
 * Adam steps on at most train_samples records (none when freeze is set).
 * Frames use sample indices first_sample, first_sample + 1, ...  On the
 * wavefront schedule (the default) up to 8 frames (2^23 paths) render as
 * one wave, and the steps of its frames follow the wave, each frame's on its
 * share of the wave's records. */
typedef struct {
    uint32_t query_vertex;   /* 1 */
    uint32_t train_every;    /* 0 = adaptive: the spacing that yields about
                                train_samples records per frame, re-aimed after
                                every frame from the records it produced */
    uint32_t train_samples;  /* 8192 (path suffixes per frame; 0 = 8192) */
    uint32_t train_steps;    /* 1 */
    uint32_t freeze;         /* 1 = render with the cache as it is, no training */
    float scene_min[3];      /* position normalisation box; scene_max <= scene_min */
    float scene_max[3];      /* selects the scene's bounds */
} cr_cache_config;
typedef struct {
    uint64_t frames;
    uint64_t queries;
    uint64_t train_records;
    float last_loss;
    uint32_t last_train_every;  /* training-path spacing of the last frame */
} cr_cache_stats;
/* stats (may be NULL) is added to, not reset. */
int cr_render_cached(cr_scene* scene, const cr_integrator_config* cfg,
                     const cr_cache_config* cache, cr_mlp* mlp, uint32_t frames,
                     uint32_t first_sample, void* stream, cr_cache_stats* stats);

/* ---- batched rendering (no counterpart in the reference) ----
 * Many scenes (each with its camera and film set) rendered from captured
 * CUDA graphs, on one of two schedules:
 *   - persistent megakernel (wave_log2 = 0): one persistent launch whose
 *     blocks take work items (scene, pixel tile, run of spp_per_item sample
 *     indices) from one queue, largest scenes first;
 *   - wavefront (wave_log2 = 16..25): the paths of all scenes with fewer
 *     than 2^wave_log2 paths form one sequence, rendered in waves of
 *     2^wave_log2 paths; every bounce sorts the live paths by (scene,
 *     material), so a wave mixes scenes and the small ones fill the GPU
 *     together.  One captured graph of a wave is replayed wave after wave.
 *     A scene with at least one whole wave of paths renders on its own
 *     single-scene wavefront, as cr_render does.
 * Each scene's film receives exactly the samples cr_render(scene, config,
 * spp, first_sample) would add; the k-th cr_batch_render of a batch uses
 * sample indices first_sample + k*spp.  cr_batch_autotune times every
 * (tile 8|16) x (spp_per_item 1,2,4,8,16) and the wave sizes 2^20 and
 * 2^22..2^25 on the batch itself, keeps the fastest and clears the films it
 * rendered into.  The scenes must outlive the batch and keep their camera
 * size. */
typedef struct cr_batch cr_batch;
typedef struct {
    cr_integrator_config config;
    uint32_t spp;
    uint32_t first_sample;
} cr_batch_item;
typedef struct {
    uint32_t tile;          /* persistent: 8 or 16 pixels square */
    uint32_t spp_per_item;  /* persistent: sample indices per work item */
    uint32_t blocks_per_sm; /* persistent: 0 = as many as fit */
    uint32_t wave_log2;     /* 0 = persistent megakernel; 16..25 = wavefront waves of 2^wave_log2 paths */
} cr_batch_tuning;
typedef struct {
    cr_batch_tuning tuning;
    float ms;
} cr_batch_tuning_result;
int cr_batch_create(cr_scene* const* scenes, const cr_batch_item* items,
                    uint32_t n, cr_batch** out);
int cr_batch_destroy(cr_batch* batch);
int cr_batch_set_tuning(cr_batch* batch, const cr_batch_tuning* tuning);
int cr_batch_get_tuning(const cr_batch* batch, cr_batch_tuning* tuning);
/* stream NULL: the batch's own stream, waited for before returning */
int cr_batch_render(cr_batch* batch, void* stream);
/* The batch rendered with the radiance cache (cr_render_cached per scene):
 * scene i renders items[i].spp cached frames (one sample per pixel each, the
 * k-th render of the batch starting at sample index first_sample + k*spp)
 * with its own network mlps[i], all with the cache settings `cache`; the
 * scenes' configs must allow caching (RGB, query_vertex < max_depth).  The
 * scenes advance wave by wave together, each on a stream of its own, so that
 * the small scenes' waves, inference and training overlap the large ones'.
 * Each scene's film receives the samples cr_render_cached would add.  stats
 * (may be NULL) is an array of n entries, added to.  Returns when done. */
int cr_batch_render_cached(cr_batch* batch, cr_mlp* const* mlps,
                           const cr_cache_config* cache, cr_cache_stats* stats);
int cr_batch_autotune(cr_batch* batch, cr_batch_tuning* best,
                      cr_batch_tuning_result* results, uint32_t max_results,
                      uint32_t* n_results);

/* Read bandwidth (GB/s) of the memory level a buffer of `bytes` lives in:
 * the buffer is read `passes` times by persistent blocks with 16-byte loads
 * cached in L2 only, after one untimed pass; CUDA events time the passes.
 * Below the L2 size this is the L2 read bandwidth, the peak the ray queries
 * on L2-resident scenes are measured against; far above it, HBM's.  No
 * counterpart in the reference (a measurement aid for the roofline). */
int cr_device_read_bandwidth(uint64_t bytes, uint32_t passes, double* gbs);

/* Number of kernel launches this library issued since the process started
 * (all entry points); for launch accounting in benchmarks. */
uint64_t cr_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
