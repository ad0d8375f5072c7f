/*
 * lmgpu: C ABI of the GB300 (sm_103a) ray-intersection and path-sampling
 * library.  Plain C types only; every entry point returns an int status
 * (LMGPU_OK == 0) and never throws.  On failure lmgpu_last_error() returns a
 * message for the calling thread.
 *
 * Each entry point names the reference interface it stands in for
 * (Lightmetrica v2, file:line within that project).
 *
 * Buffer conventions
 *   triangles : float[ntri * 9], vertices p1, p2, p3 of each triangle after the
 *               primitive transform, in global triangle order (primitives in
 *               scene order, faces in mesh order: accel_naive.cpp:62-87).
 *   rays      : float[n * 8] = (ox, oy, oz, tmin, dx, dy, dz, tmax).
 *   hits      : lmgpu_hit[n]; prim == -1 (0xFFFFFFFF) means no hit in
 *               [tmin, tmax].  b1, b2 weight vertices p2 and p3, the (u, v)
 *               IntersectionUtils::CreateTriangleIntersection takes
 *               (intersectionutils.h:59, :115-124).
 *   "_device" entry points take device pointers and a cudaStream_t passed
 *   as void* (NULL = legacy default stream); the others take host pointers
 *   and include the host<->device copies.
 */
#ifndef LMGPU_H
#define LMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LMGPU_OK 0
#define LMGPU_ERR_INVALID 1     /* bad argument */
#define LMGPU_ERR_CUDA 2        /* a CUDA runtime call failed */
#define LMGPU_ERR_NOT_BUILT 3   /* accel used before a successful build */
#define LMGPU_ERR_OVERFLOW 4    /* a device-side bound (traversal stack) was exceeded, or the
                                   tree is malformed; the accel keeps this state until its next
                                   build, so later queries on it return it too */
#define LMGPU_ERR_NO_DEVICE 5   /* no CUDA device visible */

typedef struct {
    float t;
    int32_t prim;   /* global triangle id, -1 = miss */
    float b1, b2;
} lmgpu_hit;

typedef struct lmgpu_accel lmgpu_accel;

/* Properties of a built accel. */
typedef struct {
    uint64_t num_triangles;
    uint64_t num_binary_nodes;  /* nodes of the binned-SAH binary tree */
    uint64_t num_wide_nodes;    /* 8-wide compressed nodes (80 bytes each) */
    uint64_t node_bytes;
    uint64_t triangle_bytes;
    int32_t binary_depth;
    int32_t wide_depth;
    double build_ms;            /* device time of the last build */
} lmgpu_accel_info;

/* Traversal counters of one instrumented launch (sums over all rays). */
typedef struct {
    uint64_t rays;
    uint64_t node_fetches;      /* wide nodes loaded (80 bytes each) */
    uint64_t triangle_fetches;  /* triangles tested (48 bytes each) */
    uint64_t hits;
} lmgpu_trace_stats;

/* Version string of the library. */
const char* lmgpu_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char* lmgpu_last_error(void);

/* Creates an empty accel on the current device.
 * Stands in for Accel::Initialize (include/lightmetrica/accel.h:67);
 * the reference accels take no parameters (accel_naive.cpp:53-57). */
int lmgpu_accel_create(lmgpu_accel** out);

/* Frees an accel and its device buffers (accel_embree.cpp:68-78 frees its
 * device scene in the destructor the same way).  NULL is ignored. */
void lmgpu_accel_destroy(lmgpu_accel* accel);

/* Builds a binned-SAH BVH on the GPU and collapses it into 8-wide
 * compressed nodes.  Host triangle buffer.
 * Stands in for Accel::Build (include/lightmetrica/accel.h:79). */
int lmgpu_accel_build(lmgpu_accel* accel, const float* triangles, uint64_t ntri);

/* As lmgpu_accel_build, with the triangle buffer already on the device. */
int lmgpu_accel_build_device(lmgpu_accel* accel, const float* d_triangles, uint64_t ntri, void* stream);

/* One primitive's indexed triangle mesh (TriangleMesh::Positions / Faces,
 * include/lightmetrica/trianglemesh.h:60-90) with the primitive's transform
 * (Primitive::transform, include/lightmetrica/primitive.h:56-80):
 * positions float[3 * num_vertices], faces uint32[3 * num_faces] (vertex
 * indices), transform column-major m[column][row] = transform[4 column + row],
 * the layout of the reference's Mat4. */
typedef struct {
    const float* positions;
    const uint32_t* faces;
    uint32_t num_vertices;
    uint32_t num_faces;
    float transform[16];
} lmgpu_mesh;

/* Flattens n meshes on the GPU into d_triangles (float[9 * total faces]) in
 * global order -- meshes in order, faces in mesh order, as the reference's
 * accels enumerate them (accel_naive.cpp:59-90) -- and, if d_tri_prim is not
 * NULL, each triangle's mesh index into it.  positions and faces are device
 * pointers.  Vertices go through the transform with the reference's
 * single-precision arithmetic (Mat4 x Vec4, math.h:1268-1279: every product
 * and sum rounded, no fused multiply-add), so the triangles equal the
 * reference's bit for bit.  A face index outside its mesh returns
 * LMGPU_ERR_INVALID.  Returns after the flattening has finished. */
int lmgpu_flatten_meshes_device(const lmgpu_mesh* meshes, uint32_t n, float* d_triangles, int32_t* d_tri_prim,
                                void* stream);

/* Builds the accel from host meshes: checks the face indices, uploads
 * positions and faces (12 bytes per vertex and per face instead of 36 per
 * flattened triangle), flattens them on the GPU as
 * lmgpu_flatten_meshes_device does, and builds.  Stands in for Accel::Build
 * (include/lightmetrica/accel.h:79) with its triangle enumeration. */
int lmgpu_accel_build_meshes(lmgpu_accel* accel, const lmgpu_mesh* meshes, uint32_t n);

/* Fills *info for a built accel. */
int lmgpu_accel_get_info(const lmgpu_accel* accel, lmgpu_accel_info* info);

/* Closest hit (anyhit = 0) or any hit (anyhit = 1) for n rays, host buffers,
 * copies included.  Closest hit stands in for Accel3::Intersect
 * (include/lightmetrica/accel3.h:68); any hit for Scene3::Visible
 * (include/lightmetrica/scene3.h:107-116), which the reference answers with a
 * full closest-hit query.  Ties at equal t resolve to the higher global
 * triangle id, the order accel::naive keeps (accel_naive.cpp:99-110).
 * Queries of at most 256 rays (a single-ray Intersect) go through a pinned,
 * device-mapped buffer: one launch and one synchronisation per call.  Larger
 * ones on page-locked buffers (cudaHostAlloc, cudaHostRegister) are traced in
 * place, the kernel reading the rays and writing the hits across the host
 * link; on pageable memory they are staged through device memory in
 * overlapped batches.  Calls on one accel from several threads are
 * serialised. */
int lmgpu_trace(const lmgpu_accel* accel, const float* rays, lmgpu_hit* hits, uint64_t n, int anyhit);

/* As lmgpu_trace on device buffers (rays 16-byte aligned), asynchronous on
 * `stream`; the status of device-side bounds is checked by the next
 * lmgpu_accel_check or synchronous call. */
int lmgpu_trace_device(const lmgpu_accel* accel, const float* d_rays, lmgpu_hit* d_hits, uint64_t n,
                       int anyhit, void* stream);

/* Runs the instrumented traversal once (device buffers) and returns its
 * counters; used to state the algorithmic bytes per ray. */
int lmgpu_trace_stats_device(const lmgpu_accel* accel, const float* d_rays, lmgpu_hit* d_hits, uint64_t n,
                             int anyhit, void* stream, lmgpu_trace_stats* stats);

/* Sets the traversal kernel's scheduling knobs for this accel: a warp takes
 * new rays once `refill` of its 32 lanes are idle (1..32), and postpones
 * triangle tests while fewer than `postpone` lanes have triangle work
 * (0..32, 0 = never postpone).  Results do not depend on them; speed does.
 * No counterpart in the reference (its accels trace one ray per call). */
int lmgpu_accel_set_tuning(lmgpu_accel* accel, int refill, int postpone);

/* Synchronises `stream` and reports device-side errors (stack overflow)
 * raised by earlier asynchronous launches. */
int lmgpu_accel_check(const lmgpu_accel* accel, void* stream);

/* ---- Path tracing (renderer::pt) -------------------------------------- */

#define LMGPU_BSDF_NULL 0           /* bsdf::null: paths end here (bsdf_null.cpp) */
#define LMGPU_BSDF_DIFFUSE 1        /* bsdf::diffuse, reflectance R (bsdf_diffuse.cpp) */
#define LMGPU_BSDF_DIELECTRIC 2     /* bsdf::flesnel, R, eta1 (outside), eta2 (inside) */
#define LMGPU_BSDF_COOK_TORRANCE 3  /* bsdf::cook_torrance: GGX, R, conductor eta/k, roughness */

/* One scene primitive (Primitive, include/lightmetrica/primitive.h:56-80):
 * its BSDF and, if is_light, an area light (light::area, light_area.cpp)
 * with radiance Le over its triangles, emitting on the front side.
 * Parameter defaults of the reference: eta1 1, eta2 2 (bsdf_flesnel.cpp:49-50);
 * ct_eta (0.14, 0.129, 0.1585), ct_k (4.58625, 3.348125, 2.329375),
 * roughness 0.1 (bsdf_cooktorrance.cpp:58-63). */
typedef struct {
    int32_t bsdf;
    int32_t is_light;
    float R[3];
    float Le[3];
    float eta1, eta2;
    float ct_eta[3], ct_k[3];
    float roughness;
} lmgpu_prim;

/* Pinhole sensor at a lookat node (scene3.cpp:213-221, sensor_pinhole.cpp):
 * vertical fov in degrees, film width x height. */
typedef struct {
    float eye[3], center[3], up[3];
    float fov_deg;
    int32_t width, height;
} lmgpu_camera;

/* Renderer parameters (renderer_pt.cpp:56-62 and the same in the other
 * renderers): samples per pixel (the reference's num_samples = width *
 * height * spp), max_num_vertices (-1 = unbounded), the seed of the
 * counter-based random numbers, and min_num_vertices (0 = none; paths with
 * fewer vertices contribute nothing, as each renderer applies it:
 * renderer_pt.cpp:186, renderer_ptmis.cpp:132, :247, renderer_bdpt.cpp:892;
 * renderer::ptdirect and renderer::ltdirect have no minimum). */
typedef struct {
    uint64_t spp;
    int32_t max_num_vertices;
    uint32_t seed;
    int32_t min_num_vertices;
    int32_t reserved;
} lmgpu_pt_params;

typedef struct lmgpu_scene lmgpu_scene;

/* Uploads a scene (triangles in global order, the primitive of each, the
 * primitives, the camera) and builds its BVH on the GPU.  Stands in for
 * Scene::Initialize (include/lightmetrica/scene.h:59) with Accel::Build. */
int lmgpu_scene_create(const float* triangles, const int32_t* tri_prim, uint64_t ntri, const lmgpu_prim* prims,
                       uint32_t nprims, const lmgpu_camera* camera, lmgpu_scene** out);

/* Frees a scene and everything it owns.  NULL is ignored. */
void lmgpu_scene_destroy(lmgpu_scene* scene);

/* Adds (Le != NULL) or removes a constant environment light (light::env
 * without an envmap, light_env.cpp): radiance Le arrives from every
 * direction on the scene's bounding sphere (scene3.cpp:52-78), which rays
 * meet when they leave the geometry (scene3.cpp:464-475). */
int lmgpu_scene_set_environment(lmgpu_scene* scene, const float* Le);

/* Number of kernels the renderers have launched for this scene since it was
 * created (a diagnostic; no counterpart in the reference). */
int lmgpu_scene_launch_count(const lmgpu_scene* scene, uint64_t* count);

/* The scene's accel (owned by the scene), for ray queries on its triangles. */
int lmgpu_scene_accel(const lmgpu_scene* scene, const lmgpu_accel** accel);

/* Instrumentation of the traversal launches of a scene's renders (and of a
 * batch's, lmgpu_batch_set_trace_profile), the dominant kernel of every
 * renderer (a diagnostic; no counterpart in the reference).  Images are
 * unchanged in every mode. */
enum {
    LMGPU_TRACE_PROFILE_OFF = 0,
    LMGPU_TRACE_PROFILE_COUNT = 1, /* launch the counting traversal: rays, node and triangle fetches, hits */
    LMGPU_TRACE_PROFILE_TIME = 2   /* the production traversal, device time of each launch (CUDA events) */
};
typedef struct {
    uint64_t launches;         /* traversal launches since the last read */
    uint64_t rays;             /* COUNT: rays traced */
    uint64_t node_fetches;     /* COUNT: 80-byte node fetches */
    uint64_t triangle_fetches; /* COUNT: 48-byte triangle tests */
    uint64_t hits;             /* COUNT: rays that hit */
    double device_ms;          /* TIME: summed device time of the timed launches */
    uint64_t timed_launches;   /* TIME: launches inside device_ms (at most 4,096 between reads) */
    /* The photon-merge launches of renderer::vcm (modes vcm and bdpm), that
     * renderer's dominant kernel: */
    uint64_t merge_launches;     /* merge launches since the last read */
    uint64_t merge_queries;      /* COUNT: eye vertices that looked for photons */
    uint64_t merge_eye_vertices; /* COUNT: eye-subpath vertex records those queries read */
    uint64_t merge_entries;      /* COUNT: photon entries scanned in the queries' grid cells */
    uint64_t merges;             /* COUNT: photons within the radius, evaluated */
    double merge_ms;             /* TIME: summed device time of the merge launches */
    uint64_t merge_timed_launches; /* TIME: launches inside merge_ms (at most 512 between reads) */
} lmgpu_trace_profile;

/* Selects the mode and clears the record. */
int lmgpu_scene_set_trace_profile(lmgpu_scene* scene, int mode);

/* Waits for the device, returns the record since the last read or mode
 * change and clears it. */
int lmgpu_scene_read_trace_profile(lmgpu_scene* scene, lmgpu_trace_profile* out);

/* Renders the scene with the wavefront path tracer and writes the film
 * (height x width x 3 floats, row = raster y from the bottom, as
 * film_hdr.cpp:218-223 indexes it) and, if variance is not NULL, the
 * per-pixel variance of that estimate.  Host buffers.  Stands in for
 * Renderer::Render of renderer::pt (include/lightmetrica/renderer.h:81). */
int lmgpu_render_pt(lmgpu_scene* scene, const lmgpu_pt_params* params, float* image, float* variance);

/* As lmgpu_render_pt into device buffers on `stream` (NULL: the scene's
 * stream); returns after the render has finished. */
int lmgpu_render_pt_device(lmgpu_scene* scene, const lmgpu_pt_params* params, float* d_image, float* d_variance,
                           void* stream);

/* Renders the scene with path tracing plus next-event estimation: one light
 * sample per vertex (the sensor included) combined with BSDF sampling by the
 * balance heuristic.  Stands in for Renderer::Render of renderer::ptmis
 * (src/liblightmetrica/renderer/renderer_ptmis.cpp:68-325).  The scene needs
 * at least one area light; environment lights are not sampled by this
 * renderer (LMGPU_ERR_INVALID if the scene has one). */
int lmgpu_render_ptmis(lmgpu_scene* scene, const lmgpu_pt_params* params, float* image, float* variance);

/* As lmgpu_render_ptmis into device buffers on `stream` (NULL: the scene's
 * stream); returns after the render has finished. */
int lmgpu_render_ptmis_device(lmgpu_scene* scene, const lmgpu_pt_params* params, float* d_image, float* d_variance,
                              void* stream);

/* Renders the scene with path tracing by light samples only: one light
 * sample per vertex (the sensor included) with weight 1, and no emission
 * counted on BSDF-sampled hits.  Stands in for Renderer::Render of
 * renderer::ptdirect (src/liblightmetrica/renderer/renderer_ptdirect.cpp:72-291).
 * Same scene requirements as lmgpu_render_ptmis. */
int lmgpu_render_ptdirect(lmgpu_scene* scene, const lmgpu_pt_params* params, float* image, float* variance);

/* As lmgpu_render_ptdirect into device buffers on `stream`. */
int lmgpu_render_ptdirect_device(lmgpu_scene* scene, const lmgpu_pt_params* params, float* d_image,
                                 float* d_variance, void* stream);

/* Renders the scene by light tracing: params->spp x W x H light paths, each
 * connected to the pinhole at every vertex (weight 1), Russian roulette 0.5
 * after every hit, at most max_num_vertices vertices per full path.  Stands
 * in for Renderer::Render of renderer::ltdirect
 * (src/liblightmetrica/renderer/renderer_ltdirect.cpp:72-279; num_samples =
 * spp x W x H).  Needs an area light; scenes with an environment light are
 * rejected.  The variance is that of the image's light-path estimate. */
int lmgpu_render_ltdirect(lmgpu_scene* scene, const lmgpu_pt_params* params, float* image, float* variance);

/* As lmgpu_render_ltdirect into device buffers on `stream`. */
int lmgpu_render_ltdirect_device(lmgpu_scene* scene, const lmgpu_pt_params* params, float* d_image,
                                 float* d_variance, void* stream);

/* Renders the scene with bidirectional path tracing (all (s, t) strategies,
 * power-heuristic MIS) and writes the film as lmgpu_render_pt does.  Stands
 * in for Renderer::Render of renderer::bdpt
 * (src/liblightmetrica/renderer/renderer_bdpt.cpp:841-998).  The scene needs
 * at least one area light (LMGPU_ERR_INVALID otherwise); the environment
 * light is not part of this estimator, as in the reference.  Light and eye
 * subpaths are capped at 16 vertices each (max_num_vertices = -1 included);
 * with roulette 0.5 per step a subpath reaches that cap with probability
 * 2^-14. */
int lmgpu_render_bdpt(lmgpu_scene* scene, const lmgpu_pt_params* params, float* image, float* variance);

/* As lmgpu_render_bdpt into device buffers on `stream` (NULL: the scene's
 * stream); returns after the render has finished. */
int lmgpu_render_bdpt_device(lmgpu_scene* scene, const lmgpu_pt_params* params, float* d_image, float* d_variance,
                             void* stream);

/* MIS weights of renderer::bdpt's "mis" parameter. */
#define LMGPU_MIS_POWER 0  /* misweight::powerheuristics (renderer_bdpt.cpp:747-784), the default */
#define LMGPU_MIS_SIMPLE 1 /* misweight::simple (renderer_bdpt.cpp:711-744): one over the number of
                              strategies that can sample the path */

/* As lmgpu_render_bdpt / lmgpu_render_bdpt_device with the MIS weight
 * chosen (LMGPU_MIS_*). */
int lmgpu_render_bdpt_mis(lmgpu_scene* scene, const lmgpu_pt_params* params, int mis, float* image,
                          float* variance);
int lmgpu_render_bdpt_mis_device(lmgpu_scene* scene, const lmgpu_pt_params* params, int mis, float* d_image,
                                 float* d_variance, void* stream);

/* ---- Vertex connection and merging (renderer::vcm) ---------------------- */

/* Estimators of renderer::vcm's "mode" parameter (renderer_vcm.cpp:581-587). */
#define LMGPU_VCM_MODE_VCM 0  /* connections and merges, EvaluateMISWeight_VCM */
#define LMGPU_VCM_MODE_BDPT 1 /* connections only, EvaluateMISWeight_BDPT */
#define LMGPU_VCM_MODE_BDPM 2 /* merges only, EvaluateMISWeight_BDPM */

/* The parameters of Renderer_VCM::Initialize (renderer_vcm.cpp:573-593),
 * whose defaults are max_num_vertices 10, min_num_vertices 0,
 * num_iteration_pass 100, num_photon_trace_samples 10000,
 * num_eye_trace_samples 10000, initial_radius 0.1, alpha 0.7, mode vcm. */
typedef struct lmgpu_vcm_params {
    int32_t max_num_vertices;          /* 1 .. 16: subpaths have no roulette, so the cap is required */
    int32_t min_num_vertices;
    uint64_t num_iteration_pass;
    uint64_t num_photon_trace_samples; /* light subpaths per pass, < 2^28 */
    uint64_t num_eye_trace_samples;    /* eye samples per pass */
    float initial_radius;
    float alpha;
    int32_t mode;                      /* LMGPU_VCM_MODE_* */
    uint32_t seed;
} lmgpu_vcm_params;

/* Renders the scene with vertex connection and merging and writes the film
 * as lmgpu_render_pt does (the mean of the passes' images).  Stands in for
 * Renderer::Render of renderer::vcm (src/liblightmetrica/renderer/
 * renderer_vcm.cpp:596-790).  Per pass k the merge radius is initial_radius,
 * then sqrt((alpha + k) / (1 + k)) times the previous one; the photon
 * subpaths of the pass are put in a hashed grid of cells r wide; every eye
 * sample traces an eye subpath and a light subpath and combines them by all
 * connections and by merges with the photon vertices within r of each eye
 * vertex.  Eye samples are stratified over the pixels when
 * num_eye_trace_samples is a multiple of W x H, uniform over the film
 * otherwise.  Needs an area light; environment lights are rejected. */
int lmgpu_render_vcm(lmgpu_scene* scene, const lmgpu_vcm_params* params, float* image, float* variance);

/* As lmgpu_render_vcm into device buffers on `stream` (NULL: the scene's
 * stream); returns after the render has finished. */
int lmgpu_render_vcm_device(lmgpu_scene* scene, const lmgpu_vcm_params* params, float* d_image, float* d_variance,
                            void* stream);

/* ---- Batched path tracing: many scenes / views in one wavefront -------- */

typedef struct lmgpu_batch lmgpu_batch;

/* renderer::pt parameters for a batch (all views share them).  rr_depth:
 * Russian roulette (probability 0.5) applies once a path has more than
 * rr_depth segments; 0 reproduces renderer::pt (roulette at every hit,
 * renderer_pt.cpp:207-216).  Both are unbiased. */
typedef struct {
    uint64_t spp;
    int32_t max_num_vertices;
    uint32_t seed;
    int32_t rr_depth;
} lmgpu_batch_params;

/* Scheduling knobs of a batch: traversal refill / postpone thresholds (see
 * lmgpu_accel_set_tuning) and the number of paths per wave; probe_ms is the
 * autotuner's best probe time (output only). */
typedef struct {
    int32_t refill;
    int32_t postpone;
    uint64_t wave_paths;
    double probe_ms;
} lmgpu_batch_tuning;

/* Groups n scenes (each with its own geometry, BVH, camera and resolution;
 * 1 <= n <= 255, fewer than 2^24 pixels each) for lmgpu_batch_render_pt.  The
 * scenes are borrowed and must outlive the batch.  No counterpart in the
 * reference (its renderers render one scene per process). */
int lmgpu_batch_create(lmgpu_scene* const* scenes, uint32_t n, lmgpu_batch** out);

/* Frees a batch (not its scenes).  NULL is ignored. */
void lmgpu_batch_destroy(lmgpu_batch* batch);

/* Renders every view of the batch with renderer::pt's estimator in one
 * wavefront (paths of all views share the queues and the traversal
 * launches; the per-bounce work is replayed from CUDA graphs).  images[v]
 * (and variances[v] if variances is not NULL) receive view v's film, laid
 * out as lmgpu_render_pt's. */
int lmgpu_batch_render_pt(lmgpu_batch* batch, const lmgpu_batch_params* params, float* const* images,
                          float* const* variances);

/* As lmgpu_batch_render_pt into device buffers: the views' films one after
 * another in d_images (and d_variances, may be NULL), rendered on `stream`
 * (NULL: the batch's own stream); returns after the render has finished. */
int lmgpu_batch_render_pt_device(lmgpu_batch* batch, const lmgpu_batch_params* params, float* d_images,
                                 float* d_variances, void* stream);

/* Measures renders of `probe` over candidate tunings (coordinate descent over
 * refill, postpone and wave size), keeps the fastest and returns it. */
int lmgpu_batch_autotune(lmgpu_batch* batch, const lmgpu_batch_params* probe, lmgpu_batch_tuning* out);

/* Sets / reads the batch's tuning. */
int lmgpu_batch_set_tuning(lmgpu_batch* batch, const lmgpu_batch_tuning* tuning);
int lmgpu_batch_get_tuning(const lmgpu_batch* batch, lmgpu_batch_tuning* tuning);

/* Kernels the batch renderer has launched so far (a diagnostic). */
int lmgpu_batch_launch_count(const lmgpu_batch* batch, uint64_t* count);

/* The trace profile (lmgpu_scene_set_trace_profile) of the batch's
 * multi-scene traversal launches.  While a mode other than OFF is set, the
 * bounces are launched one by one instead of through the captured graphs,
 * so that every traversal launch can be counted or timed; images are
 * unchanged. */
int lmgpu_batch_set_trace_profile(lmgpu_batch* batch, int mode);
int lmgpu_batch_read_trace_profile(lmgpu_batch* batch, lmgpu_trace_profile* out);

/* ---- Learned path guiding: the network ----------------------------------
 * A small MLP (input: position with a 16-frequency encoding, normal,
 * outgoing direction; 4 x 64 ReLU; output: 8 von Mises-Fisher lobes) run on
 * the tensor cores, trained online with Adam.  No counterpart in the
 * reference.  Queries are float[9] each: position, normal, outgoing
 * direction; raw outputs float[40] each: per lobe (mean 3, kappa
 * pre-activation, weight logit). */

typedef struct lmgpu_guide lmgpu_guide;

/* Number of FP32 parameters (the layout is documented in guide_net.cuh). */
int lmgpu_guide_num_params(uint64_t* n);

/* Creates a network with seeded initial weights for positions in the box
 * box_lo_hi = (lo.x, lo.y, lo.z, hi.x, hi.y, hi.z). */
int lmgpu_guide_create(const float* box_lo_hi, uint32_t seed, lmgpu_guide** out);
void lmgpu_guide_destroy(lmgpu_guide* guide);

/* Copies the FP32 master parameters out / in (n = lmgpu_guide_num_params). */
int lmgpu_guide_get_params(const lmgpu_guide* guide, float* params, uint64_t n);
int lmgpu_guide_set_params(lmgpu_guide* guide, const float* params, uint64_t n);

/* Raw outputs of n queries (host buffers). */
int lmgpu_guide_forward(lmgpu_guide* guide, const float* queries, uint64_t n, float* raw);

/* Gradient of the mean loss -(1/n) sum_i weights[i] log q(dirs[i] | query i)
 * with respect to the parameters (float[num_params]) and the loss value;
 * the parameters are not changed. */
int lmgpu_guide_gradient(lmgpu_guide* guide, const float* queries, const float* dirs, const float* weights,
                         uint64_t n, float* grad, float* loss);

/* Device-buffer forms, asynchronous on `stream` (no status check; a later
 * host-buffer call reports tensor-core time-outs). */
int lmgpu_guide_forward_device(lmgpu_guide* guide, const float* d_queries, uint64_t n, float* d_raw, void* stream);
int lmgpu_guide_train_step_device(lmgpu_guide* guide, const float* d_queries, const float* d_dirs,
                                  const float* d_weights, uint64_t n, float lr, void* stream);

/* One Adam step (beta 0.9 / 0.999, learning rate lr) on that loss. */
int lmgpu_guide_train_step(lmgpu_guide* guide, const float* queries, const float* dirs, const float* weights,
                           uint64_t n, float lr, float* loss);

/* ---- Guided path tracing -------------------------------------------------- */

/* alpha: probability of BSDF sampling in the one-sample MIS mixture with the
 * network (0.5); learning_rate: Adam's (1e-3); train: nonzero to train the
 * network after every wave of passes; batch: training minibatch (2^18);
 * max_steps_per_pass: Adam steps after a wave at most; rr_mode: 0 Russian
 * roulette with survival 0.5 as renderer::pt, 1 survival min(1, max
 * throughput component). */
typedef struct {
    float alpha;
    float learning_rate;
    uint32_t train;
    uint32_t batch;
    uint32_t max_steps_per_pass;
    uint32_t rr_mode;
} lmgpu_guiding_params;

/* Renders renderer::pt's image with guided direction sampling at diffuse
 * vertices (one-sample MIS of BSDF sampling and the guide's mixture; every
 * pass unbiased), params->spp passes of one sample per pixel, training the
 * guide online between passes.  The film is written as lmgpu_render_pt's;
 * last_loss (may be NULL) receives the last training step's loss.  Films of
 * at most 2^21 pixels.  No counterpart in the reference. */
int lmgpu_render_pt_guided(lmgpu_scene* scene, lmgpu_guide* guide, const lmgpu_pt_params* params,
                           const lmgpu_guiding_params* guiding, float* image, float* variance, float* last_loss);

/* As lmgpu_render_pt_guided into device buffers on `stream`. */
int lmgpu_render_pt_guided_device(lmgpu_scene* scene, lmgpu_guide* guide, const lmgpu_pt_params* params,
                                  const lmgpu_guiding_params* guiding, float* d_image, float* d_variance,
                                  void* stream, float* last_loss);

/* ---- Surface geometry at hits ---------------------------------------------- */

/* Shading attributes for lmgpu_surface, per triangle in global order (the
 * order lmgpu_accel_build received): normals [ntri*9] = the three vertex
 * normals through the primitive's normal transform (intersectionutils.h:91-93),
 * or NULL; texcoords [ntri*6] = the three vertices' (u, v), or NULL; flags
 * [ntri] (bit 0 the triangle has normals, bit 1 texcoords) or NULL for
 * every triangle having what is given.  Host memory; call after a build
 * (a rebuild drops them).  Without attributes every triangle uses its
 * geometric normal and uv (0, 0), as for a mesh without normals or
 * texcoords.  Stands in for the per-hit mesh lookups of
 * IntersectionUtils::CreateTriangleIntersection (intersectionutils.h:59-135). */
int lmgpu_accel_set_attributes(lmgpu_accel* accel, const float* normals, const float* texcoords,
                               const uint8_t* flags, uint64_t ntri);

/* Planes of lmgpu_surface's output. */
#define LMGPU_SURFACE_PLANES 23

/* Surface geometry of n hits (lmgpu_hit from lmgpu_trace for the same rays):
 * what IntersectionUtils::CreateTriangleIntersection (intersectionutils.h:59)
 * puts in Intersection::geom for each, as LMGPU_SURFACE_PLANES planes of n
 * floats (plane k of hit i at surface[k * n + i]): p (planes 0-2, o + d t),
 * gn (3-5), sn (6-8), dpdu (9-11), dpdv (12-14), dndu (15-17), dndv (18-20),
 * uv (21-22).  ToWorld is the matrix of columns (dpdu, dpdv, sn) and ToLocal
 * its transpose.  Misses (prim < 0) give zeros.  Host buffers.
 * The per-triangle records these queries read are packed by
 * lmgpu_accel_set_attributes, or else by the first query after a build,
 * which then waits for them (under the accel's lock, so concurrent queries
 * from several threads are safe).  Page-locked buffers are read and written
 * in place by the kernel; pageable ones go through a staging buffer the
 * accel keeps, 2^20 hits at a time. */
int lmgpu_surface(const lmgpu_accel* accel, const float* rays, const lmgpu_hit* hits, uint64_t n, float* surface);

/* As lmgpu_surface on device buffers, asynchronous on `stream`, except the
 * first query after a build (or after lmgpu_accel_set_attributes failed to
 * pack): it allocates the per-triangle records and synchronises `stream`
 * while packing them, so make it before capturing surface queries into a
 * CUDA graph. */
int lmgpu_surface_device(const lmgpu_accel* accel, const float* d_rays, const lmgpu_hit* d_hits, uint64_t n,
                         float* d_surface, void* stream);

/* Largest scene lmgpu_trace_static_scene accepts. */
#define LMGPU_STATIC_MAX_TRIANGLES 16384

/* Builds the BVH of d_triangles (float[ntri*9], device) and traces d_rays
 * (float[nrays*8], device) against it, writing d_hits (device), closest hit
 * (anyhit = 0) or any hit (anyhit = 1) -- without allocating device memory.
 * No counterpart in the reference: it exists for callers that cannot
 * allocate (a plugin inside a host that owns all device memory through its
 * own pool, or a query path that must not incur the device-wide
 * synchronisation of cudaMalloc/cudaFree).  All scratch, including the BVH,
 * is one fixed library-owned device array of about 5.4 MiB, reserved on
 * every device that loads the library until the process exits; scenes
 * above LMGPU_STATIC_MAX_TRIANGLES are rejected with LMGPU_ERR_INVALID.
 * The first call on a device looks up that array's address (set-up), so
 * make it before any stream capture.  Every call shares the array and it
 * keeps the previous call's contents: calls that overlap on the GPU (other
 * host threads or streams) race and must be serialised by the caller.
 * Synchronises `stream` before returning.  Closest-hit results (the
 * triangle and t) equal those of lmgpu_accel_build_device +
 * lmgpu_trace_device on the same inputs; any-hit results agree on hit or
 * miss only, since which blocking triangle an any-hit query reports depends
 * on the tree, and this path always collapses its BVH greedily (the
 * allocating path uses the SAH-optimal collapse from 4,096 triangles on). */
int lmgpu_trace_static_scene(const float* d_triangles, uint64_t ntri, const float* d_rays, lmgpu_hit* d_hits,
                             uint64_t nrays, int anyhit, void* stream);

#ifdef __cplusplus
}
#endif
#endif
