/*
 * CPU oracle for the ray-intersection and path-sampling hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference's CPU algorithms, used by tests/ as the checker and by bench.py
 * as the timed CPU baseline.  The product (the CUDA library behind
 * include/lmgpu.h) never links, loads or calls it.
 *
 * Every function names the reference file:line it restates.  Floating-point
 * expressions keep the reference's operation order and are compiled with
 * -ffp-contract=off, so that results are bit-identical to the reference
 * compiled from its own sources (checked against fixtures in tests/golden/).
 */
#ifndef LMORACLE_H
#define LMORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* TriAccelTriangle (include/lightmetrica/triaccel.h:35-48). */
typedef struct {
    uint32_t k;
    float n_u, n_v, n_d;
    float a_u, a_v;
    float b_nu, b_nv;
    float c_nu, c_nv;
    uint32_t face_index;
    uint32_t prim_index;
} lmo_triaccel;

/* One hit record, shared by every trace routine of the oracle.
 * id = global triangle id or -1; b = barycentrics weighting vertices 2, 3;
 * p = ray.o + ray.d * t, the point the reference stores (accel_naive.cpp:118). */
typedef struct {
    int32_t id;
    float t;
    float b0, b1;
    float p[3];
} lmo_hit;

/* Ray layout of the C-ABI: ox, oy, oz, tmin, dx, dy, dz, tmax (32 bytes). */

int  lmo_triaccel_load(lmo_triaccel* tri, const float A[3], const float B[3], const float C[3]);
int  lmo_triaccel_intersect(const lmo_triaccel* tri, const float o[3], const float d[3],
                            float mint, float maxt, float* u, float* v, float* t);

/* Opaque accel built over `ntri` triangles given as 9 floats each
 * (v1, v2, v3 in global triangle order). */
typedef struct lmo_accel lmo_accel;

/* kind: 0 = accel::naive (accel_naive.cpp), 1 = accel::bvh_sahbin (accel_bvh_sahbin.cpp),
 *       2 = accel::qbvh (accel_qbvh.cpp) */
lmo_accel* lmo_accel_build(int kind, const float* tris, size_t ntri);
void       lmo_accel_free(lmo_accel* a);
/* Closest hit for n rays using `threads` POSIX threads. */
void       lmo_accel_trace(const lmo_accel* a, const float* rays, size_t n, lmo_hit* out, int threads);
/* Counts of the BVH: nodes, leaves, max binary depth (bvh_sahbin: binary nodes; qbvh: 4-wide nodes). */
void       lmo_accel_stats(const lmo_accel* a, size_t* nodes, size_t* leaves, int* depth);

/* FP64 recomputation of the ray parameter t at which the ray meets the plane
 * of triangle `tri` (9 floats), and of its barycentrics (b1, b2). */
double     lmo_plane_t_fp64(const float* tri, const float* ray, double* b1, double* b2);

/* ---- renderer::pt (lmoracle_pt.c) ---- */

#define LMO_BSDF_NULL 0
#define LMO_BSDF_DIFFUSE 1
#define LMO_BSDF_DIELECTRIC 2     /* bsdf::flesnel */
#define LMO_BSDF_COOK_TORRANCE 3  /* bsdf::cook_torrance (GGX) */

/* One scene primitive: its BSDF and, when is_light, an area light on it. */
typedef struct {
    int32_t bsdf;
    int32_t is_light;
    float R[3];
    float Le[3];
    float eta1, eta2;          /* flesnel: outside / inside index */
    float ct_eta[3], ct_k[3];  /* cook_torrance: conductor eta, k */
    float roughness;           /* cook_torrance: GGX alpha */
} lmo_pt_prim;

/* Constant environment light (light::env without an envmap). */
typedef struct {
    int32_t enabled;
    float Le[3];
} lmo_pt_env;

/* Pinhole camera from a lookat node; fov is vertical, in degrees. */
typedef struct {
    float eye[3], center[3], up[3];
    float fov_deg;
    int32_t width, height;
} lmo_pt_camera;

/* Renders num_samples paths with `threads` threads; fills per-pixel sums of
 * splatted values and of their squares (H*W*3 doubles each, row = raster y). */
uint64_t lmo_render_pt(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                       const lmo_pt_env* env, const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices,
                       uint64_t seed, int threads, double* sum, double* sumsq);

/* ---- renderer::bdpt (lmoracle_bdpt.c): area lights, pinhole, power heuristic ---- */
uint64_t lmo_render_bdpt(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims, int nprims,
                         const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices, uint64_t seed,
                         int threads, double* sum, double* sumsq);

/* ---- renderer::ptmis (lmoracle_bdpt.c): area lights, NEE + balance heuristic ---- */
uint64_t lmo_render_ptmis(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims, int nprims,
                          const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices, uint64_t seed,
                          int threads, double* sum, double* sumsq);

/* ---- renderer::ptdirect (lmoracle_bdpt.c): light samples only, weight 1 ---- */
uint64_t lmo_render_ptdirect(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                             int nprims, const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices,
                             uint64_t seed, int threads, double* sum, double* sumsq);

/* renderer::ltdirect (renderer_ltdirect.cpp:72-279): num_samples light paths,
 * sensor connections at every vertex; films as lmo_render_bdpt.  (The
 * variant with an independent emission-direction sample is
 * lmo_render_bdpt_ex with independent_light_dir = -4.) */
uint64_t lmo_render_ltdirect(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                             int nprims, const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices,
                             uint64_t seed, int threads, double* sum, double* sumsq);

/* As lmo_render_bdpt; independent_light_dir != 0 draws the light subpath's
 * first direction from its own 2D sample instead of reusing the position's
 * (the reference's light_area.cpp:73-80 reuses it).  A diagnostic that
 * isolates the effect of that reuse on the estimate. */
uint64_t lmo_render_bdpt_ex(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                            int nprims, const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices,
                            uint64_t seed, int threads, double* sum, double* sumsq, int independent_light_dir);

/* As lmo_render_bdpt_ex with renderer::bdpt's MIS weight: mis 0
 * misweight::powerheuristics (renderer_bdpt.cpp:747-784), 1 misweight::simple
 * (:711-744). */
uint64_t lmo_render_bdpt_mis(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims,
                             int nprims, const lmo_pt_camera* cam, uint64_t num_samples, int max_num_vertices,
                             uint64_t seed, int threads, double* sum, double* sumsq, int independent_light_dir,
                             int mis);

/* renderer::vcm (renderer_vcm.cpp:536-797): the parameters of
 * Renderer_VCM::Initialize (:573-593); mode 0 vcm, 1 bdpt, 2 bdpm. */
typedef struct {
    int32_t max_num_vertices;
    int32_t min_num_vertices;
    uint64_t num_iteration_pass;
    uint64_t num_photon_trace_samples;
    uint64_t num_eye_trace_samples;
    float initial_radius;
    float alpha;
    int32_t mode;
    int32_t reserved;
} lmo_vcm_params;

/* Sums over all passes of the per-sample splats (each already scaled by
 * W H / num_eye_trace_samples) and of their per-pixel squares; the
 * reference's film is sum / num_iteration_pass.  Returns the eye samples
 * processed (passes x num_eye_trace_samples); max_num_vertices outside
 * [1, 64] renders nothing. */
uint64_t lmo_render_vcm(const float* tris, const int32_t* tri_prim, size_t ntri, const lmo_pt_prim* prims, int nprims,
                        const lmo_pt_camera* cam, const lmo_vcm_params* prm, uint64_t seed, int threads, double* sum,
                        double* sumsq);

/* Surface geometry of n hits (IntersectionUtils::CreateTriangleIntersection,
 * intersectionutils.h:59-135) in double precision.  tris / normals: [ntri*9]
 * per triangle in global order, already through the primitive's transform /
 * normal transform (normals may be NULL); texcoords [ntri*6] or NULL; flags
 * [ntri] (bit 0 normals, bit 1 texcoords) or NULL; rays [n*8]; hits [n*4] =
 * (t, prim, b1, b2), prim < 0 a miss.  out [n*23] per hit: p, gn, sn, dpdu,
 * dpdv, dndu, dndv (3 each), u, v; zeros for misses. */
void lmo_surface(const double* tris, const double* normals, const double* texcoords, const uint8_t* flags,
                 const double* rays, const double* hits, size_t n, double* out);

#ifdef __cplusplus
}
#endif
#endif
