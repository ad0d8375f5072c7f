// TEST INFRASTRUCTURE ONLY: a CPU stand-in for the liblmgpu C ABI
// (include/lmgpu.h), so that the reference-side plugins (plugin/*.cpp) can be
// linked into the reference harness and executed through the reference's
// component interfaces on a machine that has the reference tree but no GPU.
// It implements the entry points the plugins call, with the documented
// semantics, on top of the CPU oracle (oracle/lmoracle_*.c):
//   accels     mesh flattening with the reference's Mat4 x Vec4 rounding,
//              closest hits by the oracle's accel::naive (ties to the higher
//              triangle id, as the GPU resolves them) or accel::bvh_sahbin
//              above 4,096 triangles, surface geometry by lmo_surface;
//   renderers  the oracle's restatements of renderer::pt, ptmis, ptdirect,
//              ltdirect, bdpt and vcm; the guided tracer's stand-in renders
//              renderer::pt (the guided estimator has the same expectation).
// It is never linked into the product library, which runs on the GPU only.
#include <lmgpu.h>

extern "C" {
#include "../lmoracle.h"
}

#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace {

thread_local std::string g_error;

int fail(int code, const std::string& msg)
{
    g_error = msg;
    return code;
}

int threads()
{
    const unsigned n = std::thread::hardware_concurrency();
    return n ? (int)n : 4;
}

}  // namespace

struct lmgpu_accel {
    std::vector<float> tris;
    lmo_accel* acc = nullptr;
    bool built = false;
    std::vector<float> normals, texcoords;
    std::vector<uint8_t> flags;
};

struct lmgpu_scene {
    std::vector<float> tris;
    std::vector<int32_t> tri_prim;
    std::vector<lmo_pt_prim> prims;
    lmo_pt_camera cam;
    lmo_pt_env env;
};

struct lmgpu_guide {
    int unused = 0;
};

extern "C" {

const char* lmgpu_version(void) { return "lmgpu CPU stand-in (test infrastructure)"; }

const char* lmgpu_last_error(void) { return g_error.c_str(); }

int lmgpu_accel_create(lmgpu_accel** out)
{
    if (!out) return fail(LMGPU_ERR_INVALID, "lmgpu_accel_create: NULL out");
    *out = new (std::nothrow) lmgpu_accel();
    return *out ? LMGPU_OK : fail(LMGPU_ERR_INVALID, "out of memory");
}

void lmgpu_accel_destroy(lmgpu_accel* a)
{
    if (!a) return;
    if (a->acc) lmo_accel_free(a->acc);
    delete a;
}

int lmgpu_accel_build(lmgpu_accel* a, const float* triangles, uint64_t ntri)
{
    if (!a || (ntri && !triangles)) return fail(LMGPU_ERR_INVALID, "lmgpu_accel_build: NULL argument");
    if (a->acc) lmo_accel_free(a->acc);
    a->tris.assign(triangles, triangles + 9 * ntri);
    a->acc = lmo_accel_build(ntri <= 4096 ? 0 : 1, a->tris.data(), (size_t)ntri);
    a->built = true;
    a->normals.clear();
    a->texcoords.clear();
    a->flags.clear();
    return LMGPU_OK;
}

int lmgpu_accel_build_meshes(lmgpu_accel* a, const lmgpu_mesh* meshes, uint32_t n)
{
    if (!a || (n && !meshes)) return fail(LMGPU_ERR_INVALID, "lmgpu_accel_build_meshes: NULL argument");
    std::vector<float> tris;
    for (uint32_t i = 0; i < n; i++) {
        const lmgpu_mesh& m = meshes[i];
        const float* T = m.transform;
        for (uint32_t f = 0; f < m.num_faces; f++)
            for (int k = 0; k < 3; k++) {
                const uint32_t v = m.faces[3 * f + k];
                if (v >= m.num_vertices) return fail(LMGPU_ERR_INVALID, "lmgpu_accel_build_meshes: face index out of range");
                const float x = m.positions[3 * v], y = m.positions[3 * v + 1], z = m.positions[3 * v + 2];
                for (int r = 0; r < 3; r++) {
                    // Mat4 x Vec4 with w = 1: every product and sum rounded
                    volatile float a0 = T[r] * x, a1 = T[4 + r] * y, a2 = T[8 + r] * z;
                    volatile float s0 = a0 + a1, s1 = a2 + T[12 + r];
                    tris.push_back(s0 + s1);
                }
            }
    }
    return lmgpu_accel_build(a, tris.data(), tris.size() / 9);
}

int lmgpu_accel_set_attributes(lmgpu_accel* a, const float* normals, const float* texcoords, const uint8_t* flags,
                               uint64_t ntri)
{
    if (!a) return fail(LMGPU_ERR_INVALID, "lmgpu_accel_set_attributes: NULL accel");
    if (!a->built) return fail(LMGPU_ERR_NOT_BUILT, "lmgpu_accel_set_attributes: accel not built");
    if (ntri != a->tris.size() / 9) return fail(LMGPU_ERR_INVALID, "lmgpu_accel_set_attributes: ntri differs");
    if (normals) a->normals.assign(normals, normals + 9 * ntri); else a->normals.clear();
    if (texcoords) a->texcoords.assign(texcoords, texcoords + 6 * ntri); else a->texcoords.clear();
    a->flags.resize(ntri);
    for (uint64_t i = 0; i < ntri; i++)
        a->flags[i] = flags ? (uint8_t)(flags[i] & 3u) : (uint8_t)((normals ? 1u : 0u) | (texcoords ? 2u : 0u));
    if (!normals) for (auto& f : a->flags) f &= (uint8_t)~1u;
    if (!texcoords) for (auto& f : a->flags) f &= (uint8_t)~2u;
    return LMGPU_OK;
}

int lmgpu_trace(const lmgpu_accel* a, const float* rays, lmgpu_hit* hits, uint64_t n, int anyhit)
{
    (void)anyhit;  // the closest hit is a valid answer to an any-hit query
    if (!a || (n && (!rays || !hits))) return fail(LMGPU_ERR_INVALID, "lmgpu_trace: NULL argument");
    if (!a->built) return fail(LMGPU_ERR_NOT_BUILT, "lmgpu_trace: accel not built");
    std::vector<lmo_hit> h((size_t)n);
    if (n) lmo_accel_trace(a->acc, rays, (size_t)n, h.data(), threads());
    for (uint64_t i = 0; i < n; i++) {
        hits[i].prim = h[i].id;
        hits[i].t = h[i].id >= 0 ? h[i].t : 0.f;
        hits[i].b1 = h[i].id >= 0 ? h[i].b0 : 0.f;
        hits[i].b2 = h[i].id >= 0 ? h[i].b1 : 0.f;
    }
    return LMGPU_OK;
}

int lmgpu_surface(const lmgpu_accel* a, const float* rays, const lmgpu_hit* hits, uint64_t n, float* surface)
{
    if (!a || (n && (!rays || !hits || !surface))) return fail(LMGPU_ERR_INVALID, "lmgpu_surface: NULL argument");
    if (!a->built) return fail(LMGPU_ERR_NOT_BUILT, "lmgpu_surface: accel not built");
    const size_t ntri = a->tris.size() / 9;
    std::vector<double> T(a->tris.begin(), a->tris.end()), N(a->normals.begin(), a->normals.end()),
        UV(a->texcoords.begin(), a->texcoords.end()), R(rays, rays + 8 * n), H(4 * n), out(23 * n);
    for (uint64_t i = 0; i < n; i++) {
        H[4 * i] = hits[i].t;
        H[4 * i + 1] = hits[i].prim;
        H[4 * i + 2] = hits[i].b1;
        H[4 * i + 3] = hits[i].b2;
    }
    const bool attrs = a->flags.size() == ntri && ntri > 0;
    lmo_surface(T.data(), attrs && !N.empty() ? N.data() : nullptr, attrs && !UV.empty() ? UV.data() : nullptr,
                attrs ? a->flags.data() : nullptr, R.data(), H.data(), (size_t)n, out.data());
    for (uint64_t i = 0; i < n; i++)
        for (int k = 0; k < LMGPU_SURFACE_PLANES; k++) surface[(uint64_t)k * n + i] = (float)out[23 * i + k];
    return LMGPU_OK;
}

int lmgpu_scene_create(const float* triangles, const int32_t* tri_prim, uint64_t ntri, const lmgpu_prim* prims,
                       uint32_t nprims, const lmgpu_camera* camera, lmgpu_scene** out)
{
    if (!out || !camera || (ntri && (!triangles || !tri_prim)) || (nprims && !prims))
        return fail(LMGPU_ERR_INVALID, "lmgpu_scene_create: NULL argument");
    static_assert(sizeof(lmgpu_prim) == sizeof(lmo_pt_prim), "primitive layouts differ");
    static_assert(sizeof(lmgpu_camera) == sizeof(lmo_pt_camera), "camera layouts differ");
    auto* s = new lmgpu_scene();
    s->tris.assign(triangles, triangles + 9 * ntri);
    s->tri_prim.assign(tri_prim, tri_prim + ntri);
    s->prims.resize(nprims);
    if (nprims) std::memcpy(s->prims.data(), prims, sizeof(lmgpu_prim) * nprims);
    std::memcpy(&s->cam, camera, sizeof(lmgpu_camera));
    std::memset(&s->env, 0, sizeof(s->env));
    *out = s;
    return LMGPU_OK;
}

void lmgpu_scene_destroy(lmgpu_scene* s) { delete s; }

int lmgpu_scene_set_environment(lmgpu_scene* s, const float* Le)
{
    if (!s) return fail(LMGPU_ERR_INVALID, "lmgpu_scene_set_environment: NULL scene");
    s->env.enabled = Le ? 1 : 0;
    for (int k = 0; k < 3; k++) s->env.Le[k] = Le ? Le[k] : 0.f;
    return LMGPU_OK;
}

}  // extern "C"

namespace {

// film = sums scaled by W H / N; variance of that estimate from the squares
// (uniform raster positions: Var(I_p) = (W H)^2 Var(X) / N)
void finish(const lmgpu_scene* s, uint64_t N, const std::vector<double>& sum, const std::vector<double>& sq,
            double scale_sum, float* image, float* variance)
{
    const double WH = (double)s->cam.width * s->cam.height;
    for (size_t i = 0; i < sum.size(); i++) {
        const double img = sum[i] * scale_sum;
        image[i] = (float)img;
        if (variance) {
            const double ex = sum[i] / (double)N, ex2 = sq[i] / (double)N;
            const double v = ex2 - ex * ex;
            variance[i] = (float)(WH * WH * (v > 0 ? v : 0) / (double)N);
        }
    }
}

typedef uint64_t (*RenderFn)(const float*, const int32_t*, size_t, const lmo_pt_prim*, int, const lmo_pt_camera*,
                             uint64_t, int, uint64_t, int, double*, double*);

int render_with(lmgpu_scene* s, const lmgpu_pt_params* p, float* image, float* variance, RenderFn fn,
                const char* who)
{
    if (!s || !p || !image) return fail(LMGPU_ERR_INVALID, std::string(who) + ": NULL argument");
    if (p->min_num_vertices != 0)
        return fail(LMGPU_ERR_INVALID, std::string(who) + ": min_num_vertices is not supported by the CPU stand-in");
    const uint64_t N = p->spp * (uint64_t)s->cam.width * (uint64_t)s->cam.height;
    std::vector<double> sum((size_t)s->cam.width * s->cam.height * 3), sq(sum.size());
    if (fn)
        fn(s->tris.data(), s->tri_prim.data(), s->tri_prim.size(), s->prims.data(), (int)s->prims.size(), &s->cam, N,
           p->max_num_vertices, p->seed, threads(), sum.data(), sq.data());
    else
        lmo_render_pt(s->tris.data(), s->tri_prim.data(), s->tri_prim.size(), s->prims.data(), &s->env, &s->cam, N,
                      p->max_num_vertices, p->seed, threads(), sum.data(), sq.data());
    finish(s, N, sum, sq, (double)s->cam.width * s->cam.height / (double)N, image, variance);
    return LMGPU_OK;
}

}  // namespace

extern "C" {

int lmgpu_render_pt(lmgpu_scene* s, const lmgpu_pt_params* p, float* image, float* variance)
{
    return render_with(s, p, image, variance, nullptr, "lmgpu_render_pt");
}

int lmgpu_render_ptmis(lmgpu_scene* s, const lmgpu_pt_params* p, float* image, float* variance)
{
    return render_with(s, p, image, variance, lmo_render_ptmis, "lmgpu_render_ptmis");
}

int lmgpu_render_ptdirect(lmgpu_scene* s, const lmgpu_pt_params* p, float* image, float* variance)
{
    return render_with(s, p, image, variance, lmo_render_ptdirect, "lmgpu_render_ptdirect");
}

int lmgpu_render_ltdirect(lmgpu_scene* s, const lmgpu_pt_params* p, float* image, float* variance)
{
    return render_with(s, p, image, variance, lmo_render_ltdirect, "lmgpu_render_ltdirect");
}

int lmgpu_render_bdpt_mis(lmgpu_scene* s, const lmgpu_pt_params* p, int mis, float* image, float* variance)
{
    if (!s || !p || !image) return fail(LMGPU_ERR_INVALID, "lmgpu_render_bdpt_mis: NULL argument");
    if (p->min_num_vertices != 0)
        return fail(LMGPU_ERR_INVALID, "lmgpu_render_bdpt_mis: min_num_vertices is not supported by the CPU stand-in");
    const uint64_t N = p->spp * (uint64_t)s->cam.width * (uint64_t)s->cam.height;
    std::vector<double> sum((size_t)s->cam.width * s->cam.height * 3), sq(sum.size());
    lmo_render_bdpt_mis(s->tris.data(), s->tri_prim.data(), s->tri_prim.size(), s->prims.data(), (int)s->prims.size(),
                        &s->cam, N, p->max_num_vertices, p->seed, threads(), sum.data(), sq.data(), 0, mis);
    finish(s, N, sum, sq, (double)s->cam.width * s->cam.height / (double)N, image, variance);
    return LMGPU_OK;
}

int lmgpu_render_bdpt(lmgpu_scene* s, const lmgpu_pt_params* p, float* image, float* variance)
{
    return lmgpu_render_bdpt_mis(s, p, LMGPU_MIS_POWER, image, variance);
}

int lmgpu_render_vcm(lmgpu_scene* s, const lmgpu_vcm_params* p, float* image, float* variance)
{
    if (!s || !p || !image) return fail(LMGPU_ERR_INVALID, "lmgpu_render_vcm: NULL argument");
    lmo_vcm_params q;
    std::memset(&q, 0, sizeof(q));
    q.max_num_vertices = p->max_num_vertices;
    q.min_num_vertices = p->min_num_vertices;
    q.num_iteration_pass = p->num_iteration_pass;
    q.num_photon_trace_samples = p->num_photon_trace_samples;
    q.num_eye_trace_samples = p->num_eye_trace_samples;
    q.initial_radius = p->initial_radius;
    q.alpha = p->alpha;
    q.mode = p->mode;
    std::vector<double> sum((size_t)s->cam.width * s->cam.height * 3), sq(sum.size());
    const uint64_t N = lmo_render_vcm(s->tris.data(), s->tri_prim.data(), s->tri_prim.size(), s->prims.data(),
                                      (int)s->prims.size(), &s->cam, &q, p->seed, threads(), sum.data(), sq.data());
    const double passes = p->num_iteration_pass ? (double)p->num_iteration_pass : 1.0;
    for (size_t i = 0; i < sum.size(); i++) {
        image[i] = (float)(sum[i] / passes);
        if (variance) {
            const double n = N ? (double)N : 1.0, m = sum[i] / n, v = sq[i] / n - m * m;
            variance[i] = (float)((v > 0 ? v : 0) * n / (passes * passes));
        }
    }
    return LMGPU_OK;
}

int lmgpu_guide_create(const float* box_lo_hi, uint32_t seed, lmgpu_guide** out)
{
    (void)box_lo_hi;
    (void)seed;
    if (!out) return fail(LMGPU_ERR_INVALID, "lmgpu_guide_create: NULL out");
    *out = new lmgpu_guide();
    return LMGPU_OK;
}

void lmgpu_guide_destroy(lmgpu_guide* g) { delete g; }

int lmgpu_render_pt_guided(lmgpu_scene* s, lmgpu_guide* g, const lmgpu_pt_params* p,
                           const lmgpu_guiding_params* guiding, float* image, float* variance, float* last_loss)
{
    if (!g || !guiding) return fail(LMGPU_ERR_INVALID, "lmgpu_render_pt_guided: NULL argument");
    if (last_loss) *last_loss = 0.f;
    return render_with(s, p, image, variance, nullptr, "lmgpu_render_pt_guided");
}

}  // extern "C"
