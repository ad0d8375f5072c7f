// Bidirectional path tracing on the GPU: the form of renderer::bdpt.
//
// Reference estimator (src/liblightmetrica/renderer/renderer_bdpt.cpp):
//   * a light subpath and an eye subpath per sample (Subpath::Sample, :80-220):
//     after the first vertex every step stores a BSDF-sampled vertex and a
//     "direct" vertex (the opposite endpoint's emitter sampled from the
//     previous vertex, kept only when visible); roulette 0.5 after each step;
//   * every strategy (s, t, direct) with direct only for s = 0 or t = 0
//     (Render, :841-998) is connected (Path::Connect, :233-333), weighted by
//     the power heuristic over all strategies of the same full path
//     (:747-784, EvaluatePDF :628-703), divided by the roulette selection
//     probability 0.5^(max(0,s-2)+max(0,t-2)) (:348-368) and splatted at
//     the raster position of the path's last segment;
//   * light::area draws its emission direction from the same 2D sample as the
//     position (light_area.cpp:73-80) and the pinhole is a delta position, so
//     t = 0 strategies carry no weight -- both kept as the reference has them.
//
// GPU structure (wavefront), per wave of up to kWaveSamples samples:
//   k_bd_start     vertex 0 of every light and eye subpath, and the rays of
//                  step 1: the extension ray and the ray to the "direct"
//                  endpoint candidate;
//   per step k     closest-hit traversal of the extension rays and any-hit
//                  traversal of the direct rays (trace.cu, persistent), then
//                  k_bd_step: store the step's vertex, roulette, sample the
//                  rays of step k + 1 for the surviving subpaths (compacted);
//   k_bd_count     per sample: the number of work items per strategy (s, t)
//                  -- the s = 0 strategies (no ray needed) and the s, t >= 1
//                  connections -- into per-strategy buckets, which
//                  k_bd_buckets lays out and k_bd_items fills, so that the
//                  warps of the next kernel each evaluate one strategy;
//   k_bd_connect   one thread per item: contribution (unweighted estimate,
//                  MIS weight, selection pdf) and, for connections, the
//                  shadow ray; any-hit traversal of all shadow rays;
//                  k_bd_splat adds the unoccluded ones; k_bd_flush merges
//                  each sample's own-pixel contributions into the film (the
//                  reference film squares per-sample sums, so the variance
//                  estimate does too).
// Subpath vertices live in HBM as 32-byte records, [vertex k][sample], so
// the kernels of one step read and write them coalesced.  Eye subpaths start
// at per-pixel stratified raster positions; random numbers are Philox keyed
// by (seed, sample, subpath, step), so every kernel draws its own without
// carried state.
#include "interact.cuh"
#include "rng.cuh"

namespace lmgpu {
namespace {

constexpr int kMaxV = 16;
// Connection work items are grouped by strategy (s, t), bucket s * kStrideST + t.
constexpr int kStrideST = kMaxV + 1;
constexpr int kBuckets = kStrideST * kStrideST;
constexpr uint64_t kWaveSamples = 1ull << 21;
// A work item: sample index (21 bits, kWaveSamples samples), d (bit 21),
// s (bits 22..26) and t (bits 27..31).
constexpr uint32_t kSampleMask = (uint32_t)kWaveSamples - 1u;
constexpr int kItemD = 21, kItemS = 22, kItemT = 27;
constexpr int kBdptThreads = 128;
constexpr uint32_t kKeyBdpt = 0x42445054u;

// EvaluateUnweightContribution (:489-591) with EvaluateCst (:375-406).
__device__ __noinline__ Spd unweighted(const Ctx& C, const PV* P, int n, int s, bool direct)
{
    const int t = n - s;
    Spd a = S1(1.0f);
    if (s > 0) {
        a = S1(1.0f / pdf_pos(C, P[0]) / emitter_pdf(C, P[0]));
        for (int i = 0; i < s - 1; i++) {
            const float3 wi = i >= 1 ? dirto(P[i], P[i - 1]) : zero3(), wo = dirto(P[i], P[i + 1]);
            const bool dl = t == 0 && i == s - 2 && direct;
            const Spd fs = eval_dir(C, P[i], P[i].type, wi, wo, DIR_LE, dl);
            if (black(fs)) return S1(0.0f);
            const float pdf = dl ? pdf_pos(C, P[i + 1]) / geometry_term(P[i + 1], P[i]) * emitter_pdf(C, P[i + 1])
                                 : pdf_dir(C, P[i], P[i].type, wi, wo);
            for (int k = 0; k < 3; k++) a.c[k] *= fs.c[k] / pdf;
        }
    }
    if (black(a)) return a;
    if (t > 0) {
        const float ae = 1.0f / pdf_pos(C, P[n - 1]) / emitter_pdf(C, P[n - 1]);
        for (int k = 0; k < 3; k++) a.c[k] *= ae;
        for (int i = n - 1; i > s; i--) {
            const float3 wi = i < n - 1 ? dirto(P[i], P[i + 1]) : zero3(), wo = dirto(P[i], P[i - 1]);
            const bool dl = s == 0 && i == 1 && direct;
            const Spd fs = eval_dir(C, P[i], P[i].type, wi, wo, DIR_EL, dl);
            if (black(fs)) return S1(0.0f);
            const float pdf = dl ? pdf_pos(C, P[i - 1]) / geometry_term(P[i - 1], P[i]) * emitter_pdf(C, P[i - 1])
                                 : pdf_dir(C, P[i], P[i].type, wi, wo);
            for (int k = 0; k < 3; k++) a.c[k] *= fs.c[k] / pdf;
        }
    }
    if (black(a)) return a;
    // Cst
    Spd cst;
    if (s == 0 && t > 0) {
        cst = eval_dir(C, P[0], P[0].type, zero3(), dirto(P[0], P[1]), DIR_EL, false);
    } else if (s > 0 && t == 0) {
        cst = S1(0.0f);  // EvaluatePosition(evalDelta = true) of the pinhole is 0
    } else {
        const PV& vL = P[s - 1];
        const PV& vE = P[s];
        const Spd fL = eval_dir(C, vL, vL.type, s - 2 >= 0 ? dirto(vL, P[s - 2]) : zero3(), dirto(vL, vE), DIR_LE, true);
        const Spd fE = eval_dir(C, vE, vE.type, s + 1 < n ? dirto(vE, P[s + 1]) : zero3(), dirto(vE, vL), DIR_EL, true);
        const float G = geometry_term(vL, vE);
        for (int k = 0; k < 3; k++) cst.c[k] = fL.c[k] * G * fE.c[k];
    }
    for (int k = 0; k < 3; k++) a.c[k] *= cst.c[k];
    return a;
}

// Samplable + EvaluatePDF (:593-703) for every strategy of one full path,
// and the power-heuristic weight of strategy (s_, d_) over them
// (MISWeight_PowerHeuristics, :747-784).  EvaluatePDF(s, d) is the product
// of the endpoint terms and of one factor per vertex,
//   light side  fL[i] = pdf_dir(P[i] -> P[i+1]) G(P[i], P[i+1]),  i < s - 1
//   eye side    fE[i] = pdf_dir(P[i] -> P[i-1]) G(P[i], P[i-1]),  i > s
// with the direct strategies swapping the factor next to the sampled
// endpoint for that endpoint's positional pdf.  The factors are evaluated
// once per path and combined through prefix / suffix products, so every
// strategy's pdf costs O(1) instead of O(n).
__device__ __noinline__ float mis_weight(const Ctx& C, const PV* P, int n, int s_, bool d_)
{
    float preL[2 * kMaxV + 1], sufE[2 * kMaxV + 1];
    const float posL = pdf_pos(C, P[0]) * emitter_pdf(C, P[0]);
    const float posE = pdf_pos(C, P[n - 1]) * emitter_pdf(C, P[n - 1]);
    // preL[k] = posL * prod_{i < k} fL[i], k = 0 .. n - 1
    preL[0] = posL;
    for (int i = 0; i + 1 < n; i++) {
        const float f = pdf_dir(C, P[i], P[i].type, i >= 1 ? dirto(P[i], P[i - 1]) : zero3(), dirto(P[i], P[i + 1])) *
                        geometry_term(P[i], P[i + 1]);
        preL[i + 1] = preL[i] * f;
    }
    // sufE[k] = posE * prod_{i >= k} fE[i], k = n .. 1
    sufE[n] = posE;
    for (int i = n - 1; i >= 1; i--) {
        const float f = pdf_dir(C, P[i], P[i].type, i + 1 < n ? dirto(P[i], P[i + 1]) : zero3(),
                                dirto(P[i], P[i - 1])) *
                        geometry_term(P[i], P[i - 1]);
        sufE[i] = sufE[i + 1] * f;
    }
    auto pdf = [&](int s, bool d) -> float {
        const int t = n - s;
        if (s > 0 && t > 0 && d) return 0.0f;
        if (t == 0 && s > 0 && d && delta_dir(C, P[n - 2], P[n - 2].type)) return 0.0f;
        if (s == 0 && t > 0 && d && delta_dir(C, P[1], P[1].type)) return 0.0f;
        if (s == 0 && t > 0) {
            if (P[0].type & T_E) return 0.0f;
        } else if (s > 0 && t == 0) {
            if (P[n - 1].type & T_E) return 0.0f;
        } else if (delta_dir(C, P[s - 1], P[s - 1].type) || delta_dir(C, P[s], P[s].type)) {
            return 0.0f;
        }
        float pl = 1.0f, pe = 1.0f;
        if (s > 0) pl = (t == 0 && d) ? preL[s - 2] * posE : preL[s - 1];
        if (t > 0) pe = (s == 0 && d) ? sufE[2] * posL : sufE[s + 1];
        return pl * pe;
    };
    if (C.mis == 1) {
        // misweight::simple (renderer_bdpt.cpp:711-744)
        int nonzero = 0;
        for (int s = 0; s <= n; s++)
            for (int d = 0; d < 2; d++) {
                if (s > 0 && n - s > 0 && d) continue;
                if (pdf(s, d != 0) > 0.0f) nonzero++;
            }
        return 1.0f / (float)nonzero;
    }
    const float ps = pdf(s_, d_);
    float inv = 0.0f;
    for (int s = 0; s <= n; s++)
        for (int d = 0; d < 2; d++) {
            if (s > 0 && n - s > 0 && d) continue;
            const float pi = pdf(s, d != 0);
            if (pi > 0.0f) {
                const float r = pi / ps;
                inv += r * r;
            }
        }
    return 1.0f / inv;
}


// ---- wave storage --------------------------------------------------------

// A stored subpath vertex: position and primitive, normal and type bits.
struct __align__(16) BVtx {
    float4 a;  // p, prim (int bits)
    float4 b;  // n, type | degen << 8 | F_SV | F_DIRECT (bits)
};
constexpr uint32_t F_SV = 1u << 16;      // the step stored a BSDF-sampled vertex
constexpr uint32_t F_DIRECT = 1u << 17;  // the step's direct endpoint was visible

__device__ __forceinline__ BVtx pack(const PV& v, uint32_t flags)
{
    BVtx r;
    r.a = make_float4(v.p.x, v.p.y, v.p.z, __int_as_float(v.prim));
    r.b = make_float4(v.n.x, v.n.y, v.n.z,
                      __uint_as_float(((uint32_t)v.type & 0xffu) | (((uint32_t)v.degen & 0xffu) << 8) | flags));
    return r;
}

__device__ __forceinline__ PV unpack(const BVtx& r)
{
    PV v;
    v.p = f3(r.a.x, r.a.y, r.a.z);
    v.n = f3(r.b.x, r.b.y, r.b.z);
    v.prim = __float_as_int(r.a.w);
    const uint32_t w = __float_as_uint(r.b.w);
    v.type = (short)(w & 0xffu);
    v.degen = (short)((w >> 8) & 0xffu);
    return v;
}

__device__ __forceinline__ uint32_t flags_of(const BVtx& r) { return __float_as_uint(r.b.w) & (F_SV | F_DIRECT); }

// Device view of one wave.  Slot j in [0, 2n) is subpath j / n (0 light,
// 1 eye) of sample j % n; vertex k of subpath d of sample i is at
// sv[d][k * stride + i] (BSDF-sampled) and dv[d][k * stride + i] (direct).
struct Wave {
    uint64_t p0;       // global index of the wave's first sample
    uint32_t n;        // samples in the wave
    uint32_t stride;   // sample capacity of the vertex arrays
    uint32_t npix;
    uint32_t seed;
    BVtx* sv[2];
    BVtx* dv[2];
    int32_t* count[2];  // vertices stored per subpath
    BVtx* pend;         // [slot] the direct endpoint candidate of the current step
    float* own;         // [3 i] sample i's contributions to its own pixel
};

// The random numbers of step k of subpath `dir` of sample p: extension
// direction (u0, u1, uc), direct endpoint (us, a0, a1), roulette (rr).
struct StepRand {
    float u0, u1, uc, us, a0, a1, rr;
};

__device__ __forceinline__ StepRand step_rand(uint64_t p, int dir, int k, uint32_t seed)
{
    const uint32_t c2 = ((uint32_t)dir << 8) | (uint32_t)k;
    const Philox4x32 A = philox4x32_10((uint32_t)p, (uint32_t)(p >> 32), c2, 0u, seed, kKeyBdpt);
    const Philox4x32 B = philox4x32_10((uint32_t)p, (uint32_t)(p >> 32), c2, 1u, seed, kKeyBdpt);
    return StepRand{u01(A.v[0]), u01(A.v[1]), u01(A.v[2]), u01(A.v[3]), u01(B.v[0]), u01(B.v[1]), u01(B.v[2])};
}

__device__ __forceinline__ void store_ray(float4* rays, uint32_t q, float3 o, float tmin, float3 d, float tmax)
{
    rays[2 * q] = make_float4(o.x, o.y, o.z, tmin);
    rays[2 * q + 1] = make_float4(d.x, d.y, d.z, tmax);
}

// A ray that meets nothing (empty [tmin, tmax]).
__device__ __forceinline__ void store_null_ray(float4* rays, uint32_t q)
{
    rays[2 * q] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    rays[2 * q + 1] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
}

// Scene3::Visible (scene3.h:107-116) as a ray: [EpsIsect, L (1 - EpsIsect)].
__device__ __forceinline__ void store_shadow_ray(float4* rays, uint32_t q, float3 a, float3 b)
{
    float3 d = b - a;
    const float L = sqrtf(dot3(d, d));
    d = d * (1.0f / L);
    store_ray(rays, q, a, 1e-4f, d, L * (1.0f - 1e-4f));
}

// The rays of step k from vertex v (Subpath::Sample, renderer_bdpt.cpp:130-200):
// the extension ray along wo (null if the direction was not sampled or its
// BSDF value is black) and the ray to the direct endpoint, drawn with step
// k's random numbers; the endpoint is kept in pend[slot], flagged F_DIRECT
// when its visibility is traced.  Visibility is traced only where the
// endpoint can contribute:
//   * light subpaths: the direct endpoint is the pinhole, used only by the
//     t = 0 strategies, which carry no weight (delta sensor position), so no
//     ray is traced;
//   * eye subpaths: not when the sampled light point faces away from v (its
//     emission towards v is zero, light_area.cpp EvaluateDirection) or v's
//     BSDF is a delta or null one (zero under evalDelta), where the (s = 0,
//     direct) strategy's contribution is zero whatever the visibility.
__device__ __forceinline__ void emit_step(const Ctx& C, const Wave& w, int dir, uint32_t slot, const PV& v, bool has_wo,
                                          float3 wo, const StepRand& r, uint32_t q, float4* ext, float4* sh)
{
    if (has_wo) store_ray(ext, q, v.p, 1e-4f, wo, FLT_MAX);
    else store_null_ray(ext, q);
    PV e;
    bool trace = false;
    if (dir == DIR_LE) {
        sensor_vertex(C, e);
    } else {
        sample_light(C, r.us, r.a0, r.a1, e);
        const bool front = dot3(v.p - e.p, e.n) > 0.0f;
        const bool conn = (v.type & T_E) || (v.type != 0 && !delta_dir(C, v, v.type));
        trace = front && conn;
    }
    if (trace) store_shadow_ray(sh, q, v.p, e.p);
    else store_null_ray(sh, q);
    w.pend[slot] = pack(e, trace ? F_DIRECT : 0u);
}

__global__ void __launch_bounds__(kBdptThreads) k_bd_start(Ctx C, Wave w, float4* __restrict__ ext,
                                                           float4* __restrict__ sh, uint32_t* __restrict__ active,
                                                           uint32_t* __restrict__ n_out)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j == 0) *n_out = C.max_v > 1 ? 2 * w.n : 0u;  // every subpath is queued for step 1
    if (j >= 2 * w.n) return;
    const int dir = j >= w.n ? DIR_EL : DIR_LE;
    const uint32_t i = dir == DIR_EL ? j - w.n : j;
    const uint64_t p = w.p0 + i;
    const StepRand r0 = step_rand(p, dir, 0, w.seed);
    PV v;
    float3 wo;
    bool has_wo;
    if (dir == DIR_LE) {
        sample_light(C, r0.us, r0.a0, r0.a1, v);
        // emission direction from the same 2D sample as the position (light_area.cpp:73-80)
        const float3 l = cosine_hemisphere(r0.a0, r0.a1);
        float3 b, c;
        basis(v.n, b, c);
        wo = b * l.x + c * l.y + v.n * l.z;
        has_wo = !black(eval_dir(C, v, T_L, zero3(), wo, DIR_LE, false));
    } else {
        sensor_vertex(C, v);
        const uint32_t W = (uint32_t)C.cam.width, H = (uint32_t)C.cam.height;
        const uint32_t pixel = (uint32_t)(p % w.npix);
        wo = camera_dir(C.cam, ((float)(pixel % W) + r0.u0) / (float)W, ((float)(pixel / W) + r0.u1) / (float)H);
        has_wo = importance(C.cam, wo) > 0.0f;
    }
    w.sv[dir][i] = pack(v, F_SV);
    w.count[dir][i] = 1;
    active[j] = j;
    emit_step(C, w, dir, j, v, has_wo, wo, step_rand(p, dir, 1, w.seed), j, ext, sh);
}

// Step k of the active subpaths: hits of the extension and direct rays in,
// the vertex stored, roulette, the rays of step k + 1 out (compacted).
__global__ void __launch_bounds__(kBdptThreads) k_bd_step(Ctx C, Wave w, int k, const uint32_t* __restrict__ n_in,
                                                          const uint32_t* __restrict__ active_in,
                                                          const float4* __restrict__ ext_in,
                                                          const lmgpu_hit* __restrict__ ext_hit,
                                                          const lmgpu_hit* __restrict__ sh_hit,
                                                          uint32_t* __restrict__ active_out,
                                                          uint32_t* __restrict__ n_out, float4* __restrict__ ext_out,
                                                          float4* __restrict__ sh_out)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    bool keep = false;
    uint32_t j = 0;
    int dir = 0;
    PV nv;
    float3 wo = zero3();
    bool has_wo = false;
    StepRand rn{};
    if (q < *n_in) {
        j = active_in[q];
        dir = j >= w.n ? DIR_EL : DIR_LE;
        const uint32_t i = dir == DIR_EL ? j - w.n : j;
        const uint64_t p = w.p0 + i;
        const int n = w.count[dir][i];
        const lmgpu_hit he = ext_hit[q];
        const bool has_sv = he.prim >= 0;
        // a traced direct endpoint, and visible
        const bool has_direct = (flags_of(w.pend[j]) & F_DIRECT) && sh_hit[q].prim < 0;
        if (has_sv) {
            const float4 r0 = ext_in[2 * q], r1 = ext_in[2 * q + 1];
            const float* T = C.sc.tris + 9 * (size_t)he.prim;
            const float3 p1 = f3(T[0], T[1], T[2]), p2 = f3(T[3], T[4], T[5]), p3 = f3(T[6], T[7], T[8]);
            nv.p = f3(r0.x, r0.y, r0.z) + f3(r1.x, r1.y, r1.z) * he.t;
            nv.n = normalize3(cross3(p2 - p1, p3 - p1));
            nv.prim = C.sc.tri_prim[he.prim];
            nv.type = (short)bsdf_type(C.sc.prims[nv.prim].bsdf);
            nv.degen = 0;
        } else {
            nv.p = zero3();
            nv.n = zero3();
            nv.prim = -1;
            nv.type = 0;
            nv.degen = 0;
        }
        if (has_sv || has_direct) {
            const size_t at = (size_t)n * w.stride + i;
            w.sv[dir][at] = pack(nv, (has_sv ? F_SV : 0u) | (has_direct ? F_DIRECT : 0u));
            if (has_direct) w.dv[dir][at] = w.pend[j];
            w.count[dir][i] = n + 1;
        }
        // roulette 0.5 after the step (renderer_bdpt.cpp:205-213); the step
        // loop ends after max_num_vertices steps
        keep = has_sv && step_rand(p, dir, k, w.seed).rr <= 0.5f && n + 1 < C.max_v;
        if (keep) {
            rn = step_rand(p, dir, k + 1, w.seed);
            const PV pv = unpack(w.sv[dir][(size_t)(n - 1) * w.stride + i]);
            const float3 wi = dirto(nv, pv);
            has_wo = sample_dir(C, nv, wi, rn.u0, rn.u1, rn.uc, wo) &&
                     !black(eval_dir(C, nv, nv.type, wi, wo, dir, false));
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    if (m == 0u) return;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned leader = __ffs(m) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(n_out, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (keep) {
        const uint32_t o = base + __popc(m & ((1u << lane) - 1u));
        active_out[o] = j;
        emit_step(C, w, dir, j, nv, has_wo, wo, rn, o, ext_out, sh_out);
    }
}

__device__ __forceinline__ uint32_t raster_pixel(const Ctx& C, const PV* P, int n)
{
    float rx = 0.0f, ry = 0.0f;
    raster_pos(C.cam, dirto(P[n - 1], P[n - 2]), rx, ry);
    const int W = C.cam.width, H = C.cam.height;
    int ix = (int)(rx * (float)W), iy = (int)(ry * (float)H);
    ix = ix < 0 ? 0 : (ix > W - 1 ? W - 1 : ix);
    iy = iy < 0 ? 0 : (iy > H - 1 ? H - 1 : iy);
    return (uint32_t)iy * (uint32_t)W + (uint32_t)ix;
}

// Contribution of one full path: unweighted estimate x MIS weight /
// SelectionPDF (renderer_bdpt.cpp:348-368, :938-947); false if black.
__device__ __forceinline__ bool path_contribution(const Ctx& C, const PV* P, int n, int s, bool d, float c[3])
{
    // min_num_vertices applies only with max_num_vertices set (renderer_bdpt.cpp:892)
    if (C.max_path >= 0 && n < C.min_path) return false;
    const Spd cs = unweighted(C, P, n, s, d);
    if (black(cs)) return false;
    const float wgt = mis_weight(C, P, n, s, d);
    if (!(wgt == wgt)) return false;
    const int t = n - s;
    float sel = 1.0f;
    for (int q = 1; q < s - 1; q++) sel *= 0.5f;
    for (int q = 1; q < t - 1; q++) sel *= 0.5f;
    bool any = false;
    for (int k = 0; k < 3; k++) {
        c[k] = cs.c[k] * wgt / sel;
        any = any || (c[k] != 0.0f && c[k] == c[k]);
    }
    return any;
}

__device__ __forceinline__ void splat_px(double* film, double* film_sq, uint32_t pix, const float c[3])
{
    for (int k = 0; k < 3; k++) {
        if (c[k] != 0.0f) {
            atomicAdd(&film[3 * (size_t)pix + k], (double)c[k]);
            atomicAdd(&film_sq[3 * (size_t)pix + k], (double)c[k] * (double)c[k]);
        }
    }
}

// Eye-subpath vertices t that light-subpath vertex count s connects to.
__device__ __forceinline__ int t_limit(int s, int nE, int max_path)
{
    int t = nE;
    if (max_path >= 0 && t > max_path - s) t = max_path - s;
    return t > 0 ? t : 0;
}

// Eye-subpath lengths t of the s = 0 strategies (the eye subpath ends on a
// light, d = 0, or its direct vertex is one, d = 1): 2 .. t_limit_s0.
__device__ __forceinline__ int t_limit_s0(int nE, int max_path)
{
    return max_path >= 0 && nE > max_path ? max_path : nE;
}

// Bucket of the s = 0 items: (0, t) for d = 0, (t, 0) for d = 1 (bins no
// connection uses).
__device__ __forceinline__ int bucket_s0(int t, int d) { return d ? t * kStrideST : t; }

__device__ __forceinline__ int num_connections(int nL, int nE, int max_path)
{
    int c = 0;
    for (int s = 1; s <= nL; s++) {
        int t = nE;
        if (max_path >= 0 && t > max_path - s) t = max_path - s;
        c += t > 0 ? t : 0;
    }
    return c;
}

// Per sample: its work items are counted, in total and per strategy bucket
// (the s = 0 strategies, where the eye subpath reaches a light or its direct
// vertex is one, and the s, t >= 1 connections), and its own-pixel
// accumulator is cleared.  t = 0 strategies carry no weight with a pinhole
// sensor (its position cannot be hit and EvaluateCst is 0).
__global__ void __launch_bounds__(kBdptThreads) k_bd_count(Ctx C, Wave w, uint32_t* __restrict__ hist,
                                                           uint32_t* __restrict__ total)
{
    __shared__ uint32_t s_hist[kBuckets];
    for (int k = threadIdx.x; k < kBuckets; k += blockDim.x) s_hist[k] = 0u;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cnt = 0;
    const int nL = i < w.n ? w.count[0][i] : 0, nE = i < w.n ? w.count[1][i] : 0;
    const int t0 = t_limit_s0(nE, C.max_path);
    if (i < w.n) {
        cnt = (uint32_t)(num_connections(nL, nE, C.max_path) + 2 * (t0 > 1 ? t0 - 1 : 0));
        for (int k = 0; k < 3; k++) w.own[3 * (size_t)i + k] = 0.0f;
    }
    // item total, and the items per strategy (s, t) for the buckets
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t wsum = __reduce_add_sync(0xffffffffu, cnt);
    if (lane == 0u && wsum > 0u) atomicAdd(total, wsum);
    const int sw = __reduce_max_sync(0xffffffffu, nL);
    for (int sl = 1; sl <= sw; sl++) {
        const int tm = sl <= nL ? t_limit(sl, nE, C.max_path) : 0;
        const int tw = __reduce_max_sync(0xffffffffu, tm);
        for (int t = 1; t <= tw; t++) {
            const unsigned m = __ballot_sync(0xffffffffu, t <= tm);
            if (lane == 0u) atomicAdd(&s_hist[sl * kStrideST + t], (uint32_t)__popc(m));
        }
    }
    const int t0w = __reduce_max_sync(0xffffffffu, t0);
    for (int t = 2; t <= t0w; t++) {
        const unsigned m = __ballot_sync(0xffffffffu, t <= t0);
        if (lane == 0u) {
            atomicAdd(&s_hist[bucket_s0(t, 0)], (uint32_t)__popc(m));
            atomicAdd(&s_hist[bucket_s0(t, 1)], (uint32_t)__popc(m));
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kBuckets; k += blockDim.x)
        if (s_hist[k]) atomicAdd(&hist[k], s_hist[k]);
}

// Bucket offsets: exclusive scan of the per-strategy counts; cursors reset.
__global__ void k_bd_buckets(uint32_t* __restrict__ hist, uint32_t* __restrict__ offset, uint32_t* __restrict__ cursor)
{
    if (threadIdx.x != 0) return;
    uint32_t acc = 0;
    for (int k = 0; k < kBuckets; k++) {
        offset[k] = acc;
        acc += hist[k];
        cursor[k] = 0u;
    }
}

// Work items, scattered into their strategy's bucket so that a warp of
// k_bd_connect evaluates one strategy (same path length, same MIS loops) at
// a time: the s, t >= 1 connections as sample | s << 22 | t << 27, and the
// s = 0 strategies (Path::Connect, :245-275; no visibility ray: the eye
// subpath's own rays found the light) as sample | d << 21 | t << 27.
// The (s, t) buckets of one sample, in a fixed order; visit(b, m, lane-has,
// item) for each, with m the warp's ballot of the samples that have it.
template <typename F>
__device__ __forceinline__ void for_each_bucket(const Ctx& C, int nL, int nE, uint32_t i, F visit)
{
    const int sw = __reduce_max_sync(0xffffffffu, nL);
    for (int s = 1; s <= sw; s++) {
        const int tm = s <= nL ? t_limit(s, nE, C.max_path) : 0;
        const int tw = __reduce_max_sync(0xffffffffu, tm);
        for (int t = 1; t <= tw; t++) {
            const bool has = t <= tm;
            const unsigned m = __ballot_sync(0xffffffffu, has);
            visit(s * kStrideST + t, m, has, i | ((uint32_t)s << kItemS) | ((uint32_t)t << kItemT));
        }
    }
    // s = 0: i | d << 21 | t << 27
    const int t0 = t_limit_s0(nE, C.max_path);
    const int t0w = __reduce_max_sync(0xffffffffu, t0);
    for (int t = 2; t <= t0w; t++) {
        const bool has = t <= t0;
        const unsigned m = __ballot_sync(0xffffffffu, has);
        for (int d = 0; d < 2; d++)
            visit(bucket_s0(t, d), m, has, i | ((uint32_t)d << kItemD) | ((uint32_t)t << kItemT));
    }
}

// Two passes over the same buckets: the block's count per bucket (shared
// atomics, one per warp and bucket), one global reservation per bucket and
// block, then each warp's positions inside the block's range.
__global__ void __launch_bounds__(256) k_bd_items(Ctx C, Wave w, const uint32_t* __restrict__ offset,
                                                  uint32_t* __restrict__ cursor, uint32_t* __restrict__ items)
{
    __shared__ uint32_t s_pos[kBuckets];
    for (int k = threadIdx.x; k < kBuckets; k += blockDim.x) s_pos[k] = 0u;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned lane = threadIdx.x & 31u;
    const int nL = i < w.n ? w.count[0][i] : 0, nE = i < w.n ? w.count[1][i] : 0;
    for_each_bucket(C, nL, nE, i, [&](int b, unsigned m, bool, uint32_t) {
        if (lane == (unsigned)(__ffs(m) - 1)) atomicAdd(&s_pos[b], (uint32_t)__popc(m));
    });
    __syncthreads();
    for (int k = threadIdx.x; k < kBuckets; k += blockDim.x) {
        const uint32_t c = s_pos[k];
        s_pos[k] = c ? offset[k] + atomicAdd(&cursor[k], c) : 0u;
    }
    __syncthreads();
    for_each_bucket(C, nL, nE, i, [&](int b, unsigned m, bool has, uint32_t item) {
        uint32_t base = 0;
        if (lane == (unsigned)(__ffs(m) - 1)) base = atomicAdd(&s_pos[b], (uint32_t)__popc(m));
        base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
        if (has) items[base + __popc(m & ((1u << lane) - 1u))] = item;
    });
}

// One connection (Path::Connect, :298-330): the full path L[0..s-1] E[t-1..0],
// its contribution and the shadow ray between the two subpath ends.
// 8 blocks per SM (64 registers): +1.5 % over the unbounded 72-register build
__global__ void __launch_bounds__(kBdptThreads, 8) k_bd_connect(Ctx C, Wave w, const uint32_t* __restrict__ items,
                                                             uint32_t n_items, float4* __restrict__ rays,
                                                             float4* __restrict__ rec)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_items) return;
    const uint32_t it = items[q];
    const uint32_t i = it & kSampleMask;
    const int s = (int)((it >> kItemS) & 0x1fu), t = (int)(it >> kItemT);
    float c[3] = {0.0f, 0.0f, 0.0f};
    PV P[2 * kMaxV];
    if (s == 0) {
        // the eye subpath ends on a light (d = 0) or its direct vertex is one
        const int d = (int)((it >> kItemD) & 1u);
        const BVtx last = w.sv[1][(size_t)(t - 1) * w.stride + i];
        bool ok0 = false;
        if (d == 0) {
            if (flags_of(last) & F_SV) {
                P[0] = unpack(last);
                ok0 = P[0].prim >= 0 && C.sc.prims[P[0].prim].is_light;
            }
        } else if (flags_of(last) & F_DIRECT) {
            P[0] = unpack(w.dv[1][(size_t)(t - 1) * w.stride + i]);
            ok0 = true;
        }
        if (ok0) {
            P[0].type = T_L;
            for (int k = 1; k < t; k++) P[k] = unpack(w.sv[1][(size_t)(t - 1 - k) * w.stride + i]);
            ok0 = path_contribution(C, P, t, 0, d != 0, c);
        }
        store_null_ray(rays, q);  // visibility known already: the splat sees a miss
        rec[q] = ok0 ? make_float4(c[0], c[1], c[2], __uint_as_float(raster_pixel(C, P, t)))
                     : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const BVtx lend = w.sv[0][(size_t)(s - 1) * w.stride + i], eend = w.sv[1][(size_t)(t - 1) * w.stride + i];
    bool ok = (flags_of(lend) & F_SV) && (flags_of(eend) & F_SV);
    const int n = s + t;
    if (ok) {
        for (int k = 0; k < s; k++) P[k] = unpack(w.sv[0][(size_t)k * w.stride + i]);
        for (int k = 0; k < t; k++) P[s + k] = unpack(w.sv[1][(size_t)(t - 1 - k) * w.stride + i]);
        ok = path_contribution(C, P, n, s, false, c);
    }
    if (ok) {
        store_shadow_ray(rays, q, P[s - 1].p, P[s].p);
        rec[q] = make_float4(c[0], c[1], c[2], __uint_as_float(raster_pixel(C, P, n)));
    } else {
        store_null_ray(rays, q);
        rec[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
}

__global__ void k_bd_splat(Wave w, const uint32_t* __restrict__ items, uint32_t n_items,
                           const float4* __restrict__ rec, const lmgpu_hit* __restrict__ hits,
                           double* __restrict__ film_x, double* __restrict__ film_x_sq)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n_items) return;
    const float4 r = rec[q];
    if ((r.x == 0.0f && r.y == 0.0f && r.z == 0.0f) || hits[q].prim >= 0) return;
    const uint32_t i = items[q] & kSampleMask;
    const uint32_t pix = __float_as_uint(r.w);
    const float c[3] = {r.x, r.y, r.z};
    if (pix == (uint32_t)((w.p0 + i) % w.npix)) {
        for (int k = 0; k < 3; k++)
            if (c[k] != 0.0f) atomicAdd(&w.own[3 * (size_t)i + k], c[k]);
    } else {
        splat_px(film_x, film_x_sq, pix, c);
    }
}

__global__ void k_bd_flush(Wave w, double* __restrict__ film, double* __restrict__ film_sq)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= w.n) return;
    const float c[3] = {w.own[3 * (size_t)i], w.own[3 * (size_t)i + 1], w.own[3 * (size_t)i + 2]};
    splat_px(film, film_sq, (uint32_t)((w.p0 + i) % w.npix), c);
}

template <typename T>
int grow_dev(T** p, uint64_t* cap, uint64_t count)
{
    if (*cap >= count) return LMGPU_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    const cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) {
        set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
        return LMGPU_ERR_CUDA;
    }
    *cap = count;
    return LMGPU_OK;
}

inline unsigned blocks(uint64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

}  // namespace

// Device buffers of the bidirectional renderer, kept by the scene between calls.
struct BdptState {
    BVtx* verts = nullptr;  // sv[0], dv[0], sv[1], dv[1], each levels * stride
    uint64_t verts_cap = 0;
    BVtx* pend = nullptr;
    uint64_t pend_cap = 0;
    int32_t* counts = nullptr;
    uint64_t counts_cap = 0;
    float* own = nullptr;
    uint64_t own_cap = 0;
    uint32_t* active[2] = {nullptr, nullptr};
    uint64_t active_cap[2] = {0, 0};
    float4* ext[2] = {nullptr, nullptr};
    uint64_t ext_cap[2] = {0, 0};
    float4* sh = nullptr;
    uint64_t sh_cap = 0;
    lmgpu_hit* ext_hit = nullptr;
    uint64_t ext_hit_cap = 0;
    lmgpu_hit* sh_hit = nullptr;
    uint64_t sh_hit_cap = 0;
    uint32_t* counter = nullptr;  // [0], [1] step queue lengths, [2] connection items
    uint64_t counter_cap = 0;
    uint32_t* h_counter = nullptr;
    uint32_t* items = nullptr;
    uint64_t items_cap = 0;
    float4* c_rays = nullptr;
    uint64_t c_rays_cap = 0;
    float4* c_rec = nullptr;
    uint64_t c_rec_cap = 0;
    lmgpu_hit* c_hit = nullptr;
    uint64_t c_hit_cap = 0;
    uint32_t* buckets = nullptr;  // per strategy: counts, offsets, cursors
    uint64_t buckets_cap = 0;
};

void free_bdpt(BdptState* b)
{
    if (!b) return;
    void* ptrs[] = {b->verts, b->pend, b->counts, b->own, b->active[0], b->active[1], b->ext[0], b->ext[1],
                    b->sh, b->ext_hit, b->sh_hit, b->counter, b->items, b->c_rays, b->c_rec, b->c_hit,
                    b->buckets};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (b->h_counter) cudaFreeHost(b->h_counter);
    delete b;
}

int render_bdpt(lmgpu_scene* sc, const lmgpu_pt_params* prm, float* d_image, float* d_variance, cudaStream_t stream)
{
    const uint32_t W = (uint32_t)sc->cam.width, H = (uint32_t)sc->cam.height;
    const uint64_t npix = (uint64_t)W * H;
    const uint64_t total = npix * prm->spp;
    if (total == 0) return LMGPU_OK;
    if (sc->lights.count == 0) {
        set_error("lmgpu_render_bdpt: the scene has no area light");
        return LMGPU_ERR_INVALID;
    }
    int rc = clear_film(sc, npix, stream);
    if (rc) return rc;
    // The connection kernels keep a full path in per-thread local memory:
    // raise the per-thread stack limit once, up front, rather than have a
    // launch resize the device's local-memory pool.
    {
        size_t need = 0;
        const void* fns[] = {(const void*)k_bd_connect, (const void*)k_bd_count, (const void*)k_bd_step};
        for (const void* f : fns) {
            cudaFuncAttributes fa{};
            LMGPU_CUDA_TRY(cudaFuncGetAttributes(&fa, f));
            need = fa.localSizeBytes > need ? fa.localSizeBytes : need;
        }
        size_t stack = 0;
        LMGPU_CUDA_TRY(cudaDeviceGetLimit(&stack, cudaLimitStackSize));
        if (stack < need) LMGPU_CUDA_TRY(cudaDeviceSetLimit(cudaLimitStackSize, need));
    }
    Ctx C;
    C.sc = scene_view(sc);
    C.lights = sc->lights;
    C.cam = sc->cam;
    C.max_v = prm->max_num_vertices < 0 || prm->max_num_vertices > kMaxV ? kMaxV : prm->max_num_vertices;
    C.max_path = prm->max_num_vertices;
    C.mis = sc->bdpt_mis;
    C.min_path = prm->min_num_vertices;
    if (C.max_v < 1) return finalize_film(sc, prm->spp, d_image, d_variance, stream);

    if (!sc->bdpt) sc->bdpt = new BdptState();
    BdptState& B = *sc->bdpt;
    // wave size: the vertex arrays (4 x levels x 32 bytes per sample) within ~2 GB
    const uint64_t levels = (uint64_t)C.max_v;
    uint64_t stride = (2048ull << 20) / (4 * levels * sizeof(BVtx));
    stride = stride > kWaveSamples ? kWaveSamples : stride;
    stride = stride < total ? stride : total;
    if ((rc = grow_dev(&B.verts, &B.verts_cap, 4 * levels * stride)) ||
        (rc = grow_dev(&B.pend, &B.pend_cap, 2 * stride)) || (rc = grow_dev(&B.counts, &B.counts_cap, 2 * stride)) ||
        (rc = grow_dev(&B.own, &B.own_cap, 3 * stride)) ||
        (rc = grow_dev(&B.active[0], &B.active_cap[0], 2 * stride)) ||
        (rc = grow_dev(&B.active[1], &B.active_cap[1], 2 * stride)) ||
        (rc = grow_dev(&B.ext[0], &B.ext_cap[0], 4 * stride)) || (rc = grow_dev(&B.ext[1], &B.ext_cap[1], 4 * stride)) ||
        (rc = grow_dev(&B.sh, &B.sh_cap, 4 * stride)) || (rc = grow_dev(&B.ext_hit, &B.ext_hit_cap, 2 * stride)) ||
        (rc = grow_dev(&B.sh_hit, &B.sh_hit_cap, 2 * stride)) || (rc = grow_dev(&B.counter, &B.counter_cap, 3)) ||
        (rc = grow_dev(&B.buckets, &B.buckets_cap, 3 * kBuckets)))
        return rc;
    if (!B.h_counter && cudaMallocHost((void**)&B.h_counter, sizeof(uint32_t)) != cudaSuccess) {
        set_error("lmgpu_render_bdpt: pinned allocation failed");
        return LMGPU_ERR_CUDA;
    }
    Wave w;
    w.stride = (uint32_t)stride;
    w.npix = (uint32_t)npix;
    w.seed = prm->seed;
    w.sv[0] = B.verts;
    w.dv[0] = B.verts + levels * stride;
    w.sv[1] = B.verts + 2 * levels * stride;
    w.dv[1] = B.verts + 3 * levels * stride;
    w.count[0] = B.counts;
    w.count[1] = B.counts + stride;
    w.pend = B.pend;
    w.own = B.own;
    auto read_counter = [&](uint32_t& out) -> int {
        LMGPU_CUDA_TRY(cudaMemcpyAsync(B.h_counter, B.counter + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
        LMGPU_CUDA_TRY(cudaStreamSynchronize(stream));
        out = *B.h_counter;
        return LMGPU_OK;
    };
    for (uint64_t p0 = 0; p0 < total; p0 += stride) {
        w.p0 = p0;
        w.n = (uint32_t)((total - p0) < stride ? (total - p0) : stride);
        // subpaths: queue lengths stay on the device (counter [0] and [1]
        // alternate), the traversal and k_bd_step read them there; a bounded
        // subpath takes at most max_v - 1 steps
        uint32_t* qn = B.counter;
        k_bd_start<<<blocks(2ull * w.n, kBdptThreads), kBdptThreads, 0, stream>>>(C, w, B.ext[0], B.sh, B.active[0],
                                                                                   qn);
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches++;
        int cur = 0;
        for (int k = 1; k < C.max_v; k++) {
            if ((rc = launch_trace_dn(sc->accel, B.ext[cur], B.ext_hit, qn + cur, 2ull * w.n, false, stream,
                                      sc->probe)) ||
                (rc = launch_trace_dn(sc->accel, B.sh, B.sh_hit, qn + cur, 2ull * w.n, true, stream, sc->probe)))
                return rc;
            LMGPU_CUDA_TRY(cudaMemsetAsync(qn + (1 - cur), 0, sizeof(uint32_t), stream));
            k_bd_step<<<blocks(2ull * w.n, kBdptThreads), kBdptThreads, 0, stream>>>(
                C, w, k, qn + cur, B.active[cur], B.ext[cur], B.ext_hit, B.sh_hit, B.active[1 - cur], qn + (1 - cur),
                B.ext[1 - cur], B.sh);
            LMGPU_CUDA_TRY(cudaGetLastError());
            sc->launches += 3;
            cur = 1 - cur;
        }
        // connections
        LMGPU_CUDA_TRY(cudaMemsetAsync(B.counter + 2, 0, sizeof(uint32_t), stream));
        LMGPU_CUDA_TRY(cudaMemsetAsync(B.buckets, 0, sizeof(uint32_t) * kBuckets, stream));
        k_bd_count<<<blocks(w.n, kBdptThreads), kBdptThreads, 0, stream>>>(C, w, B.buckets, B.counter + 2);
        LMGPU_CUDA_TRY(cudaGetLastError());
        uint32_t n_items = 0;
        if ((rc = read_counter(n_items))) return rc;
        if (n_items > 0) {
            if ((rc = grow_dev(&B.items, &B.items_cap, n_items)) ||
                (rc = grow_dev(&B.c_rays, &B.c_rays_cap, 2ull * n_items)) ||
                (rc = grow_dev(&B.c_rec, &B.c_rec_cap, n_items)) || (rc = grow_dev(&B.c_hit, &B.c_hit_cap, n_items)))
                return rc;
            k_bd_buckets<<<1, 32, 0, stream>>>(B.buckets, B.buckets + kBuckets, B.buckets + 2 * kBuckets);
            k_bd_items<<<blocks(w.n, 256), 256, 0, stream>>>(C, w, B.buckets + kBuckets, B.buckets + 2 * kBuckets,
                                                            B.items);
            k_bd_connect<<<blocks(n_items, kBdptThreads), kBdptThreads, 0, stream>>>(C, w, B.items, n_items,
                                                                                   B.c_rays, B.c_rec);
            LMGPU_CUDA_TRY(cudaGetLastError());
            if ((rc = launch_trace(sc->accel, B.c_rays, B.c_hit, n_items, true, false, stream, sc->probe))) return rc;
            k_bd_splat<<<blocks(n_items, 256), 256, 0, stream>>>(w, B.items, n_items, B.c_rec, B.c_hit, sc->film_x,
                                                                  sc->film_x_sq);
            LMGPU_CUDA_TRY(cudaGetLastError());
            sc->launches += 5;
        }
        k_bd_flush<<<blocks(w.n, 256), 256, 0, stream>>>(w, sc->film, sc->film_sq);
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches += 2;
    }
    return finalize_film(sc, prm->spp, d_image, d_variance, stream);
}

}  // namespace lmgpu
