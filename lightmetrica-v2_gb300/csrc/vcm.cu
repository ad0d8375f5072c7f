// Vertex connection and merging on the GPU: the form of renderer::vcm
// (src/liblightmetrica/renderer/renderer_vcm.cpp), the reference's naive VCM
// [Georgiev et al. 2012] in the path-space form of [Hachisuka et al. 2012].
//
// Reference estimator, per pass k (Render, :596-790):
//   * merge radius r = initial_radius, then sqrt((alpha + k) / (1 + k)) r;
//   * num_photon_trace_samples light subpaths (SubpathSampler::TraceSubpath,
//     subpathsampler.cpp:41-190: no roulette; a subpath ends on a miss, on a
//     black BSDF value or at max_num_vertices vertices; the area light's
//     position and emission direction come from the same 2D sample,
//     light_area.cpp:73-80) and a range structure over their vertices 1..
//     that are neither a delta position nor a delta direction (VCMKdTree,
//     :355-465);
//   * num_eye_trace_samples samples, each an eye subpath and a fresh light
//     subpath; for every eye vertex t the connections s in [max(0, 2 - t,
//     min - t), min(nL, max - t)] (ConnectSubpaths :73-100, EvaluateF
//     :115-211) and, in the vcm and bdpm modes, a merge with every photon
//     vertex within r (|p - x|^2 < r^2; MergeSubpaths :102-113 joins the
//     photon subpath up to the vertex before the merged one to the eye
//     vertex); each weighted by the power heuristic over the connection and
//     merge strategies of the path, merges counted num_photon_trace_samples
//     times (EvaluatePathPDF :213-276, EvaluateMISWeight_* :278-338), divided
//     by its path pdf and splatted with W H / num_eye_trace_samples;
//   * the film is the mean of the passes' images.
// One difference: where a connection's path pdf is 0 although its value is
// not (FP32 underflow), the reference ends the whole sample (:698-702); here
// only that strategy is dropped.
//
// GPU structure, per pass:
//   photons     k_vc_start, then (closest-hit traversal, k_vc_step) for each
//               further vertex; queue lengths stay on the device;
//   grid        k_vc_hash counts the mergeable photon vertices per hashed
//               cell (cells r wide, so a query visits 3 x 3 x 3 cells), an
//               exclusive scan gives each bucket its range, k_vc_scatter
//               writes (position, subpath | vertex) entries into the ranges;
//   eye waves   eye and light subpaths of up to kWave samples (as for the
//               photons), then
//               k_vc_items    one thread per sample reserves its connection
//                             items (sample | s << 20 | t << 26) on a device
//                             counter;
//               k_vc_connect  contribution and shadow ray per item, any-hit
//                             traversal, k_vc_csplat adds the unoccluded;
//               k_vc_qkeys    the merge queries (sample, eye vertex t >= 2)
//                             keyed by the Morton code of the eye vertex,
//                             radix-sorted, so neighbouring lanes scan the
//                             same cells;
//               k_vc_merge    one lane per query: the cells around the
//                             vertex, each photon vertex within r evaluated
//                             as a merge;
//               k_vc_flush    each sample's own-pixel sum into the film.
// Subpath vertices are 32-byte records [vertex k][subpath] in HBM; random
// numbers are Philox keyed by (seed, pass, subpath kind, index, step).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "interact.cuh"
#include "rng.cuh"

namespace lmgpu {

struct VcmState;
void free_vcm(VcmState* v);

namespace {

constexpr int kMaxV = 16;
constexpr int kVcThreads = 128;
constexpr uint32_t kKeyVcm = 0x56434d31u;
constexpr uint32_t kWave = 1u << 19;  // eye samples per wave: the item's sample bits
constexpr uint32_t kSampleMask = kWave - 1u;
enum : int { MODE_VCM = 0, MODE_BDPT = 1, MODE_BDPM = 2 };
enum : uint32_t { KIND_PHOTON = 0, KIND_LIGHT = 1, KIND_EYE = 2 };

struct __align__(16) VVtx {
    float4 a;  // p, prim (int bits)
    float4 b;  // n, type | degen << 8 (bits)
};

__device__ __forceinline__ VVtx vpack(const PV& v)
{
    VVtx r;
    r.a = make_float4(v.p.x, v.p.y, v.p.z, __int_as_float(v.prim));
    r.b = make_float4(v.n.x, v.n.y, v.n.z, __uint_as_float(((uint32_t)v.type & 0xffu) | (((uint32_t)v.degen & 0xffu) << 8)));
    return r;
}

__device__ __forceinline__ PV vunpack(const VVtx& r)
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

// Subpaths: vertex k of subpath i at v[k * stride + i]; n[i] vertices.
struct Subs {
    VVtx* v;
    int32_t* n;
    uint32_t stride;
};

// Constants of one pass.
struct Pass {
    float r, r2, inv_cell;  // merge radius, its square, 1 / cell width (r)
    float kernel;           // pi r^2, the merge strategies' pdf factor
    float n_photon;         // num_photon_trace_samples: the merge strategies' count
    uint32_t pass, seed;
    uint32_t table_mask;    // hashed cells - 1
    int mode;
};

// Random numbers of step k of subpath `index` of a kind in a pass.
__device__ __forceinline__ float4 vc_rand(uint64_t index, uint32_t kind, uint32_t pass, int k, uint32_t seed)
{
    const Philox4x32 r = philox4x32_10((uint32_t)index, (uint32_t)(index >> 32) ^ (kind << 28),
                                       (pass << 8) | (uint32_t)k, 0u, seed, kKeyVcm);
    return make_float4(u01(r.v[0]), u01(r.v[1]), u01(r.v[2]), u01(r.v[3]));
}

// Appends (slot, ray o + [1e-4, inf) d) to a queue with warp-aggregated
// atomics; every lane of the warp calls it.
__device__ __forceinline__ void queue_push(bool has, uint32_t slot, float3 o, float3 d, uint32_t* __restrict__ active,
                                           float4* __restrict__ rays, uint32_t* __restrict__ count)
{
    const unsigned m = __ballot_sync(0xffffffffu, has);
    if (m == 0u) return;
    const unsigned lane = threadIdx.x & 31u, leader = __ffs(m) - 1u;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (has) {
        const uint32_t q = base + __popc(m & ((1u << lane) - 1u));
        active[q] = slot;
        rays[2 * q] = make_float4(o.x, o.y, o.z, 1e-4f);
        rays[2 * q + 1] = make_float4(d.x, d.y, d.z, FLT_MAX);
    }
}

// Vertex 0 of every subpath of a set and its step-1 ray (subpathsampler.cpp:61-104):
// slots [0, nl) are the light subpaths of L, [nl, nl + ne) the eye subpaths of E.
// An eye subpath's raster position is stratified over the pixels (sample
// index mod W H) or uniform over the film; its pixel goes to own_pix.
__global__ void __launch_bounds__(kVcThreads) k_vc_start(Ctx C, Pass X, Subs L, Subs E, uint32_t nl, uint32_t ne,
                                                         uint64_t index0, uint32_t kind_l, int stratified,
                                                         uint32_t* __restrict__ own_pix, uint32_t* __restrict__ active,
                                                         float4* __restrict__ rays, uint32_t* __restrict__ count)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    bool has = false;
    float3 o = zero3(), wo = zero3();
    if (j < nl + ne) {
        const bool eye = j >= nl;
        const uint32_t i = eye ? j - nl : j;
        const uint64_t g = index0 + i;
        // uEP_C selects the emitter, uED gives the position and the direction
        const float4 u = vc_rand(g, eye ? (uint32_t)KIND_EYE : kind_l, X.pass, 0, X.seed);
        PV v;
        if (!eye) {
            sample_light(C, u.x, u.y, u.z, v);
            const float3 l = cosine_hemisphere(u.y, u.z);
            float3 b, c;
            basis(v.n, b, c);
            wo = b * l.x + c * l.y + v.n * l.z;
            has = !black(eval_dir(C, v, T_L, zero3(), wo, DIR_LE, false));
            L.v[i] = vpack(v);
            L.n[i] = 1;
        } else {
            sensor_vertex(C, v);
            const uint32_t W = (uint32_t)C.cam.width, H = (uint32_t)C.cam.height;
            float rx, ry;
            uint32_t pix;
            if (stratified) {
                pix = (uint32_t)(g % ((uint64_t)W * H));
                rx = ((float)(pix % W) + u.y) / (float)W;
                ry = ((float)(pix / W) + u.z) / (float)H;
            } else {
                rx = u.y;
                ry = u.z;
                pix = pixel_at(C.cam, rx, ry);
            }
            wo = camera_dir(C.cam, rx, ry);
            own_pix[i] = pix;
            has = importance(C.cam, wo) > 0.0f;
            E.v[i] = vpack(v);
            E.n[i] = 1;
        }
        o = v.p;
        has = has && C.max_v > 1;
    }
    queue_push(has, j, o, wo, active, rays, count);
}

// Step k: the hit of each queued ray becomes vertex k of its subpath; the
// next direction is BSDF-sampled and queued while the subpath is shorter
// than max_num_vertices and the BSDF value is not black.
__global__ void __launch_bounds__(kVcThreads) k_vc_step(Ctx C, Pass X, Subs L, Subs E, uint32_t nl, uint64_t index0,
                                                        uint32_t kind_l, int k, const uint32_t* __restrict__ active_in,
                                                        const float4* __restrict__ rays_in,
                                                        const lmgpu_hit* __restrict__ hits,
                                                        const uint32_t* __restrict__ n_in,
                                                        uint32_t* __restrict__ active_out,
                                                        float4* __restrict__ rays_out, uint32_t* __restrict__ n_out)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    bool has = false;
    uint32_t j = 0;
    float3 o = zero3(), wo = zero3();
    if (q < *n_in) {
        j = active_in[q];
        const bool eye = j >= nl;
        const uint32_t i = eye ? j - nl : j;
        const Subs& S = eye ? E : L;
        const lmgpu_hit h = hits[q];
        if (h.prim >= 0) {
            const float4 r0 = rays_in[2 * q], r1 = rays_in[2 * q + 1];
            const float* T = C.sc.tris + 9 * (size_t)h.prim;
            const float3 p1 = f3(T[0], T[1], T[2]), p2 = f3(T[3], T[4], T[5]), p3 = f3(T[6], T[7], T[8]);
            PV v;
            v.p = f3(r0.x, r0.y, r0.z) + f3(r1.x, r1.y, r1.z) * h.t;
            v.n = normalize3(cross3(p2 - p1, p3 - p1));
            v.prim = C.sc.tri_prim[h.prim];
            // Type() & ~Emitter: the BSDF's type, none for a light (bsdf::null)
            v.type = (short)bsdf_type(C.sc.prims[v.prim].bsdf);
            v.degen = 0;
            S.v[(size_t)k * S.stride + i] = vpack(v);
            S.n[i] = k + 1;
            if (k + 1 < C.max_v) {
                const PV pv = vunpack(S.v[(size_t)(k - 1) * S.stride + i]);
                const float3 wi = dirto(v, pv);
                const float4 u = vc_rand(index0 + i, eye ? (uint32_t)KIND_EYE : kind_l, X.pass, k + 1, X.seed);
                has = sample_dir(C, v, wi, u.x, u.y, u.z, wo) &&
                      !black(eval_dir(C, v, v.type, wi, wo, eye ? DIR_EL : DIR_LE, false));
                o = v.p;
            }
        }
    }
    queue_push(has, j, o, wo, active_out, rays_out, n_out);
}

// Merge bookkeeping.  A merge at eye vertex vE with photon vertex vi makes the
// path P = x_0 .. x_{s-1} (the photon subpath up to x = x_{s-1}, s = vi),
// vE = P[s], then the eye subpath back to the sensor.  With the light-side
// factors a_i = pdf_dir(P[i] -> P[i+1]) G and the eye-side factors
// b_i = pdf_dir(P[i] -> P[i-1]) G of the reference's EvaluatePathPDF, every
// strategy's pdf divided by the merge's own, p_own = PL(s-1) a_{s-1}
// sufE(s+1) pi r^2, splits into
//   photon-only factors  (a_i, b_i for i <= s - 2: the photon subpath alone),
//   four junction factors J1 = a_{s-1}, J3 = b_s, J2 = a_s, J4 = b_{s-1}
//                        (pdfs at x and vE towards each other),
//   eye-only factors     (a_i, b_i for i >= s + 1: the eye subpath alone),
// so the power-heuristic sum (EvaluateMISWeight_VCM / _BDPM) is
//   (J3 / J1)^2 (A + J4^2 B) + N + [c(s)] / (J1 K)^2 + EC0 + J2^2 (EC2 + N EM)
// with A, B per photon vertex (k_vc_prep), EC0, EC2, EM per eye vertex, N
// the photon count and K = pi r^2.  The same decomposition as the recursive
// MIS of [Georgiev 2012, "Implementing vertex connection and merging"],
// written here for this reference's pdfs and samplability rules.
constexpr int kRecWords = 5;  // float4s of a photon vertex's prefix record

// Per photon subpath: for each vertex k >= 1, the record of the light side a
// merge there needs, about x = x_{k-1}:
//   [0] x.p, prim      [1] x.n, type | degen << 8
//   [2] unit direction x -> x_{k-2} (zero for k = 1), PL(k-1)
//   [3] TL(k-1) rgb, A(k-1)     [4] B(k-1), G(x_{k-1}, x_{k-2}), 0, 0
// TL(j) = prod_{i<j} eval_dir(x_i, LE) G(x_i, x_{i+1}) (EvaluateF's fL up to
// x_j, exclusive), PL(j) = pdf_pos(x_0) emitter_pdf(x_0) prod_{i<j} a_i,
// A(j) the terms of strategies split at x_j (connection x_{j-1} -- x_j over
// K^2, vcm mode only; merge at x_j, times N), B(j) those split before x_j,
// B(j + 1) = (b_j^2 B(j) + A(j)) / a_j^2.
__global__ void k_vc_prep(Ctx C, Pass X, Subs P, uint32_t n, float4* __restrict__ rec)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nv = P.n[i];
    if (nv < 2) return;
    const float K2 = X.kernel * X.kernel;
    const bool conn = X.mode == MODE_VCM;
    PV w = vunpack(P.v[i]), x = w;  // w = x_{k-2}, x = x_{k-1}
    float tl[3] = {1.0f, 1.0f, 1.0f};
    float PL = pdf_pos(C, x) * emitter_pdf(C, x), PLprev = 1.0f, B = 0.0f, gxw = 0.0f;
    float3 wdir = zero3();
    for (int k = 1; k < nv; k++) {
        // A(k - 1)
        const int j = k - 1;
        const bool csamp = j == 0 ? !(x.type & T_E) : (!delta_dir(C, w, w.type) && !delta_dir(C, x, x.type));
        const bool msamp = j >= 1 && !(x.type & T_E) && !delta_dir(C, x, x.type);
        float A = msamp ? X.n_photon : 0.0f;
        if (conn && csamp) {
            const float q = PLprev / PL;
            A += q * q / K2;
        }
        float4* r = rec + ((size_t)k * n + i) * kRecWords;
        const VVtx xv = vpack(x);
        r[0] = xv.a;
        r[1] = xv.b;
        r[2] = make_float4(wdir.x, wdir.y, wdir.z, PL);
        r[3] = make_float4(tl[0], tl[1], tl[2], A);
        r[4] = make_float4(B, gxw, 0.0f, 0.0f);
        // advance to x_k
        const PV nx = vunpack(P.v[(size_t)k * P.stride + i]);
        const float3 u = dirto(x, nx);
        const float g = geometry_term(x, nx);
        const float a = pdf_dir(C, x, x.type, wdir, u) * g;
        const Spd fs = eval_dir(C, x, x.type, wdir, u, DIR_LE, false);
        for (int c = 0; c < 3; c++) tl[c] = tl[c] * fs.c[c] * g;
        float bb = 0.0f;
        if (j >= 1) bb = pdf_dir(C, x, x.type, u, wdir) * gxw;
        B = (bb * bb * B + A) / (a * a);
        PLprev = PL;
        PL *= a;
        wdir = dirto(nx, x);
        gxw = g;
        w = x;
        x = nx;
    }
}

__device__ __forceinline__ int3 vc_cell(float3 p, float ic)
{
    return make_int3((int)floorf(p.x * ic), (int)floorf(p.y * ic), (int)floorf(p.z * ic));
}

// Spatial hash of a cell [Teschner et al. 2003].
__device__ __forceinline__ uint32_t vc_hash(int3 c, uint32_t mask)
{
    return (((uint32_t)c.x * 73856093u) ^ ((uint32_t)c.y * 19349663u) ^ ((uint32_t)c.z * 83492791u)) & mask;
}

// Photon vertex (i, k) for thread index t of an n-subpath set: k >= 1 and
// neither a delta position nor a delta direction (VCMKdTree::Build, :388-399).
__device__ __forceinline__ bool vc_photon(const Ctx& C, const Subs& P, uint32_t n, uint64_t t, uint32_t& i, int& k,
                                          PV& v)
{
    i = (uint32_t)(t % n);
    k = (int)(t / n) + 1;
    if (k >= C.max_v || k >= P.n[i]) return false;
    v = vunpack(P.v[(size_t)k * P.stride + i]);
    return !(v.type & T_E) && !delta_dir(C, v, v.type);
}

__global__ void k_vc_hash(Ctx C, Pass X, Subs P, uint32_t n, uint64_t nt, uint32_t* __restrict__ cnt)
{
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    uint32_t i;
    int k;
    PV v;
    if (!vc_photon(C, P, n, t, i, k, v)) return;
    atomicAdd(&cnt[vc_hash(vc_cell(v.p, X.inv_cell), X.table_mask)], 1u);
}

// Each mergeable photon vertex into its bucket's range: the entry (position,
// subpath * 16 + vertex) and, alongside, the prefix record k_vc_prep made
// for it, so a query reads both contiguously.
__global__ void k_vc_scatter(Ctx C, Pass X, Subs P, uint32_t n, uint64_t nt, const uint32_t* __restrict__ start,
                             uint32_t* __restrict__ cursor, const float4* __restrict__ rec,
                             float4* __restrict__ entries, float4* __restrict__ srec)
{
    const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (t >= nt) return;
    uint32_t i;
    int k;
    PV v;
    if (!vc_photon(C, P, n, t, i, k, v)) return;
    const uint32_t h = vc_hash(vc_cell(v.p, X.inv_cell), X.table_mask);
    const uint32_t slot = start[h] + atomicAdd(&cursor[h], 1u);
    entries[slot] = make_float4(v.p.x, v.p.y, v.p.z, __uint_as_float(i * (uint32_t)kMaxV + (uint32_t)k));
    const size_t src = ((size_t)k * n + i) * kRecWords;
    for (int w = 0; w < kRecWords; w++) srec[(size_t)slot * kRecWords + w] = rec[src + w];
}

// VCMPath::EvaluateF (renderer_vcm.cpp:115-211).  EvaluatePosition is 1 for
// an area light and the pinhole, and 0 for the pinhole under evalDelta.
__device__ __noinline__ Spd vc_eval_f(const Ctx& C, const PV* P, int n, int s, bool merge)
{
    const int t = n - s;
    Spd fL = S1(1.0f);
    if (s > 0) {
        const int m = merge ? s : s - 1;
        for (int i = 0; i < m; i++) {
            const Spd fs = eval_dir(C, P[i], P[i].type, i >= 1 ? dirto(P[i], P[i - 1]) : zero3(), dirto(P[i], P[i + 1]),
                                    DIR_LE, false);
            const float G = geometry_term(P[i], P[i + 1]);
            for (int c = 0; c < 3; c++) fL.c[c] = fL.c[c] * fs.c[c] * G;
        }
    }
    if (black(fL)) return S1(0.0f);
    Spd fE = S1(1.0f);
    if (t > 0) {
        for (int i = n - 1; i > s; i--) {
            const Spd fs = eval_dir(C, P[i], P[i].type, i < n - 1 ? dirto(P[i], P[i + 1]) : zero3(),
                                    dirto(P[i], P[i - 1]), DIR_EL, false);
            const float G = geometry_term(P[i], P[i - 1]);
            for (int c = 0; c < 3; c++) fE.c[c] = fE.c[c] * fs.c[c] * G;
        }
    }
    if (black(fE)) return S1(0.0f);
    Spd cst = S1(0.0f);
    if (!merge) {
        if (s == 0 && t > 0) {
            if (!(P[0].type & T_E)) cst = eval_dir(C, P[0], P[0].type, zero3(), dirto(P[0], P[1]), DIR_EL, false);
        } else if (s > 0 && t > 0) {
            const PV& vL = P[s - 1];
            const PV& vE = P[s];
            const Spd fsL = eval_dir(C, vL, vL.type, s - 2 >= 0 ? dirto(vL, P[s - 2]) : zero3(), dirto(vL, vE), DIR_LE,
                                     true);
            const Spd fsE = eval_dir(C, vE, vE.type, s + 1 < n ? dirto(vE, P[s + 1]) : zero3(), dirto(vE, vL), DIR_EL,
                                     true);
            const float G = geometry_term(vL, vE);
            for (int c = 0; c < 3; c++) cst.c[c] = fsL.c[c] * G * fsE.c[c];
        }
        // s > 0, t == 0: the pinhole end, EvaluatePosition(evalDelta) = 0
    } else {
        const PV& v = P[s];
        cst = eval_dir(C, v, v.type, dirto(v, P[s + 1]), dirto(v, P[s - 1]), DIR_EL, true);
    }
    Spd r;
    for (int c = 0; c < 3; c++) r.c[c] = fL.c[c] * cst.c[c] * fE.c[c];
    return r;
}

// EvaluatePathPDF (renderer_vcm.cpp:213-276) of every strategy of one path
// and the power-heuristic weight of strategy (s_, merge_) over them
// (EvaluateMISWeight_VCM / _BDPT / _BDPM, :278-338; merges count
// num_photon_trace_samples times).  Light-side factors pdf_dir(P[i] -> P[i+1])
// G and eye-side factors pdf_dir(P[i] -> P[i-1]) G are combined through
// prefix / suffix products: a connection s takes preL[s - 1] sufE[s + 1], a
// merge at vertex s takes preL[s] sufE[s + 1] pi r^2.  *p_own: the pdf of
// strategy (s_, merge_) itself.
__device__ __noinline__ float vc_weight(const Ctx& C, const Pass& X, const PV* P, int n, int s_, bool merge_,
                                        float* p_own)
{
    float preL[kMaxV + 1], sufE[kMaxV + 2];
    preL[0] = pdf_pos(C, P[0]) * emitter_pdf(C, P[0]);
    for (int i = 0; i + 1 < n; i++)
        preL[i + 1] = preL[i] * (pdf_dir(C, P[i], P[i].type, i >= 1 ? dirto(P[i], P[i - 1]) : zero3(),
                                         dirto(P[i], P[i + 1])) *
                                 geometry_term(P[i], P[i + 1]));
    sufE[n] = pdf_pos(C, P[n - 1]) * emitter_pdf(C, P[n - 1]);
    for (int i = n - 1; i >= 1; i--)
        sufE[i] = sufE[i + 1] * (pdf_dir(C, P[i], P[i].type, i + 1 < n ? dirto(P[i], P[i + 1]) : zero3(),
                                         dirto(P[i], P[i - 1])) *
                                 geometry_term(P[i], P[i - 1]));
    const float kernel = 3.14159265358979323846f * X.r * X.r;
    auto pdf = [&](int s, bool merge) -> float {
        const int t = n - s;
        if (!merge) {
            if (s == 0 && t > 0) {
                if (P[0].type & T_E) return 0.0f;
            } else if (s > 0 && t == 0) {
                if (P[n - 1].type & T_E) return 0.0f;
            } else if (s > 0 && t > 0) {
                if (delta_dir(C, P[s - 1], P[s - 1].type) || delta_dir(C, P[s], P[s].type)) return 0.0f;
            }
            return (s > 0 ? preL[s - 1] : 1.0f) * (t > 0 ? sufE[s + 1] : 1.0f);
        }
        if (s == 0 || t == 0) return 0.0f;
        if ((P[s].type & T_E) || delta_dir(C, P[s], P[s].type)) return 0.0f;
        return preL[s] * sufE[s + 1] * kernel;
    };
    const float ps = pdf(s_, merge_);
    *p_own = ps;
    float inv = 0.0f;
    for (int s = 0; s <= n; s++)
        for (int m = 0; m < 2; m++) {
            if ((X.mode == MODE_BDPT && m) || (X.mode == MODE_BDPM && !m)) continue;
            const float pi = pdf(s, m != 0);
            if (pi > 0.0f) {
                const float q = pi / ps;
                inv += q * q * (m ? X.n_photon : 1.0f);
            }
        }
    return 1.0f / inv;
}

// f w / p of strategy (s, merge) of path P; false if black or undefined.
__device__ __forceinline__ bool vc_contribution(const Ctx& C, const Pass& X, const PV* P, int n, int s, bool merge,
                                                float c[3])
{
    const Spd f = vc_eval_f(C, P, n, s, merge);
    if (black(f)) return false;
    float p = 0.0f;
    const float w = vc_weight(C, X, P, n, s, merge, &p);
    if (p == 0.0f || !(w == w)) return false;
    bool any = false;
    for (int k = 0; k < 3; k++) {
        c[k] = f.c[k] * w / p;
        any = any || (c[k] != 0.0f && c[k] == c[k]);
    }
    return any;
}

// Film_HDR::Splat's pixel of the raster position of the path's last segment
// (VCMPath::RasterPosition, :340-347): `e` the sensor, `e1` the next vertex.
__device__ __forceinline__ uint32_t raster_pixel(const Ctx& C, const PV& e, const PV& e1)
{
    float rx = 0.0f, ry = 0.0f;
    raster_pos(C.cam, dirto(e, e1), rx, ry);
    return pixel_at(C.cam, rx, ry);
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

// The connection range of eye vertex count t (Render, :676-681).
__device__ __forceinline__ void conn_range(const Ctx& C, int t, int nL, int& lo, int& hi)
{
    lo = 2 - t > 0 ? 2 - t : 0;
    if (C.min_path - t > lo) lo = C.min_path - t;
    hi = nL < C.max_path - t ? nL : C.max_path - t;
}

// s = 0 needs the eye subpath's vertex t - 1 on a light (ConnectSubpaths, :80-85).
__device__ __forceinline__ bool eye_on_light(const Ctx& C, const Subs& E, uint32_t i, int t)
{
    const int prim = __float_as_int(E.v[(size_t)(t - 1) * E.stride + i].a.w);
    return prim >= 0 && C.sc.prims[prim].is_light;
}

// Per sample: its connection items, reserved as one range of a device
// counter; its own-pixel accumulator cleared.
__global__ void __launch_bounds__(kVcThreads) k_vc_items(Ctx C, Subs L, Subs E, uint32_t n, int connect,
                                                         uint32_t* __restrict__ items, uint32_t* __restrict__ count,
                                                         float* __restrict__ own)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    own[3 * (size_t)i] = own[3 * (size_t)i + 1] = own[3 * (size_t)i + 2] = 0.0f;
    if (!connect) return;
    const int nL = L.n[i], nE = E.n[i];
    uint32_t cnt = 0;
    for (int t = 1; t <= nE; t++) {
        int lo, hi;
        conn_range(C, t, nL, lo, hi);
        if (lo > hi) continue;
        cnt += (uint32_t)(hi - lo + 1);
        if (lo == 0 && !eye_on_light(C, E, i, t)) cnt--;
    }
    if (cnt == 0) return;
    uint32_t o = atomicAdd(count, cnt);
    for (int t = 1; t <= nE; t++) {
        int lo, hi;
        conn_range(C, t, nL, lo, hi);
        for (int s = lo; s <= hi; s++) {
            if (s == 0 && !eye_on_light(C, E, i, t)) continue;
            items[o++] = i | ((uint32_t)s << 20) | ((uint32_t)t << 26);
        }
    }
}

// One connection item: the full path L[0..s-1] E[t-1..0] (ConnectSubpaths,
// :73-100), its contribution and the shadow ray between the subpath ends
// (none for s = 0: the eye subpath's own ray found the light).
__global__ void __launch_bounds__(kVcThreads) k_vc_connect(Ctx C, Pass X, Subs L, Subs E,
                                                           const uint32_t* __restrict__ items,
                                                           const uint32_t* __restrict__ count,
                                                           float4* __restrict__ rays, float4* __restrict__ rec)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= *count) return;
    const uint32_t it = items[q];
    const uint32_t i = it & kSampleMask;
    const int s = (int)((it >> 20) & 0x1fu), t = (int)(it >> 26);
    const int n = s + t;
    PV P[kMaxV];
    for (int k = 0; k < s; k++) P[k] = vunpack(L.v[(size_t)k * L.stride + i]);
    for (int k = 0; k < t; k++) P[s + k] = vunpack(E.v[(size_t)(t - 1 - k) * E.stride + i]);
    if (s == 0) P[0].type = T_L;
    float c[3] = {0.0f, 0.0f, 0.0f};
    const bool ok = vc_contribution(C, X, P, n, s, false, c);
    if (ok && s > 0) {
        float3 d = P[s].p - P[s - 1].p;
        const float len = sqrtf(dot3(d, d));
        d = d * (1.0f / len);
        rays[2 * q] = make_float4(P[s - 1].p.x, P[s - 1].p.y, P[s - 1].p.z, 1e-4f);
        rays[2 * q + 1] = make_float4(d.x, d.y, d.z, len * (1.0f - 1e-4f));
    } else {
        rays[2 * q] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);  // empty [tmin, tmax]: a miss
        rays[2 * q + 1] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    }
    rec[q] = ok ? make_float4(c[0], c[1], c[2], __uint_as_float(raster_pixel(C, P[n - 1], P[n - 2])))
                : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void k_vc_csplat(const uint32_t* __restrict__ items, const uint32_t* __restrict__ count,
                            const float4* __restrict__ rec, const lmgpu_hit* __restrict__ hits,
                            const uint32_t* __restrict__ own_pix, float* __restrict__ own,
                            double* __restrict__ film_x, double* __restrict__ film_x_sq)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= *count) return;
    const float4 r = rec[q];
    if ((r.x == 0.0f && r.y == 0.0f && r.z == 0.0f) || hits[q].prim >= 0) return;
    const uint32_t i = items[q] & kSampleMask;
    const uint32_t pix = __float_as_uint(r.w);
    const float c[3] = {r.x, r.y, r.z};
    if (pix == own_pix[i]) {
        for (int k = 0; k < 3; k++)
            if (c[k] != 0.0f) atomicAdd(&own[3 * (size_t)i + k], c[k]);
    } else {
        splat_px(film_x, film_x_sq, pix, c);
    }
}

__device__ __forceinline__ uint32_t morton_spread10(uint32_t x)
{
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// Sort key of merge query q = (i, t), i = q mod n, t = q / n + 2: the Morton
// code of its eye vertex in the scene's bounding cube (10 bits per axis), so
// that the queries a warp takes after sorting lie close together and scan
// the same cells; queries without an eye vertex t sort last.
__global__ void k_vc_qkeys(Ctx C, Subs E, uint32_t n, uint32_t nq, float3 lo, float inv_size,
                           uint32_t* __restrict__ keys, uint32_t* __restrict__ vals)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const uint32_t i = q % n;
    const int t = (int)(q / n) + 2;
    uint32_t key = 0xffffffffu;
    if (t <= C.max_v && t <= E.n[i]) {
        const float4 a = E.v[(size_t)(t - 1) * E.stride + i].a;
        const float c[3] = {(a.x - lo.x) * inv_size, (a.y - lo.y) * inv_size, (a.z - lo.z) * inv_size};
        uint32_t m[3];
        for (int k = 0; k < 3; k++) m[k] = (uint32_t)fminf(fmaxf(c[k] * 1024.0f, 0.0f), 1023.0f);
        key = morton_spread10(m[0]) | (morton_spread10(m[1]) << 1) | (morton_spread10(m[2]) << 2);
    }
    keys[q] = key;
    vals[q] = q;
}

// Eye-side constants of one merge query (k_vc_merge), kept in shared memory.
struct MergeQuery {
    float4 p;   // vE.p, prim (int bits)
    float4 n;   // vE.n, type | degen << 8 (bits)
    float4 d2;  // unit direction vE -> E[t-2], G(vE, E[t-2])
    float4 fe;  // EvaluateF's eye-side product fE (rgb), SEc = sufE(s + 1)
    float4 ec;  // EC0, EC2, EM, unused
};

// f w / p of one merge of query q with the photon vertex whose prefix
// record is r (see the merge bookkeeping above k_vc_prep); vi: the photon
// vertex's index.  False if black or undefined.
__device__ __forceinline__ bool merge_eval(const Ctx& C, const Pass& X, const MergeQuery& q, const float4* r, int vi,
                                           float c[3])
{
    PV vE;
    vE.p = f3(q.p.x, q.p.y, q.p.z);
    vE.n = f3(q.n.x, q.n.y, q.n.z);
    vE.prim = __float_as_int(q.p.w);
    const uint32_t tb = __float_as_uint(q.n.w);
    vE.type = (short)(tb & 0xffu);
    vE.degen = (short)((tb >> 8) & 0xffu);
    const float3 dE2 = f3(q.d2.x, q.d2.y, q.d2.z);
    const float4 r2 = r[2], r3 = r[3], r4 = r[4];
    const PV x = vunpack(VVtx{r[0], r[1]});
    const float3 wdir = f3(r2.x, r2.y, r2.z);
    const float3 u = dirto(x, vE);
    const float3 mu = u * -1.0f;
    const float gxv = geometry_term(x, vE);
    const Spd fsx = eval_dir(C, x, x.type, wdir, u, DIR_LE, false);
    if (black(fsx)) return false;
    const Spd cst = eval_dir(C, vE, vE.type, dE2, mu, DIR_EL, true);
    if (black(cst)) return false;
    const float J1 = pdf_dir(C, x, x.type, wdir, u) * gxv;
    const float J3 = pdf_dir(C, vE, vE.type, dE2, mu) * gxv;
    const float J2 = pdf_dir(C, vE, vE.type, mu, dE2) * q.d2.w;
    const float J4 = vi >= 2 ? pdf_dir(C, x, x.type, u, wdir) * r4.y : 0.0f;
    const float p = r2.w * J1 * q.fe.w * X.kernel;
    if (p == 0.0f) return false;
    const float a = J3 / J1;
    float inv = a * a * (r3.w + J4 * J4 * r4.x) + X.n_photon + J2 * J2 * (q.ec.y + X.n_photon * q.ec.z) + q.ec.x;
    if (X.mode == MODE_VCM && !delta_dir(C, x, x.type)) {
        const float qc = 1.0f / (J1 * X.kernel);
        inv += qc * qc;
    }
    const float wgt = 1.0f / inv;
    if (!(wgt == wgt)) return false;
    const float tl[3] = {r3.x, r3.y, r3.z};
    const float fe[3] = {q.fe.x, q.fe.y, q.fe.z};
    bool nz = false;
    for (int k = 0; k < 3; k++) {
        const float fL = tl[k] * fsx.c[k] * gxv;
        c[k] = fL * cst.c[k] * fe[k] * wgt / p;
        nz = nz || (c[k] != 0.0f && c[k] == c[k]);
    }
    return nz;
}

// Merges at eye vertex t >= 2 of sample i (lane (i, t)): the photon
// vertices within r (RangeQuery, :418-461) in the cells the query sphere
// meets, each joined as photon subpath [0, vi) + eye subpath [t - 1 .. 0]
// (MergeSubpaths, :102-113, with the callback's checks, :729-763), its
// contribution f w / p (EvaluateF, EvaluatePathPDF and the MIS weight with
// merge = true) assembled from the photon vertex's prefix record, the query's
// eye-side constants and the junction factors.  A warp works in two phases:
// every lane scans its own cells one entry per step and queues the entries
// that pass (within r, path length allowed) in shared memory; whenever 32
// are queued the whole warp evaluates them, one per lane, and adds each to
// its query's shared accumulator.  So the evaluation runs on full warps
// however the candidates are spread over the lanes.
constexpr int kMergeQueue = 64;
// 6 blocks per SM (80 registers, some spills): the scan phase waits on
// memory, so occupancy beats spill-free code.  Measured on the Cornell-box
// workload: 8 blocks (64 registers) 23.45, 6 blocks 23.62, 4 blocks (106
// registers, no spills) 21.6 M eye samples/s.
// STATS: the counting instantiation of the trace profile, which also adds
// queries, eye-vertex reads, scanned entries and evaluated merges into
// stats[0..3].
template <bool STATS>
__global__ void __launch_bounds__(kVcThreads, 6) k_vc_merge(Ctx C, Pass X, Subs E, uint32_t n, uint32_t nq,
                                                         const uint32_t* __restrict__ order,
                                                         const uint32_t* __restrict__ start,
                                                         const float4* __restrict__ entries,
                                                         const float4* __restrict__ srec,
                                                         const uint32_t* __restrict__ own_pix, float* __restrict__ own,
                                                         double* __restrict__ film_x, double* __restrict__ film_x_sq,
                                                         unsigned long long* __restrict__ stats)
{
    __shared__ MergeQuery sq[kVcThreads];
    __shared__ float sacc[kVcThreads][3];
    __shared__ uint32_t qent[kVcThreads / 32][kMergeQueue];
    __shared__ uint8_t qlane[kVcThreads / 32][kMergeQueue];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t qid = slot < nq ? order[slot] : 0u;
    const uint32_t i = qid % n;
    const int t = (int)(qid / n) + 2;
    bool valid = slot < nq && t <= C.max_v && t <= E.n[i];
    PV vE;
    if (valid) {
        vE = vunpack(E.v[(size_t)(t - 1) * E.stride + i]);
        // IsDeltaPosition of the eye vertex; a delta-direction vE makes p_own 0
        valid = !(vE.type & T_E) && !delta_dir(C, vE, vE.type);
    }
    sacc[threadIdx.x][0] = sacc[threadIdx.x][1] = sacc[threadIdx.x][2] = 0.0f;
    int lo[3] = {0, 0, 0}, ext[3] = {1, 1, 1};
    if (valid) {
        const PV e2 = vunpack(E.v[(size_t)(t - 2) * E.stride + i]);  // E[t-2]
        MergeQuery q;
        const VVtx ev = vpack(vE);
        q.p = ev.a;
        q.n = ev.b;
        const float3 dE2 = dirto(vE, e2);
        q.d2 = make_float4(dE2.x, dE2.y, dE2.z, geometry_term(vE, e2));
        // eye-side constants: FE (EvaluateF's fE), SEc = sufE(s+1), and the
        // strategy sums EC0 (connection vE -- E[t-2]), EC2 (connections
        // further along the eye subpath), EM (merges at E[t-2] .. E[1])
        float fe[3] = {1.0f, 1.0f, 1.0f};
        float SEc = 1.0f;  // pdf_pos and emitter pdf of the pinhole are 1
        float EC0 = 0.0f, EC2 = 0.0f, EM = 0.0f;
        // walk E[t-2] .. E[0] (path indices j = s+1 .. n-1)
        float Pb = 1.0f, Pa = 1.0f, Pa2 = 1.0f;  // prod b_{s+1..j}, prod a_{s+1..j-1}, prod a_{s+1..j-2}
        bool dprev = false;  // vE is not a delta direction
        PV nxt = vE;         // P[j - 1]
        const float K2 = X.kernel * X.kernel;
        for (int e = t - 2; e >= 0; e--) {
            const PV cur = vunpack(E.v[(size_t)e * E.stride + i]);
            const PV prv = e >= 1 ? vunpack(E.v[(size_t)(e - 1) * E.stride + i]) : cur;  // P[j + 1]
            const float3 to_prev = e >= 1 ? dirto(cur, prv) : zero3();
            const float3 to_next = dirto(cur, nxt);
            const float g = geometry_term(cur, nxt);
            const float bb = pdf_dir(C, cur, cur.type, to_prev, to_next) * g;
            SEc *= bb;
            const Spd fs = eval_dir(C, cur, cur.type, to_prev, to_next, DIR_EL, false);
            for (int k = 0; k < 3; k++) fe[k] = fe[k] * fs.c[k] * g;
            Pb *= bb;
            const bool dcur = delta_dir(C, cur, cur.type);
            if (X.mode == MODE_VCM && !dprev && !dcur) {
                const float qq = (e == t - 2 ? 1.0f : Pa2) / Pb;
                if (e == t - 2) EC0 = qq * qq / K2;
                else EC2 += qq * qq / K2;
            }
            if (e >= 1 && !dcur) {
                const float qq = Pa / Pb;
                EM += qq * qq;
            }
            if (e >= 1) {
                const float aa = pdf_dir(C, cur, cur.type, to_next, to_prev) * geometry_term(cur, prv);
                Pa2 = Pa;
                Pa *= aa;
            }
            dprev = dcur;
            nxt = cur;
        }
        q.fe = make_float4(fe[0], fe[1], fe[2], SEc);
        q.ec = make_float4(EC0, EC2, EM, 0.0f);
        sq[threadIdx.x] = q;
        const float c3[3] = {vE.p.x, vE.p.y, vE.p.z};
        for (int a = 0; a < 3; a++) {
            lo[a] = (int)floorf(c3[a] * X.inv_cell - 1.0f - 1e-3f);
            const int hi = (int)floorf(c3[a] * X.inv_cell + 1.0f + 1e-3f);
            ext[a] = hi - lo[a] + 1;
            if (ext[a] > 4 || ext[a] < 1) valid = false;  // excluded by the host's radius check
        }
    }
    const int ncell = valid ? ext[0] * ext[1] * ext[2] : 0;
    uint32_t n_entries = 0, n_merges = 0;
    int cell = 0, cx = 0, cy = 0, cz = 0;
    uint32_t e = 0, e1 = 0;
    int qn = 0;  // queued entries (warp-uniform)
    __syncwarp();
    for (;;) {
        // scan: the next entry of this lane's query, if any
        bool has = false;
        uint32_t he = 0;
        if (valid) {
            while (e >= e1 && cell < ncell) {
                cx = lo[0] + cell % ext[0];
                cy = lo[1] + (cell / ext[0]) % ext[1];
                cz = lo[2] + cell / (ext[0] * ext[1]);
                const uint32_t h = vc_hash(make_int3(cx, cy, cz), X.table_mask);
                e = start[h];
                e1 = start[h + 1];
                cell++;
            }
            if (e < e1) {
                const float4 en = entries[e];
                const float3 lp = f3(en.x, en.y, en.z);
                const int3 lc = vc_cell(lp, X.inv_cell);
                const float3 d = lp - vE.p;
                const int np = (int)(__float_as_uint(en.w) % (uint32_t)kMaxV) + t;
                has = lc.x == cx && lc.y == cy && lc.z == cz && dot3(d, d) < X.r2 && np >= C.min_path &&
                      np <= C.max_path;
                he = e;
                e++;
                if (STATS) {
                    n_entries++;
                    n_merges += has ? 1u : 0u;
                }
            }
        }
        const bool more = valid && (e < e1 || cell < ncell);
        const unsigned m = __ballot_sync(0xffffffffu, has);
        if (has) {
            const int pos = qn + __popc(m & ((1u << lane) - 1u));
            qent[warp][pos] = he;
            qlane[warp][pos] = (uint8_t)lane;
        }
        qn += __popc(m);
        const bool any_more = __any_sync(0xffffffffu, more);
        __syncwarp();
        // evaluate: 32 queued entries at a time, or the rest at the end
        while (qn >= 32 || (!any_more && qn > 0)) {
            const int take = qn < 32 ? qn : 32;
            if ((int)lane < take) {
                const int idx = qn - take + (int)lane;
                const uint32_t ee = qent[warp][idx];
                const unsigned ql = qlane[warp][idx];
                const int vi = (int)(__float_as_uint(entries[ee].w) % (uint32_t)kMaxV);
                float c[3];
                if (merge_eval(C, X, sq[warp * 32 + ql], srec + (size_t)ee * kRecWords, vi, c))
                    for (int k = 0; k < 3; k++) atomicAdd(&sacc[warp * 32 + ql][k], c[k]);
            }
            qn -= take;
            __syncwarp();
        }
        if (!any_more) break;
    }
    __syncwarp();
    if (STATS) {
        // every lane of the warp is here: one atomic per counter and warp
        unsigned long long v[4] = {valid ? 1ull : 0ull, valid ? (unsigned long long)t : 0ull, n_entries, n_merges};
        for (int k = 0; k < 4; k++) {
            unsigned long long x = v[k];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) atomicAdd(&stats[k], x);
        }
    }
    if (!valid) return;
    const float acc[3] = {sacc[threadIdx.x][0], sacc[threadIdx.x][1], sacc[threadIdx.x][2]};
    if (acc[0] == 0.0f && acc[1] == 0.0f && acc[2] == 0.0f) return;
    const PV e0 = vunpack(E.v[i]), e1v = vunpack(E.v[(size_t)E.stride + i]);
    const uint32_t pix = raster_pixel(C, e0, e1v);
    if (pix == own_pix[i]) {
        for (int k = 0; k < 3; k++)
            if (acc[k] != 0.0f) atomicAdd(&own[3 * (size_t)i + k], acc[k]);
    } else {
        splat_px(film_x, film_x_sq, pix, acc);
    }
}

__global__ void k_vc_flush(uint32_t n, const uint32_t* __restrict__ own_pix, const float* __restrict__ own,
                           double* __restrict__ film, double* __restrict__ film_sq)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float c[3] = {own[3 * (size_t)i], own[3 * (size_t)i + 1], own[3 * (size_t)i + 2]};
    splat_px(film, film_sq, own_pix[i], c);
}

template <typename T>
int grow(T** p, uint64_t* cap, uint64_t count)
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

// Device buffers of the VCM renderer, kept by the scene between calls.
struct VcmState {
    VVtx* pool = nullptr;  // photon subpaths, levels x photons
    uint64_t pool_cap = 0;
    int32_t* pool_n = nullptr;
    uint64_t pool_n_cap = 0;
    VVtx* eye = nullptr;  // light then eye subpaths of a wave, 2 x levels x wave
    uint64_t eye_cap = 0;
    int32_t* eye_n = nullptr;
    uint64_t eye_n_cap = 0;
    uint32_t* own_pix = nullptr;
    uint64_t own_pix_cap = 0;
    float* own = nullptr;
    uint64_t own_cap = 0;
    uint32_t* active[2] = {nullptr, nullptr};
    uint64_t active_cap[2] = {0, 0};
    float4* rays[2] = {nullptr, nullptr};
    uint64_t rays_cap[2] = {0, 0};
    lmgpu_hit* hits = nullptr;
    uint64_t hits_cap = 0;
    uint32_t* counter = nullptr;  // [0], [1] queue lengths, [2] connection items
    uint64_t counter_cap = 0;
    uint32_t* cells = nullptr;  // hashed cells: counts / cursors, then starts (table + 1 each)
    uint64_t cells_cap = 0;
    float4* entries = nullptr;
    uint64_t entries_cap = 0;
    float4* rec = nullptr;  // photon prefix records, levels x photons x kRecWords
    uint64_t rec_cap = 0;
    float4* srec = nullptr;  // the same, in entry order
    uint64_t srec_cap = 0;
    void* scan_tmp = nullptr;
    uint64_t scan_tmp_cap = 0;
    uint32_t* qkeys = nullptr;  // merge query sort: keys and ids, double-buffered (4 x queries)
    uint64_t qkeys_cap = 0;
    void* sort_tmp = nullptr;
    uint64_t sort_tmp_cap = 0;
    uint32_t* items = nullptr;
    uint64_t items_cap = 0;
    float4* c_rays = nullptr;
    uint64_t c_rays_cap = 0;
    float4* c_rec = nullptr;
    uint64_t c_rec_cap = 0;
    lmgpu_hit* c_hit = nullptr;
    uint64_t c_hit_cap = 0;
};

void free_vcm(VcmState* v)
{
    if (!v) return;
    void* ptrs[] = {v->pool, v->pool_n, v->eye, v->eye_n, v->own_pix, v->own, v->active[0], v->active[1],
                    v->rays[0], v->rays[1], v->hits, v->counter, v->cells, v->entries, v->rec, v->srec,
                    v->scan_tmp, v->qkeys, v->sort_tmp, v->items,
                    v->c_rays, v->c_rec, v->c_hit};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete v;
}

namespace {

// Subpaths of one set (photons, or a wave's light and eye subpaths): vertex
// 0 and the step-1 rays, then (closest-hit traversal, step) per further
// vertex, queue lengths on the device.
int trace_subpaths(lmgpu_scene* sc, VcmState& V, const Ctx& C, const Pass& X, const Subs& L, const Subs& E,
                   uint32_t nl, uint32_t ne, uint64_t index0, uint32_t kind_l, int stratified, cudaStream_t stream)
{
    const uint32_t total = nl + ne;
    LMGPU_CUDA_TRY(cudaMemsetAsync(V.counter, 0, 2 * sizeof(uint32_t), stream));
    k_vc_start<<<blocks(total, kVcThreads), kVcThreads, 0, stream>>>(C, X, L, E, nl, ne, index0, kind_l, stratified,
                                                                     V.own_pix, V.active[0], V.rays[0], V.counter);
    LMGPU_CUDA_TRY(cudaGetLastError());
    sc->launches++;
    int cur = 0;
    for (int k = 1; k < C.max_v; k++) {
        int rc = launch_trace_dn(sc->accel, V.rays[cur], V.hits, V.counter + cur, total, false, stream, sc->probe);
        if (rc) return rc;
        LMGPU_CUDA_TRY(cudaMemsetAsync(V.counter + (1 - cur), 0, sizeof(uint32_t), stream));
        k_vc_step<<<blocks(total, kVcThreads), kVcThreads, 0, stream>>>(
            C, X, L, E, nl, index0, kind_l, k, V.active[cur], V.rays[cur], V.hits, V.counter + cur,
            V.active[1 - cur], V.rays[1 - cur], V.counter + (1 - cur));
        LMGPU_CUDA_TRY(cudaGetLastError());
        sc->launches += 2;
        cur = 1 - cur;
    }
    return LMGPU_OK;
}

uint32_t pow2_at_least(uint64_t x)
{
    uint64_t p = 1024;
    while (p < x && p < (1ull << 31)) p <<= 1;
    return (uint32_t)p;
}

int render_vcm(lmgpu_scene* sc, const lmgpu_vcm_params* prm, float* d_image, float* d_variance, cudaStream_t stream)
{
    const uint32_t W = (uint32_t)sc->cam.width, H = (uint32_t)sc->cam.height;
    const uint64_t npix = (uint64_t)W * H;
    int rc = clear_film(sc, npix, stream);
    if (rc) return rc;
    const uint64_t NE = prm->num_eye_trace_samples, passes = prm->num_iteration_pass;
    if (NE == 0 || passes == 0) return finalize_film_nx(sc, 1.0, 0.0, d_image, d_variance, stream);
    // the connection and merge kernels keep a path in per-thread local memory:
    // raise the stack limit once, up front
    {
        size_t need = 0;
        const void* fns[] = {(const void*)k_vc_connect, (const void*)k_vc_merge<false>, (const void*)k_vc_merge<true>,
                             (const void*)k_vc_prep};
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
    C.max_v = prm->max_num_vertices;
    C.max_path = prm->max_num_vertices;
    C.min_path = prm->min_num_vertices;
    const int mode = prm->mode;
    const uint64_t NL = mode == MODE_BDPT ? 0 : prm->num_photon_trace_samples;
    const uint64_t levels = (uint64_t)C.max_v;
    // connection items per sample: at most sum over t of (max - t + 1)
    const uint64_t items_per = mode == MODE_BDPM ? 0 : levels * (levels + 1) / 2;
    // wave size: a wave's subpaths and connection buffers within ~1 GB
    const uint64_t per_sample = 2 * levels * sizeof(VVtx) + 64 + items_per * 68;
    uint64_t wave = (1ull << 30) / per_sample;
    wave = wave > kWave ? kWave : wave;
    wave = wave < NE ? wave : NE;
    const uint64_t qcap = (2 * wave > NL ? 2 * wave : NL);
    const uint32_t table = NL ? pow2_at_least(NL * (levels > 1 ? levels - 1 : 1)) : 1024u;

    if (!sc->vcm) sc->vcm = new VcmState();
    VcmState& V = *sc->vcm;
    if ((rc = grow(&V.pool, &V.pool_cap, levels * (NL ? NL : 1))) || (rc = grow(&V.pool_n, &V.pool_n_cap, NL ? NL : 1)) ||
        (rc = grow(&V.eye, &V.eye_cap, 2 * levels * wave)) || (rc = grow(&V.eye_n, &V.eye_n_cap, 2 * wave)) ||
        (rc = grow(&V.own_pix, &V.own_pix_cap, wave)) || (rc = grow(&V.own, &V.own_cap, 3 * wave)) ||
        (rc = grow(&V.active[0], &V.active_cap[0], qcap)) || (rc = grow(&V.active[1], &V.active_cap[1], qcap)) ||
        (rc = grow(&V.rays[0], &V.rays_cap[0], 2 * qcap)) || (rc = grow(&V.rays[1], &V.rays_cap[1], 2 * qcap)) ||
        (rc = grow(&V.hits, &V.hits_cap, qcap)) || (rc = grow(&V.counter, &V.counter_cap, 4)) ||
        (rc = grow(&V.cells, &V.cells_cap, 2 * ((uint64_t)table + 1))) ||
        (rc = grow(&V.entries, &V.entries_cap, NL ? NL * (levels > 1 ? levels - 1 : 1) : 1)) ||
        (rc = grow(&V.rec, &V.rec_cap, NL ? NL * levels * kRecWords : 1)) ||
        (rc = grow(&V.srec, &V.srec_cap, NL ? NL * (levels > 1 ? levels - 1 : 1) * kRecWords : 1)) ||
        (rc = grow(&V.items, &V.items_cap, items_per * wave)) || (rc = grow(&V.c_rays, &V.c_rays_cap, 2 * items_per * wave)) ||
        (rc = grow(&V.c_rec, &V.c_rec_cap, items_per * wave)) || (rc = grow(&V.c_hit, &V.c_hit_cap, items_per * wave)))
        return rc;
    uint32_t* cnt = V.cells;
    uint32_t* start = V.cells + table + 1;
    size_t scan_bytes = 0;
    LMGPU_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, cnt, start, (int)(table + 1), stream));
    if ((rc = grow((char**)&V.scan_tmp, &V.scan_tmp_cap, scan_bytes))) return rc;
    // merge queries (sample, eye vertex t >= 2) of a wave, sorted by position
    const uint64_t nq_max = wave * (levels > 1 ? levels - 1 : 1);
    if ((rc = grow(&V.qkeys, &V.qkeys_cap, 4 * nq_max))) return rc;
    size_t sort_bytes = 0;
    LMGPU_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, V.qkeys, V.qkeys + nq_max, V.qkeys + 2 * nq_max,
                                                   V.qkeys + 3 * nq_max, (int)nq_max, 0, 32, stream));
    if ((rc = grow((char**)&V.sort_tmp, &V.sort_tmp_cap, sort_bytes))) return rc;
    float3 scene_lo;
    float scene_inv = 1.0f;
    {
        const float R = sc->sphere_radius > 0.0f ? sc->sphere_radius : 1.0f;
        scene_lo = make_float3(sc->sphere_center[0] - R, sc->sphere_center[1] - R, sc->sphere_center[2] - R);
        scene_inv = 1.0f / (2.0f * R);
    }

    Subs pool{V.pool, V.pool_n, (uint32_t)(NL ? NL : 1)};
    Subs eL{V.eye, V.eye_n, (uint32_t)wave};
    Subs eE{V.eye + levels * wave, V.eye_n + wave, (uint32_t)wave};
    Subs none{nullptr, nullptr, 1};
    const int stratified = NE % npix == 0;
    Pass X;
    X.r = 0.0f;
    X.n_photon = (float)prm->num_photon_trace_samples;
    X.seed = prm->seed;
    X.table_mask = table - 1;
    X.mode = mode;
    for (uint64_t pass = 0; pass < passes; pass++) {
        // merge radius of the pass (Render, :612-614), in single precision
        X.r = pass == 0 ? prm->initial_radius
                        : sqrtf((prm->alpha + (float)pass) / (1.0f + (float)pass)) * X.r;
        X.r2 = X.r * X.r;
        X.inv_cell = 1.0f / X.r;
        X.kernel = 3.14159265358979323846f * X.r * X.r;
        X.pass = (uint32_t)pass;
        if (NL) {
            if ((rc = trace_subpaths(sc, V, C, X, pool, none, (uint32_t)NL, 0, 0, KIND_PHOTON, 0, stream))) return rc;
            const uint64_t nt = NL * (levels > 1 ? levels - 1 : 1);
            k_vc_prep<<<blocks(NL, kVcThreads), kVcThreads, 0, stream>>>(C, X, pool, (uint32_t)NL, V.rec);
            LMGPU_CUDA_TRY(cudaGetLastError());
            LMGPU_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * ((size_t)table + 1), stream));
            k_vc_hash<<<blocks(nt, 256), 256, 0, stream>>>(C, X, pool, (uint32_t)NL, nt, cnt);
            LMGPU_CUDA_TRY(cudaGetLastError());
            size_t tmp = (size_t)V.scan_tmp_cap;
            LMGPU_CUDA_TRY(cub::DeviceScan::ExclusiveSum(V.scan_tmp, tmp, cnt, start, (int)(table + 1), stream));
            LMGPU_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * ((size_t)table + 1), stream));
            k_vc_scatter<<<blocks(nt, 256), 256, 0, stream>>>(C, X, pool, (uint32_t)NL, nt, start, cnt, V.rec,
                                                               V.entries, V.srec);
            LMGPU_CUDA_TRY(cudaGetLastError());
            sc->launches += 4;
        }
        for (uint64_t p0 = 0; p0 < NE; p0 += wave) {
            const uint32_t n = (uint32_t)((NE - p0) < wave ? (NE - p0) : wave);
            const uint64_t index0 = p0;
            if ((rc = trace_subpaths(sc, V, C, X, eL, eE, n, n, index0, KIND_LIGHT, stratified, stream))) return rc;
            LMGPU_CUDA_TRY(cudaMemsetAsync(V.counter + 2, 0, sizeof(uint32_t), stream));
            k_vc_items<<<blocks(n, kVcThreads), kVcThreads, 0, stream>>>(C, eL, eE, n, mode != MODE_BDPM, V.items,
                                                                         V.counter + 2, V.own);
            LMGPU_CUDA_TRY(cudaGetLastError());
            sc->launches++;
            if (mode != MODE_BDPM) {
                const uint64_t max_items = items_per * n;
                k_vc_connect<<<blocks(max_items, kVcThreads), kVcThreads, 0, stream>>>(C, X, eL, eE, V.items,
                                                                                       V.counter + 2, V.c_rays, V.c_rec);
                LMGPU_CUDA_TRY(cudaGetLastError());
                if ((rc = launch_trace_dn(sc->accel, V.c_rays, V.c_hit, V.counter + 2, max_items, true, stream,
                                          sc->probe)))
                    return rc;
                k_vc_csplat<<<blocks(max_items, 256), 256, 0, stream>>>(V.items, V.counter + 2, V.c_rec, V.c_hit,
                                                                        V.own_pix, V.own, sc->film_x, sc->film_x_sq);
                LMGPU_CUDA_TRY(cudaGetLastError());
                sc->launches += 3;
            }
            if (mode != MODE_BDPT && NL > 0 && C.max_v >= 2) {
                const uint32_t nq = (uint32_t)((uint64_t)n * (levels - 1));
                uint32_t *kin = V.qkeys, *kout = V.qkeys + nq_max, *vin = V.qkeys + 2 * nq_max,
                         *vout = V.qkeys + 3 * nq_max;
                k_vc_qkeys<<<blocks(nq, 256), 256, 0, stream>>>(C, eE, n, nq, scene_lo, scene_inv, kin, vin);
                LMGPU_CUDA_TRY(cudaGetLastError());
                size_t sb = (size_t)V.sort_tmp_cap;
                LMGPU_CUDA_TRY(cub::DeviceRadixSort::SortPairs(V.sort_tmp, sb, kin, kout, vin, vout, (int)nq, 0, 32,
                                                               stream));
                // the trace profile: counting instantiation, or events around the launch
                TraceProbe* pr = sc->probe && sc->probe->mode != TraceProbe::kOff ? sc->probe : nullptr;
                const bool count = pr && pr->mode == TraceProbe::kProbeCount;
                const bool timed = pr && pr->mode == TraceProbe::kProbeTime &&
                                   pr->merge_used + 2 <= pr->merge_events.size();
                if (pr) pr->merge_launches++;
                if (timed) LMGPU_CUDA_TRY(cudaEventRecord(pr->merge_events[pr->merge_used], stream));
                auto merge = count ? k_vc_merge<true> : k_vc_merge<false>;
                merge<<<blocks(nq, kVcThreads), kVcThreads, 0, stream>>>(
                    C, X, eE, n, nq, vout, start, V.entries, V.srec, V.own_pix, V.own, sc->film_x, sc->film_x_sq,
                    count ? pr->d_counters + TraceProbe::kMergeCounters : nullptr);
                LMGPU_CUDA_TRY(cudaGetLastError());
                if (timed) {
                    LMGPU_CUDA_TRY(cudaEventRecord(pr->merge_events[pr->merge_used + 1], stream));
                    pr->merge_used += 2;
                }
                sc->launches += 2;
            }
            k_vc_flush<<<blocks(n, 256), 256, 0, stream>>>(n, V.own_pix, V.own, sc->film, sc->film_sq);
            LMGPU_CUDA_TRY(cudaGetLastError());
            sc->launches++;
        }
    }
    // film = (1 / P) sum over passes of W H / N_E sum C: the sums over
    // N_E P / (W H) samples per pixel
    const double spp = (double)NE * (double)passes / (double)npix;
    return finalize_film_nx(sc, spp, spp * (double)(npix - 1), d_image, d_variance, stream);
}

int render_vcm_checked(const char* name, lmgpu_scene* sc, const lmgpu_vcm_params* prm, float* d_image,
                       float* d_variance, cudaStream_t s)
{
    if (!sc || !prm || !d_image) {
        set_error(std::string(name) + ": NULL argument");
        return LMGPU_ERR_INVALID;
    }
    if (prm->max_num_vertices < 1 || prm->max_num_vertices > kMaxV) {
        set_error(std::string(name) + ": max_num_vertices must be in [1, 16] (subpaths have no roulette)");
        return LMGPU_ERR_INVALID;
    }
    if (prm->mode < MODE_VCM || prm->mode > MODE_BDPM) {
        set_error(std::string(name) + ": unknown mode");
        return LMGPU_ERR_INVALID;
    }
    if (prm->mode != MODE_BDPT && prm->num_photon_trace_samples >= (1ull << 28)) {
        set_error(std::string(name) + ": num_photon_trace_samples must be below 2^28");
        return LMGPU_ERR_INVALID;
    }
    if (prm->mode != MODE_BDPT && prm->num_iteration_pass > 0 && !(prm->initial_radius > 0.0f)) {
        set_error(std::string(name) + ": initial_radius must be positive");
        return LMGPU_ERR_INVALID;
    }
    if (prm->num_iteration_pass >= (1ull << 24)) {
        set_error(std::string(name) + ": num_iteration_pass must be below 2^24");
        return LMGPU_ERR_INVALID;
    }
    if (sc->lights.count == 0) {
        set_error(std::string(name) + ": the scene has no area light");
        return LMGPU_ERR_INVALID;
    }
    if (sc->has_env) {
        set_error(std::string(name) + ": environment lights are not sampled by this renderer");
        return LMGPU_ERR_INVALID;
    }
    if (prm->mode != MODE_BDPT && prm->num_iteration_pass > 0) {
        // the smallest radius of the schedule, which the grid's cell indices
        // (exact integers in float, below 2^22 in magnitude) must resolve
        float r = prm->initial_radius;
        for (uint64_t k = 1; k < prm->num_iteration_pass; k++)
            r = sqrtf((prm->alpha + (float)k) / (1.0f + (float)k)) * r;
        float extent = sc->sphere_radius;
        for (int a = 0; a < 3; a++) extent += fabsf(sc->sphere_center[a]);
        if (!(r > 0.0f) || !(extent / r < 4194304.0f)) {
            set_error(std::string(name) + ": the merge radius schedule (initial_radius, alpha) falls to " +
                      std::to_string(r) + ", too small for the scene's extent");
            return LMGPU_ERR_INVALID;
        }
    }
    int rc = render_vcm(sc, prm, d_image, d_variance, s);
    if (rc) return rc;
    uint32_t st = 0;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(&st, sc->accel->status, sizeof(st), cudaMemcpyDeviceToHost, s));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(s));
    if (st & (kStatusBadTree | kStatusStackOverflow)) {
        set_error(std::string(name) + ": traversal status " + std::to_string(st));
        return LMGPU_ERR_OVERFLOW;
    }
    return LMGPU_OK;
}

}  // namespace
}  // namespace lmgpu

extern "C" {

int lmgpu_render_vcm_device(lmgpu_scene* sc, const lmgpu_vcm_params* prm, float* d_image, float* d_variance,
                            void* stream)
{
    lmgpu::clear_error();
    cudaStream_t s = stream ? (cudaStream_t)stream : (sc ? sc->stream : nullptr);
    return lmgpu::render_vcm_checked("lmgpu_render_vcm_device", sc, prm, d_image, d_variance, s);
}

int lmgpu_render_vcm(lmgpu_scene* sc, const lmgpu_vcm_params* prm, float* image, float* variance)
{
    lmgpu::clear_error();
    if (!sc || !prm || !image) {
        lmgpu::set_error("lmgpu_render_vcm: NULL argument");
        return LMGPU_ERR_INVALID;
    }
    const uint64_t npix = (uint64_t)sc->cam.width * sc->cam.height;
    int rc = lmgpu::ensure_film(sc, npix);
    if (rc) return rc;
    rc = lmgpu::render_vcm_checked("lmgpu_render_vcm", sc, prm, sc->d_image, variance ? sc->d_variance : nullptr,
                                   sc->stream);
    if (rc) return rc;
    LMGPU_CUDA_TRY(cudaMemcpyAsync(image, sc->d_image, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost, sc->stream));
    if (variance)
        LMGPU_CUDA_TRY(cudaMemcpyAsync(variance, sc->d_variance, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost,
                                       sc->stream));
    LMGPU_CUDA_TRY(cudaStreamSynchronize(sc->stream));
    return LMGPU_OK;
}

}  // extern "C"
