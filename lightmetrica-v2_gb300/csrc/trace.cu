// Ray traversal of the 8-wide compressed BVH (sm_103a).
//
// Replaces the per-ray Accel3::Intersect of the reference
// (include/lightmetrica/accel3.h:68; e.g. accel_bvh_sahbin.cpp:234-288,
// accel_qbvh.cpp:398-497) with a batch kernel, one thread per ray:
//
//   * node groups (child base index + 8-bit hit mask + the node's inner mask)
//     and triangle groups (triangle base + hit mask + the node's leaf mask)
//     live in a short per-thread stack; the next child is the highest set hit
//     bit, and hit bits of inner children are permuted by the ray octant so
//     that this visits children roughly front to back (the build stores
//     children in octant slots);
//   * each 80-byte node is fetched as five 16-byte read-only loads, and all
//     eight child boxes are tested with one FMA per slab
//     (t = q * (2^e / d) + (p - o) / d), two children per packed FP32 pair
//     instruction;
//   * triangles are 48-byte records, tested with the watertight algorithm of
//     Woop, Benthin and Wald (JCGT 2013): shear to ray space, edge functions
//     with unfused products (so shared edges give exactly negated values),
//     FP64 recomputation when an edge function is exactly zero;
//   * ties at equal t resolve to the higher global triangle id, the outcome
//     of accel::naive's ascending scan with "t > maxT" rejection
//     (triaccel.h:137, accel_naive.cpp:99-110).
#include "traverse.cuh"

namespace lmgpu {
namespace {

// One 1024-thread block per SM (64 registers a thread, the whole register
// file): the SM's 32 warps share one ray counter, so they stay busy until the
// SM's last rays (eight 128-thread blocks with fixed ranges left SMs idling
// as their blocks ran dry: 1,540 against 1,667 Mrays/s on the ray-cast
// benchmark).
constexpr int kTraceThreads = 1024;
// Resident blocks per SM the kernel is compiled for.
constexpr int kTraceBlocksPerSM = 1;

// Persistent traversal.  Each block owns the chunks blockIdx, blockIdx +
// grid, ... of 256 consecutive rays and its warps take rays from them
// through a shared-memory counter over the block's local index, so no global
// state outlives a launch and concurrent launches on other streams are
// independent.  The interleaving gives every block a mix of the whole range:
// renderers queue rays in an order where cost varies along the queue (the
// bidirectional tracer's connection rays are bucketed by strategy), and
// contiguous ranges left some blocks with far more work than others.
//
// Per warp, every iteration of the main loop:
//   1. refill: when at least `refill` lanes are idle, they take new rays
//      together (one shared atomic per warp);
//   2. node step: a lane with no pending triangles visits one node (or pops
//      a group from its stack, or finishes its ray);
//   3. triangle steps: lanes with pending triangles test them one at a time
//      while at least `postpone` lanes of the warp have triangle work; when
//      fewer do, lanes that also have node work push their triangles back on
//      the stack and go on traversing (after Aila & Laine 2009 and Ylitie,
//      Karras & Laine 2017), so the warp keeps doing one kind of work at once.
//
// MULTI: rays of several scenes in one launch; ray i is traced against the
// BVH tab[ray_scene[i]] (the batch renderer's views).  d_n, when not null,
// holds the ray count on the device (launches captured in CUDA graphs).
// SMALL: the same kernel as a separate function whose shared-memory
// carveout is the smallest that holds its resident blocks (the largest L1 at
// full occupancy), launched for BVHs that fit in L1.
template <bool ANYHIT, bool STATS, bool MULTI, bool SMALL = false>
__global__ void __launch_bounds__(kTraceThreads, kTraceBlocksPerSM) k_trace(const WNode* __restrict__ nodes, const WTri* __restrict__ tris,
                                                         const float4* __restrict__ rays, lmgpu_hit* __restrict__ hits,
                                                         uint64_t n, uint32_t num_nodes, uint32_t num_tris,
                                                         int refill, int postpone, uint32_t* __restrict__ status,
                                                         unsigned long long* __restrict__ counters,
                                                         const AccelView* __restrict__ tab, uint32_t ntab,
                                                         const uint8_t* __restrict__ ray_scene,
                                                         const uint32_t* __restrict__ d_n)
{
    __shared__ unsigned long long s_next;
    // inner-child hit masks permuted by octant (bit s -> bit s ^ o) for all 8
    // octants and 256 masks: one shared-memory load per node instead of the
    // three masked swaps (the ALU pipe is the busiest)
    __shared__ uint8_t s_perm[8 * 256];
    for (uint32_t i = threadIdx.x; i < 8u * 256u; i += blockDim.x) s_perm[i] = (uint8_t)permute_octant(i & 255u, i >> 8);
    if (d_n) n = *d_n;
    // the block's rays: chunks blockIdx.x, + gridDim.x, ... of kChunkRays
    // consecutive rays, counted by a local index (chunk k of the block, ray
    // o of the chunk) so that every block sees a mix of the whole range
    constexpr uint64_t kChunkRays = 256;
    const uint64_t nchunks = (n + kChunkRays - 1) / kChunkRays;
    const uint64_t my_chunks = blockIdx.x < nchunks ? (nchunks - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
    const uint64_t begin = 0, end = my_chunks * kChunkRays;
    if (threadIdx.x == 0) s_next = begin;
    __syncthreads();
    const unsigned FULL = 0xffffffffu;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned lt_mask = (1u << lane) - 1u;

    bool active = false, exhausted = false;
    uint64_t rid = 0;
    RayState R;
    float best_t = 0.0f, best_b1 = 0.0f, best_b2 = 0.0f;
    int best_id = -1;
    uint2 ng = make_uint2(0u, 0u), tg = make_uint2(0u, 0u);
    uint2 stack[kStack];
    int sp = 0;
    uint32_t budget = 0;
    uint32_t node_fetch = 0, tri_fetch = 0, nrays = 0, nhits = 0;
    // the BVH of the lane's current ray
    const WNode* lnodes = nodes;
    const WTri* ltris = tris;
    uint32_t lnn = num_nodes, lnt = num_tris;

    while (true) {
        // 1. refill idle lanes
        const unsigned idle = __ballot_sync(FULL, !active);
        if (!exhausted && __popc(idle) >= refill) {
            const unsigned leader = __ffs(idle) - 1u;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&s_next, (unsigned long long)__popc(idle));
            base = __shfl_sync(FULL, base, leader);
            if (base + __popc(idle) >= end) exhausted = true;
            if (!active) {
                const uint64_t li = base + __popc(idle & lt_mask);
                const uint64_t id = ((li / kChunkRays) * gridDim.x + blockIdx.x) * kChunkRays + li % kChunkRays;
                if (li < end && id < n) {
                    rid = id;
                    // rays and hits stream through once: cache-streaming
                    // accesses leave L1 / L2 to the BVH
                    const float4 r0 = __ldcs(rays + 2 * id);
                    const float4 r1 = __ldcs(rays + 2 * id + 1);
                    if (MULTI) {
                        const uint32_t sidx = ray_scene[id];
                        if (sidx < ntab) {
                            const AccelView av = tab[sidx];
                            lnodes = av.nodes;
                            ltris = av.tris;
                            lnn = av.num_nodes;
                            lnt = av.num_tris;
                        } else {
                            atomicOr(status, kStatusBadTree);
                            lnn = 0;
                            lnt = 0;
                        }
                    }
                    setup_ray(r0, r1, R);
                    best_t = r1.w;
                    best_id = -1;
                    best_b1 = best_b2 = 0.0f;
                    ng = make_uint2(0u, lnn > 0 ? 0x80000000u : 0u);
                    tg = make_uint2(0u, 0u);
                    sp = 0;
                    budget = lnn + 1;
                    active = true;
                    if (STATS) nrays++;
                }
            }
        }
        if (!__any_sync(FULL, active)) break;

        // 2. node step
        if (active && (tg.y & 0xffu) == 0u) {
            if (ng.y & 0xff000000u) {
                const uint32_t bit = 31u - __clz(ng.y & 0xff000000u);
                ng.y &= ~(1u << bit);
                const uint32_t slot = (bit - 24u) ^ R.oct_inv;
                const uint32_t rel = __popc(ng.y & 0xffu & ((1u << slot) - 1u));
                const uint32_t ni = ng.x + rel;
                if (ni >= lnn || budget-- == 0u) {
                    atomicOr(status, kStatusBadTree);
                    ng.y = 0u;
                    sp = 0;
                } else {
                    if (ng.y & 0xff000000u) {
                        if (sp < kStack) stack[sp++] = ng;
                        else atomicOr(status, kStatusStackOverflow);
                    }
                    uint32_t child_base, tri_base, imask, lmask;
                    const uint32_t h8 = intersect_node(lnodes, ni, R, best_t, child_base, tri_base, imask, lmask);
                    if (STATS) node_fetch++;
                    ng = make_uint2(child_base, ((uint32_t)s_perm[(R.oct_inv << 8) | (h8 & imask)] << 24) | imask);
                    tg = make_uint2(tri_base, (h8 & lmask) | (lmask << 8));
                }
            } else if (sp > 0) {
                const uint2 g = stack[--sp];
                if (g.y & 0xff000000u) ng = g;
                else tg = g;
            } else {
                lmgpu_hit h;
                h.t = best_id >= 0 ? best_t : 0.0f;
                h.prim = best_id;
                h.b1 = best_b1;
                h.b2 = best_b2;
                __stcs(reinterpret_cast<float4*>(hits) + rid, *reinterpret_cast<const float4*>(&h));
                if (STATS && best_id >= 0) nhits++;
                active = false;
            }
        }

        // 3. triangle steps
        while (true) {
            const bool has = active && (tg.y & 0xffu) != 0u;
            const unsigned m = __ballot_sync(FULL, has);
            if (m == 0u) break;
            const bool few = __popc(m) < postpone;
            if (few && has && (ng.y & 0xff000000u) && sp < kStack) {
                stack[sp++] = tg;
                tg.y = 0u;
            }
            if (active && (tg.y & 0xffu) != 0u) {
                const uint32_t slot = __ffs(tg.y) - 1u;
                tg.y &= tg.y - 1u;
                const uint32_t k = __popc((tg.y >> 8) & ((1u << slot) - 1u));
                if (tg.x + k >= lnt) {
                    atomicOr(status, kStatusBadTree);
                    tg.y = 0u;
                } else {
                    float t, b1, b2;
                    int id;
                    if (STATS) tri_fetch++;
                    if (intersect_tri(ltris, tg.x + k, R, best_t, t, b1, b2, id)) {
                        if (t < best_t || id > best_id) {
                            best_t = t;
                            best_id = id;
                            best_b1 = b1;
                            best_b2 = b2;
                        }
                        if (ANYHIT) {
                            tg.y = 0u;
                            ng.y = 0u;
                            sp = 0;
                        }
                    }
                }
            }
            if (few) break;
        }
    }
    if (STATS) {
        unsigned long long v[4] = {nrays, node_fetch, tri_fetch, nhits};
        for (int q = 0; q < 4; q++) {
            unsigned long long x = v[q];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(FULL, x, o);
            if (lane == 0) atomicAdd(&counters[q], x);
        }
    }
}

}  // namespace

namespace {

// Blocks of the persistent grid of one instantiation (SMs x resident blocks),
// looked up once per process.
template <bool ANYHIT, bool STATS, bool MULTI, bool SMALL = false>
int grid_cap_of()
{
    static int cap = 0;
    if (cap == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        LMGPU_CUDA_TRY(cudaGetDevice(&dev));
        LMGPU_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (SMALL) {
            // The smallest carveout that still holds kTraceBlocksPerSM blocks
            // (static shared memory plus the per-block reservation): the
            // carveout is honoured even where it costs occupancy (with
            // eight 128-thread blocks, the 2 KB mask table did not fit them
            // in the minimum one).
            cudaFuncAttributes fa{};
            int smem_sm = 0, reserved = 0;
            LMGPU_CUDA_TRY(cudaFuncGetAttributes(&fa, k_trace<ANYHIT, STATS, MULTI, SMALL>));
            LMGPU_CUDA_TRY(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
            LMGPU_CUDA_TRY(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev));
            const long need = (long)kTraceBlocksPerSM * ((long)fa.sharedSizeBytes + reserved);
            const int pct = smem_sm > 0 ? (int)((need * 100 + smem_sm - 1) / smem_sm) : 100;
            LMGPU_CUDA_TRY(cudaFuncSetAttribute(k_trace<ANYHIT, STATS, MULTI, SMALL>,
                                                cudaFuncAttributePreferredSharedMemoryCarveout, pct < 100 ? pct : 100));
        }
        LMGPU_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace<ANYHIT, STATS, MULTI, SMALL>,
                                                                     kTraceThreads, 0));
        if (SMALL && per_sm < kTraceBlocksPerSM) {
            // a carveout that cost occupancy after all: back to the default
            LMGPU_CUDA_TRY(cudaFuncSetAttribute(k_trace<ANYHIT, STATS, MULTI, SMALL>,
                                                cudaFuncAttributePreferredSharedMemoryCarveout,
                                                (int)cudaSharedmemCarveoutDefault));
            LMGPU_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace<ANYHIT, STATS, MULTI, SMALL>,
                                                                         kTraceThreads, 0));
        }
        cap = sms * (per_sm > 0 ? per_sm : 1);
    }
    return cap;
}

}  // namespace

int trace_grid_cap()
{
    const int caps[] = {grid_cap_of<false, false, false>(), grid_cap_of<true, false, false>(),
                        grid_cap_of<false, true, false>(),  grid_cap_of<true, true, false>(),
                        grid_cap_of<false, false, true>(),  grid_cap_of<true, false, true>()};
    int m = caps[0];
    for (int c : caps) m = c < m ? c : m;
    return m;
}

int launch_trace(const lmgpu_accel* a, const float4* d_rays, lmgpu_hit* d_hits, uint64_t n, bool anyhit, bool stats,
                 cudaStream_t stream, TraceProbe* probe)
{
    if (n == 0) return LMGPU_OK;
    if (probe && probe->mode != TraceProbe::kOff) probe->launches++;
    // a counting probe takes the counting instantiation with its counters
    unsigned long long* cnt = a->counters;
    if (probe && probe->mode == TraceProbe::kProbeCount) {
        stats = true;
        cnt = probe->d_counters;
    }
    const bool timed = probe && probe->mode == TraceProbe::kProbeTime && probe->used + 2 <= probe->events.size();
    if (probe && probe->mode == TraceProbe::kProbeTime && !timed) probe->overflow = true;
    if (timed) LMGPU_CUDA_TRY(cudaEventRecord(probe->events[probe->used], stream));
    const int grid_cap = anyhit ? (stats ? grid_cap_of<true, true, false>() : grid_cap_of<true, false, false>())
                                : (stats ? grid_cap_of<false, true, false>() : grid_cap_of<false, false, false>());
    if (grid_cap <= 0) return LMGPU_ERR_CUDA;
    const TraceConfig cfg = a->tune;
    // at least ~4 warps' worth of rays per block
    const uint64_t by_rays = (n + 4 * kTraceThreads - 1) / (4 * kTraceThreads);
    const unsigned grid = (unsigned)(by_rays < (uint64_t)grid_cap ? by_rays : (uint64_t)grid_cap);
    const uint32_t nn = a->ntri > 0 ? (uint32_t)a->num_wide : 0u;
    const uint32_t nt = (uint32_t)a->ntri;
    auto k = anyhit ? (stats ? k_trace<true, true, false> : k_trace<true, false, false>)
                    : (stats ? k_trace<false, true, false> : k_trace<false, false, false>);
    k<<<grid, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, n, nn, nt, cfg.refill, cfg.postpone,
                                          a->status, cnt, nullptr, 0u, nullptr, nullptr);
    LMGPU_CUDA_TRY(cudaGetLastError());
    if (timed) {
        LMGPU_CUDA_TRY(cudaEventRecord(probe->events[probe->used + 1], stream));
        probe->used += 2;
    }
    return LMGPU_OK;
}

int launch_trace_dn(const lmgpu_accel* a, const float4* d_rays, lmgpu_hit* d_hits, const uint32_t* d_n,
                    uint64_t max_n, bool anyhit, cudaStream_t stream, TraceProbe* probe)
{
    if (max_n == 0) return LMGPU_OK;
    if (probe && probe->mode != TraceProbe::kOff) probe->launches++;
    if (probe && probe->mode == TraceProbe::kProbeCount) {
        // the counting instantiation: the same hits, plus fetch counters
        const int cap = anyhit ? grid_cap_of<true, true, false>() : grid_cap_of<false, true, false>();
        if (cap <= 0) return LMGPU_ERR_CUDA;
        const uint64_t by_rays = (max_n + 4 * kTraceThreads - 1) / (4 * kTraceThreads);
        const unsigned grid = (unsigned)(by_rays < (uint64_t)cap ? by_rays : (uint64_t)cap);
        auto k = anyhit ? k_trace<true, true, false> : k_trace<false, true, false>;
        k<<<grid, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, max_n,
                                              a->ntri > 0 ? (uint32_t)a->num_wide : 0u, (uint32_t)a->ntri,
                                              a->tune.refill, a->tune.postpone, a->status, probe->d_counters,
                                              nullptr, 0u, nullptr, d_n);
        LMGPU_CUDA_TRY(cudaGetLastError());
        return LMGPU_OK;
    }
    const bool timed = probe && probe->mode == TraceProbe::kProbeTime && probe->used + 2 <= probe->events.size();
    if (probe && probe->mode == TraceProbe::kProbeTime && !timed) probe->overflow = true;
    if (timed) LMGPU_CUDA_TRY(cudaEventRecord(probe->events[probe->used], stream));
    // closest hit in a BVH that fits in L1 (nodes and triangles within 96 KiB)
    // runs the SMALL instantiation: the smallest shared-memory carveout that
    // holds its blocks, i.e. the largest L1 (measured +4 % on a 36-triangle
    // scene and -6 % on the 1.5M-triangle ray-cast scene)
    const bool small = !anyhit && (uint64_t)a->num_wide * sizeof(WNode) + a->ntri * sizeof(WTri) <= (96u << 10);
    const int grid_cap = small ? grid_cap_of<false, false, false, true>()
                               : (anyhit ? grid_cap_of<true, false, false>() : grid_cap_of<false, false, false>());
    if (grid_cap <= 0) return LMGPU_ERR_CUDA;
    const uint64_t by_rays = (max_n + 4 * kTraceThreads - 1) / (4 * kTraceThreads);
    const unsigned grid = (unsigned)(by_rays < (uint64_t)grid_cap ? by_rays : (uint64_t)grid_cap);
    const uint32_t nn = a->ntri > 0 ? (uint32_t)a->num_wide : 0u;
    const uint32_t nt = (uint32_t)a->ntri;
    auto k = small ? k_trace<false, false, false, true> : (anyhit ? k_trace<true, false, false> : k_trace<false, false, false>);
    k<<<grid, kTraceThreads, 0, stream>>>(a->nodes, a->tris, d_rays, d_hits, max_n, nn, nt, a->tune.refill,
                                          a->tune.postpone, a->status, nullptr, nullptr, 0u, nullptr, d_n);
    LMGPU_CUDA_TRY(cudaGetLastError());
    if (timed) {
        LMGPU_CUDA_TRY(cudaEventRecord(probe->events[probe->used + 1], stream));
        probe->used += 2;
    }
    return LMGPU_OK;
}

int launch_trace_multi(const AccelView* d_tab, uint32_t ntab, const float4* d_rays, const uint8_t* d_ray_scene,
                       lmgpu_hit* d_hits, const uint32_t* d_n, uint64_t max_n, bool anyhit, TraceConfig cfg,
                       uint32_t* d_status, cudaStream_t stream, TraceProbe* probe)
{
    if (max_n == 0) return LMGPU_OK;
    if (probe && probe->mode != TraceProbe::kOff) probe->launches++;
    const bool count = probe && probe->mode == TraceProbe::kProbeCount;
    const bool timed = probe && probe->mode == TraceProbe::kProbeTime && probe->used + 2 <= probe->events.size();
    if (probe && probe->mode == TraceProbe::kProbeTime && !timed) probe->overflow = true;
    if (timed) LMGPU_CUDA_TRY(cudaEventRecord(probe->events[probe->used], stream));
    const int grid_cap = count ? (anyhit ? grid_cap_of<true, true, true>() : grid_cap_of<false, true, true>())
                               : (anyhit ? grid_cap_of<true, false, true>() : grid_cap_of<false, false, true>());
    if (grid_cap <= 0) return LMGPU_ERR_CUDA;
    // the ray count is read on the device: the full persistent grid, each
    // block taking its share of whatever count the launch finds
    auto k = count ? (anyhit ? k_trace<true, true, true> : k_trace<false, true, true>)
                   : (anyhit ? k_trace<true, false, true> : k_trace<false, false, true>);
    k<<<(unsigned)grid_cap, kTraceThreads, 0, stream>>>(nullptr, nullptr, d_rays, d_hits, max_n, 0u, 0u, cfg.refill,
                                                         cfg.postpone, d_status, count ? probe->d_counters : nullptr,
                                                         d_tab, ntab, d_ray_scene, d_n);
    LMGPU_CUDA_TRY(cudaGetLastError());
    if (timed) {
        LMGPU_CUDA_TRY(cudaEventRecord(probe->events[probe->used + 1], stream));
        probe->used += 2;
    }
    return LMGPU_OK;
}

}  // namespace lmgpu
