/*
 * CPU oracle: TriAccel triangle test, accel::naive and accel::bvh_sahbin.
 *
 * TEST INFRASTRUCTURE ONLY (see lmoracle.h).  Restates, in C:
 *   TriAccelTriangle::Load / Intersect   include/lightmetrica/triaccel.h:50-151
 *   Bound::Intersect / SurfaceArea / ... include/lightmetrica/bound.h:39-91
 *   Accel_Naive::Build / Intersect       src/liblightmetrica/accel/accel_naive.cpp:59-124
 *   Accel_BVHSAHBin::Build / Intersect   src/liblightmetrica/accel/accel_bvh_sahbin.cpp:70-288
 *   Accel_QBVH::Build / Intersect        src/liblightmetrica/accel/accel_qbvh.cpp:152-497
 * in single precision with the reference's operation order.  Must be built
 * with -ffp-contract=off.
 */
#include "lmoracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define LMO_FLT_INF FLT_MAX /* Math::Inf() is numeric_limits<float>::max() (math.h:1663) */
#define LMO_EPS 1e-4f       /* Math::Eps<float>() (math.h:1666) */

static inline float fmin_std(float a, float b) { return (b < a) ? b : a; } /* std::min */
static inline float fmax_std(float a, float b) { return (a < b) ? b : a; } /* std::max */

/* Math::Dot for SSE Vec3 (math.h:1728-1731): _mm_dp_ps(...,0x71) sums as (x+y)+z. */
static inline float dot3(const float a[3], const float b[3])
{
    float xy = a[0] * b[0] + a[1] * b[1];
    return xy + a[2] * b[2];
}

/* Math::Cross (math.h:1784-1803). */
static inline void cross3(const float a[3], const float b[3], float r[3])
{
    r[0] = a[1] * b[2] - b[1] * a[2];
    r[1] = a[2] * b[0] - b[2] * a[0];
    r[2] = a[0] * b[1] - b[0] * a[1];
}

/* triaccel.h:50-91 */
int lmo_triaccel_load(lmo_triaccel* T, const float A[3], const float B[3], const float C[3])
{
    static const int wald_modulo[4] = {1, 2, 0, 1};
    float b[3], c[3], N[3];
    for (int i = 0; i < 3; i++) { b[i] = C[i] - A[i]; c[i] = B[i] - A[i]; }
    cross3(c, b, N);
    T->k = 0;
    for (int j = 0; j < 3; j++)
        if (fabsf(N[j]) > fabsf(N[T->k])) T->k = (uint32_t)j;
    uint32_t u = (uint32_t)wald_modulo[T->k];
    uint32_t v = (uint32_t)wald_modulo[T->k + 1];
    const float n_k = N[T->k];
    const float denom = b[u] * c[v] - b[v] * c[u];
    if (denom == 0) { T->k = 3; return 1; }
    T->n_u = N[u] / n_k;
    T->n_v = N[v] / n_k;
    T->n_d = dot3(A, N) / n_k;
    T->b_nu = b[u] / denom;
    T->b_nv = -b[v] / denom;
    T->a_u = A[u];
    T->a_v = A[v];
    T->c_nu = c[v] / denom;
    T->c_nv = -c[u] / denom;
    return 0;
}

/* triaccel.h:93-151 */
int lmo_triaccel_intersect(const lmo_triaccel* T, const float o[3], const float d[3],
                           float mint, float maxt, float* u, float* v, float* t)
{
    float o_u, o_v, o_k, d_u, d_v, d_k;
    switch (T->k) {
    case 0: o_u = o[1]; o_v = o[2]; o_k = o[0]; d_u = d[1]; d_v = d[2]; d_k = d[0]; break;
    case 1: o_u = o[2]; o_v = o[0]; o_k = o[1]; d_u = d[2]; d_v = d[0]; d_k = d[1]; break;
    case 2: o_u = o[0]; o_v = o[1]; o_k = o[2]; d_u = d[0]; d_v = d[1]; d_k = d[2]; break;
    default: return 0;
    }
    const float demon = (d_u * T->n_u + d_v * T->n_v) + d_k;
    if (demon == 0) return 0;
    *t = (((T->n_d - o_u * T->n_u) - o_v * T->n_v) - o_k) / demon;
    if (*t < mint || *t > maxt) return 0;
    const float hu = (o_u + *t * d_u) - T->a_u;
    const float hv = (o_v + *t * d_v) - T->a_v;
    *u = hv * T->b_nu + hu * T->b_nv;
    *v = hu * T->c_nu + hv * T->c_nv;
    return *u >= 0.0f && *v >= 0.0f && *u + *v <= 1.0f;
}

/* ------------------------------------------------------------------------- */

typedef struct { float mn[3], mx[3]; } lmo_bound;

static inline void bound_empty(lmo_bound* b)
{
    for (int i = 0; i < 3; i++) { b->mn[i] = LMO_FLT_INF; b->mx[i] = -LMO_FLT_INF; }
}
static inline void bound_union_b(lmo_bound* r, const lmo_bound* b)
{
    for (int i = 0; i < 3; i++) { r->mn[i] = fmin_std(r->mn[i], b->mn[i]); r->mx[i] = fmax_std(r->mx[i], b->mx[i]); }
}
static inline void bound_union_p(lmo_bound* r, const float p[3])
{
    for (int i = 0; i < 3; i++) { r->mn[i] = fmin_std(r->mn[i], p[i]); r->mx[i] = fmax_std(r->mx[i], p[i]); }
}
/* bound.h:49-53 */
static inline int bound_longest_axis(const lmo_bound* b)
{
    float d[3];
    for (int i = 0; i < 3; i++) d[i] = b->mx[i] - b->mn[i];
    return d[0] > d[1] && d[0] > d[2] ? 0 : d[1] > d[2] ? 1 : 2;
}
/* bound.h:55-59 */
static inline float bound_area(const lmo_bound* b)
{
    float d[3];
    for (int i = 0; i < 3; i++) d[i] = b->mx[i] - b->mn[i];
    return 2.0f * ((d[0] * d[1] + d[1] * d[2]) + d[2] * d[0]);
}
/* bound.h:61-64 */
static inline float bound_centroid(const lmo_bound* b, int axis)
{
    return (b->mn[axis] + b->mx[axis]) * 0.5f;
}
/* bound.h:66-91 */
static inline int bound_intersect(const lmo_bound* b, const float o[3], const float d[3], float tMin, float tMax)
{
    const float* lo = b->mn;
    const float* hi = b->mx;
    float tmin, tmax;
    const int n0 = d[0] < 0.0f, n1 = d[1] < 0.0f, n2 = d[2] < 0.0f;
    const float txmax = ((n0 ? lo : hi)[0] - o[0]) * (d[0] == 0 ? LMO_FLT_INF : 1.0f / d[0]);
    const float txmin = ((n0 ? hi : lo)[0] - o[0]) * (d[0] == 0 ? 0.0f : 1.0f / d[0]);
    tmin = txmin; tmax = txmax;
    const float tymax = ((n1 ? lo : hi)[1] - o[1]) * (d[1] == 0 ? LMO_FLT_INF : 1.0f / d[1]);
    const float tymin = ((n1 ? hi : lo)[1] - o[1]) * (d[1] == 0 ? 0.0f : 1.0f / d[1]);
    if ((tmin > tymax) || (tymin > tmax)) return 0;
    if (tymin > tmin) tmin = tymin;
    if (tymax < tmax) tmax = tymax;
    const float tzmax = ((n2 ? lo : hi)[2] - o[2]) * (d[2] == 0 ? LMO_FLT_INF : 1.0f / d[2]);
    const float tzmin = ((n2 ? hi : lo)[2] - o[2]) * (d[2] == 0 ? 0.0f : 1.0f / d[2]);
    if ((tmin > tzmax) || (tzmin > tmax)) return 0;
    if (tzmin > tmin) tmin = tzmin;
    if (tzmax < tmax) tmax = tzmax;
    return (tmin < tMax) && (tmax > tMin);
}

/* ------------------------------------------------------------------------- */

typedef struct {
    lmo_bound bound;
    int isleaf;
    int a, b; /* leaf: begin, end ; internal: child1, child2 */
} lmo_node;

/* 4-wide node of accel::qbvh (accel_qbvh.cpp:56-128): child bounds in
 * structure-of-arrays form, bmin/bmax[axis][child]; children[c] is a node
 * index (>= 0), a leaf (bit 31 set, bits 30:27 = size - 1, bits 26:0 = first
 * index into `indices`) or QBVH_EMPTY. */
typedef struct {
    float b[2][3][4];
    int children[4];
} lmo_qnode;

#define QBVH_EMPTY ((int)0xffffffff)

struct lmo_accel {
    int kind;
    size_t ntri;
    lmo_triaccel* tris;
    /* bvh_sahbin and qbvh */
    lmo_bound* bounds;
    int* indices;
    lmo_node* nodes;
    size_t nnodes, cap;
    int depth;
    /* qbvh */
    lmo_qnode* qnodes;
    size_t nq, qcap;
};

#define NUM_BINS 100
#define LEAF_NUM 10

static int push_node(lmo_accel* A)
{
    if (A->nnodes == A->cap) {
        A->cap = A->cap ? A->cap * 2 : 1024;
        A->nodes = (lmo_node*)realloc(A->nodes, A->cap * sizeof(lmo_node));
    }
    return (int)(A->nnodes++);
}

static inline int bin_of(float c, float mn, float mx)
{
    /* std::min((int)((c - min) / (max - min) * NumBins), NumBins - 1) */
    float f = (c - mn) / (mx - mn) * (float)NUM_BINS;
    int i = (int)f;
    return i < NUM_BINS - 1 ? i : NUM_BINS - 1;
}

/* accel_bvh_sahbin.cpp:120-220 (one call of the recursive Build_ lambda). */
static int build_rec(lmo_accel* A, int begin, int end, int depth)
{
    if (depth > A->depth) A->depth = depth;
    int idx = push_node(A);
    lmo_bound nb, cb;
    bound_empty(&nb);
    bound_empty(&cb);
    for (int i = begin; i < end; i++) {
        const lmo_bound* b = &A->bounds[A->indices[i]];
        bound_union_b(&nb, b);
        float c[3] = {bound_centroid(b, 0), bound_centroid(b, 1), bound_centroid(b, 2)};
        bound_union_p(&cb, c);
    }
    A->nodes[idx].bound = nb;
    if (end - begin < LEAF_NUM) {
        A->nodes[idx].isleaf = 1; A->nodes[idx].a = begin; A->nodes[idx].b = end;
        return idx;
    }
    const int axis = bound_longest_axis(&nb);
    const float mn = cb.mn[axis], mx = cb.mx[axis];
    if (!(mx > mn)) {
        /* All centroids coincide on the split axis: the reference divides
         * 0/0 there (undefined behaviour); the oracle makes a leaf. */
        A->nodes[idx].isleaf = 1; A->nodes[idx].a = begin; A->nodes[idx].b = end;
        return idx;
    }
    lmo_bound bins[NUM_BINS];
    int counts[NUM_BINS];
    for (int i = 0; i < NUM_BINS; i++) { bound_empty(&bins[i]); counts[i] = 0; }
    for (int i = begin; i < end; i++) {
        const lmo_bound* b = &A->bounds[A->indices[i]];
        int t = bin_of(bound_centroid(b, axis), mn, mx);
        bound_union_b(&bins[t], b);
        counts[t]++;
    }
    /* The reference re-unions bins 0..split and split+1..99 for every split
     * (accel_bvh_sahbin.cpp:164-191).  Unions are exact min/max, so prefix
     * and suffix sweeps give the same bounds, areas and costs bit for bit. */
    lmo_bound pre[NUM_BINS], suf[NUM_BINS];
    int npre[NUM_BINS], nsuf[NUM_BINS];
    {
        lmo_bound acc;
        int cnt = 0;
        bound_empty(&acc);
        for (int i = 0; i < NUM_BINS; i++) { bound_union_b(&acc, &bins[i]); cnt += counts[i]; pre[i] = acc; npre[i] = cnt; }
        bound_empty(&acc);
        cnt = 0;
        for (int i = NUM_BINS - 1; i >= 0; i--) { bound_union_b(&acc, &bins[i]); cnt += counts[i]; suf[i] = acc; nsuf[i] = cnt; }
    }
    float costs[NUM_BINS - 1];
    const float area = bound_area(&nb);
    for (int split = 0; split < NUM_BINS - 1; split++) {
        const lmo_bound b1 = pre[split], b2 = suf[split + 1];
        const int n1 = npre[split], n2 = nsuf[split + 1];
        const float Cb = 0.125f;
        const float C1 = n1 > 0 ? bound_area(&b1) * (float)n1 : 0.0f;
        const float C2 = n2 > 0 ? bound_area(&b2) * (float)n2 : 0.0f;
        costs[split] = Cb + (C1 + C2) / area;
    }
    int best = 0; /* std::min_element: first smallest */
    for (int s = 1; s < NUM_BINS - 1; s++)
        if (costs[s] < costs[best]) best = s;
    if (costs[best] > (float)(end - begin)) {
        A->nodes[idx].isleaf = 1; A->nodes[idx].a = begin; A->nodes[idx].b = end;
        return idx;
    }
    /* std::partition over bidirectional iterators (libstdc++ __partition):
     * the same swap sequence, so leaf order matches the reference. */
    int* first = A->indices + begin;
    int* last = A->indices + end;
    for (;;) {
        for (;;) {
            if (first == last) goto done;
            if (bin_of(bound_centroid(&A->bounds[*first], axis), mn, mx) <= best) ++first;
            else break;
        }
        --last;
        for (;;) {
            if (first == last) goto done;
            if (!(bin_of(bound_centroid(&A->bounds[*last], axis), mn, mx) <= best)) --last;
            else break;
        }
        { int tmp = *first; *first = *last; *last = tmp; }
        ++first;
    }
done:;
    const int mid = (int)(first - A->indices);
    A->nodes[idx].isleaf = 0;
    int c1 = build_rec(A, begin, mid, depth + 1);
    int c2 = build_rec(A, mid, end, depth + 1);
    A->nodes[idx].a = c1;
    A->nodes[idx].b = c2;
    return idx;
}

static int qbvh_push(lmo_accel* A);
static void qbvh_build_rec(lmo_accel* A, int begin, int end, int parent, int child, int depth);

lmo_accel* lmo_accel_build(int kind, const float* tris, size_t ntri)
{
    lmo_accel* A = (lmo_accel*)calloc(1, sizeof(lmo_accel));
    A->kind = kind;
    A->ntri = ntri;
    A->tris = (lmo_triaccel*)malloc(sizeof(lmo_triaccel) * (ntri ? ntri : 1));
    if (kind == 1 || kind == 2) {
        A->bounds = (lmo_bound*)malloc(sizeof(lmo_bound) * (ntri ? ntri : 1));
        A->indices = (int*)malloc(sizeof(int) * (ntri ? ntri : 1));
    }
    for (size_t i = 0; i < ntri; i++) {
        const float* p = tris + 9 * i;
        lmo_triaccel_load(&A->tris[i], p, p + 3, p + 6);
        A->tris[i].face_index = (uint32_t)i;
        A->tris[i].prim_index = 0;
        if (kind == 1 || kind == 2) {
            lmo_bound b;
            bound_empty(&b);
            bound_union_p(&b, p);
            bound_union_p(&b, p + 3);
            bound_union_p(&b, p + 6);
            for (int k = 0; k < 3; k++) { b.mn[k] -= LMO_EPS; b.mx[k] += LMO_EPS; }
            A->bounds[i] = b;
            A->indices[i] = (int)i;
        }
    }
    if (kind == 1 && ntri > 0) build_rec(A, 0, (int)ntri, 0);
    if (kind == 2) {
        qbvh_push(A);
        qbvh_build_rec(A, 0, (int)ntri, 0, 0, 0);
    }
    return A;
}

void lmo_accel_free(lmo_accel* A)
{
    if (!A) return;
    free(A->tris); free(A->bounds); free(A->indices); free(A->nodes); free(A->qnodes);
    free(A);
}

void lmo_accel_stats(const lmo_accel* A, size_t* nodes, size_t* leaves, int* depth)
{
    size_t nl = 0;
    if (A->kind == 2) {
        for (size_t i = 0; i < A->nq; i++)
            for (int c = 0; c < 4; c++) nl += (A->qnodes[i].children[c] < 0 && A->qnodes[i].children[c] != QBVH_EMPTY);
        if (nodes) *nodes = A->nq;
        if (leaves) *leaves = nl;
        if (depth) *depth = A->depth;
        return;
    }
    for (size_t i = 0; i < A->nnodes; i++) nl += A->nodes[i].isleaf ? 1 : 0;
    if (nodes) *nodes = A->nnodes;
    if (leaves) *leaves = nl;
    if (depth) *depth = A->depth;
}

static void finish_hit(lmo_hit* h, const float o[3], const float d[3], int id, float t, float b0, float b1)
{
    h->id = id;
    h->t = t;
    h->b0 = b0;
    h->b1 = b1;
    /* ray.o + ray.d * maxT (accel_naive.cpp:118) */
    for (int k = 0; k < 3; k++) h->p[k] = o[k] + d[k] * t;
}


/* ------------------------------------------------------------------------- */
/* accel::qbvh                                                                */

static int qbvh_push(lmo_accel* A)
{
    if (A->nq == A->qcap) {
        A->qcap = A->qcap ? A->qcap * 2 : 1024;
        A->qnodes = (lmo_qnode*)realloc(A->qnodes, A->qcap * sizeof(lmo_qnode));
    }
    lmo_qnode* q = &A->qnodes[A->nq];
    /* QBVHNode() (accel_qbvh.cpp:75-86): +inf / -inf bounds, empty children */
    for (int a = 0; a < 3; a++)
        for (int c = 0; c < 4; c++) { q->b[0][a][c] = INFINITY; q->b[1][a][c] = -INFINITY; }
    for (int c = 0; c < 4; c++) q->children[c] = QBVH_EMPTY;
    return (int)(A->nq++);
}

/* QBVHNode::SetBound (accel_qbvh.cpp:88-95) */
static void qbvh_set_bound(lmo_qnode* q, int c, const lmo_bound* b)
{
    for (int a = 0; a < 3; a++) { q->b[0][a][c] = b->mn[a]; q->b[1][a][c] = b->mx[a]; }
}

/* One call of the recursive Build_ lambda (accel_qbvh.cpp:200-373): binned
 * SAH over the longest axis of the centroid bound, leaves below 10
 * triangles, and two binary levels folded into one 4-wide node (even depths
 * open a node whose children 0 and 2 the two halves fill; odd depths fill
 * the parent's slots `child` and `child + 1`). */
static void qbvh_build_rec(lmo_accel* A, int begin, int end, int parent, int child, int depth)
{
    if (depth > A->depth) A->depth = depth;
    lmo_bound nb;
    bound_empty(&nb);
    for (int i = begin; i < end; i++) bound_union_b(&nb, &A->bounds[A->indices[i]]);
    if (end - begin < LEAF_NUM) {
        lmo_qnode* q = &A->qnodes[parent];
        qbvh_set_bound(q, child, &nb);
        /* QBVHNode::CreateLeaf (accel_qbvh.cpp:97-110) */
        const int size = end - begin;
        q->children[child] = size == 0 ? QBVH_EMPTY
                                       : (int)(0x80000000u | ((unsigned)((size - 1) & 0xf) << 27) |
                                               ((unsigned)begin & 0x07ffffffu));
        return;
    }
    lmo_bound cb;
    bound_empty(&cb);
    for (int i = begin; i < end; i++) {
        const lmo_bound* b = &A->bounds[A->indices[i]];
        float c[3] = {bound_centroid(b, 0), bound_centroid(b, 1), bound_centroid(b, 2)};
        bound_union_p(&cb, c);
    }
    const int axis = bound_longest_axis(&cb);
    const float mn = cb.mn[axis], mx = cb.mx[axis];
    int mid;
    if (!(mx > mn)) {
        /* Every centroid coincides: the reference divides 0 by 0 here and
         * indexes its bins with the converted NaN (undefined behaviour, a
         * crash on x86-64); the oracle halves the range in index order. */
        mid = begin + (end - begin) / 2;
    } else {
        lmo_bound bins[NUM_BINS];
        int counts[NUM_BINS];
        for (int i = 0; i < NUM_BINS; i++) { bound_empty(&bins[i]); counts[i] = 0; }
        for (int i = begin; i < end; i++) {
            const lmo_bound* b = &A->bounds[A->indices[i]];
            int t = bin_of(bound_centroid(b, axis), mn, mx);
            bound_union_b(&bins[t], b);
            counts[t]++;
        }
        /* prefix / suffix unions give the reference's per-split re-unions
         * (accel_qbvh.cpp:263-291) bit for bit: unions are exact min / max */
        lmo_bound pre[NUM_BINS], suf[NUM_BINS];
        int npre[NUM_BINS], nsuf[NUM_BINS];
        lmo_bound acc;
        int cnt = 0;
        bound_empty(&acc);
        for (int i = 0; i < NUM_BINS; i++) { bound_union_b(&acc, &bins[i]); cnt += counts[i]; pre[i] = acc; npre[i] = cnt; }
        bound_empty(&acc);
        cnt = 0;
        for (int i = NUM_BINS - 1; i >= 0; i--) { bound_union_b(&acc, &bins[i]); cnt += counts[i]; suf[i] = acc; nsuf[i] = cnt; }
        const float area = bound_area(&nb);
        int best = 0;
        float best_cost = 0.0f;
        for (int split = 0; split < NUM_BINS - 1; split++) {
            const int n1 = npre[split], n2 = nsuf[split + 1];
            const float C1 = n1 > 0 ? bound_area(&pre[split]) * (float)n1 : 0.0f;
            const float C2 = n2 > 0 ? bound_area(&suf[split + 1]) * (float)n2 : 0.0f;
            const float cost = 0.125f + (C1 + C2) / area;
            if (split == 0 || cost < best_cost) { best = split; best_cost = cost; } /* std::min_element */
        }
        /* std::partition (libstdc++'s bidirectional form): the same swaps */
        int* first = A->indices + begin;
        int* last = A->indices + end;
        for (;;) {
            for (;;) {
                if (first == last) goto done;
                if (bin_of(bound_centroid(&A->bounds[*first], axis), mn, mx) <= best) ++first;
                else break;
            }
            --last;
            for (;;) {
                if (first == last) goto done;
                if (!(bin_of(bound_centroid(&A->bounds[*last], axis), mn, mx) <= best)) --last;
                else break;
            }
            { int tmp = *first; *first = *last; *last = tmp; }
            ++first;
        }
done:
        mid = (int)(first - A->indices);
    }
    int current, c1, c2;
    if (depth % 2 == 1) {
        current = parent; c1 = child; c2 = child + 1;
    } else {
        current = qbvh_push(A);
        A->qnodes[parent].children[child] = current;   /* CreateIntermediateNode */
        qbvh_set_bound(&A->qnodes[parent], child, &nb);
        c1 = 0; c2 = 2;
    }
    qbvh_build_rec(A, begin, mid, current, c1, depth + 1);
    qbvh_build_rec(A, mid, end, current, c2, depth + 1);
}

/* Four-lane float vectors (SSE on x86-64, NEON on aarch64, by the compiler). */
typedef float lmo_v4f __attribute__((vector_size(16)));
typedef int lmo_v4i __attribute__((vector_size(16)));

/* _mm_max_ps / _mm_min_ps lane rule: a > b ? a : b and a < b ? a : b
 * (the second operand when either is NaN). */
static inline lmo_v4f v4_max(lmo_v4f a, lmo_v4f b)
{
    lmo_v4i m = a > b;
    return (lmo_v4f)(((lmo_v4i)a & m) | ((lmo_v4i)b & ~m));
}
static inline lmo_v4f v4_min(lmo_v4f a, lmo_v4f b)
{
    lmo_v4i m = a < b;
    return (lmo_v4f)(((lmo_v4i)a & m) | ((lmo_v4i)b & ~m));
}

/* QBVHNode::Intersect (accel_qbvh.cpp:117-128) and Accel_QBVH::Intersect
 * (accel_qbvh.cpp:398-497): iterative traversal with a stack of node words,
 * children pushed 0..3 as their slabs are hit (popped in reverse), maxT
 * narrowed by every accepted triangle, ties resolved by the last accepted. */
static void trace_qbvh(const lmo_accel* A, const float* r, lmo_hit* h)
{
    const float* o = r;
    const float* d = r + 4;
    float minT = r[3], maxT = r[7];
    int hit = 0, minIndex = 0;
    float mb0 = 0, mb1 = 0;
    lmo_v4f inv_min[3], inv_max[3], org[3];
    int sign[3];
    for (int k = 0; k < 3; k++) {
        const float im = d[k] == 0.0f ? 1e-3f /* Math::EpsLarge<float> */ : 1.0f / d[k];
        const float iM = d[k] == 0.0f ? LMO_FLT_INF : 1.0f / d[k];
        inv_min[k] = (lmo_v4f){im, im, im, im};
        inv_max[k] = (lmo_v4f){iM, iM, iM, iM};
        org[k] = (lmo_v4f){o[k], o[k], o[k], o[k]};
        sign[k] = d[k] < 0.0f;
    }
    int stack[128];
    int sp = 0;
    stack[0] = 0;
    while (sp >= 0) {
        const int data = stack[sp--];
        if (data < 0) {
            if (data == QBVH_EMPTY) continue;
            const unsigned size = (unsigned)(((data >> 27) & 0xf) + 1);
            const unsigned offset = (unsigned)data & 0x07ffffffu;
            for (unsigned i = offset; i < offset + size; i++) {
                float t, b0, b1;
                const int ti = A->indices[i];
                if (lmo_triaccel_intersect(&A->tris[ti], o, d, minT, maxT, &b0, &b1, &t)) {
                    hit = 1; maxT = t; minIndex = ti; mb0 = b0; mb1 = b1;
                }
            }
            continue;
        }
        const lmo_qnode* q = &A->qnodes[data];
        lmo_v4f vmin = (lmo_v4f){minT, minT, minT, minT};
        lmo_v4f vmax = (lmo_v4f){maxT, maxT, maxT, maxT};
        for (int k = 0; k < 3; k++) {
            lmo_v4f lo, hi;
            memcpy(&lo, q->b[sign[k]][k], 16);
            memcpy(&hi, q->b[1 - sign[k]][k], 16);
            vmin = v4_max(vmin, (lo - org[k]) * inv_min[k]);
            vmax = v4_min(vmax, (hi - org[k]) * inv_max[k]);
        }
        lmo_v4i m = vmax >= vmin;
        if (m[0]) stack[++sp] = q->children[0];
        if (m[1]) stack[++sp] = q->children[1];
        if (m[2]) stack[++sp] = q->children[2];
        if (m[3]) stack[++sp] = q->children[3];
    }
    if (!hit) { memset(h, 0, sizeof(*h)); h->id = -1; return; }
    finish_hit(h, o, d, minIndex, maxT, mb0, mb1);
}

/* accel_naive.cpp:92-124 */
static void trace_naive(const lmo_accel* A, const float* r, lmo_hit* h)
{
    const float* o = r;
    const float* d = r + 4;
    float minT = r[3], maxT = r[7];
    int hit = 0;
    size_t minIndex = 0;
    float mb0 = 0, mb1 = 0;
    for (size_t i = 0; i < A->ntri; i++) {
        float t, b0, b1;
        if (lmo_triaccel_intersect(&A->tris[i], o, d, minT, maxT, &b0, &b1, &t)) {
            hit = 1; maxT = t; minIndex = i; mb0 = b0; mb1 = b1;
        }
    }
    if (!hit) { memset(h, 0, sizeof(*h)); h->id = -1; return; }
    finish_hit(h, o, d, (int)minIndex, maxT, mb0, mb1);
}

/* accel_bvh_sahbin.cpp:234-288: depth-first, child1 before child2, maxT
 * narrowed by every accepted hit, ties resolved by the last accepted. */
static void trace_bvh(const lmo_accel* A, const float* r, lmo_hit* h)
{
    const float* o = r;
    const float* d = r + 4;
    float minT = r[3], maxT = r[7];
    int hit = 0, minIndex = 0;
    float mb0 = 0, mb1 = 0;
    int stack[256];
    int sp = 0;
    if (A->nnodes > 0) stack[sp++] = 0;
    while (sp > 0) {
        const lmo_node* node = &A->nodes[stack[--sp]];
        if (!bound_intersect(&node->bound, o, d, minT, maxT)) continue;
        if (node->isleaf) {
            for (int i = node->a; i < node->b; i++) {
                float t, b0, b1;
                int ti = A->indices[i];
                if (lmo_triaccel_intersect(&A->tris[ti], o, d, minT, maxT, &b0, &b1, &t)) {
                    hit = 1; maxT = t; minIndex = ti; mb0 = b0; mb1 = b1;
                }
            }
            continue;
        }
        stack[sp++] = node->b;
        stack[sp++] = node->a;
    }
    if (!hit) { memset(h, 0, sizeof(*h)); h->id = -1; return; }
    finish_hit(h, o, d, minIndex, maxT, mb0, mb1);
}

typedef struct {
    const lmo_accel* A;
    const float* rays;
    lmo_hit* out;
    size_t n;
    size_t next; /* shared work counter */
} trace_job;

#define TRACE_CHUNK 1024

static void* trace_worker(void* p)
{
    trace_job* J = (trace_job*)p;
    for (;;) {
        size_t b = __atomic_fetch_add(&J->next, TRACE_CHUNK, __ATOMIC_RELAXED);
        if (b >= J->n) break;
        size_t e = b + TRACE_CHUNK < J->n ? b + TRACE_CHUNK : J->n;
        for (size_t i = b; i < e; i++) {
            if (J->A->kind == 0) trace_naive(J->A, J->rays + 8 * i, &J->out[i]);
            else if (J->A->kind == 2) trace_qbvh(J->A, J->rays + 8 * i, &J->out[i]);
            else trace_bvh(J->A, J->rays + 8 * i, &J->out[i]);
        }
    }
    return NULL;
}

void lmo_accel_trace(const lmo_accel* A, const float* rays, size_t n, lmo_hit* out, int threads)
{
    trace_job J = {A, rays, out, n, 0};
    if (threads <= 1) { trace_worker(&J); return; }
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    for (int i = 0; i < threads; i++) pthread_create(&th[i], NULL, trace_worker, &J);
    for (int i = 0; i < threads; i++) pthread_join(th[i], NULL);
    free(th);
}

/* FP64 Moller-Trumbore on the same triangle: t and the barycentrics of
 * vertices 2 and 3. */
double lmo_plane_t_fp64(const float* tri, const float* ray, double* b1, double* b2)
{
    double v0[3], e1[3], e2[3], o[3], d[3];
    for (int k = 0; k < 3; k++) {
        v0[k] = tri[k];
        e1[k] = (double)tri[3 + k] - v0[k];
        e2[k] = (double)tri[6 + k] - v0[k];
        o[k] = ray[k];
        d[k] = ray[4 + k];
    }
    double pv[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
    double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
    double tv[3] = {o[0] - v0[0], o[1] - v0[1], o[2] - v0[2]};
    double u = (tv[0] * pv[0] + tv[1] * pv[1] + tv[2] * pv[2]) / det;
    double qv[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
    double v = (d[0] * qv[0] + d[1] * qv[1] + d[2] * qv[2]) / det;
    double t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) / det;
    if (b1) *b1 = u;
    if (b2) *b2 = v;
    return t;
}
