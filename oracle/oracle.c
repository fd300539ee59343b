/*
 * oracle.c -- CPU fp64 restatement of ChSchmidt99/trace pkg/pt.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline).  The
 * product never links or calls this file.  Build: oracle/Makefile, always with
 * -ffp-contract=off so that x86-64 and AArch64 give identical results.
 *
 * Deviations from the Go code, all deliberate and documented:
 *  - tie order inside runs of equal Morton codes is the stable (input index)
 *    order; Go's sort.Slice leaves it unspecified (lbvh.go:298).
 *  - the PHR initial cut is taken in FIFO breadth-first order; Go appends it
 *    from racing goroutines (phr.go:257-311).
 *  - the path tracer uses its own seeded RNG (xoshiro256**); Go seeds
 *    math/rand from the wall clock (render.go:117), so images are compared
 *    statistically.
 *  - inputs that make the Go code panic (a Morton code in bucket 4096,
 *    lbvh.go:244-245; a BVH whose root is a leaf, bvh.go:202-206) are reported
 *    as an error code or handled, not crashed on.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* small parallel-for over jobs pulled from an atomic counter (the Go code's  */
/* worker pools fed by channels, e.g. render.go:93-127, lbvh.go:36-59)       */
/* ------------------------------------------------------------------------ */
typedef void (*orc_job_fn)(void *ctx, int64_t job);
typedef struct {
    orc_job_fn fn;
    void *ctx;
    int64_t n;
    atomic_llong next;
} orc_pool;

static void *orc_worker(void *arg) {
    orc_pool *p = (orc_pool *)arg;
    for (;;) {
        int64_t j = atomic_fetch_add(&p->next, 1);
        if (j >= p->n) break;
        p->fn(p->ctx, j);
    }
    return NULL;
}

static void orc_parallel(int threads, int64_t n, orc_job_fn fn, void *ctx) {
    orc_pool p;
    p.fn = fn;
    p.ctx = ctx;
    p.n = n;
    atomic_init(&p.next, 0);
    if (threads <= 1 || n <= 1) {
        orc_worker(&p);
        return;
    }
    if (threads > 256) threads = 256;
    pthread_t tid[256];
    int started = 0;
    for (int i = 0; i < threads - 1; i++)
        if (pthread_create(&tid[started], NULL, orc_worker, &p) == 0) started++;
    orc_worker(&p);
    for (int i = 0; i < started; i++) pthread_join(tid[i], NULL);
}

/* ------------------------------------------------------------------------ */
/* vector helpers, evaluated in the operand order of pkg/pt/math.go:62-105   */
/* ------------------------------------------------------------------------ */
typedef struct { double x, y, z; } v3;
static inline v3 mk(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmul(v3 a, double f) { return mk(a.x * f, a.y * f, a.z * f); }
static inline double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double vlen(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline v3 vunit(v3 a) { double l = vlen(a); return mk(a.x / l, a.y / l, a.z / l); }
static inline v3 vinv(v3 a) { return mk(1 / a.x, 1 / a.y, 1 / a.z); }
static inline v3 vemul(v3 a, v3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }

/* util.go:47-66 */
static double min3(double a, double b, double c) {
    if (a <= b && a <= c) return a;
    if (b <= a && b <= c) return b;
    return c;
}
static double max3(double a, double b, double c) {
    if (a >= b && a >= c) return a;
    if (b >= a && b >= c) return b;
    return c;
}

/* aabb.add via MinVec/MaxVec: bounding.go:49-51, util.go:69-100 */
static void box_add(double *dst, const double *a, const double *b) {
    for (int k = 0; k < 3; k++) {
        double lo = a[k];
        if (a[k] > b[k]) lo = b[k];
        double hi = a[3 + k];
        if (a[3 + k] < b[3 + k]) hi = b[3 + k];
        dst[k] = lo;
        dst[3 + k] = hi;
    }
}

/* aabb.surface: bounding.go:45-47 with w/h/d cached by update() (:36-43) */
double orc_surface(const double b[6]) {
    double w = b[3] - b[0], h = b[4] - b[1], d = b[5] - b[2];
    return 2 * w * h + 2 * w * d + 2 * h * d;
}

/* ------------------------------------------------------------------------ */
/* primitive bounding boxes                                                 */
/* ------------------------------------------------------------------------ */
/* Triangle box: primitive.go:102-114; Sphere box: primitive.go:31-40 */
void orc_prim_boxes(const float *v, int64_t n_tri, const float *sph, int64_t n_sph, double *boxes) {
    for (int64_t i = 0; i < n_tri; i++) {
        const float *t = v + 9 * i;
        double *b = boxes + 6 * i;
        for (int k = 0; k < 3; k++) {
            double a = t[k], c = t[3 + k], e = t[6 + k];
            b[k] = min3(a, c, e);
            b[3 + k] = max3(a, c, e);
        }
    }
    for (int64_t i = 0; i < n_sph; i++) {
        const float *s = sph + 4 * i;
        double *b = boxes + 6 * (n_tri + i);
        double r = s[3];
        for (int k = 0; k < 3; k++) {
            b[k] = (double)s[k] - r;
            b[3 + k] = (double)s[k] + r;
        }
    }
}

/* enclosing(): serial fold, bounding.go:19-25 */
void orc_enclosing(const double *boxes, int64_t n, double out[6]) {
    memcpy(out, boxes, 6 * sizeof(double));
    for (int64_t i = 1; i < n; i++) box_add(out, out, boxes + 6 * i);
}

/* ------------------------------------------------------------------------ */
/* Morton codes: morton.go:6-20, lbvh.go:64-73                              */
/* ------------------------------------------------------------------------ */
/* Spread the low 21 bits of a so that bit k lands on bit 3k (morton.go:12-20).
 * Written as a plain bit loop; tests check it against the reference's own
 * byte tables (morton.go:23-129). */
uint64_t orc_split_by3(uint64_t a) {
    uint64_t x = a & 0x1fffffULL, r = 0;
    for (int k = 0; k < 21; k++) r |= ((x >> k) & 1ULL) << (3 * k);
    return r;
}

uint64_t orc_encode(uint64_t x, uint64_t y, uint64_t z) {
    return orc_split_by3(x) | (orc_split_by3(y) << 1) | (orc_split_by3(z) << 2);
}

/* Go's uint64(float64) for the quantised coordinate.  Inside the domain the
 * value is in [0, 2^21] and truncates toward zero; NaN (zero-extent axis,
 * 0/0) and anything >= 2^63 map to 0, the result Go's amd64 conversion gives
 * after splitBy3's 21-bit mask. */
static uint64_t quantise(double q) {
    if (!(q < 9223372036854775808.0)) return 0;
    if (q < 0) return 0;
    return (uint64_t)q;
}

/* aabb.barycenter = (min+max)*0.5 (bounding.go:37) */
static double bary(const double *b, int k) { return (b[k] + b[3 + k]) * (1.0 / 2.0); }

void orc_morton(const double *boxes, int64_t n, const double e[6], uint64_t *codes) {
    double w = e[3] - e[0], h = e[4] - e[1], d = e[5] - e[2];
    double sx = w / (double)(ORC_MORTON_SIZE - 1);
    double sy = h / (double)(ORC_MORTON_SIZE - 1);
    double sz = d / (double)(ORC_MORTON_SIZE - 1);
    for (int64_t i = 0; i < n; i++) {
        const double *b = boxes + 6 * i;
        double dx = fabs(e[0] - bary(b, 0));
        double dy = fabs(e[1] - bary(b, 1));
        double dz = fabs(e[2] - bary(b, 2));
        codes[i] = orc_encode(quantise(dx / sx), quantise(dy / sy), quantise(dz / sz));
    }
}

/* ------------------------------------------------------------------------ */
/* bucket sort: lbvh.go:216-301                                             */
/* ------------------------------------------------------------------------ */
typedef struct { uint64_t code; int32_t idx; int32_t pad; } orc_pair;

static int pair_cmp(const void *a, const void *b) {
    const orc_pair *p = (const orc_pair *)a, *q = (const orc_pair *)b;
    if (p->code != q->code) return p->code < q->code ? -1 : 1;
    return p->idx < q->idx ? -1 : (p->idx > q->idx);
}

typedef struct {
    orc_pair *pairs;
    const int64_t *start;
} orc_bucket_ctx;

static void bucket_job(void *c, int64_t j) {
    orc_bucket_ctx *ctx = (orc_bucket_ctx *)c;
    int64_t a = ctx->start[j], b = ctx->start[j + 1];
    if (b - a > 1) qsort(ctx->pairs + a, (size_t)(b - a), sizeof(orc_pair), pair_cmp);
}

/* fillBuckets (lbvh.go:226-253) then merge/mergeBuckets (:255-301).  Pairs
 * enter each bucket in input order (the thread batches are contiguous and are
 * concatenated in thread order), and each bucket is then sorted by code with
 * the input index as tie-break: the stable order. */
int orc_sort_pairs(const uint64_t *codes, int64_t n, int threads, uint64_t *sorted_codes, int32_t *sorted_idx) {
    const uint64_t bucket_size = ORC_MAX_MORTON_CODE / ORC_BUCKET_COUNT; /* lbvh.go:240 */
    int64_t *count = (int64_t *)calloc(ORC_BUCKET_COUNT + 1, sizeof(int64_t));
    orc_pair *pairs = (orc_pair *)malloc((size_t)(n > 0 ? n : 1) * sizeof(orc_pair));
    if (!count || !pairs) { free(count); free(pairs); return ORC_E_NOMEM; }
    for (int64_t i = 0; i < n; i++) {
        uint64_t bi = codes[i] / bucket_size;
        if (bi >= ORC_BUCKET_COUNT) { free(count); free(pairs); return ORC_E_BUCKET; }
        count[bi + 1]++;
    }
    for (int k = 0; k < ORC_BUCKET_COUNT; k++) count[k + 1] += count[k];
    int64_t *fill = (int64_t *)malloc(ORC_BUCKET_COUNT * sizeof(int64_t));
    if (!fill) { free(count); free(pairs); return ORC_E_NOMEM; }
    memcpy(fill, count, ORC_BUCKET_COUNT * sizeof(int64_t));
    for (int64_t i = 0; i < n; i++) {
        uint64_t bi = codes[i] / bucket_size;
        orc_pair *p = &pairs[fill[bi]++];
        p->code = codes[i];
        p->idx = (int32_t)i;
        p->pad = 0;
    }
    orc_bucket_ctx ctx = {pairs, count};
    orc_parallel(threads, ORC_BUCKET_COUNT, bucket_job, &ctx);
    for (int64_t i = 0; i < n; i++) {
        sorted_codes[i] = pairs[i].code;
        sorted_idx[i] = pairs[i].idx;
    }
    free(fill);
    free(count);
    free(pairs);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* BVH storage (bvh.go:14-18, 128-157), N-ary                               */
/* ------------------------------------------------------------------------ */
typedef struct {
    int32_t parent;
    int32_t nchild;
    int64_t kid_first;  /* into kids[] */
    int64_t prim_first; /* into prims[] */
    int32_t prim_count;
    int8_t is_leaf;
    int64_t size; /* subtreeSize cache (bvh.go:159-167); 0 = not computed */
    double box[6];
} orc_node;

struct orc_bvh {
    orc_node *nodes;
    int64_t n_nodes, cap_nodes;
    int32_t *kids;
    int64_t n_kids, cap_kids;
    int32_t *prims;
    int64_t n_prims, cap_prims;
    int32_t root;
    /* scene (widened to float64) */
    int64_t n_tri, n_sph;
    double *tri;     /* n_tri*9: v0 v1 v2 */
    double *tri_nrm; /* n_tri*9: per-vertex normals n0 n1 n2 */
    double *sph;     /* n_sph*4 */
    double *pbox;    /* (n_tri+n_sph)*6 */
    /* LBVH only */
    uint64_t *sorted_codes;
    int32_t *sorted_idx;
    int64_t n_sorted;
};

static int grow(void **p, int64_t *cap, int64_t need, size_t elem) {
    if (need <= *cap) return 0;
    int64_t nc = *cap ? *cap : 1024;
    while (nc < need) nc *= 2;
    void *q = realloc(*p, (size_t)nc * elem);
    if (!q) return -1;
    *p = q;
    *cap = nc;
    return 0;
}

static int32_t new_node(orc_bvh *b) {
    if (grow((void **)&b->nodes, &b->cap_nodes, b->n_nodes + 1, sizeof(orc_node))) return -1;
    orc_node *n = &b->nodes[b->n_nodes];
    memset(n, 0, sizeof(*n));
    n->parent = -1;
    return (int32_t)b->n_nodes++;
}

/* newLeaf (bvh.go:138-144) */
static int32_t new_leaf(orc_bvh *b, const int32_t *prims, int64_t count) {
    int32_t id = new_node(b);
    if (id < 0) return -1;
    if (grow((void **)&b->prims, &b->cap_prims, b->n_prims + count, sizeof(int32_t))) return -1;
    orc_node *n = &b->nodes[id];
    n->is_leaf = 1;
    n->size = 1;
    n->prim_first = b->n_prims;
    n->prim_count = (int32_t)count;
    memcpy(b->prims + b->n_prims, prims, (size_t)count * sizeof(int32_t));
    b->n_prims += count;
    return id;
}

/* newBranch (bvh.go:146-152) */
static int32_t new_branch(orc_bvh *b, int nchild) {
    int32_t id = new_node(b);
    if (id < 0) return -1;
    if (grow((void **)&b->kids, &b->cap_kids, b->n_kids + nchild, sizeof(int32_t))) return -1;
    orc_node *n = &b->nodes[id];
    n->nchild = nchild;
    n->kid_first = b->n_kids;
    for (int k = 0; k < nchild; k++) b->kids[b->n_kids + k] = -1;
    b->n_kids += nchild;
    return id;
}

/* addChild (bvh.go:154-157); parent < 0 makes the child the root */
static void add_child(orc_bvh *b, int32_t parent, int32_t child, int index) {
    if (parent < 0) {
        b->root = child;
        b->nodes[child].parent = -1;
        return;
    }
    b->kids[b->nodes[parent].kid_first + index] = child;
    b->nodes[child].parent = parent;
}

static inline int32_t kid(const orc_bvh *b, int32_t n, int k) { return b->kids[b->nodes[n].kid_first + k]; }

void orc_bvh_free(orc_bvh *b) {
    if (!b) return;
    free(b->nodes);
    free(b->kids);
    free(b->prims);
    free(b->tri);
    free(b->tri_nrm);
    free(b->sph);
    free(b->pbox);
    free(b->sorted_codes);
    free(b->sorted_idx);
    free(b);
}

/* calcNormal (primitive.go:134-138) */
static v3 calc_normal(v3 point, v3 right, v3 left) {
    v3 pa = vsub(left, point), pb = vsub(right, point);
    return vunit(vcross(pb, pa));
}

static int scene_copy(orc_bvh *b, const float *v, int64_t n_tri, const float *sph, int64_t n_sph) {
    int64_t n = n_tri + n_sph;
    b->n_tri = n_tri;
    b->n_sph = n_sph;
    b->tri = (double *)malloc((size_t)(n_tri > 0 ? n_tri : 1) * 9 * sizeof(double));
    b->tri_nrm = (double *)malloc((size_t)(n_tri > 0 ? n_tri : 1) * 9 * sizeof(double));
    b->sph = (double *)malloc((size_t)(n_sph > 0 ? n_sph : 1) * 4 * sizeof(double));
    b->pbox = (double *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(double));
    if (!b->tri || !b->tri_nrm || !b->sph || !b->pbox) return ORC_E_NOMEM;
    for (int64_t i = 0; i < n_tri * 9; i++) b->tri[i] = v[i];
    for (int64_t i = 0; i < n_sph * 4; i++) b->sph[i] = sph[i];
    /* NewTriangleWithoutNormals: one calcNormal per vertex (primitive.go:116-132) */
    for (int64_t i = 0; i < n_tri; i++) {
        const double *t = b->tri + 9 * i;
        v3 p0 = mk(t[0], t[1], t[2]), p1 = mk(t[3], t[4], t[5]), p2 = mk(t[6], t[7], t[8]);
        v3 n0 = calc_normal(p0, p1, p2), n1 = calc_normal(p1, p2, p0), n2 = calc_normal(p2, p0, p1);
        double *o = b->tri_nrm + 9 * i;
        o[0] = n0.x; o[1] = n0.y; o[2] = n0.z;
        o[3] = n1.x; o[4] = n1.y; o[5] = n1.z;
        o[6] = n2.x; o[7] = n2.y; o[8] = n2.z;
    }
    orc_prim_boxes(v, n_tri, sph, n_sph, b->pbox);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* LBVH construction: lbvh.go:76-203                                         */
/* ------------------------------------------------------------------------ */
/* findSplit (lbvh.go:184-203): index of the first pair whose code has the
 * mask bit set, by binary search. */
static int64_t find_split(const uint64_t *c, int64_t n, uint64_t mask) {
    if (c[0] & mask) return 0;
    int64_t l = 0, r = n - 1;
    while (l <= r) {
        int64_t m = (l + r) / 2;
        if ((c[m] & mask) == 0) l = m + 1;
        else if ((c[m] & mask) && (c[m - 1] & mask)) r = m - 1;
        else return m;
    }
    return n;
}

typedef struct { int64_t a, b; uint64_t mask; int32_t parent; int32_t slot; } lbvh_job;

/* lbvhJob.process (lbvh.go:133-177), run from an explicit stack */
static int construct_lbvh(orc_bvh *bv, const uint64_t *codes, const int32_t *idx, int64_t n) {
    int64_t cap = 256, top = 0;
    lbvh_job *st = (lbvh_job *)malloc((size_t)cap * sizeof(lbvh_job));
    if (!st) return ORC_E_NOMEM;
    lbvh_job j0 = {0, n, 1ULL << 62, -1, 0};
    st[top++] = j0;
    while (top > 0) {
        lbvh_job j = st[--top];
        const uint64_t *c = codes + j.a;
        int64_t len = j.b - j.a;
        if (c[0] == c[len - 1]) { /* isLeaf (lbvh.go:179-181) */
            int32_t leaf = new_leaf(bv, idx + j.a, len);
            if (leaf < 0) { free(st); return ORC_E_NOMEM; }
            add_child(bv, j.parent, leaf, j.slot);
            continue;
        }
        int64_t s = find_split(c, len, j.mask);
        if (top + 2 > cap) {
            cap *= 2;
            lbvh_job *q = (lbvh_job *)realloc(st, (size_t)cap * sizeof(lbvh_job));
            if (!q) { free(st); return ORC_E_NOMEM; }
            st = q;
        }
        if (s == 0 || s == len) { /* no split at this bit: same job, next bit */
            lbvh_job k = {j.a, j.b, j.mask >> 1, j.parent, j.slot};
            st[top++] = k;
            continue;
        }
        int32_t br = new_branch(bv, 2);
        if (br < 0) { free(st); return ORC_E_NOMEM; }
        add_child(bv, j.parent, br, j.slot);
        lbvh_job L = {j.a, j.a + s, j.mask >> 1, br, 0};
        lbvh_job R = {j.a + s, j.b, j.mask >> 1, br, 1};
        st[top++] = R;
        st[top++] = L;
    }
    free(st);
    return ORC_OK;
}

/* updateAABB (bvh.go:201-222): a leaf box is the fold of its prims' boxes in
 * leaf order (enclosingSlice, bounding.go:27-34); an inner box folds its
 * children in child order.  Post-order traversal gives the same boxes as the
 * reference's atomic last-arriver scheme because min/max folds are exact. */
static void refit(orc_bvh *b, int32_t root) {
    int64_t cap = 256, top = 0;
    int32_t *st = (int32_t *)malloc((size_t)cap * sizeof(int32_t));
    int8_t *done = (int8_t *)calloc((size_t)b->n_nodes, 1);
    st[top++] = root;
    while (top > 0) {
        int32_t ni = st[top - 1];
        orc_node *n = &b->nodes[ni];
        if (n->is_leaf) {
            const int32_t *p = b->prims + n->prim_first;
            memcpy(n->box, b->pbox + 6 * (int64_t)p[0], 6 * sizeof(double));
            for (int k = 1; k < n->prim_count; k++) box_add(n->box, n->box, b->pbox + 6 * (int64_t)p[k]);
            top--;
            continue;
        }
        if (!done[ni]) {
            done[ni] = 1;
            if (top + n->nchild > cap) {
                while (top + n->nchild > cap) cap *= 2;
                st = (int32_t *)realloc(st, (size_t)cap * sizeof(int32_t));
            }
            for (int k = 0; k < n->nchild; k++) st[top++] = kid(b, ni, k);
            continue;
        }
        memcpy(n->box, b->nodes[kid(b, ni, 0)].box, 6 * sizeof(double));
        for (int k = 1; k < n->nchild; k++) box_add(n->box, n->box, b->nodes[kid(b, ni, k)].box);
        top--;
    }
    free(st);
    free(done);
}

typedef struct { const double *boxes; const double *e; uint64_t *codes; int64_t n, chunk; } morton_ctx;
static void morton_job(void *c, int64_t j) {
    morton_ctx *m = (morton_ctx *)c;
    int64_t a = j * m->chunk, b = a + m->chunk;
    if (b > m->n) b = m->n;
    if (a < b) orc_morton(m->boxes + 6 * a, b - a, m->e, m->codes + a);
}

/* DefaultLBVH/LBVH (lbvh.go:13-25): Morton codes, sort, construction, refit. */
int orc_lbvh_build(const float *v, int64_t n_tri, const float *sph, int64_t n_sph, int threads, orc_bvh **out) {
    int64_t n = n_tri + n_sph;
    *out = NULL;
    if (n <= 0) return ORC_E_ARG;
    orc_bvh *b = (orc_bvh *)calloc(1, sizeof(orc_bvh));
    if (!b) return ORC_E_NOMEM;
    int rc = scene_copy(b, v, n_tri, sph, n_sph);
    if (rc) { orc_bvh_free(b); return rc; }
    double e[6];
    orc_enclosing(b->pbox, n, e);
    uint64_t *codes = (uint64_t *)malloc((size_t)n * sizeof(uint64_t));
    b->sorted_codes = (uint64_t *)malloc((size_t)n * sizeof(uint64_t));
    b->sorted_idx = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    b->n_sorted = n;
    if (!codes || !b->sorted_codes || !b->sorted_idx) { free(codes); orc_bvh_free(b); return ORC_E_NOMEM; }
    /* assignMortonCodes: contiguous batches per thread (lbvh.go:33-61) */
    int t = threads > 0 ? threads : 1;
    morton_ctx mc = {b->pbox, e, codes, n, (n + t - 1) / t};
    orc_parallel(t, t, morton_job, &mc);
    rc = orc_sort_pairs(codes, n, t, b->sorted_codes, b->sorted_idx);
    free(codes);
    if (rc) { orc_bvh_free(b); return rc; }
    rc = construct_lbvh(b, b->sorted_codes, b->sorted_idx, n);
    if (rc) { orc_bvh_free(b); return rc; }
    refit(b, b->root);
    *out = b;
    return ORC_OK;
}

void orc_bvh_sorted(const orc_bvh *b, uint64_t *codes, int32_t *idx) {
    if (!b->sorted_codes) return;
    memcpy(codes, b->sorted_codes, (size_t)b->n_sorted * sizeof(uint64_t));
    memcpy(idx, b->sorted_idx, (size_t)b->n_sorted * sizeof(int32_t));
}

/* ------------------------------------------------------------------------ */
/* export in depth-first pre-order, children in stored order                */
/* ------------------------------------------------------------------------ */
void orc_bvh_counts(const orc_bvh *b, int64_t out[4]) {
    /* count reachable nodes from root */
    int64_t nodes = 0, leaves = 0, refs = 0;
    int64_t cap = 256, top = 0;
    int32_t *st = (int32_t *)malloc((size_t)cap * sizeof(int32_t));
    st[top++] = b->root;
    while (top > 0) {
        int32_t ni = st[--top];
        const orc_node *n = &b->nodes[ni];
        nodes++;
        if (n->is_leaf) { leaves++; refs += n->prim_count; continue; }
        if (top + n->nchild > cap) { while (top + n->nchild > cap) cap *= 2; st = (int32_t *)realloc(st, (size_t)cap * sizeof(int32_t)); }
        for (int k = 0; k < n->nchild; k++) st[top++] = kid(b, ni, k);
    }
    free(st);
    out[0] = nodes;
    out[1] = leaves;
    out[2] = refs;
    out[3] = b->nodes[b->root].is_leaf;
}

void orc_bvh_export(const orc_bvh *b, int8_t *kind, int32_t *count, double *box, int32_t *prims) {
    int64_t cap = 256, top = 0, o = 0, po = 0;
    int32_t *st = (int32_t *)malloc((size_t)cap * sizeof(int32_t));
    st[top++] = b->root;
    while (top > 0) {
        int32_t ni = st[--top];
        const orc_node *n = &b->nodes[ni];
        kind[o] = n->is_leaf;
        count[o] = n->is_leaf ? n->prim_count : n->nchild;
        memcpy(box + 6 * o, n->box, 6 * sizeof(double));
        o++;
        if (n->is_leaf) {
            memcpy(prims + po, b->prims + n->prim_first, (size_t)n->prim_count * sizeof(int32_t));
            po += n->prim_count;
            continue;
        }
        if (top + n->nchild > cap) { while (top + n->nchild > cap) cap *= 2; st = (int32_t *)realloc(st, (size_t)cap * sizeof(int32_t)); }
        for (int k = n->nchild - 1; k >= 0; k--) st[top++] = kid(b, ni, k);
    }
    free(st);
}

/* subtreeSize (bvh.go:159-167) */
static int64_t subtree_size(orc_bvh *b, int32_t ni) {
    orc_node *n = &b->nodes[ni];
    if (n->size == 0) {
        int64_t s = 1;
        for (int k = 0; k < n->nchild; k++) s += subtree_size(b, kid(b, ni, k));
        b->nodes[ni].size = s;
    }
    return b->nodes[ni].size;
}

int64_t orc_bvh_size(orc_bvh *b) { return subtree_size(b, b->root); }

/* cost (bvh.go:226-239) */
static double node_cost(const orc_bvh *b, int32_t ni) {
    const orc_node *n = &b->nodes[ni];
    if (n->is_leaf) return 1.0 * (double)n->prim_count;
    double child_costs = 0.0;
    for (int k = 0; k < n->nchild; k++) {
        if (orc_surface(n->box) != 0) {
            const orc_node *c = &b->nodes[kid(b, ni, k)];
            double probability = orc_surface(c->box) / orc_surface(n->box);
            child_costs += probability * node_cost(b, kid(b, ni, k));
        }
    }
    return 2.0 + child_costs;
}

double orc_bvh_cost(orc_bvh *b) { return node_cost(b, b->root); }

/* ------------------------------------------------------------------------ */
/* ray queries                                                               */
/* ------------------------------------------------------------------------ */
typedef struct { v3 o, d, inv; int sign[3]; } oray;

/* newRay / reuse (camera.go:113-158) */
static oray make_ray(v3 o, v3 d) {
    oray r;
    r.o = o;
    r.d = d;
    r.inv = vinv(d);
    r.sign[0] = r.inv.x < 0;
    r.sign[1] = r.inv.y < 0;
    r.sign[2] = r.inv.z < 0;
    return r;
}

typedef struct {
    double t, u, v, det;
    int32_t prim;
    v3 point, normal;
    int front;
} ohit;

/* aabb.intersected (bounding.go:53-91) */
static int box_hit(const double *bx, const oray *r, double tmin, double tmax) {
    const double *lo = bx, *hi = bx + 3;
#define BND(s, k) ((s) ? hi[k] : lo[k])
    double txmin = (BND(r->sign[0], 0) - r->o.x) * r->inv.x;
    double txmax = (BND(1 - r->sign[0], 0) - r->o.x) * r->inv.x;
    double tymin = (BND(r->sign[1], 1) - r->o.y) * r->inv.y;
    double tymax = (BND(1 - r->sign[1], 1) - r->o.y) * r->inv.y;
    if (txmin > tymax || tymin > txmax) return 0;
    if (tymin > txmin) txmin = tymin;
    if (tymax < txmax) txmax = tymax;
    double tzmin = (BND(r->sign[2], 2) - r->o.z) * r->inv.z;
    double tzmax = (BND(1 - r->sign[2], 2) - r->o.z) * r->inv.z;
    if (txmin > tzmax || tzmin > txmax) return 0;
    if (tzmin > txmin) txmin = tzmin;
    if (tzmax < txmax) txmax = tzmax;
    if (txmax < tmin || txmin > tmax) return 0;
    return 1;
#undef BND
}

/* Triangle.intersected, Moeller-Trumbore (primitive.go:172-208).  On a hit
 * writes t,u,v and the shading normal (interpolated vertex normals flipped
 * toward the ray, primitive.go:144-150,201-205). */
static int tri_hit(const orc_bvh *b, int64_t ti, const oray *r, double tmin, double tmax, ohit *h, int want_normal) {
    const double *t = b->tri + 9 * ti;
    v3 v0 = mk(t[0], t[1], t[2]);
    v3 e1 = vsub(mk(t[3], t[4], t[5]), v0);
    v3 e2 = vsub(mk(t[6], t[7], t[8]), v0);
    v3 pvec = vcross(r->d, e2);
    double det = vdot(e1, pvec);
    if (fabs(det) <= ORC_APPROX_THRESH) return 0;
    double inv = 1 / det;
    v3 tvec = vsub(r->o, v0);
    double u = vdot(tvec, pvec) * inv;
    if (u < 0 || u > 1) return 0;
    v3 qvec = vcross(tvec, e1);
    double v = vdot(r->d, qvec) * inv;
    if (v < 0 || u + v > 1) return 0;
    double tt = vdot(e2, qvec) * inv;
    if (tt < tmin || tt > tmax) return 0;
    h->t = tt;
    h->u = u;
    h->v = v;
    h->det = det;
    h->prim = (int32_t)ti;
    if (want_normal) {
        h->point = vadd(r->o, vmul(r->d, tt));
        h->front = det > 0;
        const double *n = b->tri_nrm + 9 * ti;
        v3 nw = vmul(mk(n[0], n[1], n[2]), 1 - u - v);
        v3 nu = vmul(mk(n[3], n[4], n[5]), u);
        v3 nv = vmul(mk(n[6], n[7], n[8]), v);
        h->normal = vadd(vadd(nu, nv), nw);
        if (!h->front) h->normal = vmul(h->normal, -1);
    }
    return 1;
}

/* Sphere.intersected (primitive.go:56-86) */
static int sph_hit(const orc_bvh *b, int64_t si, const oray *r, double tmin, double tmax, ohit *h, int want_normal) {
    const double *s = b->sph + 4 * si;
    v3 c = mk(s[0], s[1], s[2]);
    double rad = s[3];
    v3 oc = vsub(r->o, c);
    double dn = vlen(r->d);
    double a = dn * dn;
    double half_b = vdot(oc, r->d);
    double ocn = vlen(oc);
    double cc = ocn * ocn - rad * rad;
    double disc = half_b * half_b - a * cc;
    if (disc < 0) return 0;
    double sq = sqrt(disc);
    double t = (-half_b - sq) / a;
    if (t <= tmin || t >= tmax) {
        t = (-half_b + sq) / a;
        if (t <= tmin || t >= tmax) return 0;
    }
    h->t = t;
    h->u = 0;
    h->v = 0;
    h->det = 0;
    h->prim = (int32_t)(b->n_tri + si);
    if (want_normal) {
        h->point = vadd(r->o, vmul(r->d, t));
        h->normal = vmul(vsub(h->point, c), 1 / rad);
        h->front = vdot(r->d, h->normal) < 0;
        if (!h->front) h->normal = vmul(h->normal, -1);
    }
    return 1;
}

static int prim_hit(const orc_bvh *b, int32_t p, const oray *r, double tmin, double tmax, ohit *h, int wn) {
    if (p < b->n_tri) return tri_hit(b, p, r, tmin, tmax, h, wn);
    return sph_hit(b, p - b->n_tri, r, tmin, tmax, h, wn);
}

/* bvhNode.intersected (bvh.go:179-199): recursive, children in stored order,
 * the running closest t narrows every later test. */
static int node_hit(const orc_bvh *b, int32_t ni, const oray *r, double tmin, double tmax, ohit *h, int wn) {
    const orc_node *n = &b->nodes[ni];
    if (!box_hit(n->box, r, tmin, tmax)) return 0;
    int did = 0;
    if (n->is_leaf) {
        for (int k = 0; k < n->prim_count; k++)
            if (prim_hit(b, b->prims[n->prim_first + k], r, tmin, h->t, h, wn)) did = 1;
    } else {
        for (int k = 0; k < n->nchild; k++)
            if (node_hit(b, kid(b, ni, k), r, tmin, h->t, h, wn)) did = 1;
    }
    return did;
}

/* BVH.intersected (bvh.go:74-77) */
static int bvh_hit(const orc_bvh *b, const oray *r, double tmin, double tmax, ohit *h, int wn) {
    h->t = tmax;
    return node_hit(b, b->root, r, tmin, tmax, h, wn);
}

typedef struct {
    const orc_bvh *b;
    const float *rays;
    int64_t n, chunk;
    int32_t *prim;
    double *t, *u, *v;
    int32_t *steps;
} trace_ctx;

static oray ray_from8(const float *q) {
    return make_ray(mk(q[0], q[1], q[2]), mk(q[4], q[5], q[6]));
}

static void trace_job(void *c, int64_t j) {
    trace_ctx *x = (trace_ctx *)c;
    int64_t a = j * x->chunk, e = a + x->chunk;
    if (e > x->n) e = x->n;
    for (int64_t i = a; i < e; i++) {
        const float *q = x->rays + 8 * i;
        oray r = ray_from8(q);
        ohit h;
        memset(&h, 0, sizeof(h));
        h.prim = -1;
        if (bvh_hit(x->b, &r, q[3], q[7], &h, 0)) {
            x->prim[i] = h.prim;
            x->t[i] = h.t;
            x->u[i] = h.u;
            x->v[i] = h.v;
        } else {
            x->prim[i] = -1;
            x->t[i] = INFINITY;
            x->u[i] = 0;
            x->v[i] = 0;
        }
    }
}

void orc_trace(const orc_bvh *b, const float *rays, int64_t n, int threads,
               int32_t *hit_prim, double *hit_t, double *hit_u, double *hit_v) {
    trace_ctx x = {b, rays, n, 4096, hit_prim, hit_t, hit_u, hit_v, NULL};
    orc_parallel(threads, (n + x.chunk - 1) / x.chunk, trace_job, &x);
}

int orc_prim_intersect(const orc_bvh *b, int32_t prim, const float *q, double *t, double *u, double *v, double *det) {
    oray r = ray_from8(q);
    ohit h;
    memset(&h, 0, sizeof(h));
    int ok = prim_hit(b, prim, &r, q[3], q[7], &h, 0);
    if (prim < b->n_tri) {
        /* report det even when rejected, for near-threshold classification */
        const double *tv = b->tri + 9 * (int64_t)prim;
        v3 v0 = mk(tv[0], tv[1], tv[2]);
        v3 e1 = vsub(mk(tv[3], tv[4], tv[5]), v0), e2 = vsub(mk(tv[6], tv[7], tv[8]), v0);
        v3 pvec = vcross(r.d, e2);
        double dd = vdot(e1, pvec);
        double inv = 1 / dd;
        v3 tvec = vsub(r.o, v0);
        v3 qvec = vcross(tvec, e1);
        *det = dd;
        *u = vdot(tvec, pvec) * inv;
        *v = vdot(r.d, qvec) * inv;
        *t = vdot(e2, qvec) * inv;
    } else {
        *t = ok ? h.t : INFINITY;
        *u = 0;
        *v = 0;
        *det = 0;
    }
    return ok;
}

/* BVH.traversalSteps (bvh.go:21-44): explicit stack, children pushed in
 * order (so popped last-first), counts inner nodes whose box is hit. */
static int32_t traversal_steps(const orc_bvh *b, const oray *r, double tmin, double tmax) {
    int32_t st[4096];
    int top = 0, count = 0;
    ohit h;
    memset(&h, 0, sizeof(h));
    h.t = tmax;
    st[top++] = b->root;
    while (top > 0) {
        int32_t ni = st[--top];
        const orc_node *n = &b->nodes[ni];
        if (!box_hit(n->box, r, tmin, h.t)) continue;
        if (n->is_leaf) {
            for (int k = 0; k < n->prim_count; k++) prim_hit(b, b->prims[n->prim_first + k], r, tmin, h.t, &h, 0);
        } else {
            for (int k = 0; k < n->nchild && top < 4096; k++) st[top++] = kid(b, ni, k);
            count++;
        }
    }
    return count;
}

static void steps_job(void *c, int64_t j) {
    trace_ctx *x = (trace_ctx *)c;
    int64_t a = j * x->chunk, e = a + x->chunk;
    if (e > x->n) e = x->n;
    for (int64_t i = a; i < e; i++) {
        oray r = ray_from8(x->rays + 8 * i);
        x->steps[i] = traversal_steps(x->b, &r, x->rays[8 * i + 3], x->rays[8 * i + 7]);
    }
}

void orc_traversal_steps(const orc_bvh *b, const float *rays, int64_t n, int threads, int32_t *steps) {
    trace_ctx x = {b, rays, n, 4096, NULL, NULL, NULL, NULL, steps};
    orc_parallel(threads, (n + x.chunk - 1) / x.chunk, steps_job, &x);
}

/* ------------------------------------------------------------------------ */
/* camera (camera.go:7-97)                                                   */
/* ------------------------------------------------------------------------ */
typedef struct { v3 origin, w, u, v, horizontal, vertical, llc; } ocam;

static ocam make_camera(const orc_camera_desc *c) {
    ocam k;
    double vh = 2.0 * tan((c->fov_deg * (M_PI / 180)) / 2); /* NewCamera, DegreesToRadians util.go:43-45 */
    double vw = c->aspect * vh;
    v3 from = mk(c->look_from[0], c->look_from[1], c->look_from[2]);
    v3 at = mk(c->look_at[0], c->look_at[1], c->look_at[2]);
    v3 up = mk(c->up[0], c->up[1], c->up[2]);
    k.w = vunit(vsub(from, at)); /* newOrientation */
    k.u = vunit(vcross(up, k.w));
    k.v = vcross(k.w, k.u);
    k.origin = from;
    k.horizontal = vmul(k.u, vw); /* SetTransformation */
    k.vertical = vmul(k.v, vh);
    k.llc = vsub(vsub(vsub(k.origin, vmul(k.horizontal, 0.5)), vmul(k.vertical, 0.5)), k.w);
    return k;
}

/* castRayReuse direction (camera.go:95-97) */
static v3 cam_dir(const ocam *k, double s, double t) {
    return vsub(vadd(vadd(k->llc, vmul(k->horizontal, s)), vmul(k->vertical, t)), k->origin);
}

void orc_camera_rays(const orc_camera_desc *cam, int32_t width, int32_t height,
                     const double *su, const double *sv, int64_t n, double *dirs, double origin[3]) {
    (void)width;
    (void)height;
    ocam k = make_camera(cam);
    origin[0] = k.origin.x;
    origin[1] = k.origin.y;
    origin[2] = k.origin.z;
    for (int64_t i = 0; i < n; i++) {
        v3 d = cam_dir(&k, su[i], sv[i]);
        dirs[3 * i] = d.x;
        dirs[3 * i + 1] = d.y;
        dirs[3 * i + 2] = d.z;
    }
}

/* HeatMapRenderer.RenderToBuffer (render.go:167-197): pixel-centre rays
 * (u = x/(w-1), v = y/(h-1)), BVH.traversalSteps from 0.001 to MaxFloat64
 * (bvh.go:21-44) and DefaultTraversalCountShader (render.go:250-257).
 * rgb: width*height*3 (row y = 0 first); counts optional. */
typedef struct {
    const orc_bvh *b;
    ocam k;
    int32_t w, h, thr;
    double *rgb;
    int32_t *counts;
} heat_ctx;

static void heat_job(void *c, int64_t y) {
    heat_ctx *x = (heat_ctx *)c;
    for (int32_t xx = 0; xx < x->w; xx++) {
        double u = (double)xx / (double)(x->w - 1), v = (double)y / (double)(x->h - 1);
        oray r = make_ray(x->k.origin, cam_dir(&x->k, u, v));
        int32_t cnt = traversal_steps(x->b, &r, 0.001, DBL_MAX);
        int64_t p = y * x->w + xx;
        double *o = x->rgb + 3 * p;
        if (cnt > x->thr) {
            o[0] = (double)cnt / (double)x->thr * 2;
            o[1] = 0;
            o[2] = 0;
        } else {
            double f = (double)cnt / ((double)x->thr * 1.25);
            o[0] = 0;
            o[1] = f;
            o[2] = 1 - f;
        }
        if (x->counts) x->counts[p] = cnt;
    }
}

void orc_heatmap(const orc_bvh *b, const orc_camera_desc *cam, int32_t width, int32_t height, int32_t threshold,
                 int threads, double *rgb, int32_t *counts) {
    heat_ctx x = {b, make_camera(cam), width, height, threshold, rgb, counts};
    orc_parallel(threads, height, heat_job, &x);
}

/* ------------------------------------------------------------------------ */
/* renderer (render.go:91-129, 199-246; material.go:13-42; util.go:15-26)    */
/* ------------------------------------------------------------------------ */
typedef struct { uint64_t s[4]; } xrng;

static uint64_t splitmix(uint64_t *x) {
    uint64_t z = (*x += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t xnext(xrng *r) {
    uint64_t res = rotl(r->s[1] * 5, 7) * 9, t = r->s[1] << 17;
    r->s[2] ^= r->s[0];
    r->s[3] ^= r->s[1];
    r->s[1] ^= r->s[2];
    r->s[0] ^= r->s[3];
    r->s[2] ^= t;
    r->s[3] = rotl(r->s[3], 45);
    return res;
}
static double xf64(xrng *r) { return (double)(xnext(r) >> 11) * 0x1.0p-53; }
static double xnorm(xrng *r) { /* Box-Muller standing in for rand.NormFloat64 */
    double u1 = 1.0 - xf64(r), u2 = xf64(r);
    return sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
}
static void xseed(xrng *r, uint64_t seed, uint64_t a, uint64_t b) {
    uint64_t x = seed ^ (a * 0xd1b54a32d192ed03ULL) ^ (b * 0x8cb92ba72f3d8dd7ULL);
    for (int i = 0; i < 4; i++) r->s[i] = splitmix(&x);
}

/* RandomUnitVector (util.go:15-26) */
static v3 random_unit_vector(xrng *r) {
    double u = xf64(r);
    double x1 = xnorm(r), x2 = xnorm(r), x3 = xnorm(r);
    double mag = sqrt(x1 * x1 + x2 * x2 + x3 * x3);
    x1 /= mag;
    x2 /= mag;
    x3 /= mag;
    double c = cbrt(u);
    return vunit(mk(x1 * c, x2 * c, x3 * c));
}

typedef struct {
    const orc_bvh *b;
    const int32_t *prim_mat, *mat_type;
    const double *mat_color, *mat_param;
    const orc_render_desc *rd;
    ocam cam;
    double *acc; /* running mean per pixel (PixelBuffer) */
    int32_t *samples;
    atomic_llong rays;
} render_ctx;

static _Thread_local int64_t tl_rays; /* rays traced by this thread's current row */

static v3 miss_color(const render_ctx *x, const oray *r) { /* render.go:228-246 */
    switch (x->rd->miss_mode) {
    case 1: return mk(1, 1, 1);
    case 2: {
        v3 unit = vunit(r->d);
        double t = 0.5 * (unit.y + 1);
        return vadd(vmul(mk(0.8, 0.8, 0.8), 1.0 - t), vmul(mk(0.25, 0.35, 0.5), t));
    }
    case 3: return mk(x->rd->miss_color[0], x->rd->miss_color[1], x->rd->miss_color[2]);
    default: return mk(0, 0, 0);
    }
}

/* reflect, refract, reflectance (Schlick): material.go:88-106 */
static v3 reflect_v(v3 v, v3 n) { return vsub(v, vmul(n, vdot(v, n) * 2)); }
static v3 refract_v(v3 uv, v3 n, double eta) {
    double c = fmin(vdot(vmul(uv, -1), n), 1.0);
    v3 perp = vmul(vadd(uv, vmul(n, c)), eta);
    v3 par = vmul(n, -sqrt(fabs(1.0 - vdot(perp, perp))));
    return vadd(perp, par);
}
static double reflectance(double cosine, double ratio) {
    double r0 = (1 - ratio) / (1 + ratio);
    r0 = r0 * r0;
    return r0 + (1 - r0) * pow(1 - cosine, 5);
}

/* DefaultClosestHitShader (render.go:209-224) with Light (material.go:13-23),
 * Diffuse (:29-38), Reflective (:49-53) and Refractive (:63-86) scatter. */
static v3 shade(const render_ctx *x, oray r, ohit h, int depth, xrng *g) {
    if (depth > x->rd->max_depth) return mk(0, 0, 0);
    depth++;
    int m = x->prim_mat[h.prim];
    v3 col = mk(x->mat_color[3 * m], x->mat_color[3 * m + 1], x->mat_color[3 * m + 2]);
    int type = x->mat_type[m];
    if (type == 1) return col; /* Light: emits, does not scatter */
    v3 light = mk(0, 0, 0);
    v3 sd;
    if (type == 2) { /* Reflective */
        v3 refl = reflect_v(vunit(r.d), h.normal);
        sd = vadd(refl, vmul(random_unit_vector(g), x->mat_param ? x->mat_param[m] : 0.0));
        if (!(vdot(refl, h.normal) > 0)) return light;
    } else if (type == 3) { /* Refractive */
        double ratio = x->mat_param ? x->mat_param[m] : 1.0;
        if (h.front) ratio = 1 / ratio;
        v3 ud = vunit(r.d);
        double ct = fmin(vdot(vmul(ud, -1), h.normal), 1.0);
        double st = sqrt(1.0 - ct * ct);
        int cannot = ratio * st > 1.0;
        if (cannot || reflectance(ct, ratio) > xf64(g)) sd = reflect_v(ud, h.normal);
        else sd = refract_v(ud, h.normal, ratio);
    } else { /* Diffuse */
        sd = vadd(h.normal, random_unit_vector(g));
        if (fabs(sd.x) <= ORC_APPROX_THRESH && fabs(sd.y) <= ORC_APPROX_THRESH && fabs(sd.z) <= ORC_APPROX_THRESH)
            sd = h.normal;
    }
    oray r2 = make_ray(h.point, sd);
    ohit h2;
    memset(&h2, 0, sizeof(h2));
    (void)r;
    tl_rays++;
    if (bvh_hit(x->b, &r2, 0.0001, INFINITY, &h2, 1))
        return vadd(light, vemul(shade(x, r2, h2, depth, g), col));
    return vadd(light, vemul(miss_color(x, &r2), col));
}

static void render_row(void *c, int64_t job) {
    render_ctx *x = (render_ctx *)c;
    int32_t w = x->rd->width, hgt = x->rd->height;
    int64_t pass = job / hgt, y = job % hgt;
    xrng g;
    xseed(&g, x->rd->seed, (uint64_t)pass + 1, (uint64_t)y + 1);
    tl_rays = w; /* one primary ray per pixel */
    for (int32_t px = 0; px < w; px++) {
        double s = ((double)px + xf64(&g)) / (double)(w - 1); /* RandomSampling render.go:201-205 */
        double t = ((double)y + xf64(&g)) / (double)(hgt - 1);
        oray r = make_ray(x->cam.origin, cam_dir(&x->cam, s, t));
        ohit h;
        memset(&h, 0, sizeof(h));
        v3 col;
        if (bvh_hit(x->b, &r, 0.001, INFINITY, &h, 1)) col = shade(x, r, h, 0, &g);
        else col = miss_color(x, &r);
        int64_t p = y * w + px;
        /* Pixel.addSample running mean (buffer.go:19-26).  Rows of one pass
         * are distinct jobs; passes of one row are serialised by the
         * row lock below, which the reference lacks (a known race). */
        double *a = x->acc + 3 * p;
        int32_t n = __atomic_add_fetch(&x->samples[p], 1, __ATOMIC_ACQ_REL);
        if (n == 1) { a[0] = col.x; a[1] = col.y; a[2] = col.z; }
        else {
            a[0] = a[0] + (col.x - a[0]) / n;
            a[1] = a[1] + (col.y - a[1]) / n;
            a[2] = a[2] + (col.z - a[2]) / n;
        }
    }
    atomic_fetch_add(&x->rays, tl_rays);
}

typedef struct { render_ctx *x; int64_t pass; } pass_ctx;
static void pass_row(void *c, int64_t y) {
    pass_ctx *p = (pass_ctx *)c;
    render_row(p->x, p->pass * p->x->rd->height + y);
}

int orc_render(const orc_bvh *b, const int32_t *prim_mat, const int32_t *mat_type, const double *mat_color,
               const double *mat_param, const orc_camera_desc *cam, orc_render_desc *rd, double *rgb) {
    if (rd->width < 2 || rd->height < 2) return ORC_E_ARG;
    render_ctx x;
    x.b = b;
    x.prim_mat = prim_mat;
    x.mat_type = mat_type;
    x.mat_color = mat_color;
    x.mat_param = mat_param;
    x.rd = rd;
    x.cam = make_camera(cam);
    x.acc = rgb;
    atomic_init(&x.rays, 0);
    int64_t np = (int64_t)rd->width * rd->height;
    x.samples = (int32_t *)calloc((size_t)np, sizeof(int32_t));
    if (!x.samples) return ORC_E_NOMEM;
    memset(rgb, 0, (size_t)np * 3 * sizeof(double));
    /* one pass (all rows) at a time, as render.go:120-125 enqueues them; the
     * barrier between passes keeps each pixel's samples serial */
    for (int64_t pass = 0; pass < rd->spp; pass++) {
        pass_ctx pc = {&x, pass};
        orc_parallel(rd->threads, rd->height, pass_row, &pc);
    }
    rd->rays_traced = atomic_load(&x.rays);
    free(x.samples);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* float64 adjoint with the GPU's random numbers                             */
/* ------------------------------------------------------------------------ */
/* Philox-2x32-10 (Salmon et al., SC'11), as the device code uses it */
static void philox2x32(uint32_t c0, uint32_t c1, uint32_t key, uint32_t out[2]) {
    for (int i = 0; i < 10; i++) {
        uint64_t prod = (uint64_t)0xD256D193u * c0;
        uint32_t hi = (uint32_t)(prod >> 32), lo = (uint32_t)prod;
        c0 = hi ^ key ^ c1;
        c1 = lo;
        key += 0x9E3779B9u;
    }
    out[0] = c0;
    out[1] = c1;
}
static double u01_24(uint32_t x) { return (double)(x >> 8) * (1.0 / 16777216.0); }

typedef struct { int tri; v3 P, a; } adj_vertex;

typedef struct {
    const orc_bvh *b;
    const orc_render_desc *rd;
    ocam cam;
    const float *albedo, *emission, *dimg;
    double *img, *ga, *ge;
    pthread_mutex_t lock;
} adj_ctx;

/* one path: vertices, radiance L and the miss colour after the last vertex */
static int adj_path(const adj_ctx *x, uint32_t g, adj_vertex *vx, int maxv, v3 *L, v3 *miss) {
    const orc_render_desc *rd = x->rd;
    uint32_t npix = (uint32_t)rd->width * (uint32_t)rd->height, key = (uint32_t)rd->seed ^ (uint32_t)(rd->seed >> 32);
    uint32_t pix = g % npix, px = pix % (uint32_t)rd->width, py = pix / (uint32_t)rd->width;
    uint32_t rnd[2];
    philox2x32(g, 0xFFFFu, key, rnd);
    double s = ((double)px + u01_24(rnd[0])) / (double)(rd->width - 1);
    double t = ((double)py + u01_24(rnd[1])) / (double)(rd->height - 1);
    oray r = make_ray(x->cam.origin, cam_dir(&x->cam, s, t));
    double tmin = 0.001;
    v3 T = mk(1, 1, 1);
    *L = mk(0, 0, 0);
    *miss = mk(0, 0, 0);
    int nv = 0;
    for (int level = 0;; level++) {
        ohit h;
        memset(&h, 0, sizeof(h));
        if (!bvh_hit(x->b, &r, tmin, INFINITY, &h, 0)) {
            render_ctx rc;
            memset(&rc, 0, sizeof(rc));
            rc.rd = rd;
            *miss = miss_color(&rc, &r);
            *L = vadd(*L, vemul(T, *miss));
            break;
        }
        if (level > rd->max_depth || nv >= maxv) break;
        int tri = h.prim;
        double e = x->emission[tri];
        v3 a = mk(x->albedo[3 * tri], x->albedo[3 * tri + 1], x->albedo[3 * tri + 2]);
        vx[nv].tri = tri;
        vx[nv].P = T;
        vx[nv].a = a;
        nv++;
        *L = vadd(*L, vmul(T, e));
        /* geometric normal facing the ray, then normal + uniform unit vector */
        const double *tv = x->b->tri + 9 * (int64_t)tri;
        v3 v0 = mk(tv[0], tv[1], tv[2]);
        v3 ng = vcross(vsub(mk(tv[3], tv[4], tv[5]), v0), vsub(mk(tv[6], tv[7], tv[8]), v0));
        v3 n = vunit(ng);
        if (!(vdot(r.d, ng) < 0)) n = vmul(n, -1);
        philox2x32(g, (uint32_t)level, key, rnd);
        double z = 1.0 - 2.0 * u01_24(rnd[0]);
        double rr = sqrt(fmax(0.0, 1.0 - z * z));
        double phi = 2.0 * M_PI * u01_24(rnd[1]);
        v3 sd = mk(n.x + rr * cos(phi), n.y + rr * sin(phi), n.z + z);
        if (fabs(sd.x) <= ORC_APPROX_THRESH && fabs(sd.y) <= ORC_APPROX_THRESH && fabs(sd.z) <= ORC_APPROX_THRESH) sd = n;
        v3 p = vadd(r.o, vmul(r.d, h.t));
        T = vemul(T, a);
        r = make_ray(p, sd);
        tmin = 0.0001;
    }
    return nv;
}

static void adj_row(void *c, int64_t y) {
    adj_ctx *x = (adj_ctx *)c;
    const orc_render_desc *rd = x->rd;
    const uint32_t npix = (uint32_t)rd->width * (uint32_t)rd->height;
    enum { MAXV = 16 };
    adj_vertex vx[MAXV];
    v3 S[MAXV];
    int n_tri = (int)x->b->n_tri;
    double *ga = (double *)calloc((size_t)n_tri * 3, sizeof(double));
    double *ge = (double *)calloc((size_t)n_tri, sizeof(double));
    for (int32_t px = 0; px < rd->width; px++) {
        uint32_t pix = (uint32_t)y * (uint32_t)rd->width + (uint32_t)px;
        v3 sum = mk(0, 0, 0);
        v3 delta = mk(0, 0, 0);
        if (x->dimg)
            delta = mk(x->dimg[3 * pix] / rd->spp, x->dimg[3 * pix + 1] / rd->spp, x->dimg[3 * pix + 2] / rd->spp);
        for (int32_t s = 0; s < rd->spp; s++) {
            v3 L, m;
            int nv = adj_path(x, (uint32_t)s * npix + pix, vx, MAXV, &L, &m);
            sum = vadd(sum, L);
            if (!x->dimg) continue;
            v3 acc = m;
            for (int i = nv - 1; i >= 0; i--) {
                S[i] = acc;
                double e = x->emission[vx[i].tri];
                acc = vadd(mk(e, e, e), vemul(vx[i].a, acc));
            }
            for (int i = 0; i < nv; i++) {
                int t = vx[i].tri;
                v3 P = vx[i].P;
                ga[3 * t] += delta.x * P.x * S[i].x;
                ga[3 * t + 1] += delta.y * P.y * S[i].y;
                ga[3 * t + 2] += delta.z * P.z * S[i].z;
                ge[t] += delta.x * P.x + delta.y * P.y + delta.z * P.z;
            }
        }
        x->img[3 * pix] = sum.x / rd->spp;
        x->img[3 * pix + 1] = sum.y / rd->spp;
        x->img[3 * pix + 2] = sum.z / rd->spp;
    }
    if (x->dimg) {
        pthread_mutex_lock(&x->lock);
        for (int t = 0; t < n_tri; t++) {
            x->ga[3 * t] += ga[3 * t];
            x->ga[3 * t + 1] += ga[3 * t + 1];
            x->ga[3 * t + 2] += ga[3 * t + 2];
            x->ge[t] += ge[t];
        }
        pthread_mutex_unlock(&x->lock);
    }
    free(ga);
    free(ge);
}

int orc_adjoint(const orc_bvh *b, const orc_camera_desc *cam, const orc_render_desc *rd, const float *albedo,
                const float *emission, const float *dimg, double *img, double *g_albedo, double *g_emission) {
    if (b->n_sph || rd->width < 2 || rd->height < 2 || rd->spp < 1) return ORC_E_ARG;
    adj_ctx x;
    x.b = b;
    x.rd = rd;
    x.cam = make_camera(cam);
    x.albedo = albedo;
    x.emission = emission;
    x.dimg = dimg;
    x.img = img;
    x.ga = g_albedo;
    x.ge = g_emission;
    pthread_mutex_init(&x.lock, NULL);
    if (dimg) {
        memset(g_albedo, 0, (size_t)b->n_tri * 3 * sizeof(double));
        memset(g_emission, 0, (size_t)b->n_tri * sizeof(double));
    }
    orc_parallel(rd->threads, rd->height, adj_row, &x);
    pthread_mutex_destroy(&x.lock);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* PHR: phr.go:42-459                                                        */
/* ------------------------------------------------------------------------ */
/* A cut holds aux-node ids (>= 0) or, for a one-node cut made by makeLeaf,
 * the encoded output-node id -(id+1). */
typedef struct {
    int32_t *nodes;
    int64_t n;
    double box[6];
    int32_t depth;
} ocut;

typedef struct {
    orc_bvh *aux;
    orc_bvh *out;
    double alpha, delta, S;
    int bf;
    double *bc;     /* aux barycenters, 3 per node */
    int64_t max_cut;
    int64_t initial;
    int64_t build_cost; /* BuildWithCost's count (phr.go:154-255) */
    /* scratch for minCost */
    double *rbox;
    double *rcost;
    int64_t scratch_cap;
} phr_ctx;

/* DefaultThreshold (phr.go:356-358) */
static double threshold(const phr_ctx *p, int depth) {
    return p->S / pow(2, p->alpha * (double)depth + p->delta);
}

/* collectLeaves (bvh.go:169-177) appended into a prim list (makeLeaf, phr.go:340-352) */
static int collect_prims(const orc_bvh *aux, int32_t ni, int32_t **buf, int64_t *n, int64_t *cap) {
    int64_t scap = 64, top = 0;
    int32_t *st = (int32_t *)malloc((size_t)scap * sizeof(int32_t));
    if (!st) return ORC_E_NOMEM;
    st[top++] = ni;
    while (top > 0) {
        int32_t c = st[--top];
        const orc_node *nd = &aux->nodes[c];
        if (nd->is_leaf) {
            if (grow((void **)buf, cap, *n + nd->prim_count, sizeof(int32_t))) { free(st); return ORC_E_NOMEM; }
            memcpy(*buf + *n, aux->prims + nd->prim_first, (size_t)nd->prim_count * sizeof(int32_t));
            *n += nd->prim_count;
            continue;
        }
        if (top + nd->nchild > scap) {
            while (top + nd->nchild > scap) scap *= 2;
            int32_t *q = (int32_t *)realloc(st, (size_t)scap * sizeof(int32_t));
            if (!q) { free(st); return ORC_E_NOMEM; }
            st = q;
        }
        for (int k = nd->nchild - 1; k >= 0; k--) st[top++] = kid(aux, c, k);
    }
    free(st);
    return ORC_OK;
}

/* makeLeaf (phr.go:340-352): returns the new output leaf id */
static int32_t make_leaf(phr_ctx *p, const double *box, const int32_t *nodes, int64_t n) {
    int32_t *buf = NULL;
    int64_t cnt = 0, cap = 0;
    for (int64_t i = 0; i < n; i++) {
        if (nodes[i] < 0) { /* an already-made output leaf */
            const orc_node *m = &p->out->nodes[-nodes[i] - 1];
            if (grow((void **)&buf, &cap, cnt + m->prim_count, sizeof(int32_t))) { free(buf); return -1; }
            memcpy(buf + cnt, p->out->prims + m->prim_first, (size_t)m->prim_count * sizeof(int32_t));
            cnt += m->prim_count;
        } else if (collect_prims(p->aux, nodes[i], &buf, &cnt, &cap)) {
            free(buf);
            return -1;
        }
    }
    int32_t id = new_leaf(p->out, buf, cnt);
    free(buf);
    if (id >= 0) memcpy(p->out->nodes[id].box, box, 6 * sizeof(double));
    return id;
}

/* copy of an aux leaf into the output tree (the Go tree shares the node) */
static int32_t adopt_leaf(phr_ctx *p, int32_t enc) {
    if (enc < 0) return -enc - 1;
    const orc_node *a = &p->aux->nodes[enc];
    if (!a->is_leaf) { /* a one-node cut holding an inner node cannot arise; flatten defensively */
        return make_leaf(p, a->box, &enc, 1);
    }
    int32_t id = new_leaf(p->out, p->aux->prims + a->prim_first, a->prim_count);
    if (id >= 0) memcpy(p->out->nodes[id].box, a->box, 6 * sizeof(double));
    return id;
}

static const double *cut_node_box(const phr_ctx *p, int32_t enc) {
    return enc >= 0 ? p->aux->nodes[enc].box : p->out->nodes[-enc - 1].box;
}
static int64_t cut_node_size(phr_ctx *p, int32_t enc) {
    return enc >= 0 ? subtree_size(p->aux, enc) : 1;
}

/* refined (phr.go:313-338); consumes c->nodes */
static int refine(phr_ctx *p, const ocut *c, ocut *out) {
    double thr = threshold(p, c->depth);
    int64_t cap = c->n * 2 + 4, n = 0;
    int32_t *r = (int32_t *)malloc((size_t)cap * sizeof(int32_t));
    if (!r) return ORC_E_NOMEM;
    for (int64_t i = 0; i < c->n; i++) {
        int32_t e = c->nodes[i];
        if (e < 0 || p->aux->nodes[e].is_leaf || orc_surface(p->aux->nodes[e].box) < thr) {
            if (grow((void **)&r, &cap, n + 1, sizeof(int32_t))) { free(r); return ORC_E_NOMEM; }
            r[n++] = e;
        } else {
            const orc_node *a = &p->aux->nodes[e];
            if (grow((void **)&r, &cap, n + a->nchild, sizeof(int32_t))) { free(r); return ORC_E_NOMEM; }
            for (int k = 0; k < a->nchild; k++) r[n++] = kid(p->aux, e, k);
        }
    }
    if (n == 1) {
        int32_t leaf = make_leaf(p, c->box, r, 1);
        if (leaf < 0) { free(r); return ORC_E_NOMEM; }
        r[0] = -leaf - 1;
    }
    out->nodes = r;
    out->n = n;
    memcpy(out->box, c->box, sizeof(out->box));
    out->depth = c->depth + 1;
    if (n > p->max_cut) p->max_cut = n;
    return ORC_OK;
}

/* stable merge sort of cut entries by barycenter component (sort.SliceStable) */
static void stable_sort(phr_ctx *p, int32_t *a, int64_t n, int axis, int32_t *tmp) {
    if (n < 2) return;
    for (int64_t w = 1; w < n; w *= 2) {
        for (int64_t lo = 0; lo < n; lo += 2 * w) {
            int64_t mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
            int64_t i = lo, j = mid, k = lo;
            while (i < mid && j < hi) {
                double ki = p->bc[3 * (int64_t)a[i] + axis], kj = p->bc[3 * (int64_t)a[j] + axis];
                if (kj < ki) tmp[k++] = a[j++];
                else tmp[k++] = a[i++];
            }
            while (i < mid) tmp[k++] = a[i++];
            while (j < hi) tmp[k++] = a[j++];
        }
        memcpy(a, tmp, (size_t)n * sizeof(int32_t));
    }
}

typedef struct { double cost; int64_t split; double lbox[6], rbox[6]; } osah;

/* minCost (phr.go:414-459) */
static osah min_cost(phr_ctx *p, const int32_t *s, int64_t n, const double *bounding) {
    osah best;
    double *rb = p->rbox, *rc = p->rcost;
    double sa_right[6];
    memcpy(sa_right, cut_node_box(p, s[n - 1]), sizeof(sa_right));
    int64_t count = 0;
    for (int64_t i = n - 1; i > 0; i--) {
        box_add(sa_right, sa_right, cut_node_box(p, s[i]));
        count += cut_node_size(p, s[i]);
        rc[i] = orc_surface(sa_right) * (double)count;
        memcpy(rb + 6 * i, sa_right, sizeof(sa_right));
    }
    count += cut_node_size(p, s[0]);
    best.cost = orc_surface(bounding) * (double)count;
    best.split = 0;
    memcpy(best.lbox, bounding, sizeof(best.lbox));
    count = cut_node_size(p, s[0]);
    double sa_left[6];
    memcpy(sa_left, cut_node_box(p, s[0]), sizeof(sa_left));
    for (int64_t i = 1; i < n; i++) {
        double cost = rc[i] + orc_surface(sa_left) * (double)count;
        if (cost < best.cost) {
            best.cost = cost;
            best.split = i;
            memcpy(best.lbox, sa_left, sizeof(sa_left));
            memcpy(best.rbox, rb + 6 * i, sizeof(sa_left));
        }
        box_add(sa_left, sa_left, cut_node_box(p, s[i]));
        count += cut_node_size(p, s[i]);
    }
    return best;
}

/* SweepSAH (phr.go:368-405).  Produces the left and right cuts (right.n == 0
 * when not splitting is cheapest).  Reproduces which array each axis sorts
 * from, since that fixes the tie order of equal barycenters. */
static int sweep_sah(phr_ctx *p, ocut *c, ocut *left, ocut *right) {
    int64_t n = c->n;
    if (p->scratch_cap < n) {
        free(p->rbox);
        free(p->rcost);
        p->rbox = (double *)malloc((size_t)n * 6 * sizeof(double));
        p->rcost = (double *)malloc((size_t)n * sizeof(double));
        p->scratch_cap = n;
        if (!p->rbox || !p->rcost) return ORC_E_NOMEM;
    }
    int32_t *a = c->nodes;
    int32_t *s2 = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *tmp = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    if (!s2 || !tmp) { free(s2); free(tmp); return ORC_E_NOMEM; }
    stable_sort(p, a, n, 0, tmp);
    memcpy(s2, a, (size_t)n * sizeof(int32_t));
    stable_sort(p, s2, n, 1, tmp);
    osah xs = min_cost(p, a, n, c->box);
    osah ys = min_cost(p, s2, n, c->box);
    osah win;
    const int32_t *arr;
    if (xs.cost < ys.cost) {
        stable_sort(p, s2, n, 2, tmp);
        osah zs = min_cost(p, s2, n, c->box);
        if (xs.cost < zs.cost) { win = xs; arr = a; }
        else { win = zs; arr = s2; }
    } else {
        stable_sort(p, a, n, 2, tmp);
        osah zs = min_cost(p, a, n, c->box);
        if (ys.cost < zs.cost) { win = ys; arr = s2; }
        else { win = zs; arr = a; }
    }
    int64_t k = win.split == 0 ? n : win.split;
    left->nodes = (int32_t *)malloc((size_t)k * sizeof(int32_t));
    memcpy(left->nodes, arr, (size_t)k * sizeof(int32_t));
    left->n = k;
    memcpy(left->box, win.lbox, sizeof(left->box));
    left->depth = c->depth;
    if (win.split == 0) {
        right->nodes = NULL;
        right->n = 0;
    } else {
        right->nodes = (int32_t *)malloc((size_t)(n - k) * sizeof(int32_t));
        memcpy(right->nodes, arr + k, (size_t)(n - k) * sizeof(int32_t));
        right->n = n - k;
        memcpy(right->box, win.rbox, sizeof(right->box));
        right->depth = c->depth;
    }
    free(s2);
    free(tmp);
    return ORC_OK;
}

typedef struct { ocut cut; int32_t parent; int32_t slot; } phr_job;

/* buildSubTree (phr.go:92-152), jobs from an explicit stack */
static int build_subtrees(phr_ctx *p, ocut initial) {
    int64_t cap = 256, top = 0;
    phr_job *st = (phr_job *)malloc((size_t)cap * sizeof(phr_job));
    if (!st) return ORC_E_NOMEM;
    st[top].cut = initial;
    st[top].parent = -1;
    st[top].slot = 0;
    top++;
    ocut *cuts = (ocut *)malloc((size_t)(p->bf > 1 ? p->bf : 2) * sizeof(ocut));
    int rc = ORC_OK;
    while (top > 0 && rc == ORC_OK) {
        phr_job j = st[--top];
        if (j.cut.n <= 1) {
            int32_t leaf = adopt_leaf(p, j.cut.nodes[0]);
            free(j.cut.nodes);
            if (leaf < 0) { rc = ORC_E_NOMEM; break; }
            add_child(p->out, j.parent, leaf, j.slot);
            continue;
        }
        int nc = 1;
        cuts[0] = j.cut; /* the first split below always consumes it (bf >= 2) */
        while (nc < p->bf) {
            int64_t mx = 0;
            int mi = 0;
            for (int i = 0; i < nc; i++)
                if (cuts[i].n > mx) { mx = cuts[i].n; mi = i; }
            if (mx <= 1) break;
            p->build_cost += mx; /* buildSubTreeCost, phr.go:214 */
            ocut L, R;
            rc = sweep_sah(p, &cuts[mi], &L, &R);
            if (rc) break;
            free(cuts[mi].nodes);
            if (R.n > 0) {
                ocut rl, rr;
                rc = refine(p, &L, &rl);
                if (!rc) rc = refine(p, &R, &rr);
                free(L.nodes);
                free(R.nodes);
                if (rc) break;
                cuts[mi] = rl;
                cuts[nc++] = rr;
            } else {
                int32_t leaf = make_leaf(p, L.box, L.nodes, L.n);
                free(L.nodes);
                if (leaf < 0) { rc = ORC_E_NOMEM; break; }
                cuts[mi].nodes = (int32_t *)malloc(sizeof(int32_t));
                cuts[mi].nodes[0] = -leaf - 1;
                cuts[mi].n = 1;
                cuts[mi].depth = 0;
                memset(cuts[mi].box, 0, sizeof(cuts[mi].box));
            }
        }
        if (rc) break;
        int32_t br = new_branch(p->out, nc);
        if (br < 0) { rc = ORC_E_NOMEM; break; }
        memcpy(p->out->nodes[br].box, j.cut.box, 6 * sizeof(double));
        add_child(p->out, j.parent, br, j.slot);
        if (top + nc > cap) {
            while (top + nc > cap) cap *= 2;
            phr_job *q = (phr_job *)realloc(st, (size_t)cap * sizeof(phr_job));
            if (!q) { rc = ORC_E_NOMEM; break; }
            st = q;
        }
        for (int i = nc - 1; i >= 0; i--) {
            st[top].cut = cuts[i];
            st[top].parent = br;
            st[top].slot = i;
            top++;
        }
    }
    for (int64_t i = 0; i < top; i++) free(st[i].cut.nodes);
    free(cuts);
    free(st);
    return rc;
}

/* findInitialCut / processNodeInitialCut (phr.go:257-311) in FIFO order */
static int initial_cut(phr_ctx *p, ocut *c) {
    const orc_bvh *a = p->aux;
    int64_t cap = 1024, head = 0, tail = 0, n = 0, ccap = 1024;
    int32_t *q = (int32_t *)malloc((size_t)cap * sizeof(int32_t));
    int32_t *cut = (int32_t *)malloc((size_t)ccap * sizeof(int32_t));
    if (!q || !cut) { free(q); free(cut); return ORC_E_NOMEM; }
    double thr0 = threshold(p, 0);
    int64_t counter = 0;
    q[tail++] = a->root;
    while (head < tail) {
        int32_t ni = q[head++];
        const orc_node *nd = &a->nodes[ni];
        int add = 0;
        if (nd->is_leaf) add = 1;
        else if (orc_surface(nd->box) > thr0) {
            counter += nd->nchild - 1;
            if (counter >= ORC_MAX_CUT_SIZE) add = 1;
            else {
                if (tail + nd->nchild > cap) {
                    /* compact the consumed head, then grow */
                    memmove(q, q + head, (size_t)(tail - head) * sizeof(int32_t));
                    tail -= head;
                    head = 0;
                    while (tail + nd->nchild > cap) cap *= 2;
                    int32_t *qq = (int32_t *)realloc(q, (size_t)cap * sizeof(int32_t));
                    if (!qq) { free(q); free(cut); return ORC_E_NOMEM; }
                    q = qq;
                }
                for (int k = 0; k < nd->nchild; k++) q[tail++] = kid(a, ni, k);
            }
        } else add = 1;
        if (add) {
            if (grow((void **)&cut, &ccap, n + 1, sizeof(int32_t))) { free(q); free(cut); return ORC_E_NOMEM; }
            cut[n++] = ni;
        }
    }
    free(q);
    c->nodes = cut;
    c->n = n;
    memcpy(c->box, a->nodes[a->root].box, sizeof(c->box));
    c->depth = 1;
    return ORC_OK;
}

/* PhrBuilder.BuildFromAuxilary (phr.go:47-84) */
int orc_phr_build(const orc_bvh *aux, double alpha, double delta, int bf, orc_bvh **out, int64_t stats[5]) {
    *out = NULL;
    if (bf < 2 || bf > ORC_MAX_ARITY) return ORC_E_ARG;
    orc_bvh *o = (orc_bvh *)calloc(1, sizeof(orc_bvh));
    if (!o) return ORC_E_NOMEM;
    /* share the scene by copy so that the output can be traced on its own */
    int64_t n = aux->n_tri + aux->n_sph;
    o->n_tri = aux->n_tri;
    o->n_sph = aux->n_sph;
    o->tri = (double *)malloc((size_t)(aux->n_tri > 0 ? aux->n_tri : 1) * 9 * sizeof(double));
    o->tri_nrm = (double *)malloc((size_t)(aux->n_tri > 0 ? aux->n_tri : 1) * 9 * sizeof(double));
    o->sph = (double *)malloc((size_t)(aux->n_sph > 0 ? aux->n_sph : 1) * 4 * sizeof(double));
    o->pbox = (double *)malloc((size_t)(n > 0 ? n : 1) * 6 * sizeof(double));
    if (!o->tri || !o->tri_nrm || !o->sph || !o->pbox) { orc_bvh_free(o); return ORC_E_NOMEM; }
    memcpy(o->tri, aux->tri, (size_t)aux->n_tri * 9 * sizeof(double));
    memcpy(o->tri_nrm, aux->tri_nrm, (size_t)aux->n_tri * 9 * sizeof(double));
    memcpy(o->sph, aux->sph, (size_t)aux->n_sph * 4 * sizeof(double));
    memcpy(o->pbox, aux->pbox, (size_t)n * 6 * sizeof(double));

    phr_ctx p;
    memset(&p, 0, sizeof(p));
    p.aux = (orc_bvh *)aux; /* subtree sizes are cached into aux, like node.size in Go */
    p.out = o;
    p.alpha = alpha;
    p.delta = delta;
    p.bf = bf;
    p.S = orc_surface(aux->nodes[aux->root].box);
    p.bc = (double *)malloc((size_t)aux->n_nodes * 3 * sizeof(double));
    if (!p.bc) { orc_bvh_free(o); return ORC_E_NOMEM; }
    for (int64_t i = 0; i < aux->n_nodes; i++)
        for (int k = 0; k < 3; k++) p.bc[3 * i + k] = bary(aux->nodes[i].box, k);
    subtree_size(p.aux, aux->root);
    ocut c0;
    int rc = initial_cut(&p, &c0);
    if (!rc) {
        p.initial = c0.n;
        p.max_cut = c0.n;
        p.build_cost = c0.n; /* BuildWithCost, phr.go:159 */
        rc = build_subtrees(&p, c0);
    }
    free(p.bc);
    free(p.rbox);
    free(p.rcost);
    if (rc) { orc_bvh_free(o); return rc; }
    if (stats) {
        int64_t cnt[4];
        orc_bvh_counts(o, cnt);
        stats[0] = p.initial;
        stats[1] = p.max_cut;
        stats[2] = cnt[0];
        stats[3] = cnt[1];
        stats[4] = p.build_cost;
    }
    *out = o;
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* ToImage (buffer.go:60-69, 104-116) and Color.goColor (math.go:20-25)      */
/* ------------------------------------------------------------------------ */
/* Clamp (util.go:32-40): NaN compares false both ways and passes through */
static double orc_clamp(double v, double lo, double hi) {
    if (v < lo) return lo;
    if (v > hi) return hi;
    return v;
}

/* uint8(Clamp(math.Sqrt(c), 0, 1) * 255): Go truncates toward zero; a NaN gives 0 on
 * amd64 and arm64 alike */
static uint8_t orc_go_channel(double c) {
    double v = orc_clamp(sqrt(c), 0.0, 1.0) * 255.0;
    if (v != v) return 0;
    return (uint8_t)(int)v;
}

void orc_to_image(const float *rgb, int32_t width, int32_t height, uint8_t *rgba) {
    /* image.NewRGBA starts zeroed; img.Set outside the rectangle is a no-op */
    memset(rgba, 0, (size_t)width * height * 4);
    for (int64_t i = 0; i < (int64_t)width * height; i++) {
        int64_t x = i % width;
        int64_t y = height - i / width; /* buffer.go:65: row 0 maps to y = height, outside */
        if (y < 0 || y >= height) continue;
        uint8_t *px = rgba + 4 * (y * width + x);
        px[0] = orc_go_channel((double)rgb[3 * i]);
        px[1] = orc_go_channel((double)rgb[3 * i + 1]);
        px[2] = orc_go_channel((double)rgb[3 * i + 2]);
        px[3] = 255;
    }
}
