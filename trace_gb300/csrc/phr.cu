// PHR refinement on the device: pkg/pt/phr.go:47-459 (BuildFromAuxilary).
//
//   k_aux_build      unified view of the LBVH (inner nodes and leaves) with
//                    boxes, subtree sizes (bvh.go:159-167) and primitive ranges,
//                    and whether every box coordinate lies in the range where
//                    the float32 screening of phr_exact.cuh holds
//   k_initial_cut    findInitialCut (phr.go:257-311), breadth-first in FIFO
//                    order with the MAX_CUT_SIZE cap, one block
//   k_phr_level      buildSubTree (phr.go:92-152), one launch per tree level:
//                      SweepSAH (phr.go:368-405): three stable sorts by
//                      barycenter, chained x -> y -> z as the Go code chains
//                      them, each followed by minCost (phr.go:414-459): a
//                      prefix/suffix sweep of boxes and subtree sizes whose
//                      costs are taken in float32 and decided exactly, with
//                      float64 only where the float32 values cannot settle a
//                      comparison (phr_exact.cuh);
//                      refined (phr.go:313-338) and makeLeaf (phr.go:340-352).
//                    Cuts of 2..LANE_CUT nodes (bf = 2) are swept by one lane
//                    each, larger ones by a warp, the largest by a block.
//   k_phr_finalize   the N-ary tree into 64-byte binary or 128-byte 4-wide nodes
//
// The result is the oracle's tree exactly: same splits, same tie orders, same
// leaves, so SAH cost and hit ids agree with it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "gbt_internal.cuh"
#include "phr_exact.cuh"

namespace {

constexpr uint32_t MAX_CUT_SIZE = 2500;  // phr.go:11
constexpr int PT = 256;                  // threads per job block
constexpr int WIDE = 512;                // threads per job block on levels of a few large cuts
constexpr uint32_t SORT_SMEM_MAX = 8192; // largest padded cut sorted in shared memory (96 KB)
constexpr int SPEC_LEVELS = 8;           // small-cut levels launched per readback
#ifndef GBT_PHR_SPEC_BIG
#define GBT_PHR_SPEC_BIG 3                // levels of larger cuts launched per readback (branching 2)
#endif
constexpr int DEPTH_TABLE = 4096;
// Cuts of at most this many nodes are swept by a single lane (bf = 2): most
// cuts are that small (on a 1M-triangle soup 93% of the splits sort 2-16
// nodes), and a warp then works on 32 of them at once.
constexpr uint32_t LANE_CUT = 16;
// The same for the lane path of bf > 2, whose jobs' later cuts can double.
constexpr uint32_t LANE_CUT_MULTI = 32;
// Largest branching factor the lane path serves (its per-lane cut table).
constexpr int MAX_BF_LANES = 4;
// Longer record ranges of the lane path's leaves are copied by the whole warp.
constexpr uint32_t LANE_COPY = 8;

// An auxiliary-tree node in two parts: what every sweep reads (32 bytes, one
// sector) and what only leaves and refinements read.
struct AuxNode {
    float lo[3], hi[3];
    uint32_t size;  // subtree size (bvh.go:159-167)
    int32_t c0;     // first child, -1 for a leaf
};
struct AuxCold {
    uint32_t first, count;  // the subtree's primitive records
    int32_t c1;             // second child
    uint32_t pad;
};

struct PJob {
    uint32_t off, n;
    float lo[3], hi[3];
    int32_t depth, parent, slot, pad;
};

struct PNode {
    float lo[3], hi[3];
    int32_t leaf, nchild;
    int32_t child[4];
    uint32_t rec_off, rec_cnt;
};

struct PhrGlobals {
    uint32_t pnode_ctr, rec_ctr;
    int32_t root;
    uint32_t screen_bad;  // 1: some box coordinate is outside the float32 screening range
    uint32_t job_ctr[2], pool_ctr[2], max_n[2];
    unsigned long long build_cost;  // sizes of the cuts handed to Split (phr.go:214)
    // Jobs of a level are kept in two lists in one array: cuts a single lane
    // sweeps (2..LANE_CUT nodes, bf = 2) from the front (job_ctr), the others
    // from the back (job_big_ctr).
    uint32_t job_big_ctr[2];
    // Levels run in batches launched without waiting (bookkeeping in k_phr_level):
    uint32_t level_done;   // levels completed
    uint32_t blocks_done;  // blocks of the running level that have finished
    uint32_t stall;        // a launch found cuts beyond its capacity and did nothing
    uint32_t err_copy;     // the device error word when the last level completed
};

// ---------------------------------------------------------------------------
// float64 helpers, every operation rounded on its own (no contraction)
// ---------------------------------------------------------------------------
// aabb.surface (bounding.go:45-47) of a float32 box evaluated in float64
__device__ __forceinline__ double surface(const float *lo, const float *hi) {
    double w = __dsub_rn((double)hi[0], (double)lo[0]);
    double h = __dsub_rn((double)hi[1], (double)lo[1]);
    double d = __dsub_rn((double)hi[2], (double)lo[2]);
    double a = __dmul_rn(__dmul_rn(2.0, w), h);
    double b = __dmul_rn(__dmul_rn(2.0, w), d);
    double c = __dmul_rn(__dmul_rn(2.0, h), d);
    return __dadd_rn(__dadd_rn(a, b), c);
}



// The float64 paths below are taken rarely (inside the float32 screening
// band, or without screening).  Kept out of line, so that the compiler branches
// around them instead of predicating their float64 operations into every pass.
__device__ __noinline__ bool surface_below(const float *lo, const float *hi, double thr) {
    return surface(lo, hi) < thr;
}

// minCost's float64 cost of a split (phr.go:423-445): right box and count, left box and count.
__device__ __noinline__ double split_cost64(float rl0, float rl1, float rl2, float rh0, float rh1, float rh2,
                                            uint32_t rc, float ll0, float ll1, float ll2, float lh0, float lh1,
                                            float lh2, uint32_t lc) {
    const float rl[3] = {rl0, rl1, rl2}, rh[3] = {rh0, rh1, rh2};
    const float ll[3] = {ll0, ll1, ll2}, lh[3] = {lh0, lh1, lh2};
    const double rcost = __dmul_rn(surface(rl, rh), (double)rc);
    return __dadd_rn(rcost, __dmul_rn(surface(ll, lh), (double)lc));
}

struct BoxAgg {
    float lo[3], hi[3];
    uint32_t c;
};

__device__ __forceinline__ BoxAgg agg_identity() {
    BoxAgg a;
    a.lo[0] = a.lo[1] = a.lo[2] = INFINITY;
    a.hi[0] = a.hi[1] = a.hi[2] = -INFINITY;
    a.c = 0;
    return a;
}

__device__ __forceinline__ BoxAgg agg_join(const BoxAgg &a, const BoxAgg &b) {
    BoxAgg r;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        r.lo[k] = fminf(a.lo[k], b.lo[k]);
        r.hi[k] = fmaxf(a.hi[k], b.hi[k]);
    }
    r.c = a.c + b.c;
    return r;
}

__device__ __forceinline__ BoxAgg agg_shfl_up(const BoxAgg &a, int o) {
    BoxAgg r;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        r.lo[k] = __shfl_up_sync(0xffffffffu, a.lo[k], o);
        r.hi[k] = __shfl_up_sync(0xffffffffu, a.hi[k], o);
    }
    r.c = __shfl_up_sync(0xffffffffu, a.c, o);
    return r;
}

// Exclusive scan of one BoxAgg per thread in the order given by `rank`
// (0..PT-1); blockDim == PT.  s_tmp holds PT/32 aggregates.
__device__ BoxAgg block_scan_agg(BoxAgg v, int rank, BoxAgg *s_tmp, BoxAgg *s_rank) {
    // place by rank so that warps scan consecutive ranks
    s_rank[rank] = v;
    __syncthreads();
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    BoxAgg x = s_rank[t];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        BoxAgg y = agg_shfl_up(x, o);
        if (lane >= o) x = agg_join(y, x);
    }
    if (lane == 31) s_tmp[w] = x;
    __syncthreads();
    BoxAgg pre = agg_identity();
    for (int j = 0; j < w; j++) pre = agg_join(pre, s_tmp[j]);
    // exclusive value at position t: earlier warps, then earlier lanes (lane-1's inclusive)
    BoxAgg prev = agg_shfl_up(x, 1);
    BoxAgg excl = lane == 0 ? pre : agg_join(pre, prev);
    __syncthreads();
    s_rank[t] = excl;
    __syncthreads();
    BoxAgg out = s_rank[rank];
    __syncthreads();
    return out;
}

__device__ uint32_t block_scan_u32(uint32_t v, uint32_t *s_tmp, uint32_t *total) {
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_tmp[w] = x;
    __syncthreads();
    uint32_t off = 0, tot = 0;
    for (int j = 0; j < (int)(blockDim.x >> 5); j++) {
        uint32_t c = s_tmp[j];
        off += (j < w) ? c : 0u;
        tot += c;
    }
    __syncthreads();
    *total = tot;
    return off + x - v;
}

// ---------------------------------------------------------------------------
// auxiliary tree
// ---------------------------------------------------------------------------
// Inner node k of the LBVH: its children's boxes (and a leaf child's records),
// its first child, subtree size and record range; ok is cleared when a child's
// box leaves the float32 screening range.
__device__ __forceinline__ void aux_build_node(const float4 *__restrict__ nodes, const uint32_t *__restrict__ subtree,
                                               const uint2 *__restrict__ range, const uint32_t *__restrict__ run,
                                               AuxNode *aux, AuxCold *auxc, uint32_t U, uint32_t k, bool &ok) {
    const float4 *nd = nodes + 4 * (size_t)k;
    float4 n0 = nd[0], n1 = nd[1], n2 = nd[2];
    int4 n3 = *reinterpret_cast<const int4 *>(nd + 3);
    int32_t ids[2];
    for (int c = 0; c < 2; c++) {
        float4 xy = c ? n1 : n0;
        float zl = c ? n2.z : n2.x, zh = c ? n2.w : n2.y;
        int32_t ref = c ? n3.z : n3.x, cnt = c ? n3.w : n3.y;
        int32_t id = cnt > 0 ? (int32_t)(U - 1 + k + c) : ref;
        ids[c] = id;
        AuxNode &a = aux[id];
        a.lo[0] = xy.x; a.hi[0] = xy.y; a.lo[1] = xy.z; a.hi[1] = xy.w; a.lo[2] = zl; a.hi[2] = zh;
        const float cs[6] = {xy.x, xy.y, xy.z, xy.w, zl, zh};
        for (int q = 0; q < 6; q++) ok = ok && gbt_phr::phr_screen_ok(cs[q]);
        if (cnt > 0) {
            a.size = 1;
            a.c0 = -1;
            auxc[id].first = (uint32_t)ref;
            auxc[id].count = (uint32_t)cnt;
            auxc[id].c1 = -1;
        }
    }
    AuxNode &me = aux[k];
    me.c0 = ids[0];
    me.size = subtree[k];
    uint2 lr = range[k];
    auxc[k].c1 = ids[1];
    auxc[k].first = run[lr.x];
    auxc[k].count = run[lr.y + 1] - run[lr.x];
}

// Every box it writes is checked against the float32 screening range
// (phr_exact.cuh); g->screen_bad is set when some coordinate is outside.
__global__ void k_aux_build(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes,
                            const uint32_t *__restrict__ subtree, const uint2 *__restrict__ range,
                            const uint32_t *__restrict__ run, AuxNode *aux, AuxCold *auxc, uint32_t U,
                            uint32_t n_prim, PhrGlobals *g) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    bool ok = true;
    auto screen = [&](const AuxNode &a) {
        for (int c = 0; c < 3; c++) ok = ok && gbt_phr::phr_screen_ok(a.lo[c]) && gbt_phr::phr_screen_ok(a.hi[c]);
    };
    if (k == 0) {  // the root's own box lives in the header
        uint32_t rid = hdr->root_cnt > 0 ? 0u : (uint32_t)hdr->root_ref;
        AuxNode &a = aux[rid];
        for (int c = 0; c < 3; c++) {
            a.lo[c] = hdr->root_lo[c];
            a.hi[c] = hdr->root_hi[c];
        }
        screen(a);
        if (hdr->root_cnt > 0) {
            a.size = 1;
            a.c0 = -1;
            auxc[rid].first = 0;
            auxc[rid].count = n_prim;
            auxc[rid].c1 = -1;
        }
    }
    if (U >= 2 && k < U - 1) aux_build_node(nodes, subtree, range, run, aux, auxc, U, k, ok);
    if (__any_sync(0xffffffffu, !ok) && (threadIdx.x & 31) == 0) atomicOr(&g->screen_bad, 1u);
}

// ---------------------------------------------------------------------------
// initial cut: FIFO breadth-first expansion with the MAX_CUT_SIZE cap
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_initial_cut(const AuxNode *__restrict__ aux,
                                                      const AuxCold *__restrict__ auxc, int32_t root, double thr0,
                                                      uint32_t *front_a, uint32_t *front_b, uint32_t *cut,
                                                      PJob *job0, PhrGlobals *g, uint32_t cap) {
    __shared__ uint32_t s_tmp[32];
    __shared__ uint32_t s_nf;
    uint32_t *front = front_a, *next = front_b;
    uint32_t nf = 1, counter = 0, ncut = 0;
    if (threadIdx.x == 0) front[0] = (uint32_t)root;
    __syncthreads();
    while (nf > 0) {
        uint32_t nnext = 0;
        for (uint32_t base = 0; base < nf; base += blockDim.x) {
            uint32_t i = base + threadIdx.x;
            bool valid = i < nf;
            uint32_t id = valid ? front[i] : 0u;
            bool leaf = !valid || aux[id].c0 < 0;
            bool attempt = valid && !leaf && surface(aux[id].lo, aux[id].hi) > thr0;
            uint32_t tot_att, tot_exp, tot_term;
            uint32_t a_ex = block_scan_u32(attempt ? 1u : 0u, s_tmp, &tot_att);
            bool expand = attempt && (counter + a_ex + 1 < MAX_CUT_SIZE);
            bool term = valid && !expand;
            uint32_t e_ex = block_scan_u32(expand ? 1u : 0u, s_tmp, &tot_exp);
            uint32_t t_ex = block_scan_u32(term ? 1u : 0u, s_tmp, &tot_term);
            if (term && ncut + t_ex < cap) cut[ncut + t_ex] = id;
            if (expand && nnext + 2 * e_ex + 1 < cap) {
                next[nnext + 2 * e_ex] = (uint32_t)aux[id].c0;
                next[nnext + 2 * e_ex + 1] = (uint32_t)auxc[id].c1;
            }
            counter += tot_att;
            ncut += tot_term;
            nnext += 2 * tot_exp;
        }
        __syncthreads();
        uint32_t *t = front;
        front = next;
        next = t;
        nf = nnext;
        if (threadIdx.x == 0) s_nf = nf;
        __syncthreads();
        nf = s_nf;
    }
    if (threadIdx.x == 0) {
        job0->off = 0;
        job0->n = ncut;
        const AuxNode &r = aux[root];
        for (int k = 0; k < 3; k++) {
            job0->lo[k] = r.lo[k];
            job0->hi[k] = r.hi[k];
        }
        job0->depth = 1;
        job0->parent = -1;
        job0->slot = 0;
        g->job_ctr[0] = 1;
        g->pool_ctr[0] = ncut;
        g->max_n[0] = ncut;
    }
}

// ---------------------------------------------------------------------------
// one tree level: per-block scratch of the whole-block and warp sweeps
// ---------------------------------------------------------------------------
struct Scratch {
    uint32_t *ids, *ord[3];
    unsigned long long *skey;
    uint32_t *sval;
    float *lb[6], *rb[6];
    uint32_t *lc, *rc, *flag;
    float *c32;  // float32 cost of each split position of the sweep in progress
};

__host__ __device__ inline uint32_t pow2_at_least(uint32_t n) {
    uint32_t p = 1;
    while (p < n) p <<= 1;
    return p;
}

__host__ __device__ inline size_t scratch_bytes_for(uint32_t nmax) {
    size_t P = pow2_at_least(nmax > 0 ? nmax : 1);
    return (size_t)nmax * 4 * 4 + P * 12 + (size_t)nmax * 12 * 4 + (size_t)nmax * 4 * 4 + 256 * 4;
}

__device__ Scratch carve(unsigned char *base, uint32_t nmax) {
    Scratch s;
    uint32_t P = pow2_at_least(nmax > 0 ? nmax : 1);
    unsigned char *p = base;
    s.skey = reinterpret_cast<unsigned long long *>(p);
    p += (size_t)P * 8;
    s.sval = reinterpret_cast<uint32_t *>(p);
    p += (size_t)P * 4;
    s.ids = reinterpret_cast<uint32_t *>(p);
    p += (size_t)nmax * 4;
    for (int k = 0; k < 3; k++) {
        s.ord[k] = reinterpret_cast<uint32_t *>(p);
        p += (size_t)nmax * 4;
    }
    for (int k = 0; k < 6; k++) {
        s.lb[k] = reinterpret_cast<float *>(p);
        p += (size_t)nmax * 4;
    }
    for (int k = 0; k < 6; k++) {
        s.rb[k] = reinterpret_cast<float *>(p);
        p += (size_t)nmax * 4;
    }
    s.lc = reinterpret_cast<uint32_t *>(p);
    p += (size_t)nmax * 4;
    s.rc = reinterpret_cast<uint32_t *>(p);
    p += (size_t)nmax * 4;
    s.flag = reinterpret_cast<uint32_t *>(p);
    p += (size_t)nmax * 4;
    s.c32 = reinterpret_cast<float *>(p);
    return s;
}

// One compare-exchange of the bitonic network on pair (i, i + j) of the shared
// arrays, ascending when (i & k) == 0.
__device__ __forceinline__ void bitonic_cx_shared(unsigned long long *skey, uint32_t *sval, uint32_t i, uint32_t j,
                                                  uint32_t k) {
    const uint32_t l = i + j;
    const unsigned long long ki = skey[i], kl = skey[l];
    const uint32_t vi = sval[i], vl = sval[l];
    const bool gt = ki > kl || (ki == kl && vi > vl);
    if (((i & k) == 0) == gt) {
        skey[i] = kl;
        skey[l] = ki;
        sval[i] = vl;
        sval[l] = vi;
    }
}

// The bitonic network over P = E * blockDim.x (key, position) pairs of the
// shared arrays, E consecutive ones held in each thread's registers: partners
// within a thread (stride below E) swap in registers, partners in other lanes
// of the warp (stride below 32 E) are read through shuffles, and only wider
// strides go through the shared arrays, with a barrier per stage.  The pairs
// (key, position) are distinct, so the order is the one any sort gives.
template <int E>
__device__ void bitonic_regs(unsigned long long *skey, uint32_t *sval, uint32_t P) {
    const uint32_t t = threadIdx.x, base = t * E;
    unsigned long long k[E];
    uint32_t v[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
        k[e] = skey[base + e];
        v[e] = sval[base + e];
    }
    for (uint32_t kk = 2; kk <= P; kk <<= 1) {
        uint32_t j = kk >> 1;
        if (j >= 32u * E) {
            __syncthreads();  // every thread has read the arrays it wrote before
#pragma unroll
            for (int e = 0; e < E; e++) {
                skey[base + e] = k[e];
                sval[base + e] = v[e];
            }
            __syncthreads();
            for (; j >= 32u * E; j >>= 1) {
                for (uint32_t q = t; q < P / 2; q += blockDim.x)
                    bitonic_cx_shared(skey, sval, ((q & ~(j - 1)) << 1) | (q & (j - 1)), j, kk);
                __syncthreads();
            }
#pragma unroll
            for (int e = 0; e < E; e++) {
                k[e] = skey[base + e];
                v[e] = sval[base + e];
            }
        }
        for (; j >= (uint32_t)E; j >>= 1) {  // the partner: same slot, lane ^ (j / E)
            const uint32_t lx = j / E;
#pragma unroll
            for (int e = 0; e < E; e++) {
                const unsigned long long pk = __shfl_xor_sync(0xffffffffu, k[e], lx);
                const uint32_t pv = __shfl_xor_sync(0xffffffffu, v[e], lx);
                const uint32_t i = base + e;
                const bool p_less = pk < k[e] || (pk == k[e] && pv < v[e]);
                // the lower position of an ascending pair (or the upper of a descending one) keeps the smaller
                if ((((i & j) == 0) == ((i & kk) == 0)) ? p_less : !p_less) {
                    k[e] = pk;
                    v[e] = pv;
                }
            }
        }
#pragma unroll
        for (int jj = E / 2; jj > 0; jj >>= 1) {  // the partner in this thread's registers
            if ((uint32_t)jj > (kk >> 1)) continue;
#pragma unroll
            for (int e = 0; e < E; e++) {
                if ((e & jj) == 0) {
                    const int f = e | jj;
                    const bool gt = k[e] > k[f] || (k[e] == k[f] && v[e] > v[f]);
                    if ((((base + e) & kk) == 0) == gt) {
                        const unsigned long long tk = k[e];
                        k[e] = k[f];
                        k[f] = tk;
                        const uint32_t tv = v[e];
                        v[e] = v[f];
                        v[f] = tv;
                    }
                }
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int e = 0; e < E; e++) {
        skey[base + e] = k[e];
        sval[base + e] = v[e];
    }
    __syncthreads();
}

// sort.SliceStable by barycenter component: bitonic sort of (key, input
// position), so equal keys keep their input order.
__device__ void stable_sort_axis(const AuxNode *__restrict__ aux, const uint32_t *in, uint32_t n, int axis,
                                 uint32_t *out, unsigned long long *skey, uint32_t *sval) {
    uint32_t P = pow2_at_least(n);
    for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
        if (i < n) {
            // the float64 barycenter (lo + hi) * 0.5, computed exactly from the float32 bounds
            const AuxNode &x = aux[in[i]];
            skey[i] = gbt_phr::key_of_bits(gbt_phr::bary_bits(x.lo[axis], x.hi[axis]));
        } else {
            skey[i] = ~0ULL;
        }
        sval[i] = i;
    }
    __syncthreads();
    // blocks of whole warps sorting 1 to 8 pairs a thread: the network in registers
    const uint32_t E = P / blockDim.x;
    if (blockDim.x >= 64 && P >= blockDim.x && P % blockDim.x == 0 && E <= 8) {
        if (E == 1) bitonic_regs<1>(skey, sval, P);
        else if (E == 2) bitonic_regs<2>(skey, sval, P);
        else if (E == 4) bitonic_regs<4>(skey, sval, P);
        else bitonic_regs<8>(skey, sval, P);
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) out[i] = in[sval[i]];
        __syncthreads();
        return;
    }
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t i = threadIdx.x; i < P; i += blockDim.x) {
                uint32_t l = i ^ j;
                if (l > i) {
                    unsigned long long ki = skey[i], kl = skey[l];
                    uint32_t vi = sval[i], vl = sval[l];
                    bool gt = ki > kl || (ki == kl && vi > vl);
                    bool asc = (i & k) == 0;
                    if (asc == gt) {
                        skey[i] = kl;
                        skey[l] = ki;
                        sval[i] = vl;
                        sval[l] = vi;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) out[i] = in[sval[i]];
    __syncthreads();
}

// The same sort for one-warp blocks and n <= 256: a bitonic network over
// 32 * E (key, position) pairs held in registers, E consecutive ones per lane;
// partners within a lane (stride J < E) swap in registers, partners in other
// lanes are read through shuffles.
template <int E, int J>
__device__ __forceinline__ void bitonic_in_lane(unsigned long long (&key)[E], uint32_t (&val)[E], uint32_t lane,
                                                uint32_t k) {
#pragma unroll
    for (int e = 0; e < E; e++) {
        const int p = e ^ J;
        if (p > e) {
            const bool asc = ((lane * E + e) & k) == 0;
            const bool gt = key[e] > key[p] || (key[e] == key[p] && val[e] > val[p]);
            if (gt == asc) {
                const unsigned long long tk = key[e];
                key[e] = key[p];
                key[p] = tk;
                const uint32_t tv = val[e];
                val[e] = val[p];
                val[p] = tv;
            }
        }
    }
}

template <int E>
__device__ void warp_sort_axis_e(const AuxNode *__restrict__ aux, const uint32_t *in, uint32_t n, int axis,
                                 uint32_t *out) {
    const uint32_t lane = threadIdx.x & 31;
    unsigned long long key[E];
    uint32_t val[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
        const uint32_t i = lane * E + e;
        if (i < n) {
            const AuxNode &x = aux[in[i]];
            key[e] = gbt_phr::key_of_bits(gbt_phr::bary_bits(x.lo[axis], x.hi[axis]));
        } else {
            key[e] = ~0ULL;  // padding sorts last
        }
        val[e] = i;
    }
    for (uint32_t k = 2; k <= 32u * E; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            if (j >= (uint32_t)E) {
                const int lj = (int)(j / E);
#pragma unroll
                for (int e = 0; e < E; e++) {
                    const unsigned long long pk = __shfl_xor_sync(0xffffffffu, key[e], lj);
                    const uint32_t pv = __shfl_xor_sync(0xffffffffu, val[e], lj);
                    const uint32_t i = lane * E + e;
                    const bool asc = (i & k) == 0, lower = (i & j) == 0;
                    const bool gt = key[e] > pk || (key[e] == pk && val[e] > pv);
                    // the lower position keeps the smaller pair when ascending, the larger otherwise
                    if (lower ? (gt == asc) : (gt != asc)) {
                        key[e] = pk;
                        val[e] = pv;
                    }
                }
            } else if (j == 4) {
                bitonic_in_lane<E, (E > 4 ? 4 : 0)>(key, val, lane, k);
            } else if (j == 2) {
                bitonic_in_lane<E, (E > 2 ? 2 : 0)>(key, val, lane, k);
            } else {
                bitonic_in_lane<E, (E > 1 ? 1 : 0)>(key, val, lane, k);
            }
        }
    }
#pragma unroll
    for (int e = 0; e < E; e++) {
        const uint32_t i = lane * E + e;
        if (i < n) out[i] = in[val[e]];
    }
    __syncwarp();
}

// stable_sort_axis for a one-warp block: registers up to 256 nodes, else the
// shared-scratch network.
__device__ __noinline__ void warp_sort_axis(const AuxNode *__restrict__ aux, const uint32_t *in, uint32_t n, int axis,
                               uint32_t *out, unsigned long long *skey, uint32_t *sval) {
    if (n <= 32) warp_sort_axis_e<1>(aux, in, n, axis, out);
    else if (n <= 64) warp_sort_axis_e<2>(aux, in, n, axis, out);
    else if (n <= 128) warp_sort_axis_e<4>(aux, in, n, axis, out);
    else if (n <= 256) warp_sort_axis_e<8>(aux, in, n, axis, out);
    else stable_sort_axis(aux, in, n, axis, out, skey, sval);
}

// A minCost result.  Its float64 cost is taken only when a comparison needs it
// (sah_less): from the split's boxes and subtree sizes, or for not splitting
// (split 0) from the cut's box (llo, lhi) and all of its subtree sizes (rc).
struct SahResult {
    float c32;        // float32 value of the cost
    uint32_t split;   // 0: not splitting is cheapest
    uint32_t lc, rc;  // subtree sizes left and right of the split
    float llo[3], lhi[3], rlo[3], rhi[3];
};

__device__ __noinline__ double nosplit_cost64(float l0, float l1, float l2, float h0, float h1, float h2,
                                              uint32_t total) {
    const float lo[3] = {l0, l1, l2}, hi[3] = {h0, h1, h2};
    return __dmul_rn(surface(lo, hi), (double)total);
}

__device__ __forceinline__ double sah_cost64(const SahResult &r) {
    if (r.split == 0) return nosplit_cost64(r.llo[0], r.llo[1], r.llo[2], r.lhi[0], r.lhi[1], r.lhi[2], r.rc);
    return split_cost64(r.rlo[0], r.rlo[1], r.rlo[2], r.rhi[0], r.rhi[1], r.rhi[2], r.rc, r.llo[0], r.llo[1],
                        r.llo[2], r.lhi[0], r.lhi[1], r.lhi[2], r.lc);
}

// a.cost < b.cost as the float64 values compare: decided by the float32 values
// when they are further apart than the screening slack (phr_exact.cuh)
__device__ __forceinline__ bool sah_less(const SahResult &a, const SahResult &b, bool screen) {
    if (a.split == 0 && b.split == 0) return false;  // both are the cost of not splitting the cut
    if (screen) {
        if (__fmul_rn(a.c32, gbt_phr::SCREEN_SLACK) < b.c32) return true;
        if (__fmul_rn(b.c32, gbt_phr::SCREEN_SLACK) < a.c32) return false;
    }
    return sah_cost64(a) < sah_cost64(b);
}

// Block-wide first minimum of (value, index) pairs; every thread gets it.
__device__ __forceinline__ void block_argmin_f32(float &v, uint32_t &idx, float *s_v, uint32_t *s_i) {
    for (int o = 16; o > 0; o >>= 1) {
        const float v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const uint32_t i2 = __shfl_xor_sync(0xffffffffu, idx, o);
        if (v2 < v || (v2 == v && i2 < idx)) {
            v = v2;
            idx = i2;
        }
    }
    const int t = threadIdx.x, nw = blockDim.x >> 5;
    if ((t & 31) == 0) {
        s_v[t >> 5] = v;
        s_i[t >> 5] = idx;
    }
    __syncthreads();
    for (int w = 0; w < nw; w++) {
        const float v2 = s_v[w];
        const uint32_t i2 = s_i[w];
        if (v2 < v || (v2 == v && i2 < idx)) {
            v = v2;
            idx = i2;
        }
    }
    __syncthreads();
}

// minCost (phr.go:414-459) over the order `ord`: the first split position of
// least float64 cost, or not splitting when that is not cheaper.  Every
// position's cost is taken in float32; with `screen` only the positions within
// the screening slack of the least float32 cost are candidates, and a single
// candidate needs no float64 at all (phr_exact.cuh).
// The result goes to *s_out (shared memory, written by thread 0).
__device__ __forceinline__ void min_cost(const AuxNode *__restrict__ aux, const uint32_t *ord, uint32_t n,
                                         const float *clo, const float *chi, const Scratch &s, BoxAgg *s_tmp,
                                         BoxAgg *s_rank, double *s_cost, uint32_t *s_idx, bool screen,
                                         SahResult *s_out) {
    const int t = threadIdx.x;
    const uint32_t chunk = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t a = min(n, t * chunk), b = min(n, a + chunk);
    // forward: exclusive prefix (union, count) -> left box/count at position i
    BoxAgg loc = agg_identity();
    for (uint32_t i = a; i < b; i++) {
        const AuxNode &x = aux[ord[i]];
        BoxAgg e;
        for (int k = 0; k < 3; k++) { e.lo[k] = x.lo[k]; e.hi[k] = x.hi[k]; }
        e.c = x.size;
        loc = agg_join(loc, e);
    }
    BoxAgg run = block_scan_agg(loc, t, s_tmp, s_rank);
    for (uint32_t i = a; i < b; i++) {
        for (int k = 0; k < 3; k++) { s.lb[k][i] = run.lo[k]; s.lb[3 + k][i] = run.hi[k]; }
        s.lc[i] = run.c;
        const AuxNode &x = aux[ord[i]];
        BoxAgg e;
        for (int k = 0; k < 3; k++) { e.lo[k] = x.lo[k]; e.hi[k] = x.hi[k]; }
        e.c = x.size;
        run = agg_join(run, e);
    }
    // backward: inclusive suffix from position i to the end -> right box/count, and
    // the float32 cost of splitting before position i (>= 1) with the left box and
    // count this thread wrote in the forward pass
    BoxAgg suf = block_scan_agg(loc, (int)blockDim.x - 1 - t, s_tmp, s_rank);
    float m = INFINITY;  // least float32 cost of this thread's positions, first position
    uint32_t mi = 0xffffffffu;
    for (uint32_t i = b; i > a; i--) {
        const AuxNode &x = aux[ord[i - 1]];
        BoxAgg e;
        for (int k = 0; k < 3; k++) { e.lo[k] = x.lo[k]; e.hi[k] = x.hi[k]; }
        e.c = x.size;
        suf = agg_join(suf, e);
        for (int k = 0; k < 3; k++) { s.rb[k][i - 1] = suf.lo[k]; s.rb[3 + k][i - 1] = suf.hi[k]; }
        s.rc[i - 1] = suf.c;
        if (i - 1 >= 1) {
            const float ll[3] = {s.lb[0][i - 1], s.lb[1][i - 1], s.lb[2][i - 1]};
            const float lh[3] = {s.lb[3][i - 1], s.lb[4][i - 1], s.lb[5][i - 1]};
            const float c = __fadd_rn(__fmul_rn(gbt_phr::surface32(suf.lo, suf.hi), gbt_phr::count_f32(suf.c)),
                                      __fmul_rn(gbt_phr::surface32(ll, lh), gbt_phr::count_f32(s.lc[i - 1])));
            s.c32[i - 1] = c;
            if (c <= m) {  // going backwards: an equal cost at a lower position wins
                m = c;
                mi = i - 1;
            }
        }
    }
    __syncthreads();
    auto cost32 = [&](uint32_t i) { return s.c32[i]; };
    float *s_f = reinterpret_cast<float *>(s_cost);
    block_argmin_f32(m, mi, s_f, s_idx);
    const float lim = __fmul_rn(m, gbt_phr::SCREEN_SLACK);
    uint32_t cand = 0;
    if (screen) {
        for (uint32_t i = 1 + t; i < n; i += blockDim.x) cand += cost32(i) <= lim ? 1u : 0u;
        for (int o = 16; o > 0; o >>= 1) cand += __shfl_xor_sync(0xffffffffu, cand, o);
        if ((t & 31) == 0) s_idx[t >> 5] = cand;
        __syncthreads();
        cand = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) cand += s_idx[w];
        __syncthreads();
    }
    uint32_t bidx = mi;
    if (n > 1 && (!screen || cand > 1)) {
        // float64 among the candidates (every position without screening), first minimum wins
        double best = INFINITY;
        uint32_t bi = 0xffffffffu;
        for (uint32_t i = 1 + t; i < n; i += blockDim.x) {
            if (screen && !(cost32(i) <= lim)) continue;
            const double cost = split_cost64(s.rb[0][i], s.rb[1][i], s.rb[2][i], s.rb[3][i], s.rb[4][i], s.rb[5][i],
                                             s.rc[i], s.lb[0][i], s.lb[1][i], s.lb[2][i], s.lb[3][i], s.lb[4][i],
                                             s.lb[5][i], s.lc[i]);
            if (cost < best || (cost == best && i < bi)) {
                best = cost;
                bi = i;
            }
        }
        s_cost[t] = best;
        s_idx[t] = bi;
        __syncthreads();
        for (int off = blockDim.x / 2; off > 0; off >>= 1) {
            if (t < off) {
                double c2 = s_cost[t + off];
                uint32_t i2 = s_idx[t + off];
                if (c2 < s_cost[t] || (c2 == s_cost[t] && i2 < s_idx[t])) {
                    s_cost[t] = c2;
                    s_idx[t] = i2;
                }
            }
            __syncthreads();
        }
        bidx = s_idx[0];
        __syncthreads();
    }
    if (t == 0) {
        SahResult sp, ns;  // the best split, and not splitting
        ns.split = 0;
        ns.lc = 0;
        ns.rc = s.rc[0];
        ns.c32 = __fmul_rn(gbt_phr::surface32(clo, chi), gbt_phr::count_f32(ns.rc));
        for (int k = 0; k < 3; k++) {
            ns.llo[k] = clo[k];
            ns.lhi[k] = chi[k];
            ns.rlo[k] = 0.f;
            ns.rhi[k] = 0.f;
        }
        bool split = false;
        if (n > 1 && bidx < n) {
            sp.split = bidx;
            sp.c32 = cost32(bidx);
            sp.lc = s.lc[bidx];
            sp.rc = s.rc[bidx];
            for (int k = 0; k < 3; k++) {
                sp.llo[k] = s.lb[k][bidx];
                sp.lhi[k] = s.lb[3 + k][bidx];
                sp.rlo[k] = s.rb[k][bidx];
                sp.rhi[k] = s.rb[3 + k][bidx];
            }
            split = sah_less(sp, ns, screen);
        }
        *s_out = split ? sp : ns;
    }
    __syncthreads();  // the result is out, and the next sweep may rewrite the scratch
}

struct Cut {  // a cut inside a job: a node list in the output pool, or a finished leaf
    uint32_t off, n;
    const uint32_t *src;
    float lo[3], hi[3];
    int32_t depth;
    int32_t leaf;  // >= 0: the PNode of a leaf made from this cut
};

// Block-cooperative copy of `count` records; ranges outside [0, n) are skipped
// and reported (they would mean an inconsistent tree).
__device__ void copy_records(const float4 *__restrict__ src, float4 *__restrict__ dst, uint32_t from, uint32_t count,
                             uint32_t to, uint32_t n, unsigned int *err) {
    if ((uint64_t)from + count > n || (uint64_t)to + count > n) {
        if (threadIdx.x == 0) atomicOr(err, GBT_DEVERR_BOUNDS);
        return;
    }
    for (uint32_t i = threadIdx.x; i < 3 * count; i += blockDim.x) dst[3 * (size_t)to + i] = src[3 * (size_t)from + i];
}

struct LevelArgs {
    const AuxNode *aux;
    const AuxCold *auxc;
    const float4 *aux_recs;
    float4 *recs;
    PNode *pn;
    const double *thr;
    const float *thr_lo, *thr_hi;  // thr * (1 -+ 2^-19) in float32: the screening band
    const PJob *jobs_in;
    PJob *jobs_out;
    const uint32_t *pool_in;
    uint32_t *pool_out;
    PhrGlobals *g;
    int parity;
    uint32_t pool_cap, job_cap, pnode_cap;
    uint32_t level;  // the level this launch works on (it does nothing unless it is the next one)
    uint32_t cap;    // per-block scratch capacity in cut nodes: at least the level's largest cut * 2^(bf-2)
    unsigned char *scratch;
    size_t scratch_per_block;
    uint32_t sort_smem;  // > 0: the block sort's keys and positions live in dynamic shared memory
    int bf;
    uint32_t n_prim;
    unsigned int *err;
};

__device__ int32_t new_pnode(PhrGlobals *g, uint32_t cap, unsigned int *err) {
    uint32_t id = atomicAdd(&g->pnode_ctr, 1u);
    if (id >= cap) {
        atomicOr(err, GBT_DEVERR_CAPACITY);
        return -1;
    }
    return (int32_t)id;
}

__device__ void attach(const LevelArgs &A, int32_t parent, int32_t slot, int32_t child) {
    if (parent < 0) A.g->root = child;
    else A.pn[parent].child[slot] = child;
}

// Shared state of a block working on one job at a time.
template <int BS>
struct BlockShared {
    BoxAgg tmp[BS / 32];
    BoxAgg rank[BS];
    double cost[BS];
    uint32_t idx[BS];
    uint32_t u[32];
    Cut cuts[4];
    SahResult res[3];  // minCost of the x, y and z orders
    int32_t branch, ncuts;
    uint32_t off;
};

// Whether a job goes to the lane list: a cut of 2..LANE_CUT nodes (bf = 2), or
// of 2..LANE_CUT_MULTI >> (bf - 2) nodes (bf > 2: every cut its splits sort
// then fits a lane's scratch).
__device__ __forceinline__ bool lane_cut_job(const LevelArgs &A, uint32_t n) {
    return n >= 2 && A.bf <= MAX_BF_LANES && n <= (A.bf == 2 ? LANE_CUT : (LANE_CUT_MULTI >> (A.bf - 2)));
}

// Index in jobs_out for one new job of the given list (0xffffffff: no room).
__device__ __forceinline__ uint32_t push_job_slot(const LevelArgs &A, bool lane_list) {
    const int out = A.parity ^ 1;
    const uint32_t q = atomicAdd(lane_list ? &A.g->job_ctr[out] : &A.g->job_big_ctr[out], 1u);
    if (q >= A.job_cap) {
        atomicOr(A.err, GBT_DEVERR_CAPACITY);
        return 0xffffffffu;
    }
    return lane_list ? q : A.job_cap - 1 - q;
}

__device__ __forceinline__ void store_job(const LevelArgs &A, const PJob &nj, uint32_t slot) {
    if (slot != 0xffffffffu) A.jobs_out[slot] = nj;
}

// buildSubTree (phr.go:92-152) for one job by the whole block: split the
// largest cut until BranchingFactor cuts, then the branch and its children.
// Thread 0 accumulates the build cost and the largest new cut.
template <int BS>
__device__ __forceinline__ void job_block(const LevelArgs &A, const PJob &job, uint32_t nmax, BlockShared<BS> &sh,
                                          const Scratch &S, bool screen, unsigned long long &blk_build_cost,
                                          uint32_t &blk_max_n) {
    BoxAgg *s_tmp = sh.tmp;
    BoxAgg *s_rank = sh.rank;
    double *s_cost = sh.cost;
    uint32_t *s_idx = sh.idx;
    uint32_t *s_u = sh.u;
    Cut *s_cuts = sh.cuts;
    int32_t &s_branch = sh.branch, &s_ncuts = sh.ncuts;
    uint32_t &s_off = sh.off;
    const int out = A.parity ^ 1;
    if (job.n > nmax) {
        if (threadIdx.x == 0) atomicOr(A.err, GBT_DEVERR_CAPACITY);
        return;
    }
    if (job.n <= 1) {  // only the root job when the auxiliary root is a leaf
        if (threadIdx.x == 0) {
            uint32_t id = A.pool_in[job.off];
            const AuxNode &a = A.aux[id];
            const AuxCold &ac = A.auxc[id];
            int32_t p = new_pnode(A.g, A.pnode_cap, A.err);
            if (p >= 0) {
                uint32_t ro = atomicAdd(&A.g->rec_ctr, ac.count);
                PNode &q = A.pn[p];
                for (int k = 0; k < 3; k++) { q.lo[k] = a.lo[k]; q.hi[k] = a.hi[k]; }
                q.leaf = 1;
                q.nchild = 0;
                q.rec_off = ro;
                q.rec_cnt = ac.count;
                attach(A, job.parent, job.slot, p);
                s_off = ro;
                s_u[0] = ac.first;
                s_u[1] = ac.count;
            }
        }
        __syncthreads();
        copy_records(A.aux_recs, A.recs, s_u[0], s_u[1], s_off, A.n_prim, A.err);
        __syncthreads();
        return;
    }
    if (threadIdx.x == 0) {
        int32_t b = new_pnode(A.g, A.pnode_cap, A.err);
        s_branch = b;
        if (b >= 0) {
            PNode &q = A.pn[b];
            for (int k = 0; k < 3; k++) { q.lo[k] = job.lo[k]; q.hi[k] = job.hi[k]; }
            q.leaf = 0;
            q.nchild = 0;
            attach(A, job.parent, job.slot, b);
        }
        Cut c0;
        c0.off = job.off;
        c0.n = job.n;
        c0.src = A.pool_in + job.off;
        for (int k = 0; k < 3; k++) { c0.lo[k] = job.lo[k]; c0.hi[k] = job.hi[k]; }
        c0.depth = job.depth;
        c0.leaf = -1;
        s_cuts[0] = c0;
        s_ncuts = 1;
    }
    __syncthreads();
    if (s_branch < 0) return;
    // buildSubTree's loop: split the largest cut until BranchingFactor cuts
    while (s_ncuts < A.bf) {
        int nc = s_ncuts, mi = 0;
        uint32_t mx = 0;
        for (int i = 0; i < nc; i++)
            if (s_cuts[i].n > mx) { mx = s_cuts[i].n; mi = i; }
        if (mx <= 1) break;
        if (threadIdx.x == 0) blk_build_cost += mx;
        const Cut cut = s_cuts[mi];
        const uint32_t n = cut.n;
        // a refined cut of this job can be larger than the job's own cut (bf > 2)
        if (n > A.cap) {
            if (threadIdx.x == 0) atomicOr(A.err, GBT_DEVERR_CAPACITY);
            break;
        }
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) S.ids[i] = cut.src[i];
        __syncthreads();
        // SweepSAH: x from the cut order, y from the x order, z from the y order
        // when x is cheaper than y, else from the x order
        if (BS == 32) warp_sort_axis(A.aux, S.ids, n, 0, S.ord[0], S.skey, S.sval);
        else stable_sort_axis(A.aux, S.ids, n, 0, S.ord[0], S.skey, S.sval);
        if (BS == 32) warp_sort_axis(A.aux, S.ord[0], n, 1, S.ord[1], S.skey, S.sval);
        else stable_sort_axis(A.aux, S.ord[0], n, 1, S.ord[1], S.skey, S.sval);
        SahResult *res = sh.res;  // x, y, z
        min_cost(A.aux, S.ord[0], n, cut.lo, cut.hi, S, s_tmp, s_rank, s_cost, s_idx, screen, &res[0]);
        min_cost(A.aux, S.ord[1], n, cut.lo, cut.hi, S, s_tmp, s_rank, s_cost, s_idx, screen, &res[1]);
        const bool x_first = sah_less(res[0], res[1], screen);
        const uint32_t *zsrc = x_first ? S.ord[1] : S.ord[0];
        if (BS == 32) warp_sort_axis(A.aux, zsrc, n, 2, S.ord[2], S.skey, S.sval);
        else stable_sort_axis(A.aux, zsrc, n, 2, S.ord[2], S.skey, S.sval);
        min_cost(A.aux, S.ord[2], n, cut.lo, cut.hi, S, s_tmp, s_rank, s_cost, s_idx, screen, &res[2]);
        const int warr = x_first ? (sah_less(res[0], res[2], screen) ? 0 : 2) : (sah_less(res[1], res[2], screen) ? 1 : 2);
        const SahResult &win = res[warr];
        const uint32_t *ord = warr == 0 ? S.ord[0] : (warr == 1 ? S.ord[1] : S.ord[2]);
        if (win.split == 0) {
            // makeLeaf(left.bounding, left.nodes...) over the winning order
            uint32_t loc = 0;
            const uint32_t chunk = (n + blockDim.x - 1) / blockDim.x;
            const uint32_t a = min(n, threadIdx.x * chunk), b = min(n, a + chunk);
            for (uint32_t i = a; i < b; i++) loc += A.auxc[ord[i]].count;
            uint32_t tot;
            uint32_t ex = block_scan_u32(loc, s_u, &tot);
            for (uint32_t i = a; i < b; i++) {
                S.flag[i] = ex;
                ex += A.auxc[ord[i]].count;
            }
            if (threadIdx.x == 0) {
                int32_t p = new_pnode(A.g, A.pnode_cap, A.err);
                s_off = atomicAdd(&A.g->rec_ctr, tot);
                if (p >= 0) {
                    PNode &q = A.pn[p];
                    for (int k = 0; k < 3; k++) { q.lo[k] = win.llo[k]; q.hi[k] = win.lhi[k]; }
                    q.leaf = 1;
                    q.nchild = 0;
                    q.rec_off = s_off;
                    q.rec_cnt = tot;
                }
                Cut c;
                c.n = 1;
                c.leaf = p;
                s_cuts[mi] = c;
            }
            __syncthreads();
            for (uint32_t i = 0; i < n; i++) {
                const AuxCold &x = A.auxc[ord[i]];
                copy_records(A.aux_recs, A.recs, x.first, x.count, s_off + S.flag[i], A.n_prim, A.err);
            }
            __syncthreads();
            continue;
        }
        // refined(left), refined(right)
        const uint32_t ns[2] = {win.split, n - win.split};
        const uint32_t *srcs[2] = {ord, ord + win.split};
        const double thr = A.thr[min(cut.depth, DEPTH_TABLE - 1)];
        const float thr_lo = A.thr_lo[min(cut.depth, DEPTH_TABLE - 1)];
        const float thr_hi = A.thr_hi[min(cut.depth, DEPTH_TABLE - 1)];
        if (cut.depth >= DEPTH_TABLE - 1 && threadIdx.x == 0) atomicOr(A.err, GBT_DEVERR_CAPACITY);
#pragma unroll
        for (int side = 0; side < 2; side++) {
            const uint32_t m = ns[side];
            const uint32_t *sr = srcs[side];
            const uint32_t chunk = (m + blockDim.x - 1) / blockDim.x;
            const uint32_t a = min(m, threadIdx.x * chunk), b = min(m, a + chunk);
            uint32_t loc = 0;
            for (uint32_t i = a; i < b; i++) {
                const AuxNode &x = A.aux[sr[i]];
                // surface(x) < thr, decided in float32 outside a narrow band around thr
                bool keep = x.c0 < 0;
                if (!keep) {
                    const float s32 = screen ? gbt_phr::surface32(x.lo, x.hi) : 0.f;
                    if (screen && s32 < thr_lo) keep = true;
                    else if (screen && s32 > thr_hi) keep = false;
                    else keep = surface_below(x.lo, x.hi, thr);
                }
                S.flag[i] = keep ? 1u : 2u;
                loc += S.flag[i];
            }
            uint32_t tot;
            uint32_t ex = block_scan_u32(loc, s_u, &tot);
            const float *blo = side ? win.rlo : win.llo, *bhi = side ? win.rhi : win.lhi;
            if (tot == 1) {  // a one-node cut becomes a leaf of everything below it
                if (threadIdx.x == 0) {
                    const AuxCold &x = A.auxc[sr[0]];
                    int32_t p = new_pnode(A.g, A.pnode_cap, A.err);
                    s_off = atomicAdd(&A.g->rec_ctr, x.count);
                    s_u[8] = x.first;
                    s_u[9] = x.count;
                    if (p >= 0) {
                        PNode &q = A.pn[p];
                        for (int k = 0; k < 3; k++) { q.lo[k] = blo[k]; q.hi[k] = bhi[k]; }
                        q.leaf = 1;
                        q.nchild = 0;
                        q.rec_off = s_off;
                        q.rec_cnt = x.count;
                    }
                    Cut c;
                    c.n = 1;
                    c.leaf = p;
                    s_cuts[side == 0 ? mi : s_ncuts] = c;
                }
                __syncthreads();
                copy_records(A.aux_recs, A.recs, s_u[8], s_u[9], s_off, A.n_prim, A.err);
            } else {
                if (threadIdx.x == 0) {
                    uint32_t o = atomicAdd(&A.g->pool_ctr[out], tot);
                    if (o + tot > A.pool_cap) {
                        atomicOr(A.err, GBT_DEVERR_CAPACITY);
                        o = 0xffffffffu;
                    }
                    s_off = o;
                }
                __syncthreads();
                const uint32_t o = s_off;
                if (o != 0xffffffffu) {
                    for (uint32_t i = a; i < b; i++) {
                        const AuxNode &x = A.aux[sr[i]];
                        if (S.flag[i] == 1u) {
                            A.pool_out[o + ex] = sr[i];
                            ex += 1;
                        } else {
                            A.pool_out[o + ex] = (uint32_t)x.c0;
                            A.pool_out[o + ex + 1] = (uint32_t)A.auxc[sr[i]].c1;
                            ex += 2;
                        }
                    }
                }
                if (threadIdx.x == 0) {
                    Cut c;
                    c.off = o == 0xffffffffu ? 0 : o;
                    c.n = o == 0xffffffffu ? 1 : tot;
                    c.src = A.pool_out + c.off;
                    for (int k = 0; k < 3; k++) { c.lo[k] = blo[k]; c.hi[k] = bhi[k]; }
                    c.depth = cut.depth + 1;
                    c.leaf = o == 0xffffffffu ? -2 : -1;
                    s_cuts[side == 0 ? mi : s_ncuts] = c;
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) s_ncuts = s_ncuts + 1;
        __syncthreads();
    }
    // the branch and its children
    if (threadIdx.x == 0) {
        const int32_t b = s_branch;
        const int nc = s_ncuts;
        A.pn[b].nchild = nc;
        for (int i = 0; i < nc; i++) {
            const Cut &c = s_cuts[i];
            if (c.leaf >= 0) {
                A.pn[b].child[i] = c.leaf;
            } else if (c.leaf == -1) {
                PJob nj;
                nj.off = c.off;
                nj.n = c.n;
                for (int k = 0; k < 3; k++) { nj.lo[k] = c.lo[k]; nj.hi[k] = c.hi[k]; }
                nj.depth = c.depth;
                nj.parent = b;
                nj.slot = i;
                nj.pad = 0;
                store_job(A, nj, push_job_slot(A, lane_cut_job(A, nj.n)));
                blk_max_n = max(blk_max_n, c.n);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// lane path: one lane sweeps one cut of at most LANE_CUT nodes (bf = 2)
// ---------------------------------------------------------------------------
// The same SweepSAH, minCost, refined and makeLeaf as job_block, for one cut
// per lane.  Costs are taken in float32 and decided exactly: a comparison
// whose float32 values are further apart than the screening slack is decided
// by them (phr_exact.cuh), any other one by the float64 values, recomputed for
// just those candidates; without screening every cost is float64.

// Per-lane scratch, index-major so that the lanes of a warp use different banks.
template <uint32_t CUT_>
struct LaneScratchT {
    static constexpr uint32_t CUT = CUT_;  // the largest cut a lane sorts
    union {
        unsigned long long key[CUT][32];  // sort keys
        float c32[CUT][32];               // float32 split costs of a sweep
    };
    uint32_t id[CUT][32];       // the cut's node ids, in cut order
    uint8_t ord[3][CUT][32];    // x, y, z orders: positions into id
};
using LaneScratch = LaneScratchT<LANE_CUT>;             // bf = 2
using LaneScratchMulti = LaneScratchT<LANE_CUT_MULTI>;  // bf > 2

struct LaneBox {
    float lo[3], hi[3];
};

__device__ __forceinline__ void lbox_empty(LaneBox &b) {
    b.lo[0] = b.lo[1] = b.lo[2] = INFINITY;
    b.hi[0] = b.hi[1] = b.hi[2] = -INFINITY;
}

__device__ __forceinline__ void lbox_add(LaneBox &b, const AuxNode &x) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
        b.lo[k] = fminf(b.lo[k], x.lo[k]);
        b.hi[k] = fmaxf(b.hi[k], x.hi[k]);
    }
}

struct LaneCut {
    uint32_t n, total;   // nodes, sum of their subtree sizes
    float lo[3], hi[3];  // the cut's box
    float ns32;          // float32 cost of not splitting
};

// A minCost result: split position (0: not splitting is cheapest) of order k,
// with the float32 value of its cost.
struct LanePick {
    float c32;
    uint32_t split;
    int k;
};

template <class LS>
__device__ __forceinline__ const AuxNode &lane_node(const AuxNode *__restrict__ aux, const LS &L, int k,
                                                    uint32_t i, int ln) {
    return aux[L.id[L.ord[k][i][ln]][ln]];
}

template <class LS>
__device__ __forceinline__ const AuxCold &lane_cold(const AuxCold *__restrict__ auxc, const LS &L, int k,
                                                    uint32_t i, int ln) {
    return auxc[L.id[L.ord[k][i][ln]][ln]];
}

// sort.SliceStable by barycenter component `axis`: insertion sort of the
// order `src` (-1: the cut order) into `dst`; equal keys keep their order.
template <class LS>
__device__ void lane_sort(const AuxNode *__restrict__ aux, LS &L, int src, int dst, int axis, uint32_t n,
                          int ln) {
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t p = src < 0 ? i : L.ord[src][i][ln];
        const AuxNode &x = aux[L.id[p][ln]];
        const unsigned long long key = gbt_phr::key_of_bits(gbt_phr::bary_bits(x.lo[axis], x.hi[axis]));
        uint32_t j = i;
        while (j > 0 && L.key[j - 1][ln] > key) {
            L.key[j][ln] = L.key[j - 1][ln];
            L.ord[dst][j][ln] = L.ord[dst][j - 1][ln];
            j--;
        }
        L.key[j][ln] = key;
        L.ord[dst][j][ln] = (uint8_t)p;
    }
}

// The float64 costs are evaluated out of line (see surface_below).
// minCost's float64 cost of splitting order k before position i (phr.go:423-445).
template <class LS>
__device__ __noinline__ double lane_split_cost64(const AuxNode *__restrict__ aux, const LS &L, int k,
                                                 uint32_t n, uint32_t i, int ln) {
    LaneBox l, r;
    lbox_empty(l);
    lbox_empty(r);
    uint32_t lc = 0, rc = 0;
    for (uint32_t t = 0; t < n; t++) {
        const AuxNode &x = lane_node(aux, L, k, t, ln);
        if (t < i) {
            lbox_add(l, x);
            lc += x.size;
        } else {
            lbox_add(r, x);
            rc += x.size;
        }
    }
    const double rcost = __dmul_rn(surface(r.lo, r.hi), (double)rc);
    return __dadd_rn(rcost, __dmul_rn(surface(l.lo, l.hi), (double)lc));
}

// The float64 cost of a pick: its split's, or not splitting's (phr.go:432-439).
template <class LS>
__device__ __forceinline__ double lane_pick_cost64(const AuxNode *__restrict__ aux, const LS &L,
                                                   const LaneCut &c, int k, uint32_t split, int ln) {
    return split ? lane_split_cost64(aux, L, k, c.n, split, ln) : __dmul_rn(surface(c.lo, c.hi), (double)c.total);
}

template <class LS>
__device__ __noinline__ bool lane_less64(const AuxNode *__restrict__ aux, const LS &L, LaneCut c, int ka,
                                         uint32_t sa, int kb, uint32_t sb, int ln) {
    return lane_pick_cost64(aux, L, c, ka, sa, ln) < lane_pick_cost64(aux, L, c, kb, sb, ln);
}

// a.cost < b.cost as the float64 values compare: decided by the float32 values
// when they are further apart than the screening slack
template <class LS>
__device__ __forceinline__ bool lane_less(const LanePick &a, const LanePick &b, const AuxNode *__restrict__ aux,
                                          const LS &L, const LaneCut &c, bool screen, int ln) {
    if (a.split == 0 && b.split == 0) return false;  // both are the cost of not splitting
    if (screen) {
        if (__fmul_rn(a.c32, gbt_phr::SCREEN_SLACK) < b.c32) return true;
        if (__fmul_rn(b.c32, gbt_phr::SCREEN_SLACK) < a.c32) return false;
    }
    if (a.split && b.split) {
        // two orders that split the cut into the same two sides (always so for two
        // nodes) give bit-equal costs: the same unions, sizes and float64 sum
        uint32_t ma = 0, mb = 0;
        for (uint32_t i = 0; i < a.split; i++) ma |= 1u << L.ord[a.k][i][ln];
        for (uint32_t i = 0; i < b.split; i++) mb |= 1u << L.ord[b.k][i][ln];
        const uint32_t full = c.n >= 32 ? 0xffffffffu : (1u << c.n) - 1u;
        if (ma == mb || ma == (full ^ mb)) return false;
    }
    return lane_less64(aux, L, c, a.k, a.split, b.k, b.split, ln);
}

// The first position of least float64 cost among those whose float32 cost is
// at most `lim` (all positions when lim is +inf).
template <class LS>
__device__ __noinline__ uint32_t lane_first_min64(const AuxNode *__restrict__ aux, const LS &L, int k,
                                                  uint32_t n, float lim, bool all, int ln) {
    double bc = INFINITY;
    uint32_t bi = 1;
    for (uint32_t i = 1; i < n; i++) {
        if (!all && !(L.c32[i][ln] <= lim)) continue;
        const double d = lane_split_cost64(aux, L, k, n, i, ln);
        if (d < bc) {
            bc = d;
            bi = i;
        }
    }
    return bi;
}

// minCost (phr.go:414-459) over order k: the first cheapest split position,
// or not splitting when that is not cheaper.
template <class LS>
__device__ LanePick lane_min_cost(const AuxNode *__restrict__ aux, LS &L, int k, const LaneCut &c,
                                  bool screen, int ln) {
    const uint32_t n = c.n;
    LanePick best;
    best.k = k;
    // float32 costs of every split position
    LaneBox r;
    lbox_empty(r);
    uint32_t rc = 0;
    for (uint32_t i = n - 1; i >= 1; i--) {
        const AuxNode &x = lane_node(aux, L, k, i, ln);
        lbox_add(r, x);
        rc += x.size;
        L.c32[i][ln] = __fmul_rn(gbt_phr::surface32(r.lo, r.hi), gbt_phr::count_f32(rc));
    }
    LaneBox l;
    lbox_empty(l);
    uint32_t lc = 0, mi = 1;
    float m = INFINITY;
    for (uint32_t i = 1; i < n; i++) {
        const AuxNode &x = lane_node(aux, L, k, i - 1, ln);
        lbox_add(l, x);
        lc += x.size;
        const float cc = __fadd_rn(L.c32[i][ln], __fmul_rn(gbt_phr::surface32(l.lo, l.hi), gbt_phr::count_f32(lc)));
        L.c32[i][ln] = cc;
        if (cc < m) {
            m = cc;
            mi = i;
        }
    }
    // positions whose float32 cost is within the slack of the least one
    const float lim = __fmul_rn(m, gbt_phr::SCREEN_SLACK);
    uint32_t cand = 0;
    for (uint32_t i = 1; i < n; i++) cand += L.c32[i][ln] <= lim ? 1u : 0u;
    best.split = mi;
    if (!screen || cand > 1) {  // decided in float64 (among the candidates), first minimum wins
        best.split = lane_first_min64(aux, L, k, n, lim, !screen, ln);
    }
    best.c32 = L.c32[best.split][ln];
    LanePick ns;
    ns.k = k;
    ns.split = 0;
    ns.c32 = c.ns32;
    if (lane_less(best, ns, aux, L, c, screen, ln)) return best;
    return ns;
}

__device__ __forceinline__ uint32_t warp_incl_sum(uint32_t v, int ln) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (ln >= o) v += y;
    }
    return v;
}

// Allocates `v` entries of a counter for every lane with one atomic per warp;
// returns this lane's first index (the warp's base + the lanes before it).
__device__ __forceinline__ uint32_t warp_alloc(uint32_t *ctr, uint32_t v, int ln) {
    const uint32_t incl = warp_incl_sum(v, ln);
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0;
    if (ln == 0 && total) base = atomicAdd(ctr, total);
    base = __shfl_sync(0xffffffffu, base, 0);
    return base + incl - v;
}

// Record copy by one lane (copy_records for a single thread).
__device__ void lane_copy_records(const float4 *__restrict__ src, float4 *__restrict__ dst, uint32_t from,
                                  uint32_t count, uint32_t to, uint32_t n, unsigned int *err) {
    if ((uint64_t)from + count > n || (uint64_t)to + count > n) {
        atomicOr(err, GBT_DEVERR_BOUNDS);
        return;
    }
    for (uint32_t i = 0; i < 3 * count; i++) dst[3 * (size_t)to + i] = src[3 * (size_t)from + i];
}

// One job per lane for the lanes with `mine`; every lane of the warp calls
// this (the allocations are warp-wide).  Each lane accumulates its build cost
// and largest new cut.
// SweepSAH (phr.go:368-405) of the lane's cut in L.id: x from the cut order,
// y from the x order, z from the y order when x is cheaper than y, else from
// the x order; the winning order and split (0: not splitting).
template <class LS>
__device__ __forceinline__ LanePick lane_sweep_sah(const AuxNode *__restrict__ aux, LS &L, const LaneCut &c,
                                                   bool screen, int ln) {
    const uint32_t n = c.n;
    lane_sort(aux, L, -1, 0, 0, n, ln);
    LanePick xs = lane_min_cost(aux, L, 0, c, screen, ln);
    lane_sort(aux, L, 0, 1, 1, n, ln);
    LanePick ys = lane_min_cost(aux, L, 1, c, screen, ln);
    const bool x_first = lane_less(xs, ys, aux, L, c, screen, ln);
    lane_sort(aux, L, x_first ? 1 : 0, 2, 2, n, ln);
    LanePick zs = lane_min_cost(aux, L, 2, c, screen, ln);
    LanePick other = x_first ? xs : ys;
    return lane_less(other, zs, aux, L, c, screen, ln) ? other : zs;
}

// refined (phr.go:313-338) of both sides of a split of order k: per side the
// nodes kept (bit per position) and the refined size (a node replaced by its
// two children counts 2), against the threshold of the cut's depth.
template <class LS>
__device__ __forceinline__ void lane_refine(const LevelArgs &A, const LS &L, int k, uint32_t split,
                                            uint32_t n, int32_t depth, bool screen, int ln, uint32_t (&tot)[2],
                                            uint32_t (&keep)[2]) {
    const int di = min(depth, DEPTH_TABLE - 1);
    if (depth >= DEPTH_TABLE - 1) atomicOr(A.err, GBT_DEVERR_CAPACITY);
    const double thr = A.thr[di];
    const float thr_lo = A.thr_lo[di], thr_hi = A.thr_hi[di];
#pragma unroll
    for (int s = 0; s < 2; s++) {
        const uint32_t a = s ? split : 0, e = s ? n : split;
        for (uint32_t i = a; i < e; i++) {
            const AuxNode &x = lane_node(A.aux, L, k, i, ln);
            bool kept = x.c0 < 0;
            if (!kept) {
                const float s32 = screen ? gbt_phr::surface32(x.lo, x.hi) : 0.f;
                if (screen && s32 < thr_lo) kept = true;
                else if (screen && s32 > thr_hi) kept = false;
                else kept = surface_below(x.lo, x.hi, thr);
            }
            if (kept) keep[s] |= 1u << (i - a);
            tot[s] += kept ? 1u : 2u;
        }
    }
}

// The long record ranges of the lanes' leaves (split 0: every node of order k
// in one leaf; else the sides that became leaves), lane by lane, copied by
// the whole warp in the order the lane allocated them from rec_start.
template <class LS>
__device__ __forceinline__ void lane_long_copies(const LevelArgs &A, const LS &L, bool long_copy,
                                                 uint32_t rec_start, uint32_t split, uint32_t n, int k, uint32_t tot0,
                                                 uint32_t tot1) {
    unsigned pending = __ballot_sync(0xffffffffu, long_copy);
    while (pending) {
        const int l = __ffs(pending) - 1;
        pending &= pending - 1;
        const uint32_t r0 = __shfl_sync(0xffffffffu, rec_start, l), sp = __shfl_sync(0xffffffffu, split, l);
        const uint32_t nl = __shfl_sync(0xffffffffu, n, l);
        const int kl = __shfl_sync(0xffffffffu, k, l);
        const uint32_t t0 = __shfl_sync(0xffffffffu, tot0, l), t1 = __shfl_sync(0xffffffffu, tot1, l);
        uint32_t r = r0;
        const uint32_t walk = sp == 0 ? nl : 2;
        for (uint32_t q = 0; q < walk; q++) {
            if (sp != 0 && (q ? t1 : t0) != 1) continue;  // that side is a cut, not a leaf
            const uint32_t pos = sp == 0 ? q : (q ? sp : 0);
            const AuxCold &x = A.auxc[L.id[L.ord[kl][pos][l]][l]];
            if (x.count > LANE_COPY) copy_records(A.aux_recs, A.recs, x.first, x.count, r, A.n_prim, A.err);
            r += x.count;
        }
    }
}

__device__ void lane_jobs(const LevelArgs &A, uint32_t j, bool mine, LaneScratch &L, bool screen,
                          unsigned long long &my_build_cost, uint32_t &my_max_n) {
    const int ln = threadIdx.x & 31;
    const AuxNode *__restrict__ aux = A.aux;
    uint32_t n_pn = 0, n_rec = 0, n_pool = 0, n_lane_jobs = 0, n_big_jobs = 0;
    uint32_t n = 0, split = 0, tot[2] = {0, 0}, keep[2] = {0, 0};
    int k = 0;
    if (mine) {
        // SweepSAH (phr.go:368-405)
        const PJob &job = A.jobs_in[j];
        LaneCut c;
        c.n = n = job.n;
        c.total = 0;
        const uint32_t off = job.off;
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t id = A.pool_in[off + i];
            L.id[i][ln] = id;
            c.total += aux[id].size;
        }
        for (int a = 0; a < 3; a++) {
            c.lo[a] = job.lo[a];
            c.hi[a] = job.hi[a];
        }
        c.ns32 = __fmul_rn(gbt_phr::surface32(c.lo, c.hi), gbt_phr::count_f32(c.total));
        const LanePick win = lane_sweep_sah(aux, L, c, screen, ln);
        my_build_cost += n;
        k = win.k;
        split = win.split;
        if (split == 0) {  // makeLeaf over the winning order
            n_pn = 2;
            for (uint32_t i = 0; i < n; i++) n_rec += lane_cold(A.auxc, L, k, i, ln).count;
        } else {  // refined(left), refined(right)
            lane_refine(A, L, k, split, n, job.depth, screen, ln, tot, keep);
            n_pn = 1;
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const uint32_t a = s ? split : 0;
                if (tot[s] == 1) {  // a one-node cut becomes a leaf of everything below it
                    n_pn++;
                    n_rec += lane_cold(A.auxc, L, k, a, ln).count;
                } else {
                    n_pool += tot[s];
                    if (lane_cut_job(A, tot[s])) n_lane_jobs++;
                    else n_big_jobs++;
                }
            }
        }
    }
    // one atomic per counter and warp
    const int out = A.parity ^ 1;
    uint32_t pn = warp_alloc(&A.g->pnode_ctr, n_pn, ln);
    uint32_t rec = warp_alloc(&A.g->rec_ctr, n_rec, ln);
    uint32_t pool = warp_alloc(&A.g->pool_ctr[out], n_pool, ln);
    uint32_t qs = warp_alloc(&A.g->job_ctr[out], n_lane_jobs, ln);
    uint32_t qb = warp_alloc(&A.g->job_big_ctr[out], n_big_jobs, ln);
    bool ok = mine;
    if (ok && ((uint64_t)pn + n_pn > A.pnode_cap || (uint64_t)pool + n_pool > A.pool_cap ||
               (uint64_t)qs + n_lane_jobs > A.job_cap || (uint64_t)qb + n_big_jobs > A.job_cap)) {
        atomicOr(A.err, GBT_DEVERR_CAPACITY);
        ok = false;
    }
    // leaves' records: a lane copies ranges of up to LANE_COPY records itself and
    // leaves longer ones to the whole warp below
    const uint32_t rec_start = rec;
    bool long_copy = false;
    if (ok) {
        const PJob &job = A.jobs_in[j];
        const int32_t b = (int32_t)pn++;
        {
            PNode &q = A.pn[b];
            for (int a = 0; a < 3; a++) {
                q.lo[a] = job.lo[a];
                q.hi[a] = job.hi[a];
            }
            q.leaf = 0;
            q.nchild = split ? 2 : 1;
            attach(A, job.parent, job.slot, b);
        }
        if (split == 0) {
            const int32_t p = (int32_t)pn;
            PNode &q = A.pn[p];
            for (int a = 0; a < 3; a++) {
                q.lo[a] = job.lo[a];
                q.hi[a] = job.hi[a];
            }
            q.leaf = 1;
            q.nchild = 0;
            q.rec_off = rec;
            q.rec_cnt = n_rec;
            A.pn[b].child[0] = p;
            for (uint32_t i = 0; i < n; i++) {
                const AuxCold &x = lane_cold(A.auxc, L, k, i, ln);
                if (x.count <= LANE_COPY) lane_copy_records(A.aux_recs, A.recs, x.first, x.count, rec, A.n_prim, A.err);
                else long_copy = true;
                rec += x.count;
            }
        } else {
            const int32_t depth = job.depth;
#pragma unroll
            for (int s = 0; s < 2; s++) {
                const uint32_t a = s ? split : 0, e = s ? n : split;
                LaneBox box;  // the side's box: union of its nodes before refinement
                lbox_empty(box);
                for (uint32_t i = a; i < e; i++) lbox_add(box, lane_node(aux, L, k, i, ln));
                if (tot[s] == 1) {
                    const AuxCold &x = lane_cold(A.auxc, L, k, a, ln);
                    const int32_t p = (int32_t)pn++;
                    PNode &q = A.pn[p];
                    for (int d = 0; d < 3; d++) {
                        q.lo[d] = box.lo[d];
                        q.hi[d] = box.hi[d];
                    }
                    q.leaf = 1;
                    q.nchild = 0;
                    q.rec_off = rec;
                    q.rec_cnt = x.count;
                    A.pn[b].child[s] = p;
                    if (x.count <= LANE_COPY) lane_copy_records(A.aux_recs, A.recs, x.first, x.count, rec, A.n_prim, A.err);
                    else long_copy = true;
                    rec += x.count;
                } else {
                    PJob nj;
                    nj.off = pool;
                    nj.n = tot[s];
                    for (int d = 0; d < 3; d++) {
                        nj.lo[d] = box.lo[d];
                        nj.hi[d] = box.hi[d];
                    }
                    nj.depth = depth + 1;
                    nj.parent = b;
                    nj.slot = s;
                    nj.pad = 0;
                    for (uint32_t i = a; i < e; i++) {
                        const uint32_t id = L.id[L.ord[k][i][ln]][ln];
                        if (keep[s] >> (i - a) & 1u) {
                            A.pool_out[pool++] = id;
                        } else {
                            A.pool_out[pool++] = (uint32_t)aux[id].c0;
                            A.pool_out[pool++] = (uint32_t)A.auxc[id].c1;
                        }
                    }
                    if (lane_cut_job(A, tot[s])) A.jobs_out[qs++] = nj;
                    else A.jobs_out[A.job_cap - 1 - qb++] = nj;
                    my_max_n = max(my_max_n, tot[s]);
                }
            }
        }
    }
    lane_long_copies(A, L, long_copy, rec_start, split, n, k, tot[0], tot[1]);
}

// The lane path for bf > 2: a job is up to bf - 1 splits (buildSubTree's
// loop, phr.go:92-152: split the largest cut, the first of equal ones, until
// bf cuts).  The lanes of a warp take their jobs' splits in rounds, with one
// allocation per round; a cut a split makes goes to the output pool at once
// (as in job_block), and the lane's next round reads it back from there.  A
// job qualifies when its cut has at most LANE_CUT_MULTI >> (bf - 2) nodes, so that
// every cut it sorts fits the lane scratch (a refinement at most doubles one).
struct LaneCuts {  // per lane, index-major
    uint32_t off[MAX_BF_LANES][32];    // pool offset; bit 31: in the output pool
    uint32_t n[MAX_BF_LANES][32];      // nodes; 1 for a leaf
    float box[6][MAX_BF_LANES][32];    // lo.xyz, hi.xyz
    int32_t depth[MAX_BF_LANES][32];
    int32_t leaf[MAX_BF_LANES][32];    // >= 0: the leaf's PNode; -1: a cut
};

__device__ void lane_jobs_multi(const LevelArgs &A, uint32_t j, bool mine, LaneScratchMulti &L, LaneCuts &C, bool screen,
                                unsigned long long &my_build_cost, uint32_t &my_max_n) {
    const int ln = threadIdx.x & 31;
    const AuxNode *__restrict__ aux = A.aux;
    const int out = A.parity ^ 1;
    int ncuts = 0;
    int32_t branch = -1;
    bool ok = mine;
    if (mine) {
        const PJob &job = A.jobs_in[j];
        C.off[0][ln] = job.off;
        C.n[0][ln] = job.n;
        for (int a = 0; a < 3; a++) {
            C.box[a][0][ln] = job.lo[a];
            C.box[3 + a][0][ln] = job.hi[a];
        }
        C.depth[0][ln] = job.depth;
        C.leaf[0][ln] = -1;
        ncuts = 1;
    }
    for (int round = 0; round < A.bf - 1; round++) {  // the same count for every lane
        int mi = 0;
        uint32_t n = 0;
        if (ok)
            for (int i = 0; i < ncuts; i++) {
                const uint32_t ni = C.n[i][ln];
                if (ni > n) {
                    n = ni;
                    mi = i;
                }
            }
        if (ok && n > LANE_CUT_MULTI) {  // cannot happen for a qualifying job; the scratch holds LANE_CUT_MULTI
            atomicOr(A.err, GBT_DEVERR_CAPACITY);
            ok = false;
        }
        const bool act = ok && n > 1;
        uint32_t n_pn = (round == 0 && ok) ? 1u : 0u;  // the branch comes with the first round
        uint32_t n_rec = 0, n_pool = 0, split = 0, tot[2] = {0, 0}, keep[2] = {0, 0};
        int k = 0;
        if (act) {
            const uint32_t off = C.off[mi][ln];
            const uint32_t *src = (off >> 31) ? A.pool_out : A.pool_in;
            LaneCut c;
            c.n = n;
            c.total = 0;
            for (uint32_t i = 0; i < n; i++) {
                const uint32_t id = src[(off & 0x7fffffffu) + i];
                L.id[i][ln] = id;
                c.total += aux[id].size;
            }
            for (int a = 0; a < 3; a++) {
                c.lo[a] = C.box[a][mi][ln];
                c.hi[a] = C.box[3 + a][mi][ln];
            }
            c.ns32 = __fmul_rn(gbt_phr::surface32(c.lo, c.hi), gbt_phr::count_f32(c.total));
            const LanePick win = lane_sweep_sah(aux, L, c, screen, ln);
            my_build_cost += n;
            k = win.k;
            split = win.split;
            if (split == 0) {  // makeLeaf over the winning order
                n_pn += 1;
                for (uint32_t i = 0; i < n; i++) n_rec += lane_cold(A.auxc, L, k, i, ln).count;
            } else {
                lane_refine(A, L, k, split, n, C.depth[mi][ln], screen, ln, tot, keep);
#pragma unroll
                for (int s = 0; s < 2; s++) {
                    if (tot[s] == 1) {
                        n_pn++;
                        n_rec += lane_cold(A.auxc, L, k, s ? split : 0, ln).count;
                    } else {
                        n_pool += tot[s];
                    }
                }
            }
        }
        uint32_t pn = warp_alloc(&A.g->pnode_ctr, n_pn, ln);
        uint32_t rec = warp_alloc(&A.g->rec_ctr, n_rec, ln);
        uint32_t pool = warp_alloc(&A.g->pool_ctr[out], n_pool, ln);
        if (ok && ((uint64_t)pn + n_pn > A.pnode_cap || (uint64_t)pool + n_pool > A.pool_cap)) {
            atomicOr(A.err, GBT_DEVERR_CAPACITY);
            ok = false;
        }
        const uint32_t rec_start = rec;
        bool long_copy = false;
        if (ok && round == 0) {  // the branch node of this job
            const PJob &job = A.jobs_in[j];
            branch = (int32_t)pn++;
            PNode &q = A.pn[branch];
            for (int a = 0; a < 3; a++) {
                q.lo[a] = job.lo[a];
                q.hi[a] = job.hi[a];
            }
            q.leaf = 0;
            q.nchild = 0;
            attach(A, job.parent, job.slot, branch);
        }
        if (ok && act) {
            if (split == 0) {
                const int32_t p = (int32_t)pn++;
                PNode &q = A.pn[p];
                for (int a = 0; a < 3; a++) {
                    q.lo[a] = C.box[a][mi][ln];
                    q.hi[a] = C.box[3 + a][mi][ln];
                }
                q.leaf = 1;
                q.nchild = 0;
                q.rec_off = rec;
                q.rec_cnt = n_rec;
                for (uint32_t i = 0; i < n; i++) {
                    const AuxCold &x = lane_cold(A.auxc, L, k, i, ln);
                    if (x.count <= LANE_COPY) lane_copy_records(A.aux_recs, A.recs, x.first, x.count, rec, A.n_prim, A.err);
                    else long_copy = true;
                    rec += x.count;
                }
                C.n[mi][ln] = 1;
                C.leaf[mi][ln] = p;
            } else {
                const int32_t depth = C.depth[mi][ln] + 1;
#pragma unroll
                for (int s = 0; s < 2; s++) {
                    const uint32_t a = s ? split : 0, e = s ? n : split;
                    const int slot = s ? ncuts : mi;
                    LaneBox box;  // the side's box: union of its nodes before refinement
                    lbox_empty(box);
                    for (uint32_t i = a; i < e; i++) lbox_add(box, lane_node(aux, L, k, i, ln));
                    for (int d = 0; d < 3; d++) {
                        C.box[d][slot][ln] = box.lo[d];
                        C.box[3 + d][slot][ln] = box.hi[d];
                    }
                    C.depth[slot][ln] = depth;
                    if (tot[s] == 1) {
                        const AuxCold &x = lane_cold(A.auxc, L, k, a, ln);
                        const int32_t p = (int32_t)pn++;
                        PNode &q = A.pn[p];
                        for (int d = 0; d < 3; d++) {
                            q.lo[d] = box.lo[d];
                            q.hi[d] = box.hi[d];
                        }
                        q.leaf = 1;
                        q.nchild = 0;
                        q.rec_off = rec;
                        q.rec_cnt = x.count;
                        if (x.count <= LANE_COPY) lane_copy_records(A.aux_recs, A.recs, x.first, x.count, rec, A.n_prim, A.err);
                        else long_copy = true;
                        rec += x.count;
                        C.n[slot][ln] = 1;
                        C.leaf[slot][ln] = p;
                    } else {
                        C.off[slot][ln] = pool | 0x80000000u;
                        C.n[slot][ln] = tot[s];
                        C.leaf[slot][ln] = -1;
                        for (uint32_t i = a; i < e; i++) {
                            const uint32_t id = L.id[L.ord[k][i][ln]][ln];
                            if (keep[s] >> (i - a) & 1u) {
                                A.pool_out[pool++] = id;
                            } else {
                                A.pool_out[pool++] = (uint32_t)aux[id].c0;
                                A.pool_out[pool++] = (uint32_t)A.auxc[id].c1;
                            }
                        }
                    }
                }
                ncuts++;
            }
        }
        lane_long_copies(A, L, long_copy, rec_start, split, n, k, tot[0], tot[1]);
    }
    // the branch's children: leaves, and a job for each cut
    uint32_t n_lane_jobs = 0, n_big_jobs = 0;
    if (ok)
        for (int i = 0; i < ncuts; i++)
            if (C.leaf[i][ln] < 0) {
                if (lane_cut_job(A, C.n[i][ln])) n_lane_jobs++;
                else n_big_jobs++;
            }
    uint32_t qs = warp_alloc(&A.g->job_ctr[out], n_lane_jobs, ln);
    uint32_t qb = warp_alloc(&A.g->job_big_ctr[out], n_big_jobs, ln);
    if (ok && ((uint64_t)qs + n_lane_jobs > A.job_cap || (uint64_t)qb + n_big_jobs > A.job_cap)) {
        atomicOr(A.err, GBT_DEVERR_CAPACITY);
        ok = false;
    }
    if (!ok) return;
    PNode &B = A.pn[branch];
    B.nchild = ncuts;
    for (int i = 0; i < ncuts; i++) {
        const int32_t lf = C.leaf[i][ln];
        if (lf >= 0) {
            B.child[i] = lf;
            continue;
        }
        PJob nj;
        nj.off = C.off[i][ln] & 0x7fffffffu;
        nj.n = C.n[i][ln];
        for (int d = 0; d < 3; d++) {
            nj.lo[d] = C.box[d][i][ln];
            nj.hi[d] = C.box[3 + d][i][ln];
        }
        nj.depth = C.depth[i][ln];
        nj.parent = branch;
        nj.slot = i;
        nj.pad = 0;
        if (lane_cut_job(A, nj.n)) A.jobs_out[qs++] = nj;
        else A.jobs_out[A.job_cap - 1 - qb++] = nj;
        my_max_n = max(my_max_n, nj.n);
    }
}

// One tree level.  256-thread blocks take one job at a time (levels with a
// cut of more than PHR_SMALL_CUT nodes).  One-warp blocks take either one job
// of the second list, swept by the whole warp, or 32 jobs of the lane list,
// one per lane; a job of the lane list whose cut does not qualify (the root
// job) is swept by the whole warp after them.
// Shared memory of a level block: with a lane path, its scratch and the
// whole-block state take turns, so they share the space.
template <int BS, int LMODE>
struct LevelSmem {
    BlockShared<BS> block;
};
template <int BS>
struct LevelSmem<BS, 1> {
    union {
        BlockShared<BS> block;
        LaneScratch lane;
    };
};
struct LaneMulti {
    LaneScratchMulti lane;
    LaneCuts cuts;
};
template <int BS>
struct LevelSmem<BS, 2> {
    union {
        BlockShared<BS> block;
        LaneMulti lm;
    };
};

// LMODE (one-warp blocks): 1 the lane path for bf = 2, 2 the lane path for
// bf > 2 in rounds, 0 none (a one-warp block then holds less state and more
// of them are resident).
#ifndef GBT_PHR_LANE_MINB
#define GBT_PHR_LANE_MINB 20  // resident one-warp blocks per SM the lane path's registers are sized for
                              // (24 and 32, with spills, measured slower)
#endif
template <int BS, int LMODE = (BS == 32 ? 1 : 0)>
__global__ void __launch_bounds__(BS, BS == 32 ? (LMODE ? GBT_PHR_LANE_MINB : 32) : (BS == PT ? 2 : 1)) k_phr_level(LevelArgs A) {
    constexpr bool LANES = LMODE != 0;
    __shared__ LevelSmem<BS, LMODE> smem;
    BlockShared<BS> &sh = smem.block;
    const int in = A.parity, out = A.parity ^ 1;
    // Run only as the next level, after no stall and no device error, and only
    // when the level's cuts fit this launch's scratch (else flag a stall: the
    // host relaunches the level with a larger capacity).  Every block decides
    // the same way, so a level runs whole or not at all.
    __shared__ uint32_t s_go, s_nmax;
    if (threadIdx.x == 0) {
        const volatile PhrGlobals *vg = A.g;
        uint32_t go = vg->stall == 0 && vg->level_done == A.level && *(volatile unsigned int *)A.err == 0;
        const uint32_t nm = vg->max_n[in];
        if (go && ((uint64_t)nm << (A.bf > 2 ? A.bf - 2 : 0)) > A.cap) {
            atomicOr(&A.g->stall, 1u);
            go = 0;
        }
        s_go = go;
        s_nmax = nm;
    }
    __syncthreads();
    if (!s_go) return;
    const uint32_t nmax = s_nmax;
    const uint32_t n_lane = A.g->job_ctr[in], n_big = A.g->job_big_ctr[in];
    Scratch S = carve(A.scratch + A.scratch_per_block * blockIdx.x, A.cap);
    if (A.sort_smem) {  // every stage of the bitonic network then reads shared memory, not L2
        extern __shared__ unsigned long long dyn_smem[];
        const uint32_t P = pow2_at_least(A.cap > 0 ? A.cap : 1);
        S.skey = dyn_smem;
        S.sval = reinterpret_cast<uint32_t *>(dyn_smem + P);
    }
    const bool screen = A.g->screen_bad == 0;
    unsigned long long my_build_cost = 0;  // this thread's sums (thread 0 for whole-block jobs)
    uint32_t my_max_n = 0;
    // Work items: one-warp blocks take a second-list job or 32 lane-list jobs (the
    // lanes' own ones first, then any that do not qualify, by the whole warp); wider
    // blocks take one job of either list.  job_block has a single call site.
    const uint32_t items = LANES ? n_big + (n_lane + 31) / 32 : n_lane + n_big;
    for (uint32_t it = blockIdx.x; it < items; it += gridDim.x) {
        uint32_t base = 0;   // the group's first lane-list job
        unsigned rest = 1u;  // bit l: job base + l still to be done by the whole block
        if constexpr (!LANES) {
            base = it < n_lane ? it : A.job_cap - 1 - (it - n_lane);
        } else {
            if (it < n_big) {
                base = A.job_cap - 1 - it;
            } else {
                base = (it - n_big) * 32;
                const uint32_t j = base + threadIdx.x;
                const bool valid = j < n_lane;
                bool mine = false;
                if (valid) {
                    const uint32_t n = A.jobs_in[j].n;
                    mine = lane_cut_job(A, n) && n <= nmax;
                }
                if constexpr (LMODE == 1) lane_jobs(A, j, mine, smem.lane, screen, my_build_cost, my_max_n);
                else lane_jobs_multi(A, j, mine, smem.lm.lane, smem.lm.cuts, screen, my_build_cost, my_max_n);
                rest = __ballot_sync(0xffffffffu, valid && !mine);
            }
        }
        while (rest) {
            const int l = __ffs(rest) - 1;
            rest &= rest - 1;
            job_block<BS>(A, A.jobs_in[base + l], nmax, sh, S, screen, my_build_cost, my_max_n);
        }
    }
    // the block's totals, one atomic each (per-split atomics on these counters contend)
    if (threadIdx.x < 32) {
        for (int o = 16; o > 0; o >>= 1) {
            my_build_cost += __shfl_xor_sync(0xffffffffu, my_build_cost, o);
            my_max_n = max(my_max_n, __shfl_xor_sync(0xffffffffu, my_max_n, o));
        }
        if (threadIdx.x == 0) {
            if (my_build_cost) atomicAdd(&A.g->build_cost, my_build_cost);
            if (my_max_n) atomicMax(&A.g->max_n[out], my_max_n);
        }
    }
    // The last block to finish clears this level's input counters (the output
    // counters of the level after next) and marks the level done.
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&A.g->blocks_done, 1u) == gridDim.x - 1) {
            __threadfence();
            A.g->job_ctr[in] = 0;
            A.g->job_big_ctr[in] = 0;
            A.g->pool_ctr[in] = 0;
            A.g->max_n[in] = 0;
            A.g->err_copy = *(volatile unsigned int *)A.err;
            A.g->blocks_done = 0;
            __threadfence();
            A.g->level_done = A.level + 1;
        }
    }
}

// ---------------------------------------------------------------------------
// traversal nodes
// ---------------------------------------------------------------------------
// Also the parent of every inner node (-1 for the root) and -2 for the entries
// of leaves, which hold no node.
__global__ void k_phr_finalize(const PNode *__restrict__ pn, const PhrGlobals *__restrict__ g, float4 *nodes, int arity,
                               BvhHeader *hdr, uint32_t n_prim, int32_t *__restrict__ parent, unsigned int *err) {
    const uint32_t count = g->pnode_ctr;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        if (g->root < 0 || (uint32_t)g->root >= count) {
            atomicOr(err, GBT_DEVERR_BOUNDS);
            return;
        }
        const PNode &r = pn[g->root];
        hdr->root_ref = r.leaf ? (int32_t)r.rec_off : g->root;
        hdr->root_cnt = r.leaf ? (int32_t)r.rec_cnt : 0;
        for (int k = 0; k < 3; k++) {
            hdr->root_lo[k] = r.lo[k];
            hdr->root_hi[k] = r.hi[k];
        }
        hdr->root_lo[3] = hdr->root_hi[3] = 0.f;
        hdr->n_nodes = count;
        hdr->n_unique = 0;
        hdr->sorted_sel = 0;
    }
    if (i >= count) return;
    const PNode &b = pn[i];
    if (b.leaf) {
        parent[i] = -2;
        return;
    }
    if ((int32_t)i == g->root) parent[i] = -1;
    for (int c = 0; c < b.nchild && c < 4; c++) {
        const int32_t ci = b.child[c];
        if (ci >= 0 && (uint32_t)ci < count && !pn[ci].leaf) parent[ci] = (int32_t)i;
    }
    float lo[4][3], hi[4][3];
    int32_t ref[4], cnt[4];
    for (int c = 0; c < 4; c++) {
        const int32_t ci = c < b.nchild ? b.child[c] : -1;
        if (c < b.nchild && (ci < 0 || (uint32_t)ci >= count)) atomicOr(err, GBT_DEVERR_BOUNDS);
        if (c < b.nchild && ci >= 0 && (uint32_t)ci < count) {
            const PNode &ch = pn[ci];
            for (int k = 0; k < 3; k++) { lo[c][k] = ch.lo[k]; hi[c][k] = ch.hi[k]; }
            ref[c] = ch.leaf ? (int32_t)ch.rec_off : b.child[c];
            cnt[c] = ch.leaf ? (int32_t)ch.rec_cnt : 0;
        } else {
            for (int k = 0; k < 3; k++) { lo[c][k] = INFINITY; hi[c][k] = -INFINITY; }
            ref[c] = 0;
            cnt[c] = -1;
        }
    }
    if (arity == 2) {
        float4 *nd = nodes + 4 * (size_t)i;
        nd[0] = make_float4(lo[0][0], hi[0][0], lo[0][1], hi[0][1]);
        nd[1] = make_float4(lo[1][0], hi[1][0], lo[1][1], hi[1][1]);
        nd[2] = make_float4(lo[0][2], hi[0][2], lo[1][2], hi[1][2]);
        reinterpret_cast<int4 *>(nd)[3] = make_int4(ref[0], cnt[0], ref[1], cnt[1]);
    } else {
        float4 *nd = nodes + 8 * (size_t)i;
        nd[0] = make_float4(lo[0][0], lo[1][0], lo[2][0], lo[3][0]);
        nd[1] = make_float4(hi[0][0], hi[1][0], hi[2][0], hi[3][0]);
        nd[2] = make_float4(lo[0][1], lo[1][1], lo[2][1], lo[3][1]);
        nd[3] = make_float4(hi[0][1], hi[1][1], hi[2][1], hi[3][1]);
        nd[4] = make_float4(lo[0][2], lo[1][2], lo[2][2], lo[3][2]);
        nd[5] = make_float4(hi[0][2], hi[1][2], hi[2][2], hi[3][2]);
        reinterpret_cast<int4 *>(nd)[6] = make_int4(ref[0], ref[1], ref[2], ref[3]);
        reinterpret_cast<int4 *>(nd)[7] = make_int4(cnt[0], cnt[1], cnt[2], cnt[3]);
    }
    (void)n_prim;
}

}  // namespace

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
// One device allocation for the temporaries of a build, carved in 256-byte
// aligned pieces.
struct Arena {
    size_t used = 0;
    char *base = nullptr;
    template <class T>
    void take(T **p, size_t count) {
        *p = reinterpret_cast<T *>(base + used);
        used += gbt_align((count ? count : 1) * sizeof(T));
    }
};

int gbt_phr_run(gbt_ctx *ctx, gbt_bvh *aux, double alpha, double delta, int bf, gbt_bvh *out) {
    cudaStream_t st = ctx->stream;
    // the level loop reads the counters back through the context's pinned buffer
    struct Readback {
        PhrGlobals g;
    };
    static_assert(sizeof(Readback) <= GBT_PINNED_BYTES, "readback exceeds the pinned buffer");
    Readback *hb = static_cast<Readback *>(gbt_pinned(ctx));
    if (!hb) return gbt_fail(ctx, GBT_ENOMEM, "phr: pinned host allocation");
    BvhHeader h;
    GBT_CUDA(ctx, cudaMemcpyAsync(&h, aux->d_hdr, sizeof(h), cudaMemcpyDeviceToHost, st));
    GBT_CUDA(ctx, cudaStreamSynchronize(st));
    const uint32_t U = h.n_unique, N = aux->n_prim;
    const uint32_t n_aux = U > 0 ? 2 * U - 1 : 1;
    // the temporaries live in the context's PHR workspace (grow-only, kept unless
    // GBT_OPT_KEEP_WORKSPACE is 0)
    auto cleanup = [&]() {
        if (!ctx->keep_workspace) {
            cudaStreamSynchronize(st);
            gbt_phr_release(ctx);
        }
    };
    // outputs
    out->n_prim = N;
    const size_t per_node = bf == 2 ? 4 : 8;
    const uint32_t pnode_cap = 2 * n_aux + 2;
    {  // the tree's arrays in one allocation
        const size_t b_prims = gbt_align((size_t)N * 3 * sizeof(float4));
        const size_t b_nodes = gbt_align((size_t)pnode_cap * per_node * sizeof(float4));
        const size_t b_parent = gbt_align((size_t)pnode_cap * sizeof(int32_t));
        void *bp = nullptr;
        size_t got = 0;
        if (gbt_block_get(ctx, b_prims + b_nodes + b_parent + sizeof(BvhHeader), &bp, &got) != cudaSuccess) {
            cudaGetLastError();
            return gbt_fail(ctx, GBT_ENOMEM, "phr: output allocation");
        }
        char *blk = static_cast<char *>(bp);
        out->d_block = blk;
        out->d_block_bytes = got;
        out->d_prims = reinterpret_cast<float4 *>(blk);
        out->d_nodes = reinterpret_cast<float4 *>(blk + b_prims);
        out->d_parent = reinterpret_cast<int32_t *>(blk + b_prims + b_nodes);
        out->d_hdr = reinterpret_cast<BvhHeader *>(blk + b_prims + b_nodes + b_parent);
    }
    out->node_cap = pnode_cap;
    AuxNode *d_aux;
    AuxCold *d_auxc;
    PNode *d_pn;
    PhrGlobals *d_g;
    uint32_t *d_front[2], *d_pool[2];
    PJob *d_jobs[2];
    double *d_thr;
    const uint32_t pool_cap = 3 * n_aux + 4096, job_cap = n_aux + 16;
    Arena ar;
    for (int pass = 0; pass < 2; pass++) {  // sizes, then pointers
        ar.used = 0;
        ar.take(&d_aux, n_aux);
        ar.take(&d_auxc, n_aux);
        ar.take(&d_pn, pnode_cap);
        ar.take(&d_g, 1);
        for (int i = 0; i < 2; i++) ar.take(&d_front[i], 2 * (size_t)n_aux + 2);
        for (int i = 0; i < 2; i++) ar.take(&d_pool[i], pool_cap);
        for (int i = 0; i < 2; i++) ar.take(&d_jobs[i], job_cap);
        ar.take(&d_thr, 2 * DEPTH_TABLE);  // the table, then its float32 band edges
        if (pass == 0) {
            if (ctx->phr_ws_bytes < ar.used) {
                cudaStreamSynchronize(st);
                cudaFree(ctx->phr_ws);
                ctx->phr_ws = nullptr;
                ctx->phr_ws_bytes = 0;
                if (cudaMalloc(&ctx->phr_ws, ar.used) != cudaSuccess) {
                    cudaGetLastError();
                    ctx->phr_ws = nullptr;
                    return gbt_fail(ctx, GBT_ENOMEM, "phr: device allocation of " + std::to_string(ar.used) + " bytes");
                }
                ctx->phr_ws_bytes = ar.used;
            }
            ar.base = static_cast<char *>(ctx->phr_ws);
        }
    }
    // DefaultThreshold table (phr.go:356-358), host float64
    double S;
    {
        const float *lo = h.root_lo, *hi = h.root_hi;
        double w = (double)hi[0] - (double)lo[0], hh = (double)hi[1] - (double)lo[1], d = (double)hi[2] - (double)lo[2];
        S = 2 * w * hh + 2 * w * d + 2 * hh * d;
    }
    std::vector<double> thr(2 * DEPTH_TABLE);
    float *band = reinterpret_cast<float *>(thr.data() + DEPTH_TABLE);
    for (int d = 0; d < DEPTH_TABLE; d++) {
        thr[d] = S / std::pow(2.0, alpha * (double)d + delta);
        band[d] = (float)(thr[d] * gbt_phr::THR_LO);
        band[DEPTH_TABLE + d] = (float)(thr[d] * gbt_phr::THR_HI);
    }
    GBT_CUDA(ctx, cudaMemcpyAsync(d_thr, thr.data(), 2 * DEPTH_TABLE * sizeof(double), cudaMemcpyHostToDevice, st));
    GBT_CUDA(ctx, cudaMemsetAsync(d_g, 0, sizeof(PhrGlobals), st));
    GBT_CUDA(ctx, cudaMemsetAsync(d_g, 0xff, offsetof(PhrGlobals, screen_bad), st));  // counters 0, root -1 below
    GBT_CUDA(ctx, cudaMemsetAsync(d_g, 0, offsetof(PhrGlobals, root), st));
    // The auxiliary nodes need no clearing: k_aux_build writes every field the
    // refinement reads, of every node.  Neither do the output nodes: a level writes
    // each node it allocates (children as their jobs attach them), and
    // k_phr_finalize reads only allocated nodes and attached children.
    k_aux_build<<<(U + 255) / 256 + 1, 256, 0, st>>>(aux->d_hdr, aux->d_nodes, aux->d_size, aux->d_range, aux->d_run,
                                                     d_aux, d_auxc, U, N, d_g);
    const int32_t root = h.root_cnt > 0 ? 0 : h.root_ref;
    k_initial_cut<<<1, 1024, 0, st>>>(d_aux, d_auxc, root, thr[0], d_front[0], d_front[1], d_pool[0], d_jobs[0], d_g, 2 * n_aux + 2);
    GBT_CUDA(ctx, cudaGetLastError());
    GBT_CUDA(ctx, cudaMemcpyAsync(&hb->g, d_g, sizeof(PhrGlobals), cudaMemcpyDeviceToHost, st));
    GBT_CUDA(ctx, cudaStreamSynchronize(st));  // also: the threshold table's pageable source is consumed
    const PhrGlobals &g = hb->g;
    uint32_t n_lane = g.job_ctr[0], n_big = g.job_big_ctr[0], nmax = g.max_n[0];
    uint32_t n_jobs = n_lane + n_big;
    const uint64_t initial_cut = g.pool_ctr[0];
    // whole-block jobs sort in dynamic shared memory up to SORT_SMEM_MAX keys
    GBT_CUDA(ctx, cudaFuncSetAttribute(k_phr_level<PT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       SORT_SMEM_MAX * 12));
    GBT_CUDA(ctx, cudaFuncSetAttribute(k_phr_level<WIDE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       SORT_SMEM_MAX * 12));
    // Levels whose cuts are all small run in batches of SPEC_LEVELS launches
    // with one readback: the next levels' sizes are read on the device, and a
    // launch whose level turns out to have larger cuts does nothing and flags
    // a stall, after which that level is relaunched here with wider blocks.
    uint32_t level = 0;
    int parity = 0;
    // lane path of one-warp levels: bf = 2 one split per lane; bf 3..4 rounds of splits (their
    // cut table marks output-pool offsets with bit 31)
    const int lmode = bf == 2 ? 1 : (bf <= MAX_BF_LANES && pool_cap < 0x80000000u ? 2 : 0);
    while (n_jobs > 0) {
        // one-warp blocks when every cut is small; WIDE-thread blocks for levels of a few
        // large cuts (the first ones), PT-thread blocks otherwise
        const uint32_t small_cut = (uint32_t)ctx->phr_small_cut;
        const int variant = nmax <= small_cut ? 0 : (n_jobs * 4 <= (uint32_t)ctx->num_sms ? 2 : 1);
        // (with branching 2: 4.57 against 4.67 ms per refinement of the 1M soup; branching 4
        // measured no faster)
        const int batch = variant == 0 ? SPEC_LEVELS : (bf == 2 ? GBT_PHR_SPEC_BIG : 1);
        // splits after the first one of a job (bf > 2) sort refined cuts: each refinement at
        // most doubles a cut (binary auxiliary nodes), so bf - 2 of them bound the size
        if (nmax > (1u << 28)) {
            cleanup();
            return gbt_fail(ctx, GBT_ENOMEM, "phr: cut too large");
        }
        // levels of larger cuts launched ahead of their readback get twice the largest cut
        // known now (refinement can grow a cut from one level to the next; a level whose
        // cuts still do not fit flags a stall and is relaunched here), unless the headroom
        // would push the cut's sort out of shared memory
        const uint32_t shift = bf > 2 ? (uint32_t)(bf - 2) : 0u;
        const uint32_t big = batch > 1 && pow2_at_least((2 * nmax) << shift) <= SORT_SMEM_MAX ? 2 * nmax : nmax;
        const uint32_t cap = (variant == 0 ? small_cut : big) << shift;
        const uint32_t sort_p = pow2_at_least(cap > 0 ? cap : 1);
        const size_t dyn = variant != 0 && sort_p <= SORT_SMEM_MAX ? (size_t)sort_p * 12 : 0;
        // grid: at most the blocks that are resident at once
        int per_sm = 0;
        if (variant == 0 && lmode == 1) GBT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_phr_level<32, 1>, 32, 0));
        else if (variant == 0 && lmode == 2) GBT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_phr_level<32, 2>, 32, 0));
        else if (variant == 0) GBT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_phr_level<32, 0>, 32, 0));
        else if (variant == 1) GBT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_phr_level<PT>, PT, dyn));
        else GBT_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_phr_level<WIDE>, WIDE, dyn));
        const uint32_t max_grid = (uint32_t)ctx->num_sms * (uint32_t)std::max(1, per_sm);
        // work items: one-warp blocks with lanes (bf = 2) take a second-list job or 32
        // lane-list jobs; the batch's later levels are not known yet and get the full grid
        const uint32_t items = variant == 0 && lmode ? n_big + (n_lane + 31) / 32 : n_jobs;
        const uint32_t grid0 = std::min<uint32_t>(items, max_grid);
        const size_t per_block = gbt_align(scratch_bytes_for(cap));
        const uint32_t blocks = batch > 1 ? max_grid : grid0;
        if (per_block * blocks > ctx->phr_scr_bytes) {
            // sized for every block the variant can have resident, so that later
            // levels seldom need to grow it
            const size_t need = per_block * max_grid;
            cudaStreamSynchronize(st);
            cudaFree(ctx->phr_scr);
            ctx->phr_scr = nullptr;
            ctx->phr_scr_bytes = 0;
            if (cudaMalloc(&ctx->phr_scr, need) != cudaSuccess) {
                cudaGetLastError();
                ctx->phr_scr = nullptr;
                cleanup();
                return gbt_fail(ctx, GBT_ENOMEM, "phr: scratch");
            }
            ctx->phr_scr_bytes = need;
        }
        void *scratch = ctx->phr_scr;
        for (int bi = 0; bi < batch; bi++) {
            const uint32_t lv = level + (uint32_t)bi;
            const int par = (int)(lv & 1u), o = par ^ 1;
            LevelArgs A;
            A.aux = d_aux;
            A.auxc = d_auxc;
            A.aux_recs = aux->d_prims;
            A.recs = out->d_prims;
            A.pn = d_pn;
            A.thr = d_thr;
            A.thr_lo = reinterpret_cast<const float *>(d_thr + DEPTH_TABLE);
            A.thr_hi = A.thr_lo + DEPTH_TABLE;
            A.jobs_in = d_jobs[par];
            A.jobs_out = d_jobs[o];
            A.pool_in = d_pool[par];
            A.pool_out = d_pool[o];
            A.g = d_g;
            A.parity = par;
            A.pool_cap = pool_cap;
            A.job_cap = job_cap;
            A.pnode_cap = pnode_cap;
            A.level = lv;
            A.cap = cap;
            A.scratch = static_cast<unsigned char *>(scratch);
            A.scratch_per_block = per_block;
            A.sort_smem = dyn ? 1u : 0u;
            A.bf = bf;
            A.n_prim = N;
            A.err = ctx->d_error;
            const uint32_t grid = bi == 0 ? grid0 : max_grid;
            if (variant == 0 && lmode == 1) k_phr_level<32, 1><<<grid, 32, 0, st>>>(A);
            else if (variant == 0 && lmode == 2) k_phr_level<32, 2><<<grid, 32, 0, st>>>(A);
            else if (variant == 0) k_phr_level<32, 0><<<grid, 32, 0, st>>>(A);
            else if (variant == 1) k_phr_level<PT><<<grid, PT, dyn, st>>>(A);
            else k_phr_level<WIDE><<<grid, WIDE, dyn, st>>>(A);
            GBT_CUDA(ctx, cudaGetLastError());
        }
        GBT_CUDA(ctx, cudaMemcpyAsync(&hb->g, d_g, sizeof(PhrGlobals), cudaMemcpyDeviceToHost, st));
        GBT_CUDA(ctx, cudaStreamSynchronize(st));
        if (g.err_copy) break;  // reported by the caller's device-error check
        if (g.level_done == level) {  // the first launch of a batch always fits: nothing moved
            unsigned int flags = 0;
            GBT_CUDA(ctx, cudaMemcpy(&flags, ctx->d_error, sizeof(flags), cudaMemcpyDeviceToHost));
            if (flags) break;  // an earlier device error: reported by the caller's check
            cleanup();
            return gbt_fail(ctx, GBT_EDEVICE, "phr: a level made no progress");
        }
        level = g.level_done;
        parity = (int)(level & 1u);
        if (g.stall) GBT_CUDA(ctx, cudaMemsetAsync(reinterpret_cast<char *>(d_g) + offsetof(PhrGlobals, stall), 0, 4, st));
        n_lane = g.job_ctr[parity];
        n_big = g.job_big_ctr[parity];
        if ((uint64_t)n_lane + n_big > job_cap) {  // the two lists met
            const unsigned int flags = GBT_DEVERR_CAPACITY;
            GBT_CUDA(ctx, cudaMemcpy(ctx->d_error, &flags, sizeof(flags), cudaMemcpyHostToDevice));
            break;
        }
        n_jobs = n_lane + n_big;
        nmax = g.max_n[parity];
    }
    k_phr_finalize<<<(pnode_cap + 255) / 256, 256, 0, st>>>(d_pn, d_g, out->d_nodes, bf == 2 ? 2 : 4, out->d_hdr, N,
                                                            out->d_parent,
                                                            ctx->d_error);
    GBT_CUDA(ctx, cudaGetLastError());
    GBT_CUDA(ctx, cudaMemcpyAsync(&hb->g, d_g, sizeof(PhrGlobals), cudaMemcpyDeviceToHost, st));
    GBT_CUDA(ctx, cudaStreamSynchronize(st));
    out->n_nodes_host = g.pnode_ctr;
    out->build_cost = (int64_t)(initial_cut + g.build_cost);  // BuildWithCost (phr.go:154-192)
    cleanup();
    return GBT_OK;
}

void gbt_phr_release(gbt_ctx *ctx) {
    cudaFree(ctx->phr_ws);
    cudaFree(ctx->phr_scr);
    ctx->phr_ws = nullptr;
    ctx->phr_scr = nullptr;
    ctx->phr_ws_bytes = 0;
    ctx->phr_scr_bytes = 0;
}
