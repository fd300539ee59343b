// Closest-hit ray traversal (pkg/pt/bvh.go:74-77, 179-199 BVH.intersected).
//
// One thread per ray walks the tree with a local stack, nearer child first.
// A 64-byte binary node is four float4 loaded with 128-bit loads:
//   n0 = (L.lo.x, L.hi.x, L.lo.y, L.hi.y)   n1 = same for R
//   n2 = (L.lo.z, L.hi.z, R.lo.z, R.hi.z)   n3 = (L.ref, L.cnt, R.ref, R.cnt)
// A child with cnt > 0 is a leaf of cnt primitive records starting at ref;
// cnt == 0 is the inner node ref; cnt < 0 is an empty slot.
// A 128-byte 4-wide node (PHR with branching factor 3 or 4) is eight float4:
//   m0..m5 = lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4], hi.z[4]
//   m6 = ref[4], m7 = cnt[4]
// Primitive records are three float4 (r0 = v0|id, r1 = v1|kind, r2 = v2);
// a sphere record holds (centre|id, radius|kind).
//
// The primitive tests are pkg/pt/primitive.go:172-208 (Moeller-Trumbore with
// the absolute |det| <= 1e-7 rejection, u in [0,1], v >= 0, u+v <= 1,
// tmin <= t <= tmax) and :56-86 (sphere, exclusive t bounds), in float32.
#include <cuda_runtime.h>

#include <type_traits>

#include "gbt_internal.cuh"
#include "traverse.cuh"

namespace {

template <bool COUNT>
__device__ __forceinline__ void flush_work(const gbt_dev::Work &w, unsigned long long *counters) {
    if (!COUNT) return;
    // every lane of the warp reaches this point (no early return in the kernels)
    __syncwarp();
    unsigned long long a = w.nodes, b = w.prims;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counters, a);
        atomicAdd(counters + 1, b);
    }
}

template <bool COUNT>
__global__ void __launch_bounds__(128) k_trace2(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes,
                                                const float4 *__restrict__ recs, const float4 *__restrict__ rays,
                                                float4 *__restrict__ hits, uint32_t n, const uint32_t *__restrict__ d_count,
                                                int out_mode, unsigned int *err, unsigned long long *counters) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cnt = d_count ? *d_count : n;
    gbt_dev::Work w;
    if (i < cnt) {
        gbt_dev::Ray ray = gbt_dev::load_ray(rays, i);
        gbt_dev::Hit h = gbt_dev::closest_hit2<64, COUNT>(*hdr, nodes, recs, ray, err, &w);
        gbt_dev::store_hit(hits, i, h, recs, out_mode);
    }
    flush_work<COUNT>(w, counters);
}

template <bool COUNT>
__global__ void __launch_bounds__(128) k_trace4(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes,
                                                const float4 *__restrict__ recs, const float4 *__restrict__ rays,
                                                float4 *__restrict__ hits, uint32_t n, const uint32_t *__restrict__ d_count,
                                                int out_mode, unsigned int *err, unsigned long long *counters) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cnt = d_count ? *d_count : n;
    gbt_dev::Work w;
    if (i < cnt) {
        gbt_dev::Ray ray = gbt_dev::load_ray(rays, i);
        gbt_dev::Hit h = gbt_dev::closest_hit4<96, COUNT>(*hdr, nodes, recs, ray, err, &w);
        gbt_dev::store_hit(hits, i, h, recs, out_mode);
    }
    flush_work<COUNT>(w, counters);
}

// 1: packet warps whose rays share an octant run the loop instantiated for it.
#ifndef GBT_PACKET_OCT
#define GBT_PACKET_OCT 1
#endif

// The node loop of k_trace_packet4 from `node` on: the warp's stack is se/st in
// shared memory.  OCT in 0..7 when every ray of the warp lies in that octant
// (the slab tests then pick planes by sign), -1 otherwise.
template <bool COUNT, int OCT>
__device__ __forceinline__ void packet4_loop(int2 node, const float4 *__restrict__ nodes,
                                             const float4 *__restrict__ recs, const gbt_dev::Ray &r, gbt_dev::Hit &h,
                                             int2 *se, float *st, int lane, unsigned int *err, gbt_dev::Work &w) {
    constexpr int PSTACK = 96;
    constexpr uint32_t FULL = 0xffffffffu;
    const float MISS = __int_as_float(0x7f800000);
    int sp = 0;
    auto pop = [&]() -> int2 {
        while (sp > 0) {
            --sp;
            const float t = st[sp];
            const int2 e = se[sp];
            if (__any_sync(FULL, t <= h.t * 1.0000005f)) return e;
        }
        return make_int2(0, -1);
    };
    for (;;) {
        if (node.y == 0) {
            if (COUNT && lane == 0) w.nodes++;
            const float4 *nd = nodes + 8 * (size_t)node.x;
            float4 lx, hx, ly, hy, lz, hz, rff, cnf;
            gbt_dev::ldg256(nd, lx, hx);
            gbt_dev::ldg256(nd + 2, ly, hy);
            gbt_dev::ldg256(nd + 4, lz, hz);
            gbt_dev::ldg256(nd + 6, rff, cnf);
            float t;
            // per lane entry distance (+0 for -0, so that unsigned min orders them), MISS if missed
            const float t0 = (__float_as_int(cnf.x) >= 0 && gbt_dev::slab_sel<OCT>(lx.x, ly.x, lz.x, hx.x, hy.x, hz.x, r, h.t, t)) ? t + 0.f : MISS;
            const float t1 = (__float_as_int(cnf.y) >= 0 && gbt_dev::slab_sel<OCT>(lx.y, ly.y, lz.y, hx.y, hy.y, hz.y, r, h.t, t)) ? t + 0.f : MISS;
            const float t2 = (__float_as_int(cnf.z) >= 0 && gbt_dev::slab_sel<OCT>(lx.z, ly.z, lz.z, hx.z, hy.z, hz.z, r, h.t, t)) ? t + 0.f : MISS;
            const float t3 = (__float_as_int(cnf.w) >= 0 && gbt_dev::slab_sel<OCT>(lx.w, ly.w, lz.w, hx.w, hy.w, hz.w, r, h.t, t)) ? t + 0.f : MISS;
            // the children any lane hits, as one warp-wide mask: none -> pop, one -> take it;
            // only two or more need the warp's entry distances and the sorting network
            const uint32_t hm = __reduce_or_sync(FULL, (t0 != MISS ? 1u : 0u) | (t1 != MISS ? 2u : 0u) |
                                                           (t2 != MISS ? 4u : 0u) | (t3 != MISS ? 8u : 0u));
            if (hm == 0) {
                node = pop();
                continue;
            }
            if ((hm & (hm - 1)) == 0) {
                const int k = __ffs(hm) - 1;
                node = make_int2(__float_as_int(k == 0 ? rff.x : k == 1 ? rff.y : k == 2 ? rff.z : rff.w),
                                 __float_as_int(k == 0 ? cnf.x : k == 1 ? cnf.y : k == 2 ? cnf.z : cnf.w));
                continue;
            }
            if (__popc(hm) == 2) {  // two: the nearer taken, the farther pushed
                const int ka = __ffs(hm) - 1, kb = __ffs(hm & (hm - 1)) - 1;
                const float ta = __uint_as_float(__reduce_min_sync(
                    FULL, __float_as_uint(ka == 0 ? t0 : ka == 1 ? t1 : ka == 2 ? t2 : t3)));
                const float tb = __uint_as_float(__reduce_min_sync(
                    FULL, __float_as_uint(kb == 1 ? t1 : kb == 2 ? t2 : t3)));
                const int2 ea = make_int2(__float_as_int(ka == 0 ? rff.x : ka == 1 ? rff.y : rff.z),
                                          __float_as_int(ka == 0 ? cnf.x : ka == 1 ? cnf.y : cnf.z));
                const int2 eb = make_int2(__float_as_int(kb == 1 ? rff.y : kb == 2 ? rff.z : rff.w),
                                          __float_as_int(kb == 1 ? cnf.y : kb == 2 ? cnf.z : cnf.w));
                const bool a_first = !(tb < ta);
                if (sp + 1 > PSTACK) {
                    if (lane == 0) atomicOr(err, GBT_DEVERR_STACK);
                } else {
                    if (lane == 0) {
                        se[sp] = a_first ? eb : ea;
                        st[sp] = a_first ? tb : ta;
                    }
                    sp += 1;
                    __syncwarp();
                }
                node = a_first ? ea : eb;
                continue;
            }
            gbt_dev::Cand c0, c1, c2, c3;
            c0.t = __uint_as_float(__reduce_min_sync(FULL, __float_as_uint(t0)));
            c1.t = __uint_as_float(__reduce_min_sync(FULL, __float_as_uint(t1)));
            c2.t = __uint_as_float(__reduce_min_sync(FULL, __float_as_uint(t2)));
            c3.t = __uint_as_float(__reduce_min_sync(FULL, __float_as_uint(t3)));
            c0.e = make_int2(__float_as_int(rff.x), __float_as_int(cnf.x));
            c1.e = make_int2(__float_as_int(rff.y), __float_as_int(cnf.y));
            c2.e = make_int2(__float_as_int(rff.z), __float_as_int(cnf.z));
            c3.e = make_int2(__float_as_int(rff.w), __float_as_int(cnf.w));
            gbt_dev::cx(c0, c1);
            gbt_dev::cx(c2, c3);
            gbt_dev::cx(c0, c2);
            gbt_dev::cx(c1, c3);
            gbt_dev::cx(c1, c2);
            const int np = (c1.t != MISS) + (c2.t != MISS) + (c3.t != MISS);
            if (sp + np > PSTACK) {
                if (lane == 0) atomicOr(err, GBT_DEVERR_STACK);
            } else {
                if (lane == 0) {
                    int q = sp;
                    if (c3.t != MISS) { se[q] = c3.e; st[q] = c3.t; ++q; }
                    if (c2.t != MISS) { se[q] = c2.e; st[q] = c2.t; ++q; }
                    if (c1.t != MISS) { se[q] = c1.e; st[q] = c1.t; ++q; }
                }
                sp += np;
                __syncwarp();
            }
            node = c0.e;
        } else if (node.y > 0) {
            if (COUNT && lane == 0) w.prims += (uint32_t)node.y;
            gbt_dev::leaf(recs, node.x, node.y, r, h);
            node = pop();
        } else {
            break;
        }
    }
}

// Packet traversal of a 4-wide tree for coherent rays (camera rays of one 8x4
// pixel tile per warp): the warp walks one node sequence with a stack in shared
// memory; each lane tests every child box against its own ray and closest hit,
// the children that any lane hits are taken nearest first by the warp's
// smallest entry distance, and a popped entry is skipped when no lane can
// still reach it.  Control flow is uniform across the warp.  Each lane keeps
// its own closest hit, so the hits equal the single-ray kernels' (exact ties
// go to the lower record whatever the order).  A warp whose rays share one
// octant (almost every tile of a pinhole camera) runs the loop instantiated
// for that octant.  Counters (profiling level 2) count the warp's node
// fetches and leaf visits.
template <bool COUNT>
__global__ void __launch_bounds__(128) k_trace_packet4(const BvhHeader *__restrict__ hdr,
                                                       const float4 *__restrict__ nodes, const float4 *__restrict__ recs,
                                                       const float4 *__restrict__ rays, float4 *__restrict__ hits,
                                                       uint32_t n, int out_mode, unsigned int *err,
                                                       unsigned long long *counters) {
    constexpr int PSTACK = 96;
    constexpr uint32_t FULL = 0xffffffffu;
    __shared__ int2 s_e[4][PSTACK];
    __shared__ float s_t[4][PSTACK];
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t id = blockIdx.x * 128 + threadIdx.x;
    const bool live = id < n;
    gbt_dev::Work w;
    gbt_dev::Ray r;
    if (live) {
        r = gbt_dev::load_ray(rays, id);
    } else {  // a ray that hits nothing keeps the lane in step (tmin > tmax: every slab test fails)
        r.o = make_float3(0.f, 0.f, 0.f);
        r.d = make_float3(1.f, 1.f, 1.f);
        r.tmin = 1.f;
        r.tmax = 0.f;
        gbt_dev::finish_ray(r);
    }
    gbt_dev::Hit h;
    h.t = r.tmax;
    h.u = h.v = 0.f;
    h.rec = -1;
    float te;
    const bool root_hit = gbt_dev::slab(hdr->root_lo[0], hdr->root_lo[1], hdr->root_lo[2], hdr->root_hi[0],
                                        hdr->root_hi[1], hdr->root_hi[2], r, h.t, te);
    const int2 node = __any_sync(FULL, root_hit) ? make_int2(hdr->root_ref, hdr->root_cnt) : make_int2(0, -1);
    const uint32_t octs = __reduce_or_sync(FULL, live ? 1u << gbt_dev::octant(r) : 0u);
    const int oct = GBT_PACKET_OCT && __popc(octs) == 1 ? __ffs(octs) - 1 : -1;
    int2 *se = s_e[wp];
    float *st = s_t[wp];
    switch (oct) {
        case 0: packet4_loop<COUNT, 0>(node, nodes, recs, r, h, se, st, lane, err, w); break;
        case 1: packet4_loop<COUNT, 1>(node, nodes, recs, r, h, se, st, lane, err, w); break;
        case 2: packet4_loop<COUNT, 2>(node, nodes, recs, r, h, se, st, lane, err, w); break;
        case 3: packet4_loop<COUNT, 3>(node, nodes, recs, r, h, se, st, lane, err, w); break;
        case 4: packet4_loop<COUNT, 4>(node, nodes, recs, r, h, se, st, lane, err, w); break;
        case 5: packet4_loop<COUNT, 5>(node, nodes, recs, r, h, se, st, lane, err, w); break;
        case 6: packet4_loop<COUNT, 6>(node, nodes, recs, r, h, se, st, lane, err, w); break;
        case 7: packet4_loop<COUNT, 7>(node, nodes, recs, r, h, se, st, lane, err, w); break;
        default: packet4_loop<COUNT, -1>(node, nodes, recs, r, h, se, st, lane, err, w); break;
    }
    if (live) gbt_dev::store_hit(hits, id, h, recs, out_mode);
    flush_work<COUNT>(w, counters);
}

// One packet walk over a 4-wide tree by a warp of a 128-thread block: every
// lane takes part (a lane without a ray carries one that misses everything).
// The warp's stack lives in shared memory; the node loop is k_trace_packet4's
// general one (instantiated per octant as well, it left this kernel spilling).
template <bool COUNT>
__device__ __forceinline__ void packet_walk4(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes,
                                             const float4 *__restrict__ recs, const gbt_dev::Ray &r, gbt_dev::Hit &h,
                                             unsigned int *err, gbt_dev::Work &w) {
    constexpr int PSTACK = 96;
    constexpr uint32_t FULL = 0xffffffffu;
    __shared__ int2 s_e[4][PSTACK];
    __shared__ float s_t[4][PSTACK];
    const int wp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float te;
    const bool root_hit = gbt_dev::slab(hdr->root_lo[0], hdr->root_lo[1], hdr->root_lo[2], hdr->root_hi[0],
                                        hdr->root_hi[1], hdr->root_hi[2], r, h.t, te);
    const int2 node = __any_sync(FULL, root_hit) ? make_int2(hdr->root_ref, hdr->root_cnt) : make_int2(0, -1);
    packet4_loop<COUNT, -1>(node, nodes, recs, r, h, s_e[wp], s_t[wp], lane, err, w);
    __syncwarp();  // the stack is free for the warp's next walk
}

__device__ __forceinline__ gbt_dev::Ray missing_ray() {  // a ray that hits nothing keeps a lane in step
    gbt_dev::Ray r;
    r.o = make_float3(0.f, 0.f, 0.f);
    r.d = make_float3(1.f, 1.f, 1.f);
    r.tmin = 1.f;
    r.tmax = 0.f;
    gbt_dev::finish_ray(r);
    return r;
}

// The packet traversal over camera rays of many trees (a batched frame, the
// tree index in aux[2 i + 1].w): a warp walks once per distinct tree among its
// 32 rays, with the other lanes carrying missing rays.  Hits are (t, u, v, record).
__global__ void __launch_bounds__(128) k_trace_packet4_multi(const TreeRef *__restrict__ trees, uint32_t stride,
                                                             const float4 *__restrict__ rays,
                                                             const float4 *__restrict__ aux, float4 *__restrict__ hits,
                                                             uint32_t n, unsigned int *err) {
    const uint32_t id = blockIdx.x * 128 + threadIdx.x;
    const bool live = id < n;
    gbt_dev::Work w;
    const int item = live ? __float_as_int(__ldg(&aux[2 * (size_t)id + 1].w)) : -1;
    const gbt_dev::Ray mine = live ? gbt_dev::load_ray(rays, id) : missing_ray();
    gbt_dev::Hit out;
    uint32_t todo = __ballot_sync(0xffffffffu, live);
    while (todo) {
        const int it = __shfl_sync(0xffffffffu, item, __ffs(todo) - 1);
        const bool in = live && item == it;
        todo &= ~__ballot_sync(0xffffffffu, in);
        const TreeRef tr = *reinterpret_cast<const TreeRef *>(reinterpret_cast<const unsigned char *>(trees) +
                                                              (size_t)it * stride);
        const gbt_dev::Ray r = in ? mine : missing_ray();
        gbt_dev::Hit h;
        h.t = r.tmax;
        h.u = h.v = 0.f;
        h.rec = -1;
        packet_walk4<false>(tr.hdr, tr.nodes, tr.recs, r, h, err, w);
        if (in) out = h;
    }
    if (live) gbt_dev::store_hit(hits, id, out, nullptr, 1);
}

__device__ __forceinline__ uint32_t lane_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Resident blocks per SM the register budget is sized for (64 registers a thread at 8).
// A warp refills its idle lanes with new rays once fewer than this many are busy.
#ifndef GBT_PT_DYN
#define GBT_PT_DYN 16
#endif
#ifndef GBT_PT_MINB
#define GBT_PT_MINB 8
#endif
// Stack entries of each thread kept in shared memory (the bottom SH slots); 0: all local.
#ifndef GBT_PT_SH
#define GBT_PT_SH 12
#endif
// The same two settings for the any-hit queries past MaxDepth (their own instantiation).
#ifndef GBT_PT_DYN_ANY
#define GBT_PT_DYN_ANY GBT_PT_DYN
#endif
#ifndef GBT_PT_SH_ANY
#define GBT_PT_SH_ANY GBT_PT_SH
#endif


// AM 0: closest hit.  AM 1: stop at the first hit found (for rays whose shading only
// needs hit or miss).
template <int W, bool COUNT, int DYN, int AM>
__global__ void __launch_bounds__(128, GBT_PT_MINB) k_trace_pt(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes,
                                                  const float4 *__restrict__ recs, const float4 *__restrict__ rays,
                                                  float4 *__restrict__ hits, uint32_t n,
                                                  const uint32_t *__restrict__ d_count, int out_mode, unsigned int *err,
                                                  unsigned long long *counters, uint32_t *fetch) {
    constexpr int STACK = W == 2 ? 64 : 96;
    constexpr int SH = AM > 0 ? GBT_PT_SH_ANY : GBT_PT_SH;
    constexpr bool ANY = AM > 0;
    const uint32_t total = d_count ? *d_count : n;
    const uint32_t lane = threadIdx.x & 31;
    using StackT = typename std::conditional<(SH > 0), gbt_dev::SharedTopStack<STACK, (SH > 0 ? SH : 1)>,
                                             gbt_dev::LocalStack<STACK>>::type;
    StackT st;
    if constexpr (SH > 0) {
        __shared__ int2 s_se[SH * 128];
        __shared__ float s_st[SH * 128];
        st.se = s_se + threadIdx.x;
        st.st = s_st + threadIdx.x;
        st.stride = 128;
    }
    int sp = 0;
    int2 node = make_int2(0, -1), leaf = make_int2(0, 0);
    gbt_dev::Ray r;
    gbt_dev::Hit h;
    gbt_dev::Work w;
    h.t = 0.f;
    h.u = h.v = 0.f;
    h.rec = -1;
    uint32_t rid = 0xffffffffu;
    bool pool_empty = false;  // warp-uniform
    for (;;) {
        if (node.y < 0 && leaf.y <= 0 && rid != 0xffffffffu) {  // this lane's ray is done
            gbt_dev::store_hit(hits, rid, h, recs, out_mode);
            rid = 0xffffffffu;
        }
        const bool want = rid == 0xffffffffu && !pool_empty;
        const uint32_t need = __ballot_sync(0xffffffffu, want);
        if (need) {
            const int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if (lane == (uint32_t)leader) base = atomicAdd(fetch, (uint32_t)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            bool empty_here = false;
            if (want) {
                const uint32_t id = base + __popc(need & lane_lt());
                if (id < total) {
                    rid = id;
                    r = gbt_dev::load_ray(rays, id);
                    h.t = r.tmax;
                    h.u = h.v = 0.f;
                    h.rec = -1;
                    sp = 0;
                    leaf = make_int2(0, 0);
                    float te;
                    const float *lo = hdr->root_lo, *hi = hdr->root_hi;
                    node = gbt_dev::slab(lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], r, h.t, te)
                               ? make_int2(hdr->root_ref, hdr->root_cnt)
                               : make_int2(0, -1);
                    if (node.y > 0) {  // a leaf root
                        leaf = node;
                        node = make_int2(0, -1);
                    }
                } else {
                    empty_here = true;
                }
            }
            pool_empty = __any_sync(0xffffffffu, empty_here) || pool_empty;
        }
        if (__all_sync(0xffffffffu, rid == 0xffffffffu)) break;
        while (node.y >= 0 || leaf.y > 0) {
            while (node.y == 0) {
                if (COUNT) w.nodes++;
                node = W == 2 ? gbt_dev::step2(nodes, node, st, sp, r, h.t, err)
                              : gbt_dev::step4(nodes, node, st, sp, r, h.t, err);
                if (node.y > 0 && leaf.y <= 0) {  // postpone the leaf, keep descending
                    leaf = node;
                    node = st.pop(sp, h.t);
                }
                if (!__any_sync(__activemask(), leaf.y <= 0)) break;  // every lane here holds a leaf
            }
            while (leaf.y > 0) {
                if (COUNT) w.prims += (uint32_t)leaf.y;
                gbt_dev::leaf(recs, leaf.x, leaf.y, r, h);
                if (ANY && h.rec >= 0) {  // any hit ends the query
                    node = make_int2(0, -1);
                    leaf = make_int2(0, 0);
                    sp = 0;
                } else if (node.y > 0) {
                    leaf = node;
                    node = st.pop(sp, h.t);
                } else {
                    leaf = make_int2(0, 0);
                }
            }
            if (DYN > 0 && !pool_empty && __popc(__activemask()) < DYN) break;
        }
    }
    flush_work<COUNT>(w, counters);
}

// The persistent traversal over the rays of many trees (a batched frame):
// each lane takes its tree, and whether its ray is an any-hit query, from the
// tree table when it fetches a ray.  Hits are written as (t, u, v, record).
template <int W, int DYN>
__global__ void __launch_bounds__(128, GBT_PT_MINB) k_trace_multi(const TreeRef *__restrict__ trees, uint32_t stride,
                                                                  const float4 *__restrict__ rays,
                                                                  const float4 *__restrict__ aux,
                                                                  float4 *__restrict__ hits, uint32_t n,
                                                                  const uint32_t *__restrict__ d_count, int level,
                                                                  unsigned int *err, uint32_t *fetch) {
    constexpr int STACK = W == 2 ? 64 : 96;
    constexpr int SH = GBT_PT_SH;
    const uint32_t total = d_count ? *d_count : n;
    const uint32_t lane = threadIdx.x & 31;
    __shared__ int2 s_se[SH * 128];
    __shared__ float s_st[SH * 128];
    gbt_dev::SharedTopStack<STACK, SH> st;
    st.se = s_se + threadIdx.x;
    st.st = s_st + threadIdx.x;
    st.stride = 128;
    int sp = 0;
    int2 node = make_int2(0, -1), leaf = make_int2(0, 0);
    gbt_dev::Ray r;
    gbt_dev::Hit h;
    h.t = 0.f;
    h.u = h.v = 0.f;
    h.rec = -1;
    const float4 *nodes = nullptr, *recs = nullptr;
    bool any = false;
    uint32_t rid = 0xffffffffu;
    bool pool_empty = false;  // warp-uniform
    for (;;) {
        if (node.y < 0 && leaf.y <= 0 && rid != 0xffffffffu) {
            gbt_dev::store_hit(hits, rid, h, recs, 1);
            rid = 0xffffffffu;
        }
        const bool want = rid == 0xffffffffu && !pool_empty;
        const uint32_t need = __ballot_sync(0xffffffffu, want);
        if (need) {
            const int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if (lane == (uint32_t)leader) base = atomicAdd(fetch, (uint32_t)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            bool empty_here = false;
            if (want) {
                const uint32_t id = base + __popc(need & lane_lt());
                if (id < total) {
                    const TreeRef tr = *reinterpret_cast<const TreeRef *>(
                        reinterpret_cast<const unsigned char *>(trees) +
                        (size_t)__float_as_int(__ldg(&aux[2 * (size_t)id + 1].w)) * stride);
                    rid = id;
                    r = gbt_dev::load_ray(rays, id);
                    nodes = tr.nodes;
                    recs = tr.recs;
                    any = tr.any_level == level;
                    h.t = r.tmax;
                    h.u = h.v = 0.f;
                    h.rec = -1;
                    sp = 0;
                    leaf = make_int2(0, 0);
                    float te;
                    const float *lo = tr.hdr->root_lo, *hi = tr.hdr->root_hi;
                    node = gbt_dev::slab(lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], r, h.t, te)
                               ? make_int2(tr.hdr->root_ref, tr.hdr->root_cnt)
                               : make_int2(0, -1);
                    if (node.y > 0) {
                        leaf = node;
                        node = make_int2(0, -1);
                    }
                } else {
                    empty_here = true;
                }
            }
            pool_empty = __any_sync(0xffffffffu, empty_here) || pool_empty;
        }
        if (__all_sync(0xffffffffu, rid == 0xffffffffu)) break;
        while (node.y >= 0 || leaf.y > 0) {
            while (node.y == 0) {
                node = W == 2 ? gbt_dev::step2(nodes, node, st, sp, r, h.t, err)
                              : gbt_dev::step4(nodes, node, st, sp, r, h.t, err);
                if (node.y > 0 && leaf.y <= 0) {
                    leaf = node;
                    node = st.pop(sp, h.t);
                }
                if (!__any_sync(__activemask(), leaf.y <= 0)) break;
            }
            while (leaf.y > 0) {
                gbt_dev::leaf(recs, leaf.x, leaf.y, r, h);
                if (any && h.rec >= 0) {  // any hit ends the query
                    node = make_int2(0, -1);
                    leaf = make_int2(0, 0);
                    sp = 0;
                } else if (node.y > 0) {
                    leaf = node;
                    node = st.pop(sp, h.t);
                } else {
                    leaf = make_int2(0, 0);
                }
            }
            if (DYN > 0 && !pool_empty && __popc(__activemask()) < DYN) break;
        }
    }
}

template <int W, bool COUNT, int DYN, int AM>
void launch_pt(gbt_ctx *ctx, const BvhHeader *hdr, const float4 *nodes, const float4 *recs, const float4 *rays,
               float4 *hits, uint32_t n, const uint32_t *d_count, int out_mode, unsigned long long *counters,
               cudaStream_t s) {
    static int per_sm = 0;  // resident blocks per SM of this instantiation
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_pt<W, COUNT, DYN, AM>, 128, 0);
        if (per_sm <= 0) per_sm = 1;
    }
    uint32_t *fetch = reinterpret_cast<uint32_t *>(ctx->d_counters + 3);
    cudaMemsetAsync(fetch, 0, sizeof(uint32_t), s);
    uint32_t grid = (uint32_t)(ctx->num_sms * per_sm);
    uint32_t need = (n + 127) / 128;
    if (need < grid) grid = need;
    k_trace_pt<W, COUNT, DYN, AM><<<grid, 128, 0, s>>>(hdr, nodes, recs, rays, hits, n, d_count, out_mode, ctx->d_error,
                                                     counters, fetch);
}

template <int W, int DYN>
void launch_pt_any(gbt_ctx *ctx, const BvhHeader *hdr, const float4 *nodes, const float4 *recs, const float4 *rays,
                   float4 *hits, uint32_t n, const uint32_t *d_count, int out_mode, unsigned long long *counters,
                   cudaStream_t s, bool any) {
    constexpr int DYN_ANY = DYN > 0 ? GBT_PT_DYN_ANY : 0;
    if (any) {
        if (counters) launch_pt<W, true, DYN_ANY, 1>(ctx, hdr, nodes, recs, rays, hits, n, d_count, out_mode, counters, s);
        else launch_pt<W, false, DYN_ANY, 1>(ctx, hdr, nodes, recs, rays, hits, n, d_count, out_mode, nullptr, s);
    } else {
        if (counters) launch_pt<W, true, DYN, 0>(ctx, hdr, nodes, recs, rays, hits, n, d_count, out_mode, counters, s);
        else launch_pt<W, false, DYN, 0>(ctx, hdr, nodes, recs, rays, hits, n, d_count, out_mode, nullptr, s);
    }
}

}  // namespace

void gbt_launch_traverse(const gbt_bvh *bvh, const float4 *rays, float4 *hits, uint32_t n, const uint32_t *d_count,
                         int out_mode, unsigned int *d_error, cudaStream_t s, unsigned long long *counters, bool any) {
    if (n == 0) return;
    uint32_t blocks = (n + 127) / 128;
    gbt_ctx *ctx = bvh->ctx;
    if (ctx && ctx->traversal != 1) {  // persistent kernels
        const bool four = bvh->has_nodes4 || bvh->arity == 4;
        const BvhHeader *hd = bvh->has_nodes4 ? bvh->d_hdr4 : bvh->d_hdr;
        const float4 *nd = bvh->has_nodes4 ? bvh->d_nodes4 : bvh->d_nodes;
        const bool dyn = ctx->traversal == 0;
        if (four) {
            if (dyn) launch_pt_any<4, GBT_PT_DYN>(ctx, hd, nd, bvh->d_prims, rays, hits, n, d_count, out_mode, counters, s, any);
            else launch_pt_any<4, 0>(ctx, hd, nd, bvh->d_prims, rays, hits, n, d_count, out_mode, counters, s, any);
        } else {
            if (dyn) launch_pt_any<2, GBT_PT_DYN>(ctx, hd, nd, bvh->d_prims, rays, hits, n, d_count, out_mode, counters, s, any);
            else launch_pt_any<2, 0>(ctx, hd, nd, bvh->d_prims, rays, hits, n, d_count, out_mode, counters, s, any);
        }
        return;
    }
    (void)d_error;
    if (bvh->has_nodes4) {  // the 4-wide view of a binary tree
        if (counters)
            k_trace4<true><<<blocks, 128, 0, s>>>(bvh->d_hdr4, bvh->d_nodes4, bvh->d_prims, rays, hits, n, d_count, out_mode, d_error, counters);
        else
            k_trace4<false><<<blocks, 128, 0, s>>>(bvh->d_hdr4, bvh->d_nodes4, bvh->d_prims, rays, hits, n, d_count, out_mode, d_error, nullptr);
    } else if (bvh->arity == 4) {
        if (counters)
            k_trace4<true><<<blocks, 128, 0, s>>>(bvh->d_hdr, bvh->d_nodes, bvh->d_prims, rays, hits, n, d_count, out_mode, d_error, counters);
        else
            k_trace4<false><<<blocks, 128, 0, s>>>(bvh->d_hdr, bvh->d_nodes, bvh->d_prims, rays, hits, n, d_count, out_mode, d_error, nullptr);
    } else {
        if (counters)
            k_trace2<true><<<blocks, 128, 0, s>>>(bvh->d_hdr, bvh->d_nodes, bvh->d_prims, rays, hits, n, d_count, out_mode, d_error, counters);
        else
            k_trace2<false><<<blocks, 128, 0, s>>>(bvh->d_hdr, bvh->d_nodes, bvh->d_prims, rays, hits, n, d_count, out_mode, d_error, nullptr);
    }
}

void gbt_launch_traverse_multi(gbt_ctx *ctx, const TreeRef *trees, size_t stride, int width, const float4 *rays,
                               const float4 *aux, float4 *hits, uint32_t n, const uint32_t *d_count, int level,
                               cudaStream_t s) {
    if (n == 0) return;
    static int per_sm[2] = {0, 0};
    const int w = width == 4 ? 1 : 0;
    if (per_sm[w] == 0) {
        if (w) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[w], k_trace_multi<4, GBT_PT_DYN>, 128, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm[w], k_trace_multi<2, GBT_PT_DYN>, 128, 0);
        if (per_sm[w] <= 0) per_sm[w] = 1;
    }
    uint32_t *fetch = reinterpret_cast<uint32_t *>(ctx->d_counters + 3);
    cudaMemsetAsync(fetch, 0, sizeof(uint32_t), s);
    uint32_t grid = (uint32_t)(ctx->num_sms * per_sm[w]);
    const uint32_t need = (n + 127) / 128;
    if (need < grid) grid = need;
    if (w) k_trace_multi<4, GBT_PT_DYN><<<grid, 128, 0, s>>>(trees, (uint32_t)stride, rays, aux, hits, n, d_count, level,
                                                                   ctx->d_error, fetch);
    else k_trace_multi<2, GBT_PT_DYN><<<grid, 128, 0, s>>>(trees, (uint32_t)stride, rays, aux, hits, n, d_count, level,
                                                                   ctx->d_error, fetch);
}

void gbt_launch_traverse_packets_multi(const TreeRef *trees, size_t stride, const float4 *rays, const float4 *aux,
                                      float4 *hits, uint32_t n, unsigned int *d_error, cudaStream_t s) {
    if (n == 0) return;
    k_trace_packet4_multi<<<(n + 127) / 128, 128, 0, s>>>(trees, (uint32_t)stride, rays, aux, hits, n, d_error);
}

bool gbt_launch_traverse_packets(const gbt_bvh *bvh, const float4 *rays, float4 *hits, uint32_t n, int out_mode,
                                 unsigned int *d_error, cudaStream_t s, unsigned long long *counters) {
    if (!(bvh->has_nodes4 || bvh->arity == 4)) return false;
    if (n == 0) return true;
    const BvhHeader *hd = bvh->has_nodes4 ? bvh->d_hdr4 : bvh->d_hdr;
    const float4 *nd = bvh->has_nodes4 ? bvh->d_nodes4 : bvh->d_nodes;
    const uint32_t blocks = (n + 127) / 128;
    if (counters)
        k_trace_packet4<true><<<blocks, 128, 0, s>>>(hd, nd, bvh->d_prims, rays, hits, n, out_mode, d_error, counters);
    else
        k_trace_packet4<false><<<blocks, 128, 0, s>>>(hd, nd, bvh->d_prims, rays, hits, n, out_mode, d_error, nullptr);
    return true;
}

int gbt_trace_enqueue(gbt_ctx *ctx, const gbt_bvh *bvh, const gbt_ray *d_rays, uint32_t n, gbt_hit *d_hits) {
    gbt_prof_begin(ctx);
    gbt_launch_traverse(bvh, reinterpret_cast<const float4 *>(d_rays), reinterpret_cast<float4 *>(d_hits), n, nullptr,
                        0, ctx->d_error, ctx->stream, ctx->profiling >= 2 ? ctx->d_counters : nullptr);
    gbt_prof_end(ctx);
    GBT_CUDA(ctx, cudaGetLastError());
    return GBT_OK;
}
