// Device-side ray/BVH queries shared by the trace and render kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbt_internal.cuh"

namespace gbt_dev {

struct Ray {
    float3 o, d, inv, oi;
    float tmin, tmax;
};

struct Hit {
    float t, u, v;
    int rec;  // primitive record index, -1 for a miss
};

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 add3(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 mul3(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 emul3(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Reciprocal direction for the slab test.  A zero component is replaced by a
// tiny one of the same sign, so the slab test stays finite (the box test only
// culls; the primitive tests use the exact direction).
__device__ __forceinline__ void finish_ray(Ray &r) {
    const float eps = 1e-20f;
    float dx = fabsf(r.d.x) > eps ? r.d.x : copysignf(eps, r.d.x);
    float dy = fabsf(r.d.y) > eps ? r.d.y : copysignf(eps, r.d.y);
    float dz = fabsf(r.d.z) > eps ? r.d.z : copysignf(eps, r.d.z);
    r.inv = f3(1.0f / dx, 1.0f / dy, 1.0f / dz);
    r.oi = f3(r.o.x * r.inv.x, r.o.y * r.inv.y, r.o.z * r.inv.z);
}

__device__ __forceinline__ Ray load_ray(const float4 *__restrict__ rays, uint32_t i) {
    float4 a = __ldg(rays + 2 * (size_t)i), b = __ldg(rays + 2 * (size_t)i + 1);
    Ray r;
    r.o = f3(a.x, a.y, a.z);
    r.tmin = a.w;
    r.d = f3(b.x, b.y, b.z);
    r.tmax = b.w;
    finish_ray(r);
    return r;
}

// Slab test against [tmin, tmax]; returns the entry distance.  The far
// distance is widened by a few ulp so that a primitive lying on the box
// boundary is never culled by float32 rounding.
// Two float4 of a node in one 256-bit read-only load (sm_100 and later; p is
// 32-byte aligned: node arrays come from cudaMalloc and nodes are 64 or 128 bytes).
__device__ __forceinline__ void ldg256(const float4 *p, float4 &a, float4 &b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

__device__ __forceinline__ bool slab(float lx, float ly, float lz, float hx, float hy, float hz, const Ray &r,
                                     float tmax, float &tenter) {
    float tx0 = fmaf(lx, r.inv.x, -r.oi.x), tx1 = fmaf(hx, r.inv.x, -r.oi.x);
    float ty0 = fmaf(ly, r.inv.y, -r.oi.y), ty1 = fmaf(hy, r.inv.y, -r.oi.y);
    float tz0 = fmaf(lz, r.inv.z, -r.oi.z), tz1 = fmaf(hz, r.inv.z, -r.oi.z);
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), r.tmin));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    tenter = tn;
    return tn <= tf * 1.0000005f;
}

// The direction signs of a ray as three bits (bit a set: negative along axis a),
// read from the reciprocal, whose sign finish_ray fixes also for zero components.
__device__ __forceinline__ uint32_t octant(const Ray &r) {
    return (__float_as_uint(r.inv.x) >> 31) | ((__float_as_uint(r.inv.y) >> 31) << 1) |
           ((__float_as_uint(r.inv.z) >> 31) << 2);
}

// slab() for a ray whose octant is OCT, known at compile time: on each axis the
// near and far planes are picked by the sign instead of ordered by min/max.
// For a box with lo <= hi and finite distances the entry distance and the
// answer equal slab()'s, since the rounded products keep the order of the planes.
template <int OCT>
__device__ __forceinline__ bool slab_oct(float lx, float ly, float lz, float hx, float hy, float hz, const Ray &r,
                                         float tmax, float &tenter) {
    const float tnx = fmaf((OCT & 1) ? hx : lx, r.inv.x, -r.oi.x), tfx = fmaf((OCT & 1) ? lx : hx, r.inv.x, -r.oi.x);
    const float tny = fmaf((OCT & 2) ? hy : ly, r.inv.y, -r.oi.y), tfy = fmaf((OCT & 2) ? ly : hy, r.inv.y, -r.oi.y);
    const float tnz = fmaf((OCT & 4) ? hz : lz, r.inv.z, -r.oi.z), tfz = fmaf((OCT & 4) ? lz : hz, r.inv.z, -r.oi.z);
    const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, r.tmin));
    const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
    tenter = tn;
    return tn <= tf * 1.0000005f;
}

// slab() or, for OCT in 0..7, slab_oct<OCT>().
template <int OCT>
__device__ __forceinline__ bool slab_sel(float lx, float ly, float lz, float hx, float hy, float hz, const Ray &r,
                                         float tmax, float &tenter) {
    if constexpr (OCT < 0)
        return slab(lx, ly, lz, hx, hy, hz, r, tmax, tenter);
    else
        return slab_oct<OCT>(lx, ly, lz, hx, hy, hz, r, tmax, tenter);
}

// Moeller-Trumbore (primitive.go:172-208) on record s; narrows h on a hit.
__device__ __forceinline__ void test_record(const float4 *__restrict__ recs, int s, const Ray &r, Hit &h) {
    const float4 *p = recs + 3 * (size_t)s;
    float4 r0 = __ldg(p), r1 = __ldg(p + 1);
    if (__float_as_int(r1.w) == 0) {
        float4 r2 = __ldg(p + 2);
        float3 v0 = f3(r0.x, r0.y, r0.z);
        float3 e1 = f3(r1.x - r0.x, r1.y - r0.y, r1.z - r0.z);
        float3 e2 = f3(r2.x - r0.x, r2.y - r0.y, r2.z - r0.z);
        float3 pv = cross3(r.d, e2);
        float det = dot3(e1, pv);
        if (fabsf(det) <= 1e-7f) return;
        float inv = __frcp_rn(det);  // the correctly rounded 1 / det
        float3 tv = sub3(r.o, v0);
        float u = dot3(tv, pv) * inv;
        if (u < 0.f || u > 1.f) return;
        float3 qv = cross3(tv, e1);
        float v = dot3(r.d, qv) * inv;
        if (v < 0.f || u + v > 1.f) return;
        float t = dot3(e2, qv) * inv;
        if (t < r.tmin || t > h.t) return;
        // an exact tie with the current hit goes to the lower record, whatever the visiting order
        // (the reference keeps the last one its own order finds)
        if (t == h.t && h.rec >= 0 && s > h.rec) return;
        h.t = t;
        h.u = u;
        h.v = v;
        h.rec = s;
    } else {  // Sphere.intersected (primitive.go:56-86)
        float3 c = f3(r0.x, r0.y, r0.z);
        float rad = r1.x;
        float3 oc = sub3(r.o, c);
        float dn = sqrtf(dot3(r.d, r.d));
        float a = dn * dn;
        float hb = dot3(oc, r.d);
        float ocn = sqrtf(dot3(oc, oc));
        float cc = ocn * ocn - rad * rad;
        float disc = hb * hb - a * cc;
        if (disc < 0.f) return;
        float sq = sqrtf(disc);
        float t = (-hb - sq) / a;
        if (t <= r.tmin || t >= h.t) {
            t = (-hb + sq) / a;
            if (t <= r.tmin || t >= h.t) return;
        }
        h.t = t;
        h.u = 0.f;
        h.v = 0.f;
        h.rec = s;
    }
}

__device__ __forceinline__ void leaf(const float4 *__restrict__ recs, int first, int cnt, const Ray &r, Hit &h) {
    for (int s = first; s < first + cnt; ++s) test_record(recs, s, r, h);
}

// Per-thread traversal work counters (profiling level 2).
struct Work {
    uint32_t nodes = 0, prims = 0;
};

template <int STACK, bool COUNT = false>
__device__ __forceinline__ Hit closest_hit2(const BvhHeader &hdr, const float4 *__restrict__ nodes,
                                            const float4 *__restrict__ recs, const Ray &r, unsigned int *err,
                                            Work *work = nullptr) {
    Hit h;
    h.t = r.tmax;
    h.u = h.v = 0.f;
    h.rec = -1;
    float te;
    if (!slab(hdr.root_lo[0], hdr.root_lo[1], hdr.root_lo[2], hdr.root_hi[0], hdr.root_hi[1], hdr.root_hi[2], r, h.t, te))
        return h;
    int2 stack[STACK];
    float stack_t[STACK];
    int sp = 0;
    int2 cur = make_int2(hdr.root_ref, hdr.root_cnt);
    for (;;) {
        if (cur.y == 0) {
            if (COUNT) work->nodes++;
            const float4 *nd = nodes + 4 * (size_t)cur.x;
            float4 n0, n1, n2, n3f;
            ldg256(nd, n0, n1);
            ldg256(nd + 2, n2, n3f);
            const int4 n3 = make_int4(__float_as_int(n3f.x), __float_as_int(n3f.y), __float_as_int(n3f.z),
                                      __float_as_int(n3f.w));
            float t0, t1;
            bool h0 = n3.y >= 0 && slab(n0.x, n0.z, n2.x, n0.y, n0.w, n2.y, r, h.t, t0);
            bool h1 = n3.w >= 0 && slab(n1.x, n1.z, n2.z, n1.y, n1.w, n2.w, r, h.t, t1);
            if (h0 && h1) {
                int2 a = make_int2(n3.x, n3.y), b = make_int2(n3.z, n3.w);
                float tb = t1;
                if (t1 < t0) {
                    int2 tmp = a;
                    a = b;
                    b = tmp;
                    tb = t0;
                }
                if (sp < STACK) {
                    stack[sp] = b;
                    stack_t[sp] = tb;
                    ++sp;
                } else {
                    atomicOr(err, GBT_DEVERR_STACK);
                }
                cur = a;
                continue;
            }
            if (h0) { cur = make_int2(n3.x, n3.y); continue; }
            if (h1) { cur = make_int2(n3.z, n3.w); continue; }
        } else if (cur.y > 0) {
            if (COUNT) work->prims += (uint32_t)cur.y;
            leaf(recs, cur.x, cur.y, r, h);
        }
        bool found = false;
        while (sp > 0) {
            --sp;
            if (stack_t[sp] <= h.t * 1.0000005f) {
                cur = stack[sp];
                found = true;
                break;
            }
        }
        if (!found) break;
    }
    return h;
}

// ---------------------------------------------------------------------------
// Persistent traversal: each warp keeps its lanes busy by fetching new rays as
// old ones finish, and runs inner-node steps until every busy lane holds a leaf
// before testing primitives ("while-while" with postponed leaves, after Aila &
// Laine, HPG 2009), so inner-node and leaf work are not interleaved across
// lanes of one warp.  The scalar state (current entry, postponed leaf, stack
// depth) stays in registers; only the stack arrays live in local memory.
// ---------------------------------------------------------------------------
// Traversal stacks: entries (ref, cnt) with the entry distance used to skip
// subtrees that lie beyond the current closest hit.
template <int STACK>
struct LocalStack {  // all entries in local memory, one 16-byte word each (ref, cnt, t)
    int4 e[STACK];
    __device__ __forceinline__ void push(int &sp, int2 v, float tv, unsigned int *err) {
        if (sp < STACK) {
            e[sp] = make_int4(v.x, v.y, __float_as_int(tv), 0);
            ++sp;
        } else {
            atomicOr(err, GBT_DEVERR_STACK);
        }
    }
    __device__ __forceinline__ int2 pop(int &sp, float tmax) {
        while (sp > 0) {
            --sp;
            const int4 w = e[sp];
            if (__int_as_float(w.z) <= tmax * 1.0000005f) return make_int2(w.x, w.y);
        }
        return make_int2(0, -1);
    }
};

// The first SH slots of each thread's stack, where a shallow traversal does
// all its pushes and pops, in shared memory (column `thread` of a [SH][stride]
// array); deeper slots in local memory.
template <int STACK, int SH>
struct SharedTopStack {
    int2 *se;
    float *st;
    int stride;
    int4 e[STACK - SH];
    __device__ __forceinline__ void push(int &sp, int2 v, float tv, unsigned int *err) {
        if (sp < SH) {
            se[sp * stride] = v;
            st[sp * stride] = tv;
            ++sp;
        } else if (sp < STACK) {
            e[sp - SH] = make_int4(v.x, v.y, __float_as_int(tv), 0);
            ++sp;
        } else {
            atomicOr(err, GBT_DEVERR_STACK);
        }
    }
    __device__ __forceinline__ int2 pop(int &sp, float tmax) {
        while (sp > 0) {
            --sp;
            if (sp < SH) {
                if (st[sp * stride] <= tmax * 1.0000005f) return se[sp * stride];
            } else {
                const int4 w = e[sp - SH];
                if (__int_as_float(w.z) <= tmax * 1.0000005f) return make_int2(w.x, w.y);
            }
        }
        return make_int2(0, -1);
    }
};

// One inner-node step on a binary node: returns the next entry.
template <class StackT>
__device__ __forceinline__ int2 step2(const float4 *__restrict__ nodes, int2 node, StackT &st, int &sp, const Ray &r,
                                      float tmax, unsigned int *err) {
    const float4 *nd = nodes + 4 * (size_t)node.x;
    float4 n0, n1, n2, n3f;
    ldg256(nd, n0, n1);
    ldg256(nd + 2, n2, n3f);
    const int4 n3 = make_int4(__float_as_int(n3f.x), __float_as_int(n3f.y), __float_as_int(n3f.z), __float_as_int(n3f.w));
    float t0, t1;
    bool h0 = n3.y >= 0 && slab(n0.x, n0.z, n2.x, n0.y, n0.w, n2.y, r, tmax, t0);
    bool h1 = n3.w >= 0 && slab(n1.x, n1.z, n2.z, n1.y, n1.w, n2.w, r, tmax, t1);
    if (h0 && h1) {
        int2 a = make_int2(n3.x, n3.y), b = make_int2(n3.z, n3.w);
        if (t1 < t0) {
            st.push(sp, a, t0, err);
            return b;
        }
        st.push(sp, b, t1, err);
        return a;
    }
    if (h0) return make_int2(n3.x, n3.y);
    if (h1) return make_int2(n3.z, n3.w);
    return st.pop(sp, tmax);
}

struct Cand {
    float t;
    int2 e;
};

__device__ __forceinline__ void cx(Cand &a, Cand &b) {  // compare-exchange, ascending by t
    if (b.t < a.t) {
        Cand x = a;
        a = b;
        b = x;
    }
}

// One inner-node step on a 4-wide node: children sorted near to far by a
// register sorting network, the nearest taken, the others pushed far first.
template <class StackT>
__device__ __forceinline__ int2 step4(const float4 *__restrict__ nodes, int2 node, StackT &st, int &sp, const Ray &r,
                                      float tmax, unsigned int *err) {
    const float4 *nd = nodes + 8 * (size_t)node.x;
    float4 lx, hx, ly, hy, lz, hz, rff, cnf;
    ldg256(nd, lx, hx);
    ldg256(nd + 2, ly, hy);
    ldg256(nd + 4, lz, hz);
    ldg256(nd + 6, rff, cnf);
    const int4 rf = make_int4(__float_as_int(rff.x), __float_as_int(rff.y), __float_as_int(rff.z), __float_as_int(rff.w));
    const int4 cn = make_int4(__float_as_int(cnf.x), __float_as_int(cnf.y), __float_as_int(cnf.z), __float_as_int(cnf.w));
    const float MISS = __int_as_float(0x7f800000);
    Cand c0, c1, c2, c3;
    float t;
    c0.t = (cn.x >= 0 && slab(lx.x, ly.x, lz.x, hx.x, hy.x, hz.x, r, tmax, t)) ? t : MISS;
    c1.t = (cn.y >= 0 && slab(lx.y, ly.y, lz.y, hx.y, hy.y, hz.y, r, tmax, t)) ? t : MISS;
    c2.t = (cn.z >= 0 && slab(lx.z, ly.z, lz.z, hx.z, hy.z, hz.z, r, tmax, t)) ? t : MISS;
    c3.t = (cn.w >= 0 && slab(lx.w, ly.w, lz.w, hx.w, hy.w, hz.w, r, tmax, t)) ? t : MISS;
    c0.e = make_int2(rf.x, cn.x);
    c1.e = make_int2(rf.y, cn.y);
    c2.e = make_int2(rf.z, cn.z);
    c3.e = make_int2(rf.w, cn.w);
    cx(c0, c1);
    cx(c2, c3);
    cx(c0, c2);
    cx(c1, c3);
    cx(c1, c2);
    if (c0.t == MISS) return st.pop(sp, tmax);
    if (c3.t != MISS) st.push(sp, c3.e, c3.t, err);
    if (c2.t != MISS) st.push(sp, c2.e, c2.t, err);
    if (c1.t != MISS) st.push(sp, c1.e, c1.t, err);
    return c0.e;
}

// One ray through a 4-wide tree: the sorting-network step with the given stack.
// ANY: stop at the first hit found (a query that only needs hit or miss).
template <bool COUNT, class StackT, bool ANY = false>
__device__ __forceinline__ Hit closest_hit4_with(const BvhHeader &hdr, const float4 *__restrict__ nodes,
                                                 const float4 *__restrict__ recs, const Ray &r, unsigned int *err,
                                                 Work *work, StackT &st) {
    Hit h;
    h.t = r.tmax;
    h.u = h.v = 0.f;
    h.rec = -1;
    float te;
    if (!slab(hdr.root_lo[0], hdr.root_lo[1], hdr.root_lo[2], hdr.root_hi[0], hdr.root_hi[1], hdr.root_hi[2], r, h.t, te))
        return h;
    int sp = 0;
    int2 node = make_int2(hdr.root_ref, hdr.root_cnt);
    for (;;) {
        if (node.y == 0) {
            if (COUNT) work->nodes++;
            node = step4(nodes, node, st, sp, r, h.t, err);
        } else if (node.y > 0) {
            if (COUNT) work->prims += (uint32_t)node.y;
            leaf(recs, node.x, node.y, r, h);
            if (ANY && h.rec >= 0) break;
            node = st.pop(sp, h.t);
        } else {
            break;
        }
    }
    return h;
}

// ... with a local-memory stack
template <int STACK, bool COUNT = false>
__device__ __forceinline__ Hit closest_hit4(const BvhHeader &hdr, const float4 *__restrict__ nodes,
                                            const float4 *__restrict__ recs, const Ray &r, unsigned int *err,
                                            Work *work = nullptr) {
    LocalStack<STACK> st;
    return closest_hit4_with<COUNT>(hdr, nodes, recs, r, err, work, st);
}

// out_mode 0: gbt_hit (primitive id, t, u, v); 1: (t, u, v, record) for the renderer
__device__ __forceinline__ void store_hit(float4 *__restrict__ hits, uint32_t i, const Hit &h,
                                          const float4 *__restrict__ recs, int out_mode) {
    if (out_mode == 0) {
        int id = h.rec >= 0 ? __float_as_int(__ldg(recs + 3 * (size_t)h.rec).w) : -1;
        float t = h.rec >= 0 ? h.t : __int_as_float(0x7f800000);
        hits[i] = make_float4(__int_as_float(id), t, h.u, h.v);
    } else {
        hits[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.rec));
    }
}

}  // namespace gbt_dev
