// BVH.Cost (pkg/pt/bvh.go:226-239) on the device, over the tree as built
// (binary LBVH or PHR nodes; not the 4-wide traversal view):
//   leaf:  INTERSECTION_COST * #prims            (1 * count)
//   inner: TRAVERSAL_COST + sum_c A(c)/A(n) * C(c)  (2 + ..., children in order,
//          the sum skipped when A(n) == 0)
// evaluated bottom-up: every inner node counts its inner children; nodes whose
// children are all leaves start, and the last child to finish (an acq_rel
// counter) evaluates its parent, reading the children's costs in child order.
// Each node thus performs the recursion's float64 operations in the
// recursion's order, so the result is bit-identical to the recursive
// definition.  Surfaces are aabb.surface (bounding.go:45-47) of the float32
// boxes evaluated in float64.
#include <cuda_runtime.h>

#include "gbt_internal.cuh"

namespace {

struct Slot {
    int32_t ref, cnt;
    float lo[3], hi[3];
};

// non-empty child slots of node p, in order
__device__ int node_slots(const float4 *__restrict__ nodes, int arity, int32_t p, Slot out[4]) {
    int k = 0;
    if (arity == 2) {
        const float4 *nd = nodes + 4 * (size_t)p;
        const float4 z = __ldg(nd + 2);
        const int4 rc = __ldg(reinterpret_cast<const int4 *>(nd + 3));
        for (int c = 0; c < 2; c++) {
            const int32_t cnt = c ? rc.w : rc.y;
            if (cnt < 0) continue;
            const float4 xy = __ldg(nd + c);
            Slot s;
            s.ref = c ? rc.z : rc.x;
            s.cnt = cnt;
            s.lo[0] = xy.x; s.hi[0] = xy.y; s.lo[1] = xy.z; s.hi[1] = xy.w;
            s.lo[2] = c ? z.z : z.x;
            s.hi[2] = c ? z.w : z.y;
            out[k++] = s;
        }
    } else {
        const float *f = reinterpret_cast<const float *>(nodes + 8 * (size_t)p);
        for (int c = 0; c < 4; c++) {
            const int32_t cnt = __float_as_int(__ldg(f + 28 + c));
            if (cnt < 0) continue;
            Slot s;
            s.ref = __float_as_int(__ldg(f + 24 + c));
            s.cnt = cnt;
            for (int a = 0; a < 3; a++) {
                s.lo[a] = __ldg(f + 8 * a + c);
                s.hi[a] = __ldg(f + 8 * a + 4 + c);
            }
            out[k++] = s;
        }
    }
    return k;
}

__device__ __forceinline__ double surface(const float *lo, const float *hi) {
    const double w = __dsub_rn((double)hi[0], (double)lo[0]);
    const double h = __dsub_rn((double)hi[1], (double)lo[1]);
    const double d = __dsub_rn((double)hi[2], (double)lo[2]);
    return __dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(2.0, w), h), __dmul_rn(__dmul_rn(2.0, w), d)),
                     __dmul_rn(__dmul_rn(2.0, h), d));
}

__device__ __forceinline__ int32_t add_acq_rel(int32_t *p, int32_t v) {
    int32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// node i is an inner node of the tree: LBVH nodes all are; PHR entries of leaves are marked -2
__device__ __forceinline__ bool is_inner(const int32_t *parent, uint32_t i) { return parent[i] != -2; }

__global__ void k_cost_init(const float4 *__restrict__ nodes, int arity, const int32_t *__restrict__ parent,
                            uint32_t n, int32_t *__restrict__ pending, uint8_t *__restrict__ start) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!is_inner(parent, i)) {
        start[i] = 0;
        return;
    }
    Slot s[4];
    const int k = node_slots(nodes, arity, (int32_t)i, s);
    int inner = 0;
    for (int c = 0; c < k; c++) inner += s[c].cnt == 0;
    pending[i] = inner;
    start[i] = inner == 0;
}

__global__ void k_cost_up(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes, int arity,
                          const int32_t *__restrict__ parent, uint32_t n, int32_t *pending,
                          const uint8_t *__restrict__ start, double *cost, unsigned int *err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !start[i]) return;
    int32_t node = (int32_t)i;
    for (int guard = 0; guard < 1 << 20; guard++) {
        // this node's own box: the header's for the root, else the parent's slot that refers to it
        const int32_t p = parent[node];
        float lo[3], hi[3];
        bool found = p < 0;
        if (p < 0) {
            for (int a = 0; a < 3; a++) { lo[a] = hdr->root_lo[a]; hi[a] = hdr->root_hi[a]; }
        } else {
            Slot ps[4];
            const int kp = node_slots(nodes, arity, p, ps);
            for (int c = 0; c < kp; c++)
                if (ps[c].cnt == 0 && ps[c].ref == node) {
                    for (int a = 0; a < 3; a++) { lo[a] = ps[c].lo[a]; hi[a] = ps[c].hi[a]; }
                    found = true;
                    break;
                }
        }
        if (!found) {
            atomicOr(err, GBT_DEVERR_BOUNDS);
            return;
        }
        const double sn = surface(lo, hi);
        Slot s[4];
        const int k = node_slots(nodes, arity, node, s);
        double acc = 0.0;
        for (int c = 0; c < k; c++) {
            const double cc = s[c].cnt > 0 ? (double)s[c].cnt : __ldcg(cost + s[c].ref);
            if (sn != 0.0) acc = __dadd_rn(acc, __dmul_rn(__ddiv_rn(surface(s[c].lo, s[c].hi), sn), cc));
        }
        cost[node] = __dadd_rn(2.0, acc);
        if (p < 0) return;  // the root
        if (add_acq_rel(pending + p, -1) != 1) return;  // a sibling is still working
        node = p;
    }
    atomicOr(err, GBT_DEVERR_BOUNDS);
}

}  // namespace

int gbt_cost_device(gbt_ctx *ctx, gbt_bvh *bvh, double *out) {
    BvhHeader h;
    GBT_CUDA(ctx, cudaMemcpyAsync(&h, bvh->d_hdr, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (h.root_cnt > 0) {  // the root is a leaf
        *out = (double)h.root_cnt;
        return GBT_OK;
    }
    if (!bvh->d_parent) return gbt_fail(ctx, GBT_EINVAL, "cost: tree without parent links");
    const uint32_t n = h.n_nodes;
    const size_t off_pending = 0, off_start = gbt_align((size_t)n * 4), off_cost = gbt_align(off_start + n);
    void *scr = nullptr;
    int rc = gbt_scratch(ctx, off_cost + (size_t)n * 8, &scr);
    if (rc) return rc;
    unsigned char *b = static_cast<unsigned char *>(scr);
    int32_t *pending = reinterpret_cast<int32_t *>(b + off_pending);
    uint8_t *start = b + off_start;
    double *cost = reinterpret_cast<double *>(b + off_cost);
    const uint32_t blocks = (n + 255) / 256;
    k_cost_init<<<blocks, 256, 0, ctx->stream>>>(bvh->d_nodes, bvh->arity, bvh->d_parent, n, pending, start);
    k_cost_up<<<blocks, 256, 0, ctx->stream>>>(bvh->d_hdr, bvh->d_nodes, bvh->arity, bvh->d_parent, n, pending, start,
                                                cost, ctx->d_error);
    GBT_CUDA(ctx, cudaGetLastError());
    GBT_CUDA(ctx, cudaMemcpyAsync(out, cost + h.root_ref, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    return gbt_check_device_error(ctx, "cost");
}
