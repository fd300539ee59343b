// Four-wide traversal view of a binary BVH.
//
// The binary tree (LBVH, or PHR with branching factor 2) is what the
// reference builds and what parity checks export.  For traversal it is
// collapsed top-down into 128-byte 4-wide nodes: starting from a node's two
// children, the inner child with the largest surface area is repeatedly
// replaced by its own two children until there are four.  Closest-hit results
// do not depend on the node layout; only the number of node fetches does.
#include <cuda_runtime.h>

#include "gbt_internal.cuh"

namespace {

struct Child {
    float lo[3], hi[3];
    int32_t ref, cnt;
};

__device__ __forceinline__ void load_slots(const float4 *__restrict__ bin, int32_t node, Child &a, Child &b) {
    const float4 *nd = bin + 4 * (size_t)node;
    float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2);
    int4 n3 = __ldg(reinterpret_cast<const int4 *>(nd + 3));
    a.lo[0] = n0.x; a.hi[0] = n0.y; a.lo[1] = n0.z; a.hi[1] = n0.w; a.lo[2] = n2.x; a.hi[2] = n2.y;
    a.ref = n3.x; a.cnt = n3.y;
    b.lo[0] = n1.x; b.hi[0] = n1.y; b.lo[1] = n1.z; b.hi[1] = n1.w; b.lo[2] = n2.z; b.hi[2] = n2.w;
    b.ref = n3.z; b.cnt = n3.w;
}

__device__ __forceinline__ float area(const Child &c) {
    float w = c.hi[0] - c.lo[0], h = c.hi[1] - c.lo[1], d = c.hi[2] - c.lo[2];
    return w * h + w * d + h * d;
}

// A queued binary node becomes the 4-wide node already assigned to it; its
// inner children are queued for the next level.  A queue slot whose child was
// dropped for lack of capacity holds (-1, -1) and is skipped.
__device__ void collapse_one(const float4 *__restrict__ bin, int2 e, int2 *__restrict__ q_out, uint32_t *n_out,
                             uint32_t *n_nodes4, float4 *__restrict__ out, uint32_t cap, unsigned int *err) {
    // e = (binary node, 4-wide node)
    if (e.x < 0 || e.y < 0 || (uint32_t)e.y >= cap) return;
    Child c[4];
    load_slots(bin, e.x, c[0], c[1]);
    int nc = 0;
    if (c[0].cnt >= 0) nc++;
    if (c[1].cnt >= 0) { c[nc] = c[1]; nc++; }
    while (nc < 4) {
        int best = -1;
        float ba = -1.f;
        for (int k = 0; k < nc; k++)
            if (c[k].cnt == 0) {
                float a = area(c[k]);
                if (a > ba) { ba = a; best = k; }
            }
        if (best < 0) break;
        Child x, y;
        load_slots(bin, c[best].ref, x, y);  // slot 0 is always filled; slot 1 is empty for a one-child PHR branch
        if (y.cnt >= 0) {  // replace in place, the second grandchild right after it
            for (int k = nc; k > best + 1; k--) c[k] = c[k - 1];
            c[best] = x;
            c[best + 1] = y;
            nc++;
        } else {
            c[best] = x;
        }
    }
    float lo[3][4], hi[3][4];
    int32_t ref[4], cnt[4];
    for (int k = 0; k < 4; k++) {
        if (k < nc) {
            for (int a = 0; a < 3; a++) { lo[a][k] = c[k].lo[a]; hi[a][k] = c[k].hi[a]; }
            cnt[k] = c[k].cnt;
            ref[k] = c[k].ref;
            if (c[k].cnt == 0) {
                uint32_t idx = atomicAdd(n_nodes4, 1u);
                uint32_t q = atomicAdd(n_out, 1u);
                if (idx >= cap || q >= cap) {
                    atomicOr(err, GBT_DEVERR_CAPACITY);
                    if (q < cap) q_out[q] = make_int2(-1, -1);
                    cnt[k] = -1;
                    continue;
                }
                q_out[q] = make_int2(c[k].ref, (int32_t)idx);
                ref[k] = (int32_t)idx;
            }
        } else {
            for (int a = 0; a < 3; a++) { lo[a][k] = INFINITY; hi[a][k] = -INFINITY; }
            ref[k] = 0;
            cnt[k] = -1;
        }
    }
    float4 *nd = out + 8 * (size_t)e.y;
    nd[0] = make_float4(lo[0][0], lo[0][1], lo[0][2], lo[0][3]);
    nd[1] = make_float4(hi[0][0], hi[0][1], hi[0][2], hi[0][3]);
    nd[2] = make_float4(lo[1][0], lo[1][1], lo[1][2], lo[1][3]);
    nd[3] = make_float4(hi[1][0], hi[1][1], hi[1][2], hi[1][3]);
    nd[4] = make_float4(lo[2][0], lo[2][1], lo[2][2], lo[2][3]);
    nd[5] = make_float4(hi[2][0], hi[2][1], hi[2][2], hi[2][3]);
    reinterpret_cast<int4 *>(nd)[6] = make_int4(ref[0], ref[1], ref[2], ref[3]);
    reinterpret_cast<int4 *>(nd)[7] = make_int4(cnt[0], cnt[1], cnt[2], cnt[3]);
}

// Counters: [0], [1] the two queues' sizes, [2] 4-wide nodes, [3] the input queue of the
// current level, [4] levels done, [5] blocks of the running level done (outside a graph).
constexpr uint32_t MAX_LEVELS = 4096;  // a tree deeper than this is reported, not walked
constexpr int COLLAPSE_BATCH = 8;      // levels launched per readback (gbt_collapse4)

// One level of the graph form over a fixed grid: the input queue is ctr[3]'s.
__global__ void k_collapse_level_gs(const float4 *__restrict__ bin, int2 *q0, int2 *q1, uint32_t *ctr,
                                    float4 *__restrict__ out, uint32_t cap, unsigned int *err) {
    const uint32_t par = ctr[3];
    const uint32_t n = min(ctr[par], cap);  // a full queue counted past its capacity (reported)
    const int2 *q_in = par ? q1 : q0;
    int2 *q_out = par ? q0 : q1;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        collapse_one(bin, q_in[i], q_out, ctr + (par ^ 1), ctr + 2, out, cap, err);
}

// After a level: the output queue becomes the input, and the loop goes on while it is non-empty.
__global__ void k_collapse_advance(uint32_t *ctr, cudaGraphConditionalHandle loop, unsigned int *err) {
    const uint32_t par = ctr[3], next = par ^ 1;
    ctr[par] = 0;
    ctr[3] = next;
    const uint32_t levels = ++ctr[4];
    const bool more = ctr[next] > 0;
    if (more && levels >= MAX_LEVELS) atomicOr(err, GBT_DEVERR_CAPACITY);
    cudaGraphSetConditional(loop, more && levels < MAX_LEVELS ? 1u : 0u);
}

__device__ void k_collapse_root_body(const BvhHeader *__restrict__ hdr, BvhHeader *hdr4, int2 *q, uint32_t *n_q,
                                     uint32_t *n_nodes4) {
    *hdr4 = *hdr;
    if (hdr->root_cnt == 0) {  // an inner root becomes 4-wide node 0
        q[0] = make_int2(hdr->root_ref, 0);
        *n_q = 1;
        *n_nodes4 = 1;
        hdr4->root_ref = 0;
    } else {
        *n_q = 0;
        *n_nodes4 = 0;
    }
}

// The graph form's counters set up outside a graph (gbt_collapse4).
__global__ void k_collapse_root_gs(const BvhHeader *__restrict__ hdr, BvhHeader *hdr4, int2 *q0, uint32_t *ctr) {
    k_collapse_root_body(hdr, hdr4, q0, ctr + 0, ctr + 2);
    ctr[1] = 0;
    ctr[3] = 0;
    ctr[4] = 0;
    ctr[5] = 0;
}

// One level outside a graph, ending with k_collapse_advance's step taken by the grid's
// last block to finish (ctr[5] counts finished blocks): the output queue becomes the
// input.  After the last level the next ones find an empty queue and do nothing.
__global__ void k_collapse_level_step(const float4 *__restrict__ bin, int2 *q0, int2 *q1, uint32_t *ctr,
                                      float4 *__restrict__ out, uint32_t cap, unsigned int *err) {
    __shared__ bool s_last;
    const uint32_t par = ctr[3];
    const uint32_t n = min(ctr[par], cap);  // a full queue counted past its capacity (reported)
    const int2 *q_in = par ? q1 : q0;
    int2 *q_out = par ? q0 : q1;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        collapse_one(bin, q_in[i], q_out, ctr + (par ^ 1), ctr + 2, out, cap, err);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();  // this block's queue appends before its count
        s_last = atomicAdd(&ctr[5], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (threadIdx.x != 0 || !s_last) return;
    __threadfence();  // every block's appends before the counters are read
    const uint32_t next = par ^ 1;
    volatile uint32_t *vc = ctr;
    vc[par] = 0;
    vc[3] = next;
    vc[5] = 0;
    const uint32_t levels = vc[4] + 1;
    vc[4] = levels;
    if (vc[next] > 0 && levels >= MAX_LEVELS) atomicOr(err, GBT_DEVERR_CAPACITY);
}

__global__ void k_collapse_root_graph(const BvhHeader *__restrict__ hdr, BvhHeader *hdr4, int2 *q0, uint32_t *ctr,
                                      cudaGraphConditionalHandle loop) {
    k_collapse_root_body(hdr, hdr4, q0, ctr + 0, ctr + 2);
    ctr[1] = 0;
    ctr[3] = 0;
    ctr[4] = 0;
    cudaGraphSetConditional(loop, ctr[0] > 0 ? 1u : 0u);
}

}  // namespace

static int reserve4(gbt_ctx *ctx, gbt_bvh *bvh, uint32_t cap) {
    if (bvh->nodes4_cap < cap) {
        gbt_block_put(ctx, bvh->d_nodes4, bvh->nodes4_bytes);
        bvh->d_nodes4 = nullptr;
        bvh->nodes4_cap = 0;
        bvh->nodes4_bytes = 0;
        void *p = nullptr;
        size_t got = 0;
        if (gbt_block_get(ctx, (size_t)cap * 8 * sizeof(float4), &p, &got) != cudaSuccess) {
            cudaGetLastError();
            return gbt_fail(ctx, GBT_ENOMEM, "collapse: node allocation");
        }
        bvh->d_nodes4 = static_cast<float4 *>(p);
        bvh->nodes4_bytes = got;
        bvh->nodes4_cap = (uint32_t)(got / (8 * sizeof(float4)));
    }
    if (!bvh->d_hdr4 && cudaMalloc(&bvh->d_hdr4, sizeof(BvhHeader)) != cudaSuccess) {
        cudaGetLastError();
        return gbt_fail(ctx, GBT_ENOMEM, "collapse: header allocation");
    }
    return GBT_OK;
}

static size_t queue_bytes(uint32_t cap) { return gbt_align((size_t)cap * sizeof(int2)); }

int gbt_collapse4(gbt_ctx *ctx, gbt_bvh *bvh) {
    if (bvh->arity != 2) return GBT_OK;
    cudaStream_t st = ctx->stream;
    BvhHeader h;
    GBT_CUDA(ctx, cudaMemcpyAsync(&h, bvh->d_hdr, sizeof(h), cudaMemcpyDeviceToHost, st));
    GBT_CUDA(ctx, cudaStreamSynchronize(st));
    const uint32_t cap = h.n_nodes + 1;  // a 4-wide tree never has more nodes than the binary one
    int rc0 = reserve4(ctx, bvh, cap);
    if (rc0) return rc0;
    // the work-list capacity the kernels check against (a testing aid can lower it below what
    // was allocated; children past it are dropped and reported, never written)
    const uint32_t kcap = ctx->collapse_cap && ctx->collapse_cap < cap ? ctx->collapse_cap : cap;
    // queues (two halves), counters
    size_t qbytes = queue_bytes(cap);
    void *scr = nullptr;
    int rc = gbt_scratch(ctx, 2 * qbytes + 256, &scr);
    if (rc) return rc;
    unsigned char *sb = static_cast<unsigned char *>(scr);
    int2 *q0 = reinterpret_cast<int2 *>(sb), *q1 = reinterpret_cast<int2 *>(sb + qbytes);
    uint32_t *ctr = reinterpret_cast<uint32_t *>(sb + 2 * qbytes);  // the graph form's counters
    uint32_t *hc = static_cast<uint32_t *>(gbt_pinned(ctx));
    if (!hc) return gbt_fail(ctx, GBT_ENOMEM, "collapse: pinned host allocation");
    k_collapse_root_gs<<<1, 1, 0, st>>>(bvh->d_hdr, bvh->d_hdr4, q0, ctr);
    // levels in batches of COLLAPSE_BATCH launches between readbacks of the counters
    for (;;) {
        for (int b = 0; b < COLLAPSE_BATCH; b++)
            k_collapse_level_step<<<(unsigned)ctx->num_sms * 4, 128, 0, st>>>(bvh->d_nodes, q0, q1, ctr,
                                                                              bvh->d_nodes4, kcap, ctx->d_error);
        GBT_CUDA(ctx, cudaGetLastError());
        GBT_CUDA(ctx, cudaMemcpyAsync(hc, ctr, 5 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        GBT_CUDA(ctx, cudaStreamSynchronize(st));
        if (hc[hc[3] & 1u] == 0 || hc[4] >= MAX_LEVELS) break;
    }
    bvh->has_nodes4 = 1;
    return GBT_OK;
}

int gbt_collapse4_reserve(gbt_ctx *ctx, gbt_bvh *bvh, size_t *scratch_bytes) {
    *scratch_bytes = 0;
    if (bvh->arity != 2) return GBT_OK;
    BvhHeader h;
    GBT_CUDA(ctx, cudaMemcpyAsync(&h, bvh->d_hdr, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    GBT_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const uint32_t cap = h.n_nodes + 1;  // rebuilds over the same scene keep the node count
    int rc = reserve4(ctx, bvh, cap);
    if (rc) return rc;
    *scratch_bytes = 2 * queue_bytes(cap) + 256;
    return GBT_OK;
}

int gbt_collapse4_enqueue(gbt_ctx *ctx, gbt_bvh *bvh) {
    if (bvh->arity != 2) return GBT_OK;
    cudaStream_t st = ctx->stream;
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    GBT_CUDA(ctx, cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd));
    if (cs != cudaStreamCaptureStatusActive) return gbt_fail(ctx, GBT_EINVAL, "collapse: enqueue outside a capture");
    const uint32_t cap = bvh->nodes4_cap;
    if (cap == 0 || !bvh->d_hdr4) return gbt_fail(ctx, GBT_EINVAL, "collapse: view not reserved");
    const size_t qbytes = queue_bytes(cap);
    void *scr = nullptr;
    int rc = gbt_scratch(ctx, 2 * qbytes + 256, &scr);
    if (rc) return rc;
    unsigned char *sb = static_cast<unsigned char *>(scr);
    int2 *q0 = reinterpret_cast<int2 *>(sb), *q1 = reinterpret_cast<int2 *>(sb + qbytes);
    uint32_t *ctr = reinterpret_cast<uint32_t *>(sb + 2 * qbytes);
    cudaGraphConditionalHandle loop;
    GBT_CUDA(ctx, cudaGraphConditionalHandleCreate(&loop, g, 0, cudaGraphCondAssignDefault));
    k_collapse_root_graph<<<1, 1, 0, st>>>(bvh->d_hdr, bvh->d_hdr4, q0, ctr, loop);
    GBT_CUDA(ctx, cudaGetLastError());
    // the WHILE node after the root, its body captured on the side stream
    GBT_CUDA(ctx, cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd));
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = loop;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    GBT_CUDA(ctx, cudaGraphAddNode(&node, g, deps, nullptr, nd, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    GBT_CUDA(ctx, cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    if (!ctx->side) GBT_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking));
    GBT_CUDA(ctx, cudaStreamBeginCaptureToGraph(ctx->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    k_collapse_level_gs<<<(unsigned)ctx->num_sms * 4, 128, 0, ctx->side>>>(bvh->d_nodes, q0, q1, ctr, bvh->d_nodes4, cap,
                                                                          ctx->d_error);
    k_collapse_advance<<<1, 1, 0, ctx->side>>>(ctr, loop, ctx->d_error);
    const cudaError_t le = cudaGetLastError();
    cudaGraph_t captured = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(ctx->side, &captured);
    if (le != cudaSuccess || ee != cudaSuccess)
        return gbt_fail(ctx, GBT_ECUDA, std::string("collapse: body capture: ") +
                                            cudaGetErrorString(le != cudaSuccess ? le : ee));
    return GBT_OK;
}
