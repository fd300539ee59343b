// Batched rendering: many scenes and many independent renders as one frame.
//
// Every (scene, path) pair of the batch is one entry of a work range (the
// concatenated path ranges of the items).  Two forms trace it:
//   megakernel  one persistent launch; each lane of a resident warp pulls a
//               path from a device queue, runs it to completion -- camera ray,
//               closest hit, shading, next bounce (shade.cuh) -- and pulls the
//               next one; lanes are refilled with warp-aggregated atomics;
//   wavefront   the per-scene wavefront over all items at once: per bounce
//               level one camera/shading kernel over the live paths of every
//               item and one persistent traversal over all their trees
//               (k_trace_multi), so each level is two launches whatever the
//               number of items.
// The paths are the ones the per-scene wavefront renderer traces (same
// Philox counters), so the images agree up to the order of float additions.
// The per-frame sequence can be captured in a CUDA graph together with
// in-place LBVH rebuilds.  The form and its launch parameters come from a
// small autotuner.
//
// The reference renders one scene at a time (render.go:91-129); batching has
// no counterpart there.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <cstring>
#include <vector>

#include "gbt_internal.cuh"
#include "shade.cuh"

using namespace gbt_dev;

namespace {

constexpr int MAX_ITEMS = 1024;

struct ItemDev {
    TreeRef tree;  // first member: the item table doubles as the traversal's tree table
    const uint32_t *prim_mat;
    const float4 *mats;
    const float *normals;
    float *acc;
    float *out;
    CamF cam;
    ShadeParams sp;
    uint32_t path_base;  // first queue entry of this item
    uint32_t pix_base;   // first accumulator float of this item / 3
    float inv_spp;
    uint32_t pad;
};

__device__ __forceinline__ uint32_t lane_lt_mask() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// item of queue entry q: last item whose path_base <= q (binary search in shared memory)
__device__ __forceinline__ int find_item(const uint32_t *s_base, int n, uint32_t q) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (s_base[mid] <= q) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int W, int BLOCK, int DYN, int SH>
__global__ void __launch_bounds__(BLOCK) k_batch(const ItemDev *__restrict__ items, int n_items, uint32_t total,
                                                 uint32_t *fetch, unsigned int *err, unsigned long long *ray_total) {
    constexpr int STACK = W == 2 ? 64 : 96;
    __shared__ uint32_t s_base[MAX_ITEMS];
    __shared__ int2 s_se[SH > 0 ? SH * BLOCK : 1];
    __shared__ float s_st[SH > 0 ? SH * BLOCK : 1];
    for (int i = threadIdx.x; i < n_items; i += BLOCK) s_base[i] = items[i].path_base;
    __syncthreads();
    using StackT = typename std::conditional<(SH > 0), SharedTopStack<STACK, (SH > 0 ? SH : 1)>, LocalStack<STACK>>::type;
    StackT st;
    if constexpr (SH > 0) {
        st.se = s_se + threadIdx.x;
        st.st = s_st + threadIdx.x;
        st.stride = BLOCK;
    }
    const uint32_t lane = threadIdx.x & 31;
    int sp = 0;
    int2 node = make_int2(0, -1), leaf = make_int2(0, 0);
    Ray r;
    Hit h;
    h.t = 0.f;
    h.u = h.v = 0.f;
    h.rec = -1;
    // path state
    int item = -1;  // -1: no path
    uint32_t g = 0;
    int level = 0;
    bool any = false;  // the current ray only needs hit or miss (level past MaxDepth)
    float3 T = f3(1.f, 1.f, 1.f), L = f3(0.f, 0.f, 0.f);
    const float4 *nodes = nullptr, *recs = nullptr;
    uint32_t rays = 0;
    bool pool_empty = false;
    for (;;) {
        // a finished ray: shade it, continue the path or end it
        if (item >= 0 && node.y < 0 && leaf.y <= 0) {
            const ItemDev &it = items[item];
            float3 no, nd;
            bool cont = shade_step(it.sp, level, g, r.o, r.d, h.t, h.u, h.v, h.rec, recs, it.prim_mat, it.mats,
                                   it.normals, T, L, no, nd);
            if (cont) {
                level++;
                any = it.sp.any_last && level == it.sp.max_depth + 1;
                r.o = no;
                r.d = nd;
                r.tmin = 0.0001f;
                r.tmax = __int_as_float(0x7f800000);
                finish_ray(r);
                h.t = r.tmax;
                h.rec = -1;
                sp = 0;
                leaf = make_int2(0, 0);
                float te;
                const BvhHeader *hd = it.tree.hdr;
                node = slab(hd->root_lo[0], hd->root_lo[1], hd->root_lo[2], hd->root_hi[0], hd->root_hi[1],
                            hd->root_hi[2], r, h.t, te)
                           ? make_int2(hd->root_ref, hd->root_cnt)
                           : make_int2(0, -1);
                if (node.y > 0) {
                    leaf = node;
                    node = make_int2(0, -1);
                }
                rays++;
            } else {
                deposit(it.acc, g % it.sp.npix, L);
                item = -1;
            }
        }
        // refill lanes without a path from the queue
        const bool want = item < 0 && !pool_empty;
        const uint32_t need = __ballot_sync(0xffffffffu, want);
        if (need) {
            const int leader = __ffs(need) - 1;
            uint32_t base = 0;
            if (lane == (uint32_t)leader) base = atomicAdd(fetch, (uint32_t)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            bool empty_here = false;
            if (want) {
                const uint32_t q = base + __popc(need & lane_lt_mask());
                if (q < total) {
                    item = find_item(s_base, n_items, q);
                    const ItemDev &it = items[item];
                    g = path_id(it.sp, q - it.path_base);
                    nodes = it.tree.nodes;
                    recs = it.tree.recs;
                    level = 0;
                    any = false;
                    T = f3(1.f, 1.f, 1.f);
                    L = f3(0.f, 0.f, 0.f);
                    primary_ray(it.cam, it.sp, g, r.o, r.d);
                    r.tmin = 0.001f;
                    r.tmax = __int_as_float(0x7f800000);
                    finish_ray(r);
                    h.t = r.tmax;
                    h.u = h.v = 0.f;
                    h.rec = -1;
                    sp = 0;
                    leaf = make_int2(0, 0);
                    float te;
                    const BvhHeader *hd = it.tree.hdr;
                    node = slab(hd->root_lo[0], hd->root_lo[1], hd->root_lo[2], hd->root_hi[0], hd->root_hi[1],
                                hd->root_hi[2], r, h.t, te)
                               ? make_int2(hd->root_ref, hd->root_cnt)
                               : make_int2(0, -1);
                    if (node.y > 0) {
                        leaf = node;
                        node = make_int2(0, -1);
                    }
                    rays++;
                } else {
                    empty_here = true;
                }
            }
            pool_empty = __any_sync(0xffffffffu, empty_here) || pool_empty;
        }
        if (__all_sync(0xffffffffu, item < 0)) break;
        // closest-hit traversal of the current rays (while-while, postponed leaves)
        while (node.y >= 0 || leaf.y > 0) {
            while (node.y == 0) {
                node = W == 2 ? step2(nodes, node, st, sp, r, h.t, err) : step4(nodes, node, st, sp, r, h.t, err);
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
    // rays traced, for the statistics
    __syncwarp();
    unsigned long long c = rays;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) atomicAdd(ray_total, c);
}

__global__ void k_resolve_batch(const ItemDev *__restrict__ items, int n_items, uint32_t total_floats) {
    __shared__ uint32_t s_pb[MAX_ITEMS];
    for (int i = threadIdx.x; i < n_items; i += blockDim.x) s_pb[i] = items[i].pix_base * 3;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total_floats; i += gridDim.x * blockDim.x) {
        int it = find_item(s_pb, n_items, i);
        const ItemDev &d = items[it];
        uint32_t k = i - s_pb[it];
        d.out[k] = d.acc[k] * d.inv_spp;
    }
}

// wavefront form: camera rays of queue entries [g0, g0 + count); the item index rides in aux[2 i + 1].w
__global__ void __launch_bounds__(256) k_raygen_batch(const ItemDev *__restrict__ items, int n_items, uint32_t g0,
                                                      uint32_t count, float4 *__restrict__ rays,
                                                      float4 *__restrict__ aux, uint32_t *counts) {
    __shared__ uint32_t s_base[MAX_ITEMS];
    for (int k = threadIdx.x; k < n_items; k += blockDim.x) s_base[k] = items[k].path_base;
    __syncthreads();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) counts[0] = count;
    if (i >= count) return;
    const uint32_t q = g0 + i;
    const int item = find_item(s_base, n_items, q);
    const ItemDev &it = items[item];
    const uint32_t g = path_id(it.sp, q - it.path_base);
    float3 o, d;
    primary_ray(it.cam, it.sp, g, o, d);
    rays[2 * (size_t)i] = make_float4(o.x, o.y, o.z, 0.001f);
    rays[2 * (size_t)i + 1] = make_float4(d.x, d.y, d.z, __int_as_float(0x7f800000));
    aux[2 * (size_t)i] = make_float4(1.f, 1.f, 1.f, __int_as_float((int)g));
    aux[2 * (size_t)i + 1] = make_float4(0.f, 0.f, 0.f, __int_as_float(item));
}

// wavefront form: shade the level's hits of every item, compact the live paths into the next level
__global__ void __launch_bounds__(256) k_shade_batch(const ItemDev *__restrict__ items, int level,
                                                     const float4 *__restrict__ rays_in,
                                                     const float4 *__restrict__ aux_in, const float4 *__restrict__ hits,
                                                     const uint32_t *__restrict__ count_in,
                                                     float4 *__restrict__ rays_out, float4 *__restrict__ aux_out,
                                                     uint32_t *count_out, uint32_t cap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = *count_in;
    bool alive = false;
    float4 out_r0, out_r1, out_a0, out_a1;
    if (i < n) {
        const float4 a0 = aux_in[2 * (size_t)i], a1 = aux_in[2 * (size_t)i + 1];
        const ItemDev &it = items[__float_as_int(a1.w)];
        float3 T = f3(a0.x, a0.y, a0.z), L = f3(a1.x, a1.y, a1.z);
        const uint32_t g = (uint32_t)__float_as_int(a0.w);
        const float4 h = hits[i];
        const float4 ro = rays_in[2 * (size_t)i], rd = rays_in[2 * (size_t)i + 1];
        float3 o = f3(ro.x, ro.y, ro.z), d = f3(rd.x, rd.y, rd.z), no, nd;
        alive = shade_step(it.sp, level, g, o, d, h.x, h.y, h.z, __float_as_int(h.w), it.tree.recs, it.prim_mat,
                           it.mats, it.normals, T, L, no, nd);
        if (alive) {
            out_r0 = make_float4(no.x, no.y, no.z, 0.0001f);
            out_r1 = make_float4(nd.x, nd.y, nd.z, __int_as_float(0x7f800000));
            out_a0 = make_float4(T.x, T.y, T.z, a0.w);
            out_a1 = make_float4(L.x, L.y, L.z, a1.w);
        } else {
            deposit(it.acc, g % it.sp.npix, L);
        }
    }
    const uint32_t ball = __ballot_sync(0xffffffffu, alive);
    if (ball == 0) return;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == (uint32_t)(__ffs(ball) - 1)) base = atomicAdd(count_out, (uint32_t)__popc(ball));
    base = __shfl_sync(0xffffffffu, base, __ffs(ball) - 1);
    if (alive) {
        const uint32_t slot = base + __popc(ball & lane_lt_mask());
        if (slot < cap) {
            rays_out[2 * (size_t)slot] = out_r0;
            rays_out[2 * (size_t)slot + 1] = out_r1;
            aux_out[2 * (size_t)slot] = out_a0;
            aux_out[2 * (size_t)slot + 1] = out_a1;
        }
    }
}

__global__ void k_sum_levels(const uint32_t *counts, int levels, unsigned long long *total) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        unsigned long long s = 0;
        for (int i = 0; i < levels; i++) s += counts[i];
        *total += s;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct gbt_graph {
    gbt_ctx *ctx = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void *pinned_items = nullptr;  // page-locked source of the graph's descriptor upload
    void *state = nullptr;         // the graph's own descriptors, accumulators and path buffers
    int pins_scratch = 0;          // its rebuilds use the context's scratch
    uint64_t paths = 0;
};

namespace {

using Launcher = void (*)(const ItemDev *, int, uint32_t, uint32_t *, unsigned int *, unsigned long long *, int,
                          cudaStream_t);

template <int W, int BLOCK, int DYN, int SH>
void launch_batch(const ItemDev *items, int n, uint32_t total, uint32_t *fetch, unsigned int *err,
                  unsigned long long *rays, int num_sms, cudaStream_t s) {
    static int per_sm = 0;
    if (per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<W, BLOCK, DYN, SH>, BLOCK, 0);
        if (per_sm <= 0) per_sm = 1;
    }
    uint32_t grid = (uint32_t)(num_sms * per_sm);
    uint32_t need = (total + BLOCK - 1) / BLOCK;
    if (need < grid) grid = need;
    if (grid == 0) grid = 1;
    k_batch<W, BLOCK, DYN, SH><<<grid, BLOCK, 0, s>>>(items, n, total, fetch, err, rays);
}

// megakernel config: block in {64,128,256} x fetch_min in {0,16} x stack in {local, first 12 entries in shared memory}
template <int W>
Launcher pick(const gbt_batch_config &c) {
    const int b = c.block, d = c.fetch_min > 0 ? 1 : 0, s = c.stack ? 1 : 0;
#define GBT_PICK(B, D, S) \
    if (b == B && d == (D > 0) && s == (S > 0)) return &launch_batch<W, B, D, S>;
    GBT_PICK(64, 0, 0) GBT_PICK(64, 0, 12) GBT_PICK(64, 16, 0) GBT_PICK(64, 16, 12)
    GBT_PICK(128, 0, 0) GBT_PICK(128, 0, 12) GBT_PICK(128, 16, 0) GBT_PICK(128, 16, 12)
    GBT_PICK(256, 0, 0) GBT_PICK(256, 0, 12) GBT_PICK(256, 16, 0) GBT_PICK(256, 16, 12)
#undef GBT_PICK
    return nullptr;
}

int check_items(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n, int *width) {
    if (!items || n == 0 || n > (uint32_t)MAX_ITEMS) return gbt_fail(ctx, GBT_EINVAL, "batch: 1..1024 items");
    int w = -1;
    uint64_t paths = 0;
    for (uint32_t i = 0; i < n; i++) {
        const gbt_batch_item &it = items[i];
        if (!it.bvh || !it.d_rgb) return gbt_fail(ctx, GBT_EINVAL, "batch: item without BVH or output");
        const gbt_render_params &p = it.params;
        if (p.width < 2 || p.height < 2 || p.spp < 1 || p.max_depth < 0 || p.max_depth > 60)
            return gbt_fail(ctx, GBT_EINVAL, "batch: width/height >= 2, spp >= 1, 0 <= max_depth <= 60");
        int wi = (it.bvh->has_nodes4 || it.bvh->arity == 4) ? 4 : 2;
        if (w < 0) w = wi;
        if (wi != w) return gbt_fail(ctx, GBT_EINVAL, "batch: all BVHs need the same traversal layout");
        paths += (uint64_t)p.width * p.height * p.spp;
    }
    if (paths >= (1ull << 32)) return gbt_fail(ctx, GBT_EINVAL, "batch: more than 2^32 paths");
    *width = w;
    return GBT_OK;
}

int check_config(gbt_ctx *ctx, const gbt_batch_config &c, int width) {
    if (c.mode == GBT_BATCH_WAVEFRONT && (c.packets == 0 || c.packets == 1)) return GBT_OK;
    if (c.mode != GBT_BATCH_MEGAKERNEL || !(width == 4 ? pick<4>(c) : pick<2>(c)))
        return gbt_fail(ctx, GBT_EINVAL, "batch: unsupported configuration");
    return GBT_OK;
}

// camera rays of this tree go as packets (when the frame's form allows them): the context forces
// them, or the tree's measured or set choice says so
bool packet_tree(const gbt_ctx *ctx, const gbt_bvh *b) {
    return ctx->primary_packets == 1 || (ctx->primary_packets == 2 && b->packet_choice == 1);
}

// Item descriptors of one frame; acc pointers are set by place().  Items whose
// tree traces camera rays faster as packets come first (in their given order),
// so that their paths form one leading range of the queue; the accumulators
// follow the same order.  The order changes nothing but float summation order.
int describe(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n, std::vector<ItemDev> &hi, uint64_t *total_paths,
             size_t *acc_floats) {
    hi.resize(n);
    std::vector<uint32_t> order;
    order.reserve(n);
    for (int pass = 0; pass < 2; pass++)
        for (uint32_t i = 0; i < n; i++)
            if (packet_tree(ctx, items[i].bvh) == (pass == 0)) order.push_back(i);
    uint64_t paths = 0, pix = 0;
    for (uint32_t k = 0; k < n; k++) {
        const uint32_t i = order[k];
        const gbt_batch_item &it = items[i];
        const gbt_bvh *b = it.bvh;
        ItemDev &d = hi[k];
        d.tree.hdr = b->has_nodes4 ? b->d_hdr4 : b->d_hdr;
        d.tree.nodes = b->has_nodes4 ? b->d_nodes4 : b->d_nodes;
        d.tree.recs = b->d_prims;
        d.tree.any_level = ctx->anyhit_last ? it.params.max_depth + 1 : -1;
        d.tree.packets = packet_tree(ctx, b) ? 1 : 0;
        d.prim_mat = b->scene->d_prim_mat;
        d.mats = b->scene->d_mats;
        d.normals = b->scene->d_normals;
        d.acc = nullptr;
        d.out = it.d_rgb;
        d.cam = gbt_make_cam(&it.camera);
        d.sp = gbt_make_shade_params(&it.params, b->scene->n_tri);
        d.sp.tiles = ctx->primary_tiles ? 1u : 0u;
        d.sp.any_last = ctx->anyhit_last ? 1u : 0u;
        d.path_base = (uint32_t)paths;
        d.pix_base = (uint32_t)pix;
        d.inv_spp = 1.0f / it.params.spp;
        d.pad = 0;
        paths += (uint64_t)it.params.width * it.params.height * it.params.spp;
        pix += (uint64_t)it.params.width * it.params.height;
    }
    *total_paths = paths;
    *acc_floats = pix * 3;
    if (pix * 3 >= (1ull << 32)) return gbt_fail(ctx, GBT_EINVAL, "batch: too many pixels");
    return GBT_OK;
}

// Device buffers of one frame: descriptors, accumulators and, for the wavefront form, the path buffers.
struct FrameBufs {
    ItemDev *items = nullptr;
    float *acc = nullptr;
    RenderState rs{};  // rs.cap == 0: no path buffers
};

size_t head_bytes(size_t n, size_t acc_floats) {
    return gbt_align(n * sizeof(ItemDev)) + gbt_align(acc_floats * sizeof(float));
}

void bind_head(void *base, size_t n, FrameBufs *fb) {
    unsigned char *b = static_cast<unsigned char *>(base);
    fb->items = reinterpret_cast<ItemDev *>(b);
    fb->acc = reinterpret_cast<float *>(b + gbt_align(n * sizeof(ItemDev)));
}

void place(std::vector<ItemDev> &hi, float *acc) {
    for (auto &d : hi) d.acc = acc + (size_t)d.pix_base * 3;
}

// the context's batch state (grow-only) and, for the wavefront form, its render path buffers
int context_bufs(gbt_ctx *ctx, size_t n, size_t acc_floats, uint64_t paths, bool waves, FrameBufs *fb) {
    const size_t need = head_bytes(n, acc_floats);
    if (ctx->bstate_bytes < need) {
        if (ctx->bstate) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->bstate);
        }
        ctx->bstate = nullptr;
        ctx->bstate_bytes = 0;
        if (cudaMalloc(&ctx->bstate, need) != cudaSuccess) {
            cudaGetLastError();
            return gbt_fail(ctx, GBT_ENOMEM, "batch: state allocation");
        }
        ctx->bstate_bytes = need;
    }
    bind_head(ctx->bstate, n, fb);
    fb->rs = RenderState{};
    if (waves) return gbt_render_buffers(ctx, paths, 0, &fb->rs);
    return GBT_OK;
}

int enqueue_frame(gbt_ctx *ctx, const FrameBufs &fb, const ItemDev *h_items, size_t n_items, uint64_t paths,
                  size_t acc_floats, const gbt_batch_config &cfg, int width) {
    cudaStream_t st = ctx->stream;
    GBT_CUDA(ctx, cudaMemcpyAsync(fb.items, h_items, n_items * sizeof(ItemDev), cudaMemcpyHostToDevice, st));
    GBT_CUDA(ctx, cudaMemsetAsync(fb.acc, 0, acc_floats * sizeof(float), st));
    uint64_t launches = 0, trav = 0;
    if (cfg.mode == GBT_BATCH_MEGAKERNEL) {
        Launcher f = width == 4 ? pick<4>(cfg) : pick<2>(cfg);
        if (!f) return gbt_fail(ctx, GBT_EINVAL, "batch: unsupported configuration");
        uint32_t *fetch = reinterpret_cast<uint32_t *>(ctx->d_counters + 3);
        GBT_CUDA(ctx, cudaMemsetAsync(fetch, 0, sizeof(uint32_t), st));
        f(fb.items, (int)n_items, (uint32_t)paths, fetch, ctx->d_error, ctx->d_counters + 2, ctx->num_sms, st);
        launches++;
    } else {
        const RenderState &rs = fb.rs;
        if (rs.cap == 0) return gbt_fail(ctx, GBT_EINVAL, "batch: wavefront form without path buffers");
        int levels = 0;           // surfaces at depth 0..MaxDepth+1 of the deepest item
        uint64_t packet_paths = 0;  // the leading range of paths whose camera rays go as packets
        for (size_t i = 0; i < n_items; i++) {
            levels = std::max(levels, h_items[i].sp.max_depth + 2);
            if (h_items[i].tree.packets)
                packet_paths = (uint64_t)h_items[i].path_base + (uint64_t)h_items[i].sp.npix * h_items[i].sp.spp;
        }
        if (!cfg.packets || width != 4) packet_paths = 0;
        for (uint64_t g0 = 0; g0 < paths; g0 += rs.cap) {
            const uint32_t count = (uint32_t)std::min<uint64_t>(paths - g0, rs.cap);
            const uint32_t blocks = (count + 255) / 256;
            GBT_CUDA(ctx, cudaMemsetAsync(rs.counts, 0, 64 * sizeof(uint32_t), st));
            k_raygen_batch<<<blocks, 256, 0, st>>>(fb.items, (int)n_items, (uint32_t)g0, count, rs.rays[0], rs.aux[0],
                                                   rs.counts);
            launches++;
            for (int lv = 0; lv < levels; lv++) {
                const int a = lv & 1;
                // level 0 (every path has its camera ray, in queue order): the wave's leading rays of packet
                // trees as packets, the rest one per lane
                const uint32_t np = lv == 0 && packet_paths > g0 ? (uint32_t)std::min<uint64_t>(packet_paths - g0, count) : 0;
                if (np > 0) {
                    gbt_launch_traverse_packets_multi(&fb.items->tree, sizeof(ItemDev), rs.rays[0], rs.aux[0], rs.hits,
                                                      np, ctx->d_error, st);
                    launches++;
                }
                if (np == 0)
                    gbt_launch_traverse_multi(ctx, &fb.items->tree, sizeof(ItemDev), width, rs.rays[a], rs.aux[a],
                                              rs.hits, count, rs.counts + lv, lv, st);
                else if (np < count)
                    gbt_launch_traverse_multi(ctx, &fb.items->tree, sizeof(ItemDev), width, rs.rays[0] + 2 * (size_t)np,
                                              rs.aux[0] + 2 * (size_t)np, rs.hits + np, count - np, nullptr, 0, st);
                k_shade_batch<<<blocks, 256, 0, st>>>(fb.items, lv, rs.rays[a], rs.aux[a], rs.hits, rs.counts + lv,
                                                      rs.rays[a ^ 1], rs.aux[a ^ 1], rs.counts + lv + 1,
                                                      (uint32_t)rs.cap);
                launches += 2;
                trav++;
            }
            k_sum_levels<<<1, 32, 0, st>>>(rs.counts, levels, ctx->d_counters + 2);
            launches++;
        }
    }
    k_resolve_batch<<<ctx->num_sms * 4, 256, 0, st>>>(fb.items, (int)n_items, (uint32_t)acc_floats);
    launches++;
    GBT_CUDA(ctx, cudaGetLastError());
    ctx->last_stats.paths += paths;
    ctx->last_stats.kernel_launches += launches;
    ctx->last_stats.traverse_launches += trav;
    return GBT_OK;
}

gbt_batch_config default_config(const gbt_ctx *ctx) {
    if (ctx->batch_tuned) return ctx->batch_cfg;
    gbt_batch_config c;
    c.block = 128;
    c.fetch_min = 16;
    c.stack = 0;
    c.mode = GBT_BATCH_WAVEFRONT;
    c.packets = ctx->primary_packets && ctx->primary_tiles ? 1 : 0;
    return c;
}

// the measured camera-ray packet choice of every item's tree (once per tree)
int measure_items(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        int rc = gbt_measure_packets(ctx, items[i].bvh, &items[i].camera, &items[i].params);
        if (rc) return rc;
    }
    return GBT_OK;
}

// descriptors and the context's buffers for one frame in form cfg
int setup(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n, bool waves, std::vector<ItemDev> &hi,
          uint64_t *paths, size_t *accf, FrameBufs *fb) {
    int rc = describe(ctx, items, n, hi, paths, accf);
    if (rc) return rc;
    rc = context_bufs(ctx, n, *accf, *paths, waves, fb);
    if (rc) return rc;
    place(hi, fb->acc);
    return GBT_OK;
}

}  // namespace

extern "C" int gbt_render_batch_async(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n,
                                      const gbt_batch_config *cfg) {
    if (!ctx) return GBT_EINVAL;
    int width;
    int rc = check_items(ctx, items, n, &width);
    if (rc) return rc;
    const gbt_batch_config c = cfg ? *cfg : default_config(ctx);
    rc = check_config(ctx, c, width);
    if (rc) return rc;
    if (c.mode == GBT_BATCH_WAVEFRONT && c.packets && width == 4 && ctx->primary_packets == 2) {
        rc = measure_items(ctx, items, n);
        if (rc) return rc;
    }
    std::vector<ItemDev> hi;
    uint64_t paths;
    size_t accf;
    FrameBufs fb;
    rc = setup(ctx, items, n, c.mode == GBT_BATCH_WAVEFRONT, hi, &paths, &accf, &fb);
    if (rc) return rc;
    // a copy from pageable memory is staged before cudaMemcpyAsync returns, so hi may go
    return enqueue_frame(ctx, fb, hi.data(), hi.size(), paths, accf, c, width);
}

extern "C" int gbt_render_batch_plain_async(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n) {
    if (!ctx) return GBT_EINVAL;
    int width;
    int rc = check_items(ctx, items, n, &width);
    if (rc) return rc;
    for (uint32_t i = 0; i < n; i++) {
        rc = gbt_render_enqueue(ctx, items[i].bvh, &items[i].camera, &items[i].params, items[i].d_rgb);
        if (rc) return rc;
    }
    return GBT_OK;
}

extern "C" int gbt_batch_autotune(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n, gbt_batch_config *best,
                                  double *best_ms) {
    if (!ctx || !best) return GBT_EINVAL;
    int width;
    int rc = check_items(ctx, items, n, &width);
    if (rc) return rc;
    if (width == 4 && ctx->primary_packets == 2) {
        rc = measure_items(ctx, items, n);
        if (rc) return rc;
    }
    std::vector<ItemDev> hi;
    uint64_t paths;
    size_t accf;
    FrameBufs fb;
    rc = setup(ctx, items, n, true, hi, &paths, &accf, &fb);
    if (rc) return rc;
    std::vector<gbt_batch_config> cands;
    cands.push_back(gbt_batch_config{128, 16, 0, GBT_BATCH_WAVEFRONT, 0});
    if (width == 4 && ctx->primary_packets) cands.push_back(gbt_batch_config{128, 16, 0, GBT_BATCH_WAVEFRONT, 1});
    for (int b : {64, 128, 256})
        for (int f : {0, 16})
            for (int s : {0, 1}) cands.push_back(gbt_batch_config{b, f, s, GBT_BATCH_MEGAKERNEL, 0});
    double bms = 1e30;
    gbt_batch_config bc = cands[0];
    for (const gbt_batch_config &c : cands) {
        // one untimed frame, then the best of two timed frames
        rc = enqueue_frame(ctx, fb, hi.data(), hi.size(), paths, accf, c, width);
        if (rc) return rc;
        double m = 1e30;
        for (int rep = 0; rep < 2; rep++) {
            GBT_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
            rc = enqueue_frame(ctx, fb, hi.data(), hi.size(), paths, accf, c, width);
            if (rc) return rc;
            GBT_CUDA(ctx, cudaEventRecord(ctx->ev[3], ctx->stream));
            GBT_CUDA(ctx, cudaEventSynchronize(ctx->ev[3]));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
            m = std::min(m, (double)ms);
        }
        if (m < bms) {
            bms = m;
            bc = c;
        }
    }
    rc = gbt_check_device_error(ctx, "batch_autotune");
    if (rc) return rc;
    ctx->batch_cfg = bc;
    ctx->batch_tuned = 1;
    *best = bc;
    if (best_ms) *best_ms = bms;
    return GBT_OK;
}

extern "C" int gbt_batch_graph_create(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n,
                                      const gbt_batch_config *cfg, int32_t rebuild_lbvh, gbt_graph **out) {
    if (!ctx || !out) return GBT_EINVAL;
    *out = nullptr;
    int width;
    int rc = check_items(ctx, items, n, &width);
    if (rc) return rc;
    if (rebuild_lbvh)
        for (uint32_t i = 0; i < n; i++)
            if (items[i].bvh->kind != GBT_BVH_LBVH)
                return gbt_fail(ctx, GBT_EINVAL, "batch graph: rebuilding needs LBVH items");
    const gbt_batch_config c = cfg ? *cfg : default_config(ctx);
    rc = check_config(ctx, c, width);
    if (rc) return rc;
    const bool waves = c.mode == GBT_BATCH_WAVEFRONT;
    if (waves && c.packets && width == 4 && ctx->primary_packets == 2) {
        rc = measure_items(ctx, items, n);
        if (rc) return rc;
    }
    std::vector<ItemDev> hi;
    uint64_t paths;
    size_t accf;
    rc = describe(ctx, items, n, hi, &paths, &accf);
    if (rc) return rc;
    gbt_graph *g = new gbt_graph();
    g->ctx = ctx;
    g->paths = paths;
    auto fail = [&](int code) {
        if (g->exec) cudaGraphExecDestroy(g->exec);
        if (g->graph) cudaGraphDestroy(g->graph);
        if (g->pinned_items) cudaFreeHost(g->pinned_items);
        if (g->state) cudaFree(g->state);
        delete g;
        cudaGetLastError();
        return code;
    };
    // the graph owns its buffers, so later work on the context cannot move them
    const size_t head = head_bytes(n, accf);
    const size_t bytes = head + (waves ? gbt_render_state_bytes(paths, 0) : 0);
    if (cudaMalloc(&g->state, bytes) != cudaSuccess) return fail(gbt_fail(ctx, GBT_ENOMEM, "batch graph: state"));
    FrameBufs fb;
    bind_head(g->state, n, &fb);
    if (waves) gbt_render_state_bind(static_cast<unsigned char *>(g->state) + head, paths, 0, &fb.rs);
    place(hi, fb.acc);
    if (cudaMallocHost(&g->pinned_items, hi.size() * sizeof(ItemDev)) != cudaSuccess)
        return fail(gbt_fail(ctx, GBT_ENOMEM, "batch graph: pinned descriptors"));
    std::memcpy(g->pinned_items, hi.data(), hi.size() * sizeof(ItemDev));
    // grow the scratch the captured rebuilds (and collapses into the 4-wide views) use before
    // capturing; it may not move while the graph lives
    for (uint32_t i = 0; rebuild_lbvh && i < n; i++) {
        size_t need = gbt_lbvh_scratch_bytes(items[i].bvh->n_prim), need4 = 0;
        if (width == 4) {
            rc = gbt_collapse4_reserve(ctx, items[i].bvh, &need4);
            if (rc) return fail(rc);
        }
        void *scr;
        rc = gbt_scratch(ctx, std::max(need, need4), &scr);
        if (rc) return fail(rc);
    }
    cudaStream_t st = ctx->stream;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return fail(gbt_fail(ctx, GBT_ECUDA, "batch graph: begin capture"));
    for (uint32_t i = 0; rebuild_lbvh && i < n && !rc; i++) {
        rc = gbt_lbvh_enqueue(ctx, items[i].bvh);
        if (!rc && width == 4) rc = gbt_collapse4_enqueue(ctx, items[i].bvh);
    }
    if (!rc) rc = enqueue_frame(ctx, fb, static_cast<const ItemDev *>(g->pinned_items), hi.size(), paths, accf, c, width);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    g->graph = graph;
    if (rc || e != cudaSuccess)
        return fail(rc ? rc : gbt_fail(ctx, GBT_ECUDA, std::string("batch graph: capture: ") + cudaGetErrorString(e)));
    if (cudaGraphInstantiate(&g->exec, graph, 0) != cudaSuccess)
        return fail(gbt_fail(ctx, GBT_ECUDA, "batch graph: instantiate"));
    if (rebuild_lbvh) {
        g->pins_scratch = 1;
        ctx->scratch_pins++;
    }
    ctx->last_stats.paths = 0;
    *out = g;
    return GBT_OK;
}

extern "C" int gbt_graph_launch(gbt_ctx *ctx, gbt_graph *g) {
    if (!ctx || !g || g->ctx != ctx) return GBT_EINVAL;
    GBT_CUDA(ctx, cudaGraphLaunch(g->exec, ctx->stream));
    ctx->last_stats.paths += g->paths;
    return GBT_OK;
}

extern "C" int gbt_graph_destroy(gbt_graph *g) {
    if (!g) return GBT_EINVAL;
    if (g->ctx) {
        cudaStreamSynchronize(g->ctx->stream);
        if (g->pins_scratch) g->ctx->scratch_pins--;
    }
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->pinned_items) cudaFreeHost(g->pinned_items);
    if (g->state) cudaFree(g->state);
    delete g;
    return GBT_OK;
}
