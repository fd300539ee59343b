// Internal declarations shared by the CUDA translation units of libgbtrace.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gbtrace.h"

// ---------------------------------------------------------------------------
// error plumbing
// ---------------------------------------------------------------------------
#define GBT_DEVERR_SPIN 1u       // a bounded spin-wait ran out
#define GBT_DEVERR_BOUNDS 2u     // an index check failed and the access was skipped
#define GBT_DEVERR_STACK 4u      // traversal stack overflow (deepest entries dropped)
#define GBT_DEVERR_CAPACITY 8u   // a device work list was full

// Iteration limit of every device-side spin-wait.  With the 64 ns back-off it
// bounds one wait at roughly a quarter of a second.
#define GBT_SPIN_LIMIT (1u << 22)

#define GBT_PHR_SMALL_CUT 256

#define GBT_BLOCK_CACHE 4

struct gbt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    unsigned int *d_error = nullptr;  // device error word (GBT_DEVERR_*)
    int num_sms = 0;
    // grow-only scratch, reused by every build on this context
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    int scratch_pins = 0;  // live graphs whose captured work uses the scratch: it may not move
    // render state (grow-only)
    void *rstate = nullptr;
    size_t rstate_bytes = 0;
    gbt_render_stats last_stats{};
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // profiling (gbt_ctx_set_profiling)
    int profiling = 0;
    std::vector<cudaEvent_t> prof_ev;           // pairs around traversal launches
    int n_prof_ev = 0;
    unsigned long long *d_counters = nullptr;   // [0] inner nodes fetched, [1] primitive tests, [2] rays traced
    float *d_out = nullptr;                     // gbt_render's device image (grow-only)
    size_t d_out_bytes = 0;
    // batched rendering (batch.cu): item descriptors + accumulators, autotuned launch config
    void *bstate = nullptr;
    size_t bstate_bytes = 0;
    gbt_batch_config batch_cfg{128, 16, 0, GBT_BATCH_WAVEFRONT, 0};
    cudaStream_t side = nullptr;  // captures the bodies of conditional graph nodes (created on first use)
    int batch_tuned = 0;
    // traversal kernel: 0 persistent with dynamic ray fetch (default), 1 one thread per ray,
    // 2 persistent without mid-ray refills (GBT_TRAVERSAL=simple|ww at context creation)
    int traversal = 0;
    // renderer options (gbt_ctx_set_option): answer the rays of the level past MaxDepth,
    // whose hit shades black, with an any-hit query; order camera rays in 8x4 pixel tiles
    int anyhit_last = 1;
    int primary_tiles = 1;
    // camera rays of a tiled frame as 32-ray packets: 0 never, 1 always, 2 (default) whichever
    // kernel the first render on a BVH measures faster for its camera rays
    int primary_packets = 2;
    cudaEvent_t tune_ev[3] = {nullptr, nullptr, nullptr};
    // PHR workspace (phr.cu): the build's temporaries and its per-block scratch, kept for the
    // next refinement unless GBT_OPT_KEEP_WORKSPACE is 0
    void *phr_ws = nullptr;
    size_t phr_ws_bytes = 0;
    void *phr_scr = nullptr;
    size_t phr_scr_bytes = 0;
    int keep_workspace = 1;
    // Device blocks of destroyed trees (a PHR tree's arrays, a 4-wide view), kept for the
    // next trees built on this context: a cudaMalloc and cudaFree of a tree's few hundred MB
    // take 0.1-0.5 ms.  Released with the context, when a cudaMalloc of gbt_block_get
    // fails, and at once under GBT_OPT_KEEP_WORKSPACE 0.
    void *block_cache[GBT_BLOCK_CACHE] = {};
    size_t block_cache_bytes[GBT_BLOCK_CACHE] = {};
    // largest cut of a PHR level run with one-warp blocks (GBT_OPT_PHR_SMALL_CUT, 1..GBT_PHR_SMALL_CUT)
    int phr_small_cut = GBT_PHR_SMALL_CUT;
    void *h_pin = nullptr;  // small pinned host buffer for counter readbacks (gbt_pinned)
    // bounded device waits (GBT_OPT_SPIN_LIMIT) and the testing aids that make them and the
    // work-list checks trip (GBT_OPT_TEST_WITHHOLD_TILE, GBT_OPT_TEST_COLLAPSE_CAP)
    uint32_t spin_limit = GBT_SPIN_LIMIT;
    // threads per tile of the LBVH sort's passes: 256 (16 keys each) or 512 (8 keys each)
    int sort_threads = 256;
    uint32_t withhold_tile = 0xffffffffu;
    uint32_t collapse_cap = 0;
};

// A pinned host buffer of GBT_PINNED_BYTES owned by the context (allocated on first use).
#define GBT_PINNED_BYTES 4096
void *gbt_pinned(gbt_ctx *ctx);
// Frees the PHR workspace kept on the context.
void gbt_phr_release(gbt_ctx *ctx);

// Record a profiling event pair around one traversal launch.
void gbt_prof_begin(gbt_ctx *ctx);
void gbt_prof_end(gbt_ctx *ctx);

struct gbt_scene {
    gbt_ctx *ctx = nullptr;
    uint32_t n_tri = 0, n_sph = 0, n_mat = 0;
    float *d_verts = nullptr;      // n_tri*9, input order
    float *d_normals = nullptr;    // n_tri*9 or null
    float4 *d_sph = nullptr;       // n_sph (center, radius)
    uint32_t *d_prim_mat = nullptr;
    float4 *d_mats = nullptr;      // 2 per material: (color.rgb, type), (param, 0, 0, 0)
    std::vector<gbt_material> mats;
};

// Device-resident header of a BVH: the root entry (a node or a leaf) and sizes.
struct BvhHeader {
    int32_t root_ref;  // node index, or first primitive record when root_cnt > 0
    int32_t root_cnt;  // > 0: the root is a leaf of root_cnt primitives
    uint32_t n_unique; // LBVH: distinct Morton codes (= leaves)
    uint32_t n_nodes;  // inner nodes in use
    uint32_t sorted_sel; // LBVH: which half of d_codes/d_idx holds the sorted pairs
    uint32_t pad[3];
    float root_lo[4];
    float root_hi[4];
};

#define GBT_BVH_LBVH 0
#define GBT_BVH_PHR 1

struct gbt_bvh {
    gbt_ctx *ctx = nullptr;
    gbt_scene *scene = nullptr;
    int kind = GBT_BVH_LBVH;
    int arity = 2;              // 2: 64-byte nodes; 4: 128-byte nodes
    uint32_t n_prim = 0;        // primitive records
    uint32_t node_cap = 0;      // allocated inner nodes
    float4 *d_nodes = nullptr;  // arity 2: 4 float4 per node; arity 4: 8 float4 per node
    float4 *d_prims = nullptr;  // 3 float4 per primitive record, in leaf order
    BvhHeader *d_hdr = nullptr;
    // LBVH products kept for parity checks and PHR
    uint64_t *d_codes = nullptr;    // sorted Morton codes
    uint32_t *d_idx = nullptr;      // sorted primitive indices
    uint32_t *d_run = nullptr;      // start of each distinct-code run, n_unique+1 entries
    uint64_t *d_ukey = nullptr;     // distinct codes
    int32_t *d_parent = nullptr;    // per inner node: parent node (-1 root) -- LBVH only
    uint32_t *d_size = nullptr;     // per inner node: subtree size (bvh.go:159-167)
    int32_t *d_other = nullptr;     // emission hand-off words
    uint2 *d_range = nullptr;       // per inner node: distinct-code range [l, r]
    uint32_t n_nodes_host = 0;      // PHR: nodes allocated in d_nodes
    int64_t build_cost = 0;         // PHR: BuildWithCost's count (phr.go:154-255)
    // 4-wide traversal view of a binary tree (collapse.cu); used by traversal when present
    float4 *d_nodes4 = nullptr;
    BvhHeader *d_hdr4 = nullptr;
    uint32_t nodes4_cap = 0;
    size_t nodes4_bytes = 0;        // size of the d_nodes4 block
    int has_nodes4 = 0;
    int packet_choice = 0;          // camera-ray kernel measured for this tree: 0 not yet, 1 packets, 2 single rays
    void *d_block = nullptr;        // when set: d_nodes, d_prims, d_parent and d_hdr are pieces of this allocation
    size_t d_block_bytes = 0;
};

// collapse.cu
int gbt_collapse4(gbt_ctx *ctx, gbt_bvh *bvh);
// For graph capture: gbt_collapse4_reserve allocates the 4-wide view of a tree of this size and
// returns the scratch bytes gbt_collapse4_enqueue needs; gbt_collapse4_enqueue (only while the
// context's stream is capturing) records the collapse as a conditional WHILE node over its levels.
int gbt_collapse4_reserve(gbt_ctx *ctx, gbt_bvh *bvh, size_t *scratch_bytes);
int gbt_collapse4_enqueue(gbt_ctx *ctx, gbt_bvh *bvh);
// cost.cu: BVH.Cost of the tree as built
int gbt_cost_device(gbt_ctx *ctx, gbt_bvh *bvh, double *out);

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
int gbt_fail(gbt_ctx *ctx, int code, const std::string &msg);
int gbt_cuda_fail(gbt_ctx *ctx, cudaError_t e, const char *what);
int gbt_check_device_error(gbt_ctx *ctx, const char *what);
int gbt_scratch(gbt_ctx *ctx, size_t bytes, void **out);
// A device block of at least `bytes` (its size in *got): the smallest cached block that
// fits and is at most twice as large, else a new allocation.
cudaError_t gbt_block_get(gbt_ctx *ctx, size_t bytes, void **p, size_t *got);
// Hands a block of a destroyed tree back to the context's cache (the smallest cached
// block is freed when the cache is full); frees it under GBT_OPT_KEEP_WORKSPACE 0.
void gbt_block_put(gbt_ctx *ctx, void *p, size_t bytes);
void gbt_block_release(gbt_ctx *ctx);

#define GBT_CUDA(ctx, call)                                   \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return gbt_cuda_fail((ctx), e_, #call); \
    } while (0)

static inline size_t gbt_align(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

// ---------------------------------------------------------------------------
// Programmatic dependent launch (sm_90 and later).  A kernel launched with
// gbt_launch_pdl may be scheduled while the kernel before it in the stream is
// still running: its blocks start once every block of that kernel has started
// (or called gbt_pdl_trigger), then gbt_pdl_wait() holds them until that
// kernel has completed and its writes are visible.  Such a kernel calls
// gbt_pdl_wait() first, on every path, so that its own completion still
// implies its predecessors' (the next kernel's wait relies on it).  Without
// the launch attribute the wait returns at once.
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
__device__ __forceinline__ void gbt_pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void gbt_pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// pdl false: an ordinary launch.
template <typename... KArgs, typename... Args>
static inline cudaError_t gbt_launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                                         cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
#endif

// ---------------------------------------------------------------------------
// entry points between translation units
// ---------------------------------------------------------------------------
// lbvh.cu
int gbt_lbvh_enqueue(gbt_ctx *ctx, gbt_bvh *bvh);
size_t gbt_lbvh_scratch_bytes(uint32_t n);

// traverse.cu
int gbt_trace_enqueue(gbt_ctx *ctx, const gbt_bvh *bvh, const gbt_ray *d_rays, uint32_t n, gbt_hit *d_hits);
void gbt_launch_traverse(const gbt_bvh *bvh, const float4 *rays, float4 *hits, uint32_t n,
                         const uint32_t *d_count, int out_mode, unsigned int *d_error, cudaStream_t s,
                         unsigned long long *d_counters = nullptr, bool any = false);
// One tree of a batched frame as the multi-tree traversal reads it: a ray's
// tree is the index in .w of its second path record (aux[2 i + 1].w).
struct TreeRef {
    const BvhHeader *hdr;
    const float4 *nodes;
    const float4 *recs;
    int32_t any_level;  // the level whose rays take an any-hit query (-1: none)
    int32_t packets;    // 1: this tree's camera rays trace faster as packets (its measured choice)
};
// trees: entry k at byte offset k * stride
void gbt_launch_traverse_multi(gbt_ctx *ctx, const TreeRef *trees, size_t stride, int width, const float4 *rays,
                               const float4 *aux, float4 *hits, uint32_t n, const uint32_t *d_count, int level,
                               cudaStream_t s);
// packets over the camera rays of many 4-wide trees (tree index in aux[2 i + 1].w)
void gbt_launch_traverse_packets_multi(const TreeRef *trees, size_t stride, const float4 *rays, const float4 *aux,
                                      float4 *hits, uint32_t n, unsigned int *d_error, cudaStream_t s);
// 32-ray packets per warp (coherent camera rays) over a 4-wide tree; false when the tree has no 4-wide nodes
bool gbt_launch_traverse_packets(const gbt_bvh *bvh, const float4 *rays, float4 *hits, uint32_t n, int out_mode,
                                 unsigned int *d_error, cudaStream_t s, unsigned long long *d_counters);
// render.cu: wavefront path state (ping-pong rays and path records, hits, per-level counts, accumulator)
struct RenderState {
    size_t cap;  // paths per wave
    float4 *rays[2], *aux[2];
    float4 *hits;
    uint32_t *counts;  // per level
    float *acc;
};
// bytes of the state for waves over `total` paths and npix pixels, and its layout at base
size_t gbt_render_state_bytes(size_t total, size_t npix);
void gbt_render_state_bind(void *base, size_t total, size_t npix, RenderState *rs);
int gbt_render_buffers(gbt_ctx *ctx, size_t total, size_t npix, RenderState *rs);
// Measures, once per tree, whether camera rays of this view trace faster as packets (bvh->packet_choice
// 1) or one ray per lane (2); leaves it unmeasured (0) below 65536 camera rays or while profiling.
int gbt_measure_packets(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *p);
int gbt_render_enqueue(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *p,
                       float *d_rgb);
// phr.cu
int gbt_phr_run(gbt_ctx *ctx, gbt_bvh *aux, double alpha, double delta, int bf, gbt_bvh *out);
