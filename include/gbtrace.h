/*
 * gbtrace.h -- C ABI of the GB300 (sm_103a) backend for ChSchmidt99/trace's
 * pkg/pt hot path: Morton LBVH build, PHR refinement, closest-hit tracing and
 * the path-tracing render loop.
 *
 * Conventions
 *  - Every call returns GBT_OK (0) or a negative GBT_E* code; the message of
 *    the last failure on a context is gbt_last_error(ctx).  The Go reference
 *    panics instead (obj.go:13); a binding turns non-zero codes into panics.
 *  - Handles are opaque; the library owns all device memory.  Host buffers
 *    passed in are copied; host output buffers are written before return.
 *  - All work of a context runs on its own CUDA stream (gbt_ctx_stream).
 *    Calls without the _async suffix return after the stream is idle; _async
 *    calls only enqueue, on device buffers, and never allocate.
 *  - Primitive index space: triangles [0, n_tri), then spheres
 *    [n_tri, n_tri + n_sph), the order pkg/pt/scene.go:100-114 collects
 *    tracables in.
 *  - One context per host thread; no callbacks.
 */
#ifndef GBTRACE_H
#define GBTRACE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBT_OK 0
#define GBT_EINVAL -1      /* bad argument (null handle, size out of range) */
#define GBT_ECUDA -2       /* CUDA runtime error */
#define GBT_ENOMEM -3      /* device or host allocation failed */
#define GBT_ETIMEOUT -4    /* a bounded device-side wait ran out */
#define GBT_EDEVICE -5     /* a kernel reported an internal error */
#define GBT_EUNSUPPORTED -6

typedef struct gbt_ctx gbt_ctx;
typedef struct gbt_scene gbt_scene;
typedef struct gbt_bvh gbt_bvh;

typedef struct {
    float center[3];
    float radius;
} gbt_sphere; /* pkg/pt/primitive.go:25-40 Sphere */

#define GBT_MAT_DIFFUSE 0    /* pkg/pt/material.go:25-42 Diffuse{Albedo} */
#define GBT_MAT_LIGHT 1      /* pkg/pt/material.go:13-23 Light{Color} */
#define GBT_MAT_REFLECTIVE 2 /* pkg/pt/material.go:44-57 Reflective{Albedo, Diffusion} */
#define GBT_MAT_REFRACTIVE 3 /* pkg/pt/material.go:59-106 Refractive{Albedo, Ratio} */
typedef struct {
    int32_t type;
    float color[3]; /* Albedo (Diffuse, Reflective, Refractive) or Color (Light) */
    float param;    /* Reflective.Diffusion or Refractive.Ratio; unused otherwise */
} gbt_material;

typedef struct {
    float origin[3];
    float tmin;
    float dir[3]; /* not normalised, as pkg/pt/camera.go:95-97 casts it */
    float tmax;
} gbt_ray;

typedef struct {
    int32_t prim; /* primitive index, -1 on a miss */
    float t, u, v;
} gbt_hit;

typedef struct {
    double look_from[3], look_at[3], up[3]; /* pkg/pt/camera.go:7-11 CameraTransformation */
    double aspect, fov_deg;                 /* pkg/pt/camera.go:53-59 NewCamera */
} gbt_camera;

#define GBT_MISS_BLACK 0    /* render.go:228 DefaultMissShader */
#define GBT_MISS_WHITE 1    /* render.go:232 WhiteMissShader */
#define GBT_MISS_SKY 2      /* render.go:236 SkyMissShader */
#define GBT_MISS_CONSTANT 3 /* constant colour (render.go:244 SunMissShader is one) */
typedef struct {
    int32_t width, height, spp, max_depth; /* render.go:20-30 ImageRenderer fields */
    int32_t miss_mode;
    float miss_color[3];
    uint64_t seed;
} gbt_render_params;

typedef struct {
    uint64_t rays_traced;       /* every traced segment: primary + bounces */
    uint64_t paths;
    double ms_total;            /* device time of the render (CUDA events; gbt_render only) */
    double ms_traverse;         /* device time inside traversal launches (profiling >= 1) */
    uint64_t traverse_launches; /* traversal kernels launched */
    uint64_t kernel_launches;   /* all kernels this library launched for the render */
    uint64_t nodes_visited;     /* inner nodes fetched by traversal (profiling 2) */
    uint64_t prims_tested;      /* primitive records tested (profiling 2) */
} gbt_render_stats;

/* ---- context -------------------------------------------------------- */
/* Scenes, BVHs, buffers and batches belong to the context they were made on:
 * destroy them before it (gbt_bvh_destroy hands a tree's device blocks back to
 * its context). */
int gbt_ctx_create(int device, gbt_ctx **out);
int gbt_ctx_destroy(gbt_ctx *ctx);
const char *gbt_last_error(const gbt_ctx *ctx);
void *gbt_ctx_stream(gbt_ctx *ctx); /* the context's cudaStream_t */
int gbt_ctx_sync(gbt_ctx *ctx);
/* Profiling level of later calls: 0 off; 1 CUDA events around every traversal
 * launch (ms_traverse); 2 also counts inner nodes and primitive tests (a
 * slower counting traversal).  No counterpart in the reference. */
int gbt_ctx_set_profiling(gbt_ctx *ctx, int32_t level);
/* Execution options of later calls on this context.  None of options 0-6
 * changes a result: hits, images and gradients are identical under every
 * setting (a spin limit too low for the work fails the call instead).  The
 * testing aids 7 and 8 make calls fail on purpose, with no fault.
 *   GBT_OPT_TRAVERSAL      0 persistent with dynamic ray fetch (default),
 *                          1 one thread per ray, 2 persistent without refills
 *   GBT_OPT_ANYHIT_LAST    1 (default): rays of the level past MaxDepth, whose
 *                          hit shades black (pkg/pt/render.go:210-212), stop at
 *                          the first hit found
 *   GBT_OPT_PRIMARY_TILES  1 (default): the 32 camera rays of a warp cover an
 *                          8x4 pixel tile instead of 32 pixels of one row
 *   GBT_OPT_PRIMARY_PACKETS with tiles, the camera rays of a warp traced as
 *                          one packet (a shared node sequence, each lane testing
 *                          its own ray): 0 never, 1 always, 2 (default) when
 *                          the first render on a tree measures the packet
 *                          kernel faster on its camera rays (that render traces
 *                          them with both kernels and synchronises once)
 *   GBT_OPT_KEEP_WORKSPACE 1 (default): a PHR refinement leaves its device
 *                          workspace (about 600 bytes per auxiliary-tree
 *                          triangle) on the context for the next one, and a
 *                          destroyed tree's device blocks (a PHR tree's arrays,
 *                          a 4-wide view; up to four) stay on the context for
 *                          the next trees; 0 frees both now and from then on
 *   GBT_OPT_PHR_SMALL_CUT  1..256 (default 256): PHR levels whose cuts are all
 *                          at most this many nodes run with one-warp blocks in
 *                          batches of launches; a launch that meets a larger
 *                          cut is repeated with wider blocks
 *   GBT_OPT_SPIN_LIMIT     1..4194304 (default 4194304): polls before a bounded
 *                          device-side wait (the LBVH sort's look-back) gives
 *                          up; the call then returns GBT_ETIMEOUT, the kernels
 *                          after the wait do nothing, and the context stays
 *                          usable
 *   GBT_OPT_TEST_WITHHOLD_TILE  testing aid, -1 (default) off: the LBVH sort's
 *                          tile of this index never publishes its digit counts
 *                          in the first pass, so the tiles after it wait for a
 *                          status nothing sets until GBT_OPT_SPIN_LIMIT runs out
 *   GBT_OPT_TEST_COLLAPSE_CAP   testing aid, 0 (default) off: the work list of
 *                          the 4-wide collapse holds at most this many nodes;
 *                          children past it are dropped, never written, and
 *                          the call returns GBT_EDEVICE ("work list full")
 * The environment variables GBT_TRAVERSAL (persistent|simple|ww),
 * GBT_ANYHIT_LAST, GBT_PRIMARY_TILES (0|1) and GBT_PRIMARY_PACKETS (0|1|2) set
 * the initial values.
 * No counterpart in the reference. */
#define GBT_OPT_TRAVERSAL 0
#define GBT_OPT_ANYHIT_LAST 1
#define GBT_OPT_PRIMARY_TILES 2
#define GBT_OPT_PRIMARY_PACKETS 3
#define GBT_OPT_KEEP_WORKSPACE 4
#define GBT_OPT_PHR_SMALL_CUT 5
#define GBT_OPT_SPIN_LIMIT 6
#define GBT_OPT_TEST_WITHHOLD_TILE 7
#define GBT_OPT_TEST_COLLAPSE_CAP 8
int gbt_ctx_set_option(gbt_ctx *ctx, int32_t option, int32_t value);

/* ---- scene (pkg/pt/scene.go:7-150 Scene/Mesh collected into flat arrays) */
/* verts: n_tri*9 floats (v0 v1 v2); normals: n_tri*9 per-vertex normals or
 * NULL for face normals (NewTriangleWithoutNormals, primitive.go:116-132);
 * prim_mat: n_tri+n_sph material indices into mats. */
int gbt_scene_upload(gbt_ctx *ctx, const float *verts, const float *normals, uint32_t n_tri,
                     const gbt_sphere *spheres, uint32_t n_sph, const uint32_t *prim_mat,
                     const gbt_material *mats, uint32_t n_mat, gbt_scene **out);
int gbt_scene_destroy(gbt_scene *scene);

/* OBJ loader: pkg/pt/obj.go:10-140 ParseFromPath (fan triangulation,
 * negative indices, v/vn/f).  Two calls: first with verts == NULL to get
 * *n_tri and *has_normals, then with buffers of n_tri*9 floats. */
int gbt_obj_parse(const char *path, float *verts, float *normals, uint32_t *n_tri, int32_t *has_normals);

/* ---- BVH builders --------------------------------------------------- */
/* pkg/pt/lbvh.go:13-25 DefaultLBVH: Morton codes, LSD radix sort, Karras-style
 * hierarchy emission and bottom-up refit, all on the device. */
int gbt_lbvh_build(gbt_ctx *ctx, gbt_scene *scene, gbt_bvh **out);
/* Rebuild an LBVH in place over the scene it was built from (after the scene's
 * vertices changed through gbt_scene_update_async).  Enqueue only. */
int gbt_lbvh_rebuild_async(gbt_ctx *ctx, gbt_bvh *bvh);
int gbt_scene_update_async(gbt_ctx *ctx, gbt_scene *scene, const float *d_verts);

/* pkg/pt/phr.go:47-84 PhrBuilder.BuildFromAuxilary over an LBVH from
 * gbt_lbvh_build; alpha/delta/branching as NewPHRBuilder (phr.go:30-40). */
int gbt_phr_build(gbt_ctx *ctx, gbt_bvh *aux, double alpha, double delta, int32_t branching, gbt_bvh **out);
/* pkg/pt/phr.go:154-192 PhrBuilder.BuildWithCost: the same tree plus the build
 * cost, the initial cut's size plus the size of every cut handed to Split. */
int gbt_phr_build_with_cost(gbt_ctx *ctx, gbt_bvh *aux, double alpha, double delta, int32_t branching,
                            gbt_bvh **out, int64_t *build_cost);
/* pkg/pt/optimizer.go:44-94 gridOptimizer.OptimizedPHRparams(aux, branching):
 * builds every (alphas[i], deltas[j]) (alphas outer), scores each by
 * build/max_build + omega^2 * sah/max_sah with omega = (prims/2e6)^2 *
 * (width*height/2e5), and returns the first minimum.  evals (optional,
 * 2*n_alpha*n_delta doubles) receives (SAH cost, build cost) per candidate.
 * NewDefaultGridOptimizer's grid is alphas {0.4,0.45,0.5,0.55} x deltas {6,7,8,9}. */
int gbt_phr_optimize_grid(gbt_ctx *ctx, gbt_bvh *aux, int32_t branching, const double *alphas, int32_t n_alpha,
                          const double *deltas, int32_t n_delta, int32_t frame_width, int32_t frame_height,
                          double *alpha, double *delta, double *evals);
int gbt_bvh_destroy(gbt_bvh *bvh);
/* Traversal layout of a binary tree: 4 (default after gbt_lbvh_build and a
 * branching-2 gbt_phr_build) traverses a 4-wide view collapsed from it; 2
 * traverses the binary nodes.  Results are identical; only speed differs.
 * gbt_lbvh_rebuild_async drops the 4-wide view.  No counterpart in the reference. */
int gbt_bvh_set_layout(gbt_ctx *ctx, gbt_bvh *bvh, int32_t width);
/* Camera rays of a 4-wide tree: 0 measures on the next render whether 32-ray
 * packets or one ray per lane is faster (also what a rebuild or a layout change
 * resets to), 1 packets, 2 one ray per lane.  Under GBT_OPT_PRIMARY_PACKETS 2
 * (the default) renders and batched frames follow this choice; hits are the
 * same either way.  No counterpart in the reference. */
int gbt_bvh_set_packets(gbt_ctx *ctx, gbt_bvh *bvh, int32_t choice);
int gbt_bvh_get_packets(gbt_ctx *ctx, gbt_bvh *bvh, int32_t *choice);

int gbt_bvh_cost(gbt_ctx *ctx, gbt_bvh *bvh, double *cost); /* bvh.go:46-48 BVH.Cost */
int gbt_bvh_size(gbt_ctx *ctx, gbt_bvh *bvh, int64_t *size); /* bvh.go:50-52 BVH.Size */
/* counts[0] nodes, [1] leaves, [2] primitive references, [3] root is a leaf */
int gbt_bvh_counts(gbt_ctx *ctx, gbt_bvh *bvh, int64_t counts[4]);
/* Depth-first pre-order export, children in stored order: kind (1 leaf),
 * count (children or primitives), box (lo.xyz, hi.xyz), leaf primitives. */
int gbt_bvh_export(gbt_ctx *ctx, gbt_bvh *bvh, int8_t *kind, int32_t *count, double *box, int32_t *prims);
/* LBVH only: the sorted (Morton code, primitive index) pairs (lbvh.go:216-219). */
int gbt_lbvh_sorted(gbt_ctx *ctx, gbt_bvh *bvh, uint64_t *codes, int32_t *idx);

/* The LBVH's pair sort for callers that may not allocate device memory.  No
 * counterpart in the reference.  Some callers cannot call cudaMalloc: a plugin
 * whose host application owns all device memory through its own pool, or a
 * per-frame loop that cannot take cudaMalloc's implicit synchronisation.  This
 * call sorts n 63-bit Morton codes ascending with their input positions as
 * values (stable: equal codes keep input order), exactly as the pairs
 * gbt_lbvh_build produces, and allocates nothing: the caller passes the device
 * input (d_codes_in) and outputs (d_codes_out, d_idx_out, n entries each).
 * The input must not overlap either output; it is then left unmodified (the
 * first sort pass writes the outputs while later passes still need the
 * input's order).  The scratch is a fixed static device array of about 4 MiB
 * that every GPU loading the library holds until exit, so
 * n <= GBT_NOALLOC_MAX_PAIRS, else GBT_EINVAL.  No context is needed: work is
 * queued on `stream` (a cudaStream_t, NULL for the default stream) of the
 * current device, and the call returns after that stream has finished: it
 * synchronises the stream to read the sort's error word back, so it cannot be
 * made while the stream is capturing a graph.  All calls share the one array:
 * calls whose work overlaps on the GPU race and corrupt each other's results. */
#define GBT_NOALLOC_MAX_PAIRS 262144u
int gbt_sort_morton_pairs_noalloc(void *stream, const uint64_t *d_codes_in, uint64_t *d_codes_out,
                                  uint32_t *d_idx_out, uint32_t n);

/* ---- queries -------------------------------------------------------- */
/* Closest hit per ray (bvh.go:74-77 BVH.intersected over primitive.go:56-86
 * and :172-208), host buffers. */
int gbt_trace(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_ray *rays, uint32_t n, gbt_hit *hits);
/* Same on device buffers; enqueue only. */
int gbt_trace_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_ray *d_rays, uint32_t n, gbt_hit *d_hits);

/* ---- renderer (render.go:91-129 ImageRenderer.RenderToBuffer) -------- */
/* rgb: width*height*3 floats, row y=0 is the bottom row (buffer.go:47-49
 * order); each pixel is the mean of spp samples.  A page-locked rgb
 * (gbt_host_alloc, cudaMallocHost, cudaHostRegister) is written by the
 * frame's last kernel directly; other host memory gets a copy. */
/* pkg/pt/render.go:137-197 HeatMapRenderer.RenderToBuffer: per pixel the
 * pixel-centre ray's BVH.traversalSteps (bvh.go:21-44: inner nodes whose box
 * is intersected, children popped last-first, culled by the closest hit so
 * far) coloured by DefaultTraversalCountShader (render.go:250-257) with
 * `threshold` (NewHeatMapRenderer, render.go:145-153).  Counted on the tree
 * as built (binary LBVH or PHR nodes).  rgb: width*height*3 floats, row y = 0
 * first; counts (optional): width*height int32. */
int gbt_heatmap(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, int32_t width, int32_t height, int32_t threshold,
                float *rgb, int32_t *counts);
int gbt_heatmap_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, int32_t width, int32_t height,
                      int32_t threshold, float *d_rgb, int32_t *d_counts);
int gbt_render(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *params,
               float *rgb, gbt_render_stats *stats);
/* Same into a device buffer; enqueue only; stats are read by gbt_render_last_stats. */
int gbt_render_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *params,
                     float *d_rgb);
int gbt_render_last_stats(gbt_ctx *ctx, gbt_render_stats *stats);

/* ---- render targets (pkg/pt/buffer.go) -------------------------------
 * A device-resident Buffer that RenderToBuffer adds samples to, and its
 * ToImage.  Rows are in buffer order (row y = 0 first, the bottom row of the
 * view: buffer.go:47-49).
 *   GBT_BUFFER_PIXEL  NewPxlBuffer (buffer.go:34-45): each pixel is the running
 *                     mean of every sample added to it, across calls
 *                     (Pixel.addSample, buffer.go:19-26)
 *   GBT_BUFFER_FRAME  NewFrameBuffer (buffer.go:83-89): each pixel holds the
 *                     last sample written (buffer.go:91-93), i.e. one sample of
 *                     the last call's last pass; only that pass is traced
 * The reference seeds every RenderToBuffer call from the clock
 * (render.go:117); call k on a buffer draws with params->seed + k *
 * 0x9E3779B97F4A7C15, so repeated calls with the same parameters add new
 * samples.  The first call into a PIXEL buffer gives gbt_render's image. */
typedef struct gbt_buffer gbt_buffer;
#define GBT_BUFFER_PIXEL 0
#define GBT_BUFFER_FRAME 1
int gbt_buffer_create(gbt_ctx *ctx, int32_t kind, int32_t width, int32_t height, gbt_buffer **out);
int gbt_buffer_destroy(gbt_buffer *buffer);
/* ImageRenderer.RenderToBuffer (render.go:91-129) into `buffer`; params->width
 * and height must be the buffer's.  The _async form only enqueues. */
int gbt_render_to_buffer(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *params,
                         gbt_buffer *buffer, gbt_render_stats *stats);
int gbt_render_to_buffer_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *params,
                               gbt_buffer *buffer);
/* Buffer.addSample (buffer.go:8-12) of a whole image: d_rgb (device,
 * width*height*3 floats) holds the mean of `samples` samples per pixel.  A
 * PIXEL buffer blends it into its running mean with weight samples / (samples
 * held + samples); a FRAME buffer takes it.  Enqueue only.  It is how
 * HeatMapRenderer.RenderToBuffer (render.go:155-197, one sample per pixel)
 * writes into a buffer. */
int gbt_buffer_add_async(gbt_ctx *ctx, gbt_buffer *buffer, const float *d_rgb, int32_t samples);
/* The buffer's colours (rgb: width*height*3 floats, may be NULL) and the
 * samples per pixel it holds (samples, may be NULL). */
int gbt_buffer_read(gbt_ctx *ctx, gbt_buffer *buffer, float *rgb, uint64_t *samples);
/* PixelBuffer.ToImage / FrameBuffer.ToImage (buffer.go:60-69, 104-116):
 * rgba, width*height*4 bytes, image row 0 first.  Each channel is
 * uint8(Clamp(sqrt(c), 0, 1) * 255) in float64 (Color.goColor, math.go:20-25),
 * alpha 255.  Buffer row r lands on image row height - r, so buffer row 0 is
 * dropped and image row 0 stays (0, 0, 0, 0), as in the reference. */
int gbt_buffer_to_image(gbt_ctx *ctx, gbt_buffer *buffer, uint8_t *rgba);

/* ---- batched rendering (no counterpart in the reference, which renders one
 * scene per RenderToBuffer call, render.go:91-129) ------------------------ */
typedef struct {
    gbt_bvh *bvh;              /* the scene's BVH; materials and normals come from its scene */
    gbt_camera camera;
    gbt_render_params params;  /* this render's size, spp, depth, miss shader and seed */
    float *d_rgb;              /* device image, width*height*3 floats */
} gbt_batch_item;

#define GBT_BATCH_MEGAKERNEL 0 /* one persistent launch; each lane runs whole paths from a device queue */
#define GBT_BATCH_WAVEFRONT 1  /* per bounce level one shading and one multi-tree traversal launch over all items */

typedef struct {
    int32_t block;     /* megakernel: threads per block, 64, 128 or 256 */
    int32_t fetch_min; /* megakernel: 0, a warp refills only when all its lanes are idle; 16, when fewer than 16 are busy */
    int32_t stack;     /* megakernel: 0, traversal stack in local memory; 1, its first 12 entries in shared memory */
    int32_t mode;      /* GBT_BATCH_MEGAKERNEL or GBT_BATCH_WAVEFRONT (which ignores the three fields above) */
    int32_t packets;   /* wavefront over 4-wide trees: 1 traces the camera rays of every item whose tree is
                          faster so (measured once per tree, as gbt_render_async does) as 32-ray packets */
} gbt_batch_config;

/* All items as one frame: either one persistent launch pulling (scene, path)
 * work from a device queue, each path running to completion in one lane, or
 * the wavefront over all items (two launches per bounce level).  Images equal
 * those of gbt_render_async per item up to float summation order.  cfg NULL:
 * the autotuned choice of this context, else the wavefront form with camera
 * ray packets as GBT_OPT_PRIMARY_PACKETS allows.  All BVHs
 * must share a traversal layout (gbt_bvh_set_layout).  Enqueue only; the
 * first call may grow the context's batch state and path buffers. */
int gbt_render_batch_async(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n, const gbt_batch_config *cfg);
/* The baseline: the same items as one gbt_render_async per item. */
int gbt_render_batch_plain_async(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n);
/* Times the wavefront form and every megakernel configuration on these items
 * (one warm frame, best of two timed frames), keeps the fastest for this
 * context and returns it. */
int gbt_batch_autotune(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n, gbt_batch_config *best,
                       double *best_ms);
/* A CUDA graph of one batched frame: optionally the in-place LBVH rebuild of
 * every item (for items in the 4-wide layout followed by the collapse into
 * their 4-wide view, a conditional WHILE node over its levels), then the
 * accumulator clear, the frame in form cfg and the resolve.  The graph owns
 * its descriptors, accumulators and path buffers; with rebuilds it also holds
 * the context's scratch, which cannot grow (larger builds fail with
 * GBT_EINVAL) until the graph is destroyed.  Outputs and BVHs must outlive the
 * graph, and the graph must be destroyed before its context. */
typedef struct gbt_graph gbt_graph;
int gbt_batch_graph_create(gbt_ctx *ctx, const gbt_batch_item *items, uint32_t n, const gbt_batch_config *cfg,
                           int32_t rebuild_lbvh, gbt_graph **out);
int gbt_graph_launch(gbt_ctx *ctx, gbt_graph *graph); /* enqueue one replay */
int gbt_graph_destroy(gbt_graph *graph);

/* ---- differentiable rendering (no counterpart in the reference) -------
 * Material model of these calls: every triangle t emits e_t (white, d_emission
 * n_tri floats) and scatters diffusely with albedo a_t (d_albedo n_tri*3),
 * with the camera, sampling, Diffuse scatter and MaxDepth semantics of
 * gbt_render (render.go:91-129, 209-224).  Triangle scenes only, max_depth <= 14.
 * The forward image is bitwise reproducible (each pixel sums its paths in a
 * fixed order); the backward pass re-traces the same paths from their random
 * counters (path replay) and accumulates dLoss/d(albedo, emission) given
 * dLoss/dImage.  All device buffers; enqueue only. */
int gbt_adjoint_forward_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *params,
                              const float *d_albedo, const float *d_emission, float *d_img);
int gbt_adjoint_backward_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *params,
                               const float *d_albedo, const float *d_emission, const float *d_dimg,
                               float *d_grad_albedo, float *d_grad_emission);
/* loss = sum((img - target)^2) in float64 into *d_loss; d_dimg = 2 (img - target). */
int gbt_l2_loss_async(gbt_ctx *ctx, const float *d_img, const float *d_target, uint32_t n, float *d_dimg,
                      double *d_loss);

/* ---- device memory helpers for callers without a CUDA runtime ------- */
int gbt_device_alloc(gbt_ctx *ctx, size_t bytes, void **d_ptr);
int gbt_device_free(gbt_ctx *ctx, void *d_ptr);
int gbt_host_alloc(gbt_ctx *ctx, size_t bytes, void **h_ptr); /* page-locked host memory */
int gbt_host_free(gbt_ctx *ctx, void *h_ptr);
int gbt_copy_h2d_async(gbt_ctx *ctx, void *d_dst, const void *h_src, size_t bytes);
int gbt_copy_d2h_async(gbt_ctx *ctx, void *h_dst, const void *d_src, size_t bytes);

#ifdef __cplusplus
}
#endif
#endif
