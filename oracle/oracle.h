/*
 * oracle.h -- CPU fp64 restatement of ChSchmidt99/trace pkg/pt (the path this
 * project accelerates).  TEST INFRASTRUCTURE ONLY: the pytest suite, the smoke
 * check and the CPU-baseline leg of bench.py call it as the checker.  Nothing
 * in the product (trace_gb300/) links or calls it.
 *
 * Every function names the reference file:line it restates.  Inputs follow the
 * reference's conventions: all arithmetic in float64, vertex data given as
 * float32 and widened exactly (float64(float32)).
 *
 * Primitive index space: [0, n_tri) triangles, then [n_tri, n_tri+n_sph) spheres,
 * the order in which pkg/pt/scene.go:100-114 would collect the tracables.
 *
 * Parity is pinned by the known-answer tables of pkg/pt/morton.go:23-129, the
 * cube.obj facts and hand-worked cases in tests/; the Go reference itself cannot
 * be compiled on this image (no Go toolchain).
 */
#ifndef GBT_ORACLE_H
#define GBT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MORTON_SIZE 2097152ULL                 /* morton.go:3 */
#define ORC_MAX_MORTON_CODE 9223372036854743495ULL /* morton.go:4 */
#define ORC_BUCKET_COUNT 4096                      /* lbvh.go:11 */
#define ORC_MAX_CUT_SIZE 2500                      /* phr.go:11 */
#define ORC_APPROX_THRESH 1e-7                     /* util.go:8 */
#define ORC_MAX_ARITY 16

#define ORC_OK 0
#define ORC_E_BUCKET -2   /* code >= 4096*bucketSize: the Go builder panics (lbvh.go:244-245) */
#define ORC_E_ARG -3
#define ORC_E_NOMEM -4

typedef struct orc_bvh orc_bvh;

/* ---- bounding boxes: box = {lo.x, lo.y, lo.z, hi.x, hi.y, hi.z} ---- */
void orc_prim_boxes(const float *v, int64_t n_tri, const float *sph, int64_t n_sph, double *boxes);
void orc_enclosing(const double *boxes, int64_t n, double out[6]);
double orc_surface(const double box[6]);

/* ---- Morton codes ---- */
uint64_t orc_split_by3(uint64_t a);
uint64_t orc_encode(uint64_t x, uint64_t y, uint64_t z);
void orc_morton(const double *boxes, int64_t n, const double encl[6], uint64_t *codes);

/* ---- bucket sort (stable tie order) ---- */
int orc_sort_pairs(const uint64_t *codes, int64_t n, int threads, uint64_t *sorted_codes, int32_t *sorted_idx);

/* ---- LBVH ---- */
int orc_lbvh_build(const float *v, int64_t n_tri, const float *sph, int64_t n_sph, int threads, orc_bvh **out);
void orc_bvh_free(orc_bvh *b);
void orc_bvh_counts(const orc_bvh *b, int64_t out[4]); /* n_nodes, n_leaves, n_prim_refs, root_is_leaf */
void orc_bvh_export(const orc_bvh *b, int8_t *kind, int32_t *count, double *box, int32_t *prims);
double orc_bvh_cost(orc_bvh *b);
int64_t orc_bvh_size(orc_bvh *b);
void orc_bvh_sorted(const orc_bvh *b, uint64_t *codes, int32_t *idx); /* LBVH only: sorted pairs */

/* ---- ray queries: rays[i*8] = ox oy oz tmin dx dy dz tmax (float32 widened) ---- */
void orc_trace(const orc_bvh *b, const float *rays, int64_t n, int threads,
               int32_t *hit_prim, double *hit_t, double *hit_u, double *hit_v);
int orc_prim_intersect(const orc_bvh *b, int32_t prim, const float *ray8,
                       double *t, double *u, double *v, double *det);
void orc_traversal_steps(const orc_bvh *b, const float *rays, int64_t n, int threads, int32_t *steps);

/* ---- camera / renderer ---- */
typedef struct {
    double look_from[3], look_at[3], up[3];
    double aspect, fov_deg;
} orc_camera_desc;

typedef struct {
    int32_t width, height, spp, max_depth;
    int32_t miss_mode;      /* 0 black, 1 white, 2 sky, 3 constant */
    double miss_color[3];
    uint64_t seed;
    int32_t threads;
    int64_t rays_traced; /* out: every traced segment (primary + bounces) */
} orc_render_desc;

/* materials: mat_type[m] 0 = Diffuse(albedo), 1 = Light(color); mat_color[m*3] */
/* mat_type 0 Diffuse, 1 Light, 2 Reflective, 3 Refractive; mat_param (may be
 * NULL) is Reflective.Diffusion or Refractive.Ratio per material. */
int orc_render(const orc_bvh *b, const int32_t *prim_mat, const int32_t *mat_type, const double *mat_color,
               const double *mat_param, const orc_camera_desc *cam, orc_render_desc *rd, double *rgb);
void orc_camera_rays(const orc_camera_desc *cam, int32_t width, int32_t height,
                     const double *su, const double *sv, int64_t n, double *dirs, double origin[3]);

/* ---- float64 adjoint of the differentiable render (test of the GPU adjoint) ----
 * Material model: every triangle emits emission[t] (white) and scatters
 * diffusely with albedo[3t..3t+2]; camera rays, Diffuse scatter and MaxDepth as
 * orc_render, but driven by the same counter-based random numbers as the GPU
 * (Philox-2x32-10, counter (path, level)), so both sides sample the same paths.
 * img: width*height*3; dimg: dLoss/dImage; gradients accumulate into g_*. */
int orc_adjoint(const orc_bvh *b, const orc_camera_desc *cam, const orc_render_desc *rd, const float *albedo,
                const float *emission, const float *dimg, double *img, double *g_albedo, double *g_emission);

/* HeatMapRenderer.RenderToBuffer with traversalSteps and DefaultTraversalCountShader
 * (render.go:137-197,250-257, bvh.go:21-44): rgb width*height*3, counts optional. */
void orc_heatmap(const orc_bvh *b, const orc_camera_desc *cam, int32_t width, int32_t height, int32_t threshold,
                 int threads, double *rgb, int32_t *counts);

/* ---- PHR ---- */
/* stats: initial cut size, largest cut, nodes, leaves, BuildWithCost's build cost */
/* buffer.go:60-69 / 104-116 ToImage over a buffer of width*height*3 colours (row y = 0
 * first): rgba width*height*4 bytes, image row 0 first, Color.goColor (math.go:20-25). */
void orc_to_image(const float *rgb, int32_t width, int32_t height, uint8_t *rgba);
int orc_phr_build(const orc_bvh *aux, double alpha, double delta, int bf, orc_bvh **out, int64_t stats[5]);

#ifdef __cplusplus
}
#endif
#endif
