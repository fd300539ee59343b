// Heat-map renderer: pkg/pt/render.go:137-197 (HeatMapRenderer.RenderToBuffer)
// with BVH.traversalSteps (bvh.go:21-44) and DefaultTraversalCountShader
// (render.go:250-257).
//
// One thread per pixel casts the pixel-centre ray (u = x/(w-1), v = y/(h-1),
// camera.go:95-97; the direction is formed in float64 like the reference's,
// then traced in float32) and counts the inner nodes whose box it intersects,
// in the reference's order: the children of an intersected inner node are
// pushed in order and the last one is popped first; every popped entry's box
// is tested against the closest hit found so far; leaves test their
// primitives (Moeller-Trumbore, closest hit).  The count is a property of the
// tree as built (binary LBVH or PHR nodes), not of the 4-wide traversal view.
#include <cuda_runtime.h>

#include <cmath>

#include "gbt_internal.cuh"
#include "traverse.cuh"

using namespace gbt_dev;

namespace {

constexpr int HM_STACK = 256;  // entries: depth x (arity - 1) + 1 for trees up to depth 85 at arity 4

struct HeatCam {
    double origin[3], llc[3], hor[3], ver[3];
};

// One child slot of a stored node: its box and (ref, cnt).
__device__ __forceinline__ void child_slot(const float4 *__restrict__ nodes, int arity, int32_t p, int s, float lo[3],
                                           float hi[3], int32_t &ref, int32_t &cnt) {
    if (arity == 2) {
        const float4 *nd = nodes + 4 * (size_t)p;
        const float4 xy = __ldg(nd + s), z = __ldg(nd + 2);
        const int4 rc = __ldg(reinterpret_cast<const int4 *>(nd + 3));
        lo[0] = xy.x; hi[0] = xy.y; lo[1] = xy.z; hi[1] = xy.w;
        lo[2] = s ? z.z : z.x;
        hi[2] = s ? z.w : z.y;
        ref = s ? rc.z : rc.x;
        cnt = s ? rc.w : rc.y;
    } else {
        const float *f = reinterpret_cast<const float *>(nodes + 8 * (size_t)p);
        lo[0] = __ldg(f + s); hi[0] = __ldg(f + 4 + s);
        lo[1] = __ldg(f + 8 + s); hi[1] = __ldg(f + 12 + s);
        lo[2] = __ldg(f + 16 + s); hi[2] = __ldg(f + 20 + s);
        ref = __float_as_int(__ldg(f + 24 + s));
        cnt = __float_as_int(__ldg(f + 28 + s));
    }
}

__global__ void __launch_bounds__(128) k_heatmap(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes,
                                                 int arity, const float4 *__restrict__ recs, HeatCam cam, int width,
                                                 int height, int threshold, float *__restrict__ rgb,
                                                 int32_t *__restrict__ counts, unsigned int *err) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= (uint32_t)width * (uint32_t)height) return;
    const int x = (int)(pix % (uint32_t)width), y = (int)(pix / (uint32_t)width);
    const double u = (double)x / (double)(width - 1), v = (double)y / (double)(height - 1);
    double d[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
        d[k] = __dsub_rn(__dadd_rn(__dadd_rn(cam.llc[k], __dmul_rn(cam.hor[k], u)), __dmul_rn(cam.ver[k], v)),
                         cam.origin[k]);
    Ray r;
    r.o = make_float3((float)cam.origin[0], (float)cam.origin[1], (float)cam.origin[2]);
    r.d = make_float3((float)d[0], (float)d[1], (float)d[2]);
    r.tmin = 0.001f;
    r.tmax = __int_as_float(0x7f800000);
    finish_ray(r);
    Hit h;
    h.t = r.tmax;
    h.u = h.v = 0.f;
    h.rec = -1;

    int count = 0;
    float te;
    // the root entry
    if (slab(hdr->root_lo[0], hdr->root_lo[1], hdr->root_lo[2], hdr->root_hi[0], hdr->root_hi[1], hdr->root_hi[2], r,
             h.t, te)) {
        if (hdr->root_cnt > 0) {
            leaf(recs, hdr->root_ref, hdr->root_cnt, r, h);
        } else {
            int32_t st[HM_STACK];  // (parent << 2) | slot
            int sp = 0;
            count = 1;
            for (int s = 0; s < arity; s++) st[sp++] = (hdr->root_ref << 2) | s;
            while (sp > 0) {
                const int32_t e = st[--sp];
                float lo[3], hi[3];
                int32_t ref, cnt;
                child_slot(nodes, arity, e >> 2, e & 3, lo, hi, ref, cnt);
                if (cnt < 0) continue;  // empty slot of a node with fewer children
                if (!slab(lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], r, h.t, te)) continue;
                if (cnt > 0) {
                    leaf(recs, ref, cnt, r, h);
                } else {
                    count++;
                    if (sp + arity > HM_STACK) {
                        atomicOr(err, GBT_DEVERR_STACK);
                        continue;
                    }
                    for (int s = 0; s < arity; s++) st[sp++] = (ref << 2) | s;
                }
            }
        }
    }
    // DefaultTraversalCountShader
    float c0, c1, c2;
    if (count > threshold) {
        c0 = (float)(__dmul_rn(__ddiv_rn((double)count, (double)threshold), 2.0));
        c1 = 0.f;
        c2 = 0.f;
    } else {
        const double f = __ddiv_rn((double)count, __dmul_rn((double)threshold, 1.25));
        c0 = 0.f;
        c1 = (float)f;
        c2 = (float)__dsub_rn(1.0, f);
    }
    rgb[3 * (size_t)pix] = c0;
    rgb[3 * (size_t)pix + 1] = c1;
    rgb[3 * (size_t)pix + 2] = c2;
    if (counts) counts[pix] = count;
}

HeatCam make_heat_cam(const gbt_camera *c) {
    auto sub = [](const double *a, const double *b, double *o) { for (int k = 0; k < 3; k++) o[k] = a[k] - b[k]; };
    auto unit = [](double *v) { double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); for (int k = 0; k < 3; k++) v[k] /= l; };
    auto cross = [](const double *a, const double *b, double *o) {
        o[0] = a[1] * b[2] - a[2] * b[1];
        o[1] = a[2] * b[0] - a[0] * b[2];
        o[2] = a[0] * b[1] - a[1] * b[0];
    };
    double vh = 2.0 * std::tan((c->fov_deg * (M_PI / 180)) / 2), vw = c->aspect * vh;
    double w[3], u[3], v[3];
    sub(c->look_from, c->look_at, w);
    unit(w);
    cross(c->up, w, u);
    unit(u);
    cross(w, u, v);
    HeatCam k;
    for (int i = 0; i < 3; i++) {
        k.origin[i] = c->look_from[i];
        k.hor[i] = u[i] * vw;
        k.ver[i] = v[i] * vh;
        k.llc[i] = c->look_from[i] - k.hor[i] * 0.5 - k.ver[i] * 0.5 - w[i];
    }
    return k;
}

}  // namespace

extern "C" int gbt_heatmap_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, int32_t width, int32_t height,
                                 int32_t threshold, float *d_rgb, int32_t *d_counts) {
    if (!ctx || !bvh || !cam || !d_rgb) return GBT_EINVAL;
    if (width < 2 || height < 2) return gbt_fail(ctx, GBT_EINVAL, "heatmap: width and height must be >= 2");
    if (threshold < 1) return gbt_fail(ctx, GBT_EINVAL, "heatmap: threshold must be >= 1");
    if ((uint64_t)width * (uint64_t)height >= (1ull << 31)) return gbt_fail(ctx, GBT_EINVAL, "heatmap: image too large");
    if ((uint64_t)bvh->n_prim > (1u << 29)) return gbt_fail(ctx, GBT_EINVAL, "heatmap: tree too large");
    const uint32_t n = (uint32_t)width * (uint32_t)height;
    k_heatmap<<<(n + 127) / 128, 128, 0, ctx->stream>>>(bvh->d_hdr, bvh->d_nodes, bvh->arity, bvh->d_prims,
                                                        make_heat_cam(cam), width, height, threshold, d_rgb, d_counts,
                                                        ctx->d_error);
    GBT_CUDA(ctx, cudaGetLastError());
    return GBT_OK;
}

extern "C" int gbt_heatmap(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, int32_t width, int32_t height,
                           int32_t threshold, float *rgb, int32_t *counts) {
    if (!ctx || !bvh || !cam || !rgb) return GBT_EINVAL;
    if (width < 2 || height < 2) return gbt_fail(ctx, GBT_EINVAL, "heatmap: width and height must be >= 2");
    const size_t n = (size_t)width * (size_t)height;
    float *d_rgb = nullptr;
    int32_t *d_counts = nullptr;
    if (cudaMalloc(&d_rgb, n * 3 * sizeof(float)) != cudaSuccess ||
        (counts && cudaMalloc(&d_counts, n * sizeof(int32_t)) != cudaSuccess)) {
        cudaGetLastError();
        cudaFree(d_rgb);
        return gbt_fail(ctx, GBT_ENOMEM, "heatmap: output allocation");
    }
    int rc = gbt_heatmap_async(ctx, bvh, cam, width, height, threshold, d_rgb, d_counts);
    if (!rc && cudaMemcpyAsync(rgb, d_rgb, n * 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
        rc = gbt_fail(ctx, GBT_ECUDA, "heatmap: copy");
    if (!rc && counts &&
        cudaMemcpyAsync(counts, d_counts, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess)
        rc = gbt_fail(ctx, GBT_ECUDA, "heatmap: copy");
    if (!rc) rc = gbt_check_device_error(ctx, "heatmap");
    cudaStreamSynchronize(ctx->stream);
    cudaFree(d_rgb);
    cudaFree(d_counts);
    return rc;
}
