// Differentiable rendering by path replay: gradients of an L2 image loss with
// respect to per-triangle albedo (3 floats) and emission (1 float, white).
//
// Material model (project-defined; the reference's materials either emit or
// scatter, material.go:13-42): every triangle t emits e_t and scatters
// diffusely with albedo a_t.  A path with surface vertices 0..K-1 carries
//   L = sum_k P_k * e_k  (+ P_K * miss),  P_k = prod_{j<k} a_j,
// traced with the renderer's camera rays, Diffuse scatter directions and
// MaxDepth cut-off (shade.cuh).  Sampling does not depend on a or e, so with
// fixed Philox counters the image is a polynomial in the parameters and
// central finite differences check the adjoint exactly.
//
// Forward: one thread per pixel sums its spp paths in a fixed order (no
// atomics), so the image is bitwise reproducible.
// Backward (path replay): each thread re-traces the same paths from their
// counters instead of storing them, keeps the vertices of one path in
// registers and local memory, and with S_i = sum_{k>i} (prod_{i<j<k} a_j) e_k
// (+ miss) accumulates
//   dL/da_i = P_i * S_i,  dL/de_i = sum over channels of P_i
// weighted by dLoss/dI of the pixel / spp.  Lanes of a warp that touch the
// same triangle at the same vertex index are summed before one atomicAdd.
#include <cuda_runtime.h>

#include "gbt_internal.cuh"
#include "shade.cuh"

#define GBT_TRY_ADJ(x)       \
    do {                     \
        int rc_ = (x);       \
        if (rc_) return rc_; \
    } while (0)

using namespace gbt_dev;

namespace {

constexpr int MAXV = 16;  // path vertices kept for replay (max_depth <= 14)

constexpr int SH = 12;  // traversal stack entries per thread kept in shared memory (4-wide trees)
using Stack4 = SharedTopStack<96, SH>;

// any: only hit or miss is needed (the query past MaxDepth, render.go:210-212);
// on 4-wide trees it stops at the first hit found, with the same hit-or-miss answer.
template <int W>
__device__ __forceinline__ Hit closest(const BvhHeader &hdr, const float4 *nodes, const float4 *recs, float3 o,
                                       float3 d, float tmin, bool any, unsigned int *err, Stack4 &st) {
    Ray r;
    r.o = o;
    r.d = d;
    r.tmin = tmin;
    r.tmax = __int_as_float(0x7f800000);
    finish_ray(r);
    if constexpr (W == 2) return closest_hit2<64>(hdr, nodes, recs, r, err);
    else if (any) return closest_hit4_with<false, Stack4, true>(hdr, nodes, recs, r, err, nullptr, st);
    else return closest_hit4_with<false>(hdr, nodes, recs, r, err, nullptr, st);
}

// the per-thread shared-memory bottom of the traversal stack (blocks of 128 threads)
#define ADJ_STACK(st)                          \
    __shared__ int2 s_se_[SH * 128];           \
    __shared__ float s_st_[SH * 128];          \
    Stack4 st;                                 \
    st.se = s_se_ + threadIdx.x;               \
    st.st = s_st_ + threadIdx.x;               \
    st.stride = 128

// The pixel of thread slot i: the 32 slots of a warp take an 8x4 pixel tile
// (path_id's map over one frame), so that a warp's camera rays are coherent;
// slots past the image stay past it.
__device__ __forceinline__ uint32_t adj_pixel(const ShadeParams &sp, uint32_t i) {
    if (i >= sp.npix) return i;
    ShadeParams t = sp;
    t.tiles = 1u;
    return path_id(t, i);
}

struct Vertex {
    int tri;
    float3 P;  // throughput arriving at the vertex
    float3 a;  // albedo there
};

// Trace path g: fills its vertices, returns the radiance L and the miss colour
// M seen after the last vertex (zero when the path ended otherwise).
template <int W>
__device__ __forceinline__ int trace_path(const BvhHeader &hdr, const float4 *nodes, const float4 *recs,
                                          const float *normals, const CamF &cam, const ShadeParams &sp,
                                          const float *__restrict__ albedo, const float *__restrict__ emission,
                                          uint32_t g, Vertex *vx, float3 &L, float3 &miss, unsigned int *err,
                                          Stack4 &st) {
    float3 o, d;
    primary_ray(cam, sp, g, o, d);
    float tmin = 0.001f;
    float3 T = f3(1.f, 1.f, 1.f);
    L = f3(0.f, 0.f, 0.f);
    miss = f3(0.f, 0.f, 0.f);
    int nv = 0;
    for (int level = 0;; level++) {
        Hit h = closest<W>(hdr, nodes, recs, o, d, tmin, level > sp.max_depth, err, st);
        if (h.rec < 0) {
            miss = miss_colour(sp, d);
            L = add3(L, emul3(T, miss));
            break;
        }
        if (level > sp.max_depth || nv >= MAXV) break;
        const uint32_t id = (uint32_t)__float_as_int(__ldg(recs + 3 * (size_t)h.rec).w);
        const float e = __ldg(emission + id);
        const float3 a = f3(__ldg(albedo + 3 * id), __ldg(albedo + 3 * id + 1), __ldg(albedo + 3 * id + 2));
        vx[nv].tri = (int)id;
        vx[nv].P = T;
        vx[nv].a = a;
        nv++;
        L = add3(L, mul3(T, e));
        float3 p, sd;
        diffuse_scatter(recs, normals, h.rec, o, d, h.t, h.u, h.v, g, level, sp, p, sd);
        T = emul3(T, a);
        o = p;
        d = sd;
        tmin = 0.0001f;
    }
    return nv;
}

template <int W>
__global__ void __launch_bounds__(128, 8) k_adj_forward(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes,
                                                     const float4 *__restrict__ recs, const float *__restrict__ normals,
                                                     CamF cam, ShadeParams sp, const float *__restrict__ albedo,
                                                     const float *__restrict__ emission, double *__restrict__ part,
                                                     unsigned int *err, unsigned long long *rays) {
    const uint32_t pix = adj_pixel(sp, blockIdx.x * blockDim.x + threadIdx.x);
    const uint32_t c = blockIdx.y, nc = gridDim.y;  // this thread's chunk of the pixel's samples
    const uint32_t s_lo = (uint32_t)((uint64_t)sp.spp * c / nc), s_hi = (uint32_t)((uint64_t)sp.spp * (c + 1) / nc);
    const BvhHeader H = *hdr;
    unsigned long long nr = 0;
    ADJ_STACK(st);
    if (pix < sp.npix) {
        double s0 = 0, s1 = 0, s2 = 0;
        Vertex vx[MAXV];
        for (uint32_t s = s_lo; s < s_hi; s++) {
            float3 L, m;
            int nv = trace_path<W>(H, nodes, recs, normals, cam, sp, albedo, emission, s * sp.npix + pix, vx, L, m, err, st);
            nr += (unsigned long long)nv + 1;
            s0 += L.x;
            s1 += L.y;
            s2 += L.z;
        }
        double *o = part + 3 * ((size_t)c * sp.npix + pix);
        o[0] = s0;
        o[1] = s1;
        o[2] = s2;
    }
    __syncwarp();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nr += __shfl_xor_sync(0xffffffffu, nr, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(rays, nr);
}

// The pixel's chunk sums in chunk order, divided by spp (a fixed order: the
// image is bitwise reproducible).
__global__ void k_adj_combine(const double *__restrict__ part, uint32_t npix, uint32_t nc, uint32_t spp,
                              float *__restrict__ img) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 3 * npix) return;
    double acc = 0.0;
    for (uint32_t c = 0; c < nc; c++) acc += part[(size_t)c * 3 * npix + i];
    img[i] = (float)(acc / spp);
}

// Sum four floats over the lanes of `peers` (own value first, then the other
// peers in lane order); valid in every lane of the group.  The loop runs the
// largest group's size - 1 times: not at all when every lane's triangle differs.
__device__ __forceinline__ float4 group_sum(uint32_t peers, float4 v) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t m = peers & ~(1u << lane);
    float4 s = v;
    const int iters = (int)__reduce_max_sync(0xffffffffu, (uint32_t)__popc(peers)) - 1;
    for (int it = 0; it < iters; it++) {
        const int src = m ? __ffs(m) - 1 : (int)lane;
        float4 x;
        x.x = __shfl_sync(0xffffffffu, v.x, src);
        x.y = __shfl_sync(0xffffffffu, v.y, src);
        x.z = __shfl_sync(0xffffffffu, v.z, src);
        x.w = __shfl_sync(0xffffffffu, v.w, src);
        if (m) {
            s.x += x.x;
            s.y += x.y;
            s.z += x.z;
            s.w += x.w;
            m &= m - 1;
        }
    }
    return s;
}

template <int W>
__global__ void __launch_bounds__(128, 8) k_adj_backward(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes,
                                                      const float4 *__restrict__ recs, const float *__restrict__ normals,
                                                      CamF cam, ShadeParams sp, const float *__restrict__ albedo,
                                                      const float *__restrict__ emission, const float *__restrict__ dimg,
                                                      float *__restrict__ g_albedo, float *__restrict__ g_emission,
                                                      unsigned int *err) {
    const uint32_t pix = adj_pixel(sp, blockIdx.x * blockDim.x + threadIdx.x);
    const bool live = pix < sp.npix;
    const BvhHeader H = *hdr;
    ADJ_STACK(st);
    const float inv = 1.f / (float)sp.spp;
    float3 delta = f3(0.f, 0.f, 0.f);
    if (live) delta = f3(dimg[3 * (size_t)pix] * inv, dimg[3 * (size_t)pix + 1] * inv, dimg[3 * (size_t)pix + 2] * inv);
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t c = blockIdx.y, nc = gridDim.y;  // this thread's chunk of the pixel's samples
    const uint32_t s_lo = (uint32_t)((uint64_t)sp.spp * c / nc), s_hi = (uint32_t)((uint64_t)sp.spp * (c + 1) / nc);
    Vertex vx[MAXV];
    float3 S[MAXV];
    for (uint32_t s = s_lo; s < s_hi; s++) {  // warp-uniform loop
        int nv = 0;
        if (live) {
            float3 L, m;
            nv = trace_path<W>(H, nodes, recs, normals, cam, sp, albedo, emission, s * sp.npix + pix, vx, L, m, err, st);
            // S_i: radiance beyond vertex i per unit throughput leaving it; S_{K-1} = M
            float3 acc = m;
            for (int i = nv - 1; i >= 0; i--) {
                S[i] = acc;
                const float e = __ldg(emission + vx[i].tri);
                acc = add3(f3(e, e, e), emul3(vx[i].a, acc));  // S_{i-1} = e_i + a_i * S_i
            }
        }
        // accumulate vertex by vertex; lanes that share a triangle sum first
        for (int i = 0; __any_sync(0xffffffffu, i < nv); i++) {
            const bool has = i < nv;
            const int key = has ? vx[i].tri : -1;
            float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
            if (has) {
                const float3 P = vx[i].P, Si = S[i];
                c.x = delta.x * P.x * Si.x;
                c.y = delta.y * P.y * Si.y;
                c.z = delta.z * P.z * Si.z;
                c.w = delta.x * P.x + delta.y * P.y + delta.z * P.z;
            }
            const uint32_t peers = __match_any_sync(0xffffffffu, key);
            const float4 sum = group_sum(peers, c);
            if (has && lane == (uint32_t)(__ffs(peers) - 1)) {
                atomicAdd(g_albedo + 3 * (size_t)key, sum.x);
                atomicAdd(g_albedo + 3 * (size_t)key + 1, sum.y);
                atomicAdd(g_albedo + 3 * (size_t)key + 2, sum.z);
                atomicAdd(g_emission + key, sum.w);
            }
        }
    }
}

// loss = sum (img - target)^2 in float64, dimg = 2 (img - target)
__global__ void k_l2(const float *__restrict__ img, const float *__restrict__ target, uint32_t n, float *__restrict__ dimg,
                     double *loss) {
    __shared__ double s[8];
    double acc = 0.0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float r = img[i] - target[i];
        dimg[i] = 2.f * r;
        acc += (double)r * (double)r;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
        atomicAdd(loss, t);
    }
}

int check(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_render_params *p) {
    if (bvh->scene->n_sph) return gbt_fail(ctx, GBT_EUNSUPPORTED, "adjoint: triangle scenes only");
    if (p->width < 2 || p->height < 2 || p->spp < 1 || p->max_depth < 0 || p->max_depth > MAXV - 2)
        return gbt_fail(ctx, GBT_EINVAL, "adjoint: width/height >= 2, spp >= 1, 0 <= max_depth <= 14");
    if ((uint64_t)p->width * p->height * (uint64_t)p->spp >= (1ull << 32))
        return gbt_fail(ctx, GBT_EINVAL, "adjoint: width*height*spp must be < 2^32");
    return GBT_OK;
}

// Sample chunks per pixel: enough 128-thread blocks for about eight waves of
// the resident blocks, so the last wave's idle SMs cost little.
template <class K>
uint32_t sample_chunks(gbt_ctx *ctx, K kernel, uint32_t npix, uint32_t spp) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, 0);
    if (per_sm <= 0) per_sm = 1;
    const uint64_t want = 8ull * (uint64_t)ctx->num_sms * per_sm, have = (npix + 127) / 128;
    uint64_t c = (want + have - 1) / have;
    if (c > spp) c = spp;
    if (c > 64) c = 64;
    return (uint32_t)(c < 1 ? 1 : c);
}

}  // namespace

extern "C" int gbt_adjoint_forward_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *p,
                                         const float *d_albedo, const float *d_emission, float *d_img) {
    if (!ctx || !bvh || !cam || !p || !d_albedo || !d_emission || !d_img) return GBT_EINVAL;
    int rc = check(ctx, bvh, p);
    if (rc) return rc;
    CamF cf = gbt_make_cam(cam);
    ShadeParams sp = gbt_make_shade_params(p, bvh->scene->n_tri);
    const uint32_t blocks = (sp.npix + 127) / 128;
    const bool four = bvh->has_nodes4 || bvh->arity == 4;
    const BvhHeader *hd = bvh->has_nodes4 ? bvh->d_hdr4 : bvh->d_hdr;
    const float4 *nd = bvh->has_nodes4 ? bvh->d_nodes4 : bvh->d_nodes;
    const uint32_t nc = four ? sample_chunks(ctx, k_adj_forward<4>, sp.npix, sp.spp)
                             : sample_chunks(ctx, k_adj_forward<2>, sp.npix, sp.spp);
    void *scr = nullptr;
    GBT_TRY_ADJ(gbt_scratch(ctx, (size_t)nc * sp.npix * 3 * sizeof(double), &scr));
    double *part = static_cast<double *>(scr);
    const dim3 grid(blocks, nc);
    if (four)
        k_adj_forward<4><<<grid, 128, 0, ctx->stream>>>(hd, nd, bvh->d_prims, bvh->scene->d_normals, cf, sp, d_albedo,
                                                        d_emission, part, ctx->d_error, ctx->d_counters + 2);
    else
        k_adj_forward<2><<<grid, 128, 0, ctx->stream>>>(hd, nd, bvh->d_prims, bvh->scene->d_normals, cf, sp, d_albedo,
                                                        d_emission, part, ctx->d_error, ctx->d_counters + 2);
    k_adj_combine<<<(3 * sp.npix + 255) / 256, 256, 0, ctx->stream>>>(part, sp.npix, nc, sp.spp, d_img);
    GBT_CUDA(ctx, cudaGetLastError());
    ctx->last_stats.kernel_launches += 2;
    ctx->last_stats.paths += (uint64_t)sp.npix * sp.spp;
    return GBT_OK;
}

extern "C" int gbt_adjoint_backward_async(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam,
                                          const gbt_render_params *p, const float *d_albedo, const float *d_emission,
                                          const float *d_dimg, float *d_galbedo, float *d_gemission) {
    if (!ctx || !bvh || !cam || !p || !d_albedo || !d_emission || !d_dimg || !d_galbedo || !d_gemission)
        return GBT_EINVAL;
    int rc = check(ctx, bvh, p);
    if (rc) return rc;
    CamF cf = gbt_make_cam(cam);
    ShadeParams sp = gbt_make_shade_params(p, bvh->scene->n_tri);
    const uint32_t n_tri = bvh->scene->n_tri;
    GBT_CUDA(ctx, cudaMemsetAsync(d_galbedo, 0, (size_t)n_tri * 3 * sizeof(float), ctx->stream));
    GBT_CUDA(ctx, cudaMemsetAsync(d_gemission, 0, (size_t)n_tri * sizeof(float), ctx->stream));
    const uint32_t blocks = (sp.npix + 127) / 128;
    const bool four = bvh->has_nodes4 || bvh->arity == 4;
    const BvhHeader *hd = bvh->has_nodes4 ? bvh->d_hdr4 : bvh->d_hdr;
    const float4 *nd = bvh->has_nodes4 ? bvh->d_nodes4 : bvh->d_nodes;
    const uint32_t nc = four ? sample_chunks(ctx, k_adj_backward<4>, sp.npix, sp.spp)
                             : sample_chunks(ctx, k_adj_backward<2>, sp.npix, sp.spp);
    const dim3 grid(blocks, nc);
    if (four)
        k_adj_backward<4><<<grid, 128, 0, ctx->stream>>>(hd, nd, bvh->d_prims, bvh->scene->d_normals, cf, sp, d_albedo,
                                                         d_emission, d_dimg, d_galbedo, d_gemission, ctx->d_error);
    else
        k_adj_backward<2><<<grid, 128, 0, ctx->stream>>>(hd, nd, bvh->d_prims, bvh->scene->d_normals, cf, sp, d_albedo,
                                                         d_emission, d_dimg, d_galbedo, d_gemission, ctx->d_error);
    GBT_CUDA(ctx, cudaGetLastError());
    ctx->last_stats.kernel_launches += 1;
    return GBT_OK;
}

extern "C" int gbt_l2_loss_async(gbt_ctx *ctx, const float *d_img, const float *d_target, uint32_t n, float *d_dimg,
                                 double *d_loss) {
    if (!ctx || !d_img || !d_target || !d_dimg || !d_loss) return GBT_EINVAL;
    GBT_CUDA(ctx, cudaMemsetAsync(d_loss, 0, sizeof(double), ctx->stream));
    k_l2<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(d_img, d_target, n, d_dimg, d_loss);
    GBT_CUDA(ctx, cudaGetLastError());
    return GBT_OK;
}
