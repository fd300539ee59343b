// Wavefront path tracer: pkg/pt/render.go:91-129 (ImageRenderer.RenderToBuffer)
// with DefaultClosestHitShader (render.go:209-224), Diffuse/Light materials
// (material.go:13-42) and the miss shaders (render.go:228-246).
//
// A wave is a range of path indices g in [0, W*H*spp); path g samples pixel
// g % (W*H).  Per bounce level the kernels are
//   k_raygen (level 0)  camera rays                          camera.go:95-97, render.go:201-205
//   traversal           closest hit of every live ray        traverse.cu
//   k_shade             miss / emission / Lambertian scatter render.go:209-224
//                       and compaction of the live paths into the next level
// and k_resolve divides the accumulated radiance by spp.  The recursion of the
// reference, L = Le + albedo * L(next), becomes a throughput T carried along
// the path: L += T * Le, T *= albedo.  A surface at depth > MaxDepth returns
// black (render.go:210-212); a ray that misses returns the miss colour.
#include <cuda_runtime.h>

#include <cmath>

#include "gbt_internal.cuh"
#include "shade.cuh"

using namespace gbt_dev;

namespace {

__global__ void __launch_bounds__(256) k_raygen(CamF cam, ShadeParams sp, uint32_t g0, uint32_t count,
                                                float4 *__restrict__ rays, float4 *__restrict__ aux, uint32_t *counts) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) counts[0] = count;
    if (i >= count) return;
    uint32_t g = path_id(sp, g0 + i);
    float3 o, d;
    primary_ray(cam, sp, g, o, d);
    rays[2 * (size_t)i] = make_float4(o.x, o.y, o.z, 0.001f);
    rays[2 * (size_t)i + 1] = make_float4(d.x, d.y, d.z, __int_as_float(0x7f800000));
    aux[2 * (size_t)i] = make_float4(1.f, 1.f, 1.f, __int_as_float((int)g));
    aux[2 * (size_t)i + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void __launch_bounds__(256) k_shade(ShadeParams sp, int level, const float4 *__restrict__ rays_in,
                                               const float4 *__restrict__ aux_in, const float4 *__restrict__ hits,
                                               const uint32_t *__restrict__ count_in, float4 *__restrict__ rays_out,
                                               float4 *__restrict__ aux_out, uint32_t *count_out,
                                               const float4 *__restrict__ recs, const uint32_t *__restrict__ prim_mat,
                                               const float4 *__restrict__ mats, const float *__restrict__ normals,
                                               float *__restrict__ acc, uint32_t cap) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t n = *count_in;
    bool alive = false;
    float4 out_r0, out_r1, out_a0, out_a1;
    if (i < n) {
        float4 a0 = aux_in[2 * (size_t)i], a1 = aux_in[2 * (size_t)i + 1];
        float3 T = f3(a0.x, a0.y, a0.z), L = f3(a1.x, a1.y, a1.z);
        uint32_t g = (uint32_t)__float_as_int(a0.w);
        float4 h = hits[i];
        float4 ro = rays_in[2 * (size_t)i], rd = rays_in[2 * (size_t)i + 1];
        float3 o = f3(ro.x, ro.y, ro.z), d = f3(rd.x, rd.y, rd.z), no, nd;
        alive = shade_step(sp, level, g, o, d, h.x, h.y, h.z, __float_as_int(h.w), recs, prim_mat, mats, normals, T, L,
                           no, nd);
        if (alive) {
            out_r0 = make_float4(no.x, no.y, no.z, 0.0001f);
            out_r1 = make_float4(nd.x, nd.y, nd.z, __int_as_float(0x7f800000));
            out_a0 = make_float4(T.x, T.y, T.z, a0.w);
            out_a1 = make_float4(L.x, L.y, L.z, 0.f);
        } else {
            deposit(acc, g % sp.npix, L);
        }
    }
    // compaction: one atomic per warp
    uint32_t ball = __ballot_sync(0xffffffffu, alive);
    if (ball == 0) return;
    uint32_t lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == (uint32_t)(__ffs(ball) - 1)) base = atomicAdd(count_out, (uint32_t)__popc(ball));
    base = __shfl_sync(0xffffffffu, base, __ffs(ball) - 1);
    if (alive) {
        uint32_t lt;
        asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
        uint32_t slot = base + __popc(ball & lt);
        if (slot < cap) {
            rays_out[2 * (size_t)slot] = out_r0;
            rays_out[2 * (size_t)slot + 1] = out_r1;
            aux_out[2 * (size_t)slot] = out_a0;
            aux_out[2 * (size_t)slot + 1] = out_a1;
        }
    }
}

__global__ void k_resolve(const float *__restrict__ acc, float *__restrict__ out, uint32_t n, float inv_spp) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = acc[i] * inv_spp;
}

__global__ void k_sum_counts(const uint32_t *counts, int levels, unsigned long long *total) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        unsigned long long s = 0;
        for (int i = 0; i < levels; i++) s += counts[i];
        *total += s;
    }
}

}  // namespace

CamF gbt_make_cam(const gbt_camera *c) {
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
    double hor[3], ver[3], llc[3];
    for (int k = 0; k < 3; k++) {
        hor[k] = u[k] * vw;
        ver[k] = v[k] * vh;
        llc[k] = c->look_from[k] - hor[k] * 0.5 - ver[k] * 0.5 - w[k];
    }
    CamF f;
    f.origin = make_float3((float)c->look_from[0], (float)c->look_from[1], (float)c->look_from[2]);
    f.llc = make_float3((float)llc[0], (float)llc[1], (float)llc[2]);
    f.hor = make_float3((float)hor[0], (float)hor[1], (float)hor[2]);
    f.ver = make_float3((float)ver[0], (float)ver[1], (float)ver[2]);
    return f;
}

ShadeParams gbt_make_shade_params(const gbt_render_params *p, uint32_t n_tri) {
    ShadeParams sp;
    sp.npix = (uint32_t)p->width * (uint32_t)p->height;
    sp.width = (uint32_t)p->width;
    sp.height = (uint32_t)p->height;
    sp.spp = (uint32_t)p->spp;
    sp.max_depth = p->max_depth;
    sp.miss_mode = p->miss_mode;
    sp.miss_color = make_float3(p->miss_color[0], p->miss_color[1], p->miss_color[2]);
    sp.seed_lo = (uint32_t)p->seed;
    sp.seed_hi = (uint32_t)(p->seed >> 32);
    sp.n_tri = n_tri;
    sp.tiles = 0;
    sp.any_last = 0;
    return sp;
}


static size_t render_layout(size_t cap, size_t npix, size_t *off) {
    size_t o = 0;
    off[0] = o; o = gbt_align(o + cap * 32);  // rays[0]
    off[1] = o; o = gbt_align(o + cap * 32);  // rays[1]
    off[2] = o; o = gbt_align(o + cap * 32);  // aux[0]
    off[3] = o; o = gbt_align(o + cap * 32);  // aux[1]
    off[4] = o; o = gbt_align(o + cap * 16);  // hits
    off[5] = o; o = gbt_align(o + 64 * sizeof(uint32_t));
    off[6] = o; o = gbt_align(o + npix * 3 * sizeof(float));
    return o;
}

#define GBT_TRY_R(x)         \
    do {                     \
        int rc_ = (x);       \
        if (rc_) return rc_; \
    } while (0)

static size_t wave_cap(size_t total) { return total < (size_t)(1u << 23) ? total : (size_t)(1u << 23); }

size_t gbt_render_state_bytes(size_t total, size_t npix) {
    size_t off[7];
    return render_layout(wave_cap(total), npix, off);
}

void gbt_render_state_bind(void *base, size_t total, size_t npix, RenderState *rs) {
    size_t off[7];
    const size_t cap = wave_cap(total);
    render_layout(cap, npix, off);
    unsigned char *b = static_cast<unsigned char *>(base);
    rs->cap = cap;
    rs->rays[0] = reinterpret_cast<float4 *>(b + off[0]);
    rs->rays[1] = reinterpret_cast<float4 *>(b + off[1]);
    rs->aux[0] = reinterpret_cast<float4 *>(b + off[2]);
    rs->aux[1] = reinterpret_cast<float4 *>(b + off[3]);
    rs->hits = reinterpret_cast<float4 *>(b + off[4]);
    rs->counts = reinterpret_cast<uint32_t *>(b + off[5]);
    rs->acc = reinterpret_cast<float *>(b + off[6]);
}

// The context's path buffers for waves of up to 2^23 of `total` paths and an
// accumulator of npix pixels (grow-only; a growth synchronises the stream).
int gbt_render_buffers(gbt_ctx *ctx, size_t total, size_t npix, RenderState *rs) {
    const size_t need = gbt_render_state_bytes(total, npix);
    if (ctx->rstate_bytes < need) {
        if (ctx->rstate) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->rstate);
        }
        ctx->rstate = nullptr;
        ctx->rstate_bytes = 0;
        if (cudaMalloc(&ctx->rstate, need) != cudaSuccess) {
            cudaGetLastError();
            return gbt_fail(ctx, GBT_ENOMEM, "render: state allocation");
        }
        ctx->rstate_bytes = need;
    }
    gbt_render_state_bind(ctx->rstate, total, npix, rs);
    return GBT_OK;
}

int gbt_render_check(gbt_ctx *ctx, const gbt_render_params *p);

// Times the packet and the one-ray-per-lane kernels on the same camera rays (both leave the same
// hits) and keeps the faster for this tree.  Synchronises the stream.
static void measure_packets(gbt_ctx *ctx, gbt_bvh *bvh, const float4 *rays, float4 *hits, uint32_t count,
                            const uint32_t *d_count) {
    cudaStream_t st = ctx->stream;
    cudaEventRecord(ctx->tune_ev[0], st);
    gbt_launch_traverse_packets(bvh, rays, hits, count, 1, ctx->d_error, st, nullptr);
    cudaEventRecord(ctx->tune_ev[1], st);
    gbt_launch_traverse(bvh, rays, hits, count, d_count, 1, ctx->d_error, st, nullptr);
    cudaEventRecord(ctx->tune_ev[2], st);
    float tp = 0.f, ts = 0.f;
    if (cudaEventSynchronize(ctx->tune_ev[2]) == cudaSuccess &&
        cudaEventElapsedTime(&tp, ctx->tune_ev[0], ctx->tune_ev[1]) == cudaSuccess &&
        cudaEventElapsedTime(&ts, ctx->tune_ev[1], ctx->tune_ev[2]) == cudaSuccess)
        bvh->packet_choice = tp < ts ? 1 : 2;
    else
        bvh->packet_choice = 2;
}

int gbt_measure_packets(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *p) {
    if (bvh->packet_choice != 0 || ctx->profiling != 0 || !(bvh->has_nodes4 || bvh->arity == 4)) return GBT_OK;
    int rc = gbt_render_check(ctx, p);
    if (rc) return rc;
    const size_t total = (size_t)p->width * p->height * (size_t)p->spp;
    RenderState rs;
    GBT_TRY_R(gbt_render_buffers(ctx, total, 0, &rs));
    const uint32_t count = (uint32_t)rs.cap;  // the first wave, as the renderer's own first frame
    if (count < (1u << 16)) return GBT_OK;
    ShadeParams sp = gbt_make_shade_params(p, bvh->scene->n_tri);
    sp.tiles = ctx->primary_tiles ? 1u : 0u;
    GBT_CUDA(ctx, cudaMemsetAsync(rs.counts, 0, 64 * sizeof(uint32_t), ctx->stream));
    k_raygen<<<(count + 255) / 256, 256, 0, ctx->stream>>>(gbt_make_cam(cam), sp, 0, count, rs.rays[0], rs.aux[0],
                                                             rs.counts);
    GBT_CUDA(ctx, cudaGetLastError());
    measure_packets(ctx, bvh, rs.rays[0], rs.hits, count, rs.counts);
    return gbt_check_device_error(ctx, "measure_packets");
}

int gbt_render_check(gbt_ctx *ctx, const gbt_render_params *p) {
    if (p->width < 2 || p->height < 2 || p->spp < 1 || p->max_depth < 0 || p->max_depth > 60)
        return gbt_fail(ctx, GBT_EINVAL, "render: width/height >= 2, spp >= 1, 0 <= max_depth <= 60");
    if ((uint64_t)p->width * p->height * (uint64_t)p->spp >= (1ull << 32))
        return gbt_fail(ctx, GBT_EINVAL, "render: width*height*spp must be < 2^32");
    return GBT_OK;
}

int gbt_render_enqueue(gbt_ctx *ctx, gbt_bvh *bvh, const gbt_camera *cam, const gbt_render_params *p, float *d_rgb) {
    int rc = gbt_render_check(ctx, p);
    if (rc) return rc;
    const size_t npix = (size_t)p->width * p->height;
    const size_t total = npix * (size_t)p->spp;
    RenderState rs;
    GBT_TRY_R(gbt_render_buffers(ctx, total, npix, &rs));
    const size_t cap = rs.cap;

    cudaStream_t st = ctx->stream;
    gbt_scene *sc = bvh->scene;
    CamF cf = gbt_make_cam(cam);
    ShadeParams sp = gbt_make_shade_params(p, sc->n_tri);
    sp.tiles = ctx->primary_tiles ? 1u : 0u;
    const int levels = p->max_depth + 2;  // surfaces at depth 0..MaxDepth+1 are traced

    GBT_CUDA(ctx, cudaMemsetAsync(rs.acc, 0, npix * 3 * sizeof(float), st));
    uint64_t launches = 0, trav = 0;
    unsigned long long *ctr = ctx->profiling >= 2 ? ctx->d_counters : nullptr;
    for (size_t g0 = 0; g0 < total; g0 += cap) {
        uint32_t count = (uint32_t)((total - g0) < cap ? (total - g0) : cap);
        GBT_CUDA(ctx, cudaMemsetAsync(rs.counts, 0, 64 * sizeof(uint32_t), st));
        uint32_t blocks = (count + 255) / 256;
        k_raygen<<<blocks, 256, 0, st>>>(cf, sp, (uint32_t)g0, count, rs.rays[0], rs.aux[0], rs.counts);
        launches++;
        for (int lv = 0; lv < levels; lv++) {
            int a = lv & 1;
            gbt_prof_begin(ctx);
            // past MaxDepth a hit shades black, so only hit-or-miss matters there
            const bool any = ctx->anyhit_last && lv == levels - 1;
            // camera rays of a tiled frame: one coherent 8x4 tile per warp, traced as a packet when
            // that is faster for this tree and view (both kernels give the same hits)
            const bool four = bvh->has_nodes4 || bvh->arity == 4;
            bool packets = false, done = false;
            if (lv == 0 && ctx->primary_tiles && four && ctx->primary_packets) {
                if (ctx->primary_packets == 2 && bvh->packet_choice == 0 && ctx->profiling == 0 && count >= (1u << 16)) {
                    // first render on this tree: time both kernels on this wave's camera rays
                    measure_packets(ctx, bvh, rs.rays[a], rs.hits, count, rs.counts + lv);
                    done = true;
                    launches += 1;
                }
                packets = ctx->primary_packets == 1 || bvh->packet_choice == 1;
            }
            if (!done) {
                if (packets) gbt_launch_traverse_packets(bvh, rs.rays[a], rs.hits, count, 1, ctx->d_error, st, ctr);
                else gbt_launch_traverse(bvh, rs.rays[a], rs.hits, count, rs.counts + lv, 1, ctx->d_error, st, ctr, any);
            }
            gbt_prof_end(ctx);
            k_shade<<<blocks, 256, 0, st>>>(sp, lv, rs.rays[a], rs.aux[a], rs.hits, rs.counts + lv, rs.rays[a ^ 1],
                                            rs.aux[a ^ 1], rs.counts + lv + 1, bvh->d_prims, sc->d_prim_mat, sc->d_mats,
                                            sc->d_normals, rs.acc, (uint32_t)cap);
            launches += 2;
            trav++;
        }
        k_sum_counts<<<1, 32, 0, st>>>(rs.counts, levels, ctx->d_counters + 2);
        launches++;
    }
    k_resolve<<<(uint32_t)((npix * 3 + 255) / 256), 256, 0, st>>>(rs.acc, d_rgb, (uint32_t)(npix * 3), 1.0f / p->spp);
    launches++;
    GBT_CUDA(ctx, cudaGetLastError());
    ctx->last_stats.paths += total;
    ctx->last_stats.kernel_launches += launches;
    ctx->last_stats.traverse_launches += trav;
    return GBT_OK;
}
