// Closest-hit ray traversal (pkg/pt/bvh.go:74-77, 179-199 BVH.intersected).
//
// One thread per ray walks the tree with a local stack, nearer child first.
// A 64-byte binary node is four float4 loaded with 128-bit loads:
//   n0 = (L.lo.x, L.hi.x, L.lo.y, L.hi.y)   n1 = same for R
//   n2 = (L.lo.z, L.hi.z, R.lo.z, R.hi.z)   n3 = (L.ref, L.cnt, R.ref, R.cnt)
// A child with cnt > 0 is a leaf of cnt primitive records starting at ref;
// cnt == 0 is the inner node ref; cnt < 0 is an empty slot.
// A 128-byte 4-wide node (PHR with branching factor 3 or 4) is eight float4:
//   m0..m5 = lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4], hi.z[4]
//   m6 = ref[4], m7 = cnt[4]
// Primitive records are three float4 (r0 = v0|id, r1 = v1|kind, r2 = v2);
// a sphere record holds (centre|id, radius|kind).
//
// The primitive tests are pkg/pt/primitive.go:172-208 (Moeller-Trumbore with
// the absolute |det| <= 1e-7 rejection, u in [0,1], v >= 0, u+v <= 1,
// tmin <= t <= tmax) and :56-86 (sphere, exclusive t bounds), in float32.
#include <cuda_runtime.h>

#include "gbt_internal.cuh"
#include "traverse.cuh"

namespace {

template <bool COUNT>
__device__ __forceinline__ void flush_work(const gbt_dev::Work &w, unsigned long long *counters) {
    if (!COUNT) return;
    // every lane of the warp reaches this point (no early return in the kernels)
    __syncwarp();
    unsigned long long a = w.nodes, b = w.prims;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counters, a);
        atomicAdd(counters + 1, b);
    }
}

template <bool COUNT>
__global__ void __launch_bounds__(128) k_trace2(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes,
                                                const float4 *__restrict__ recs, const float4 *__restrict__ rays,
                                                float4 *__restrict__ hits, uint32_t n, const uint32_t *__restrict__ d_count,
                                                int out_mode, unsigned int *err, unsigned long long *counters) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cnt = d_count ? *d_count : n;
    gbt_dev::Work w;
    if (i < cnt) {
        gbt_dev::Ray ray = gbt_dev::load_ray(rays, i);
        gbt_dev::Hit h = gbt_dev::closest_hit2<64, COUNT>(*hdr, nodes, recs, ray, err, &w);
        gbt_dev::store_hit(hits, i, h, recs, out_mode);
    }
    flush_work<COUNT>(w, counters);
}

template <bool COUNT>
__global__ void __launch_bounds__(128) k_trace4(const BvhHeader *__restrict__ hdr, const float4 *__restrict__ nodes,
                                                const float4 *__restrict__ recs, const float4 *__restrict__ rays,
                                                float4 *__restrict__ hits, uint32_t n, const uint32_t *__restrict__ d_count,
                                                int out_mode, unsigned int *err, unsigned long long *counters) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cnt = d_count ? *d_count : n;
    gbt_dev::Work w;
    if (i < cnt) {
        gbt_dev::Ray ray = gbt_dev::load_ray(rays, i);
        gbt_dev::Hit h = gbt_dev::closest_hit4<96, COUNT>(*hdr, nodes, recs, ray, err, &w);
        gbt_dev::store_hit(hits, i, h, recs, out_mode);
    }
    flush_work<COUNT>(w, counters);
}

}  // namespace

void gbt_launch_traverse(const gbt_bvh *bvh, const float4 *rays, float4 *hits, uint32_t n, const uint32_t *d_count,
                         int out_mode, unsigned int *d_error, cudaStream_t s, unsigned long long *counters) {
    if (n == 0) return;
    uint32_t blocks = (n + 127) / 128;
    if (bvh->arity == 4) {
        if (counters)
            k_trace4<true><<<blocks, 128, 0, s>>>(bvh->d_hdr, bvh->d_nodes, bvh->d_prims, rays, hits, n, d_count, out_mode, d_error, counters);
        else
            k_trace4<false><<<blocks, 128, 0, s>>>(bvh->d_hdr, bvh->d_nodes, bvh->d_prims, rays, hits, n, d_count, out_mode, d_error, nullptr);
    } else {
        if (counters)
            k_trace2<true><<<blocks, 128, 0, s>>>(bvh->d_hdr, bvh->d_nodes, bvh->d_prims, rays, hits, n, d_count, out_mode, d_error, counters);
        else
            k_trace2<false><<<blocks, 128, 0, s>>>(bvh->d_hdr, bvh->d_nodes, bvh->d_prims, rays, hits, n, d_count, out_mode, d_error, nullptr);
    }
}

int gbt_trace_enqueue(gbt_ctx *ctx, const gbt_bvh *bvh, const gbt_ray *d_rays, uint32_t n, gbt_hit *d_hits) {
    gbt_prof_begin(ctx);
    gbt_launch_traverse(bvh, reinterpret_cast<const float4 *>(d_rays), reinterpret_cast<float4 *>(d_hits), n, nullptr,
                        0, ctx->d_error, ctx->stream, ctx->profiling >= 2 ? ctx->d_counters : nullptr);
    gbt_prof_end(ctx);
    GBT_CUDA(ctx, cudaGetLastError());
    return GBT_OK;
}
