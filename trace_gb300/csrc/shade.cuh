// Camera rays and surface shading shared by the wavefront renderer and the
// batched persistent renderer, so that both trace exactly the same paths.
//
//   primary_ray   castRayReuse (camera.go:95-97) with RandomSampling's
//                 u = (x + xi) / (w - 1), v = (y + xi) / (h - 1) (render.go:201-205)
//   shade_step    DefaultClosestHitShader (render.go:209-224): miss colour,
//                 Light emission, Diffuse scatter = normal + uniform unit vector
//                 (material.go:29-38, util.go:15-26), MaxDepth cut-off
// Random numbers are Philox-2x32-10 keyed by the seed with counter (path, level),
// so a path is the same whichever kernel traces it.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbt_internal.cuh"
#include "traverse.cuh"

namespace gbt_dev {

struct CamF {
    float3 origin, llc, hor, ver;
};

struct ShadeParams {
    uint32_t npix, width, height, spp;
    int32_t max_depth;
    int32_t miss_mode;
    float3 miss_color;
    uint32_t seed_lo, seed_hi;
    uint32_t n_tri;
    uint32_t tiles;     // 1: launch slots map to path ids tile by tile (path_id)
    uint32_t any_last;  // 1: rays of level MaxDepth+1 take an any-hit query (batched kernel)
};

// Philox-2x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2,
// 3", SC'11): counter (path, stream) and key from the seed.
__device__ __forceinline__ uint2 philox2x32(uint32_t c0, uint32_t c1, uint32_t key) {
#pragma unroll
    for (int i = 0; i < 10; i++) {
        uint32_t hi = __umulhi(0xD256D193u, c0);
        uint32_t lo = 0xD256D193u * c0;
        c0 = hi ^ key ^ c1;
        c1 = lo;
        key += 0x9E3779B9u;
    }
    return make_uint2(c0, c1);
}
__device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// Path launched in slot g.  Path ids select the pixel (id % npix) and the random
// numbers, so the image depends only on the set of ids: with tiles the slots of
// one warp (32 consecutive g) take the ids of an 8x4 pixel tile, which keeps the
// rays of a warp coherent.  The map is a bijection on every run of npix slots:
// full tiles first, then the right strip, then the bottom strip, in scan order.
__device__ __forceinline__ uint32_t path_id(const ShadeParams &sp, uint32_t g) {
    if (!sp.tiles) return g;
    const uint32_t p = g % sp.npix, base = g - p;
    const uint32_t w8 = sp.width & ~7u, h4 = sp.height & ~3u;
    if (p >= w8 * h4) {
        uint32_t q = p - w8 * h4, rw = sp.width - w8;
        if (q < rw * h4) return base + (q / rw) * sp.width + w8 + q % rw;
        return base + h4 * sp.width + (q - rw * h4);
    }
    const uint32_t t = p >> 5, l = p & 31u, tw = w8 >> 3;
    return base + ((t / tw) * 4 + (l >> 3)) * sp.width + (t % tw) * 8 + (l & 7u);
}

// Primary ray of path id g (pixel g % npix).
__device__ __forceinline__ void primary_ray(const CamF &cam, const ShadeParams &sp, uint32_t g, float3 &o, float3 &d) {
    uint32_t pix = g % sp.npix;
    uint32_t x = pix % sp.width, y = pix / sp.width;
    uint2 rnd = philox2x32(g, 0xFFFFu, sp.seed_lo ^ sp.seed_hi);
    float s = ((float)x + u01(rnd.x)) / (float)(sp.width - 1);
    float t = ((float)y + u01(rnd.y)) / (float)(sp.height - 1);
    d = sub3(add3(add3(cam.llc, mul3(cam.hor, s)), mul3(cam.ver, t)), cam.origin);
    o = cam.origin;
}

__device__ __forceinline__ float3 miss_colour(const ShadeParams &sp, float3 d) {
    switch (sp.miss_mode) {
    case GBT_MISS_WHITE: return f3(1.f, 1.f, 1.f);
    case GBT_MISS_SKY: {
        float inv = rsqrtf(dot3(d, d));
        float t = 0.5f * (d.y * inv + 1.f);
        return f3(0.8f * (1.f - t) + 0.25f * t, 0.8f * (1.f - t) + 0.35f * t, 0.8f * (1.f - t) + 0.5f * t);
    }
    case GBT_MISS_CONSTANT: return sp.miss_color;
    default: return f3(0.f, 0.f, 0.f);
    }
}

__device__ __forceinline__ void deposit(float *__restrict__ acc, uint32_t pix, float3 L) {
    if (L.x != 0.f) atomicAdd(acc + 3 * (size_t)pix, L.x);
    if (L.y != 0.f) atomicAdd(acc + 3 * (size_t)pix + 1, L.y);
    if (L.z != 0.f) atomicAdd(acc + 3 * (size_t)pix + 2, L.z);
}

// Hit point p, the shading normal turned toward the ray and whether the ray
// hit the front face: triangles interpolate vertex normals (primitive.go:144-150)
// and front = det > 0 (:198-205); spheres use (p - c) / r (:79-84).
__device__ __forceinline__ void surface_frame(const float4 *__restrict__ recs, const float *__restrict__ normals,
                                              int rec, float3 o, float3 d, float t, float u, float v, float3 &p,
                                              float3 &nrm, bool &front) {
    const float4 *pr = recs + 3 * (size_t)rec;
    float4 r0 = __ldg(pr), r1 = __ldg(pr + 1);
    p = add3(o, mul3(d, t));  // ray.position(t)
    if (__float_as_int(r1.w) == 0) {
        float4 r2 = __ldg(pr + 2);
        float3 e1 = f3(r1.x - r0.x, r1.y - r0.y, r1.z - r0.z), e2 = f3(r2.x - r0.x, r2.y - r0.y, r2.z - r0.z);
        float3 ng = cross3(e1, e2);
        front = dot3(d, ng) < 0.f;  // det > 0
        if (normals) {
            const float *nv = normals + 9 * (size_t)(uint32_t)__float_as_int(r0.w);
            float w = 1.f - u - v;
            nrm = f3(nv[3] * u + nv[6] * v + nv[0] * w, nv[4] * u + nv[7] * v + nv[1] * w,
                     nv[5] * u + nv[8] * v + nv[2] * w);
        } else {
            nrm = mul3(ng, rsqrtf(dot3(ng, ng)));
        }
    } else {
        nrm = mul3(sub3(p, f3(r0.x, r0.y, r0.z)), 1.f / r1.x);
        front = dot3(d, nrm) < 0.f;
    }
    if (!front) nrm = mul3(nrm, -1.f);
}

// A uniform unit vector from two 32-bit random numbers (stands in for
// RandomUnitVector, util.go:15-26).
__device__ __forceinline__ float3 unit_vector(uint2 rnd) {
    float z = 1.f - 2.f * u01(rnd.x);
    float rr = sqrtf(fmaxf(0.f, 1.f - z * z));
    float sphi, cphi;
    sincospif(2.f * u01(rnd.y), &sphi, &cphi);
    return f3(rr * cphi, rr * sphi, z);
}

// reflect / refract / reflectance (Schlick), material.go:88-106
__device__ __forceinline__ float3 reflect3(float3 v, float3 n) { return sub3(v, mul3(n, dot3(v, n) * 2.f)); }

__device__ __forceinline__ float3 refract3(float3 uv, float3 n, float eta) {
    float c = fminf(-dot3(uv, n), 1.f);
    float3 perp = mul3(add3(uv, mul3(n, c)), eta);
    float3 par = mul3(n, -sqrtf(fabsf(1.f - dot3(perp, perp))));
    return add3(perp, par);
}

__device__ __forceinline__ float reflectance(float c, float ratio) {
    float r0 = (1.f - ratio) / (1.f + ratio);
    r0 = r0 * r0;
    float x = 1.f - c;
    return r0 + (1.f - r0) * (x * x * x * x * x);
}

// Material.scatter for the scattering materials: the new direction sd, or
// false when the path ends (Reflective below the surface).
//   Diffuse    material.go:29-38   n + unit vector (n if that is ~0)
//   Reflective material.go:49-53   reflect(unit d, n) + Diffusion * unit vector, if reflect . n > 0
//   Refractive material.go:63-86   Schlick choice between reflection and refraction
__device__ __forceinline__ bool scatter(int type, float param, float3 d, float3 nrm, bool front, uint2 rnd,
                                        float3 &sd) {
    if (type == GBT_MAT_REFLECTIVE) {
        float3 ud = mul3(d, rsqrtf(dot3(d, d)));
        float3 refl = reflect3(ud, nrm);
        sd = add3(refl, mul3(unit_vector(rnd), param));
        return dot3(refl, nrm) > 0.f;
    }
    if (type == GBT_MAT_REFRACTIVE) {
        float ratio = front ? 1.f / param : param;
        float3 ud = mul3(d, rsqrtf(dot3(d, d)));
        float c = fminf(-dot3(ud, nrm), 1.f);
        float sn = sqrtf(fmaxf(0.f, 1.f - c * c));
        bool cannot = ratio * sn > 1.f;
        sd = (cannot || reflectance(c, ratio) > u01(rnd.x)) ? reflect3(ud, nrm) : refract3(ud, nrm, ratio);
        return true;
    }
    float3 uv = unit_vector(rnd);
    sd = add3(nrm, uv);
    if (fabsf(sd.x) <= 1e-7f && fabsf(sd.y) <= 1e-7f && fabsf(sd.z) <= 1e-7f) sd = nrm;
    return true;
}

// Diffuse.scatter (material.go:29-38): hit point p and the new direction for
// a triangle or sphere record.
__device__ __forceinline__ void diffuse_scatter(const float4 *__restrict__ recs, const float *__restrict__ normals,
                                                int rec, float3 o, float3 d, float t, float u, float v, uint32_t g,
                                                int level, const ShadeParams &sp, float3 &p, float3 &sd) {
    float3 nrm;
    bool front;
    surface_frame(recs, normals, rec, o, d, t, u, v, p, nrm, front);
    scatter(GBT_MAT_DIFFUSE, 0.f, d, nrm, front, philox2x32(g, (uint32_t)level, sp.seed_lo ^ sp.seed_hi), sd);
}

// One shading event of path g at bounce `level` for ray (o, d) with the
// closest hit (t, u, v, rec).  Updates throughput T and radiance L.  Returns
// true when the path continues with the new ray (no, nd); false when it ends
// (L is then final).  Materials: two float4 each, (color.rgb, type), (param, ...).
__device__ __forceinline__ bool shade_step(const ShadeParams &sp, int level, uint32_t g, float3 o, float3 d, float t,
                                           float u, float v, int rec, const float4 *__restrict__ recs,
                                           const uint32_t *__restrict__ prim_mat, const float4 *__restrict__ mats,
                                           const float *__restrict__ normals, float3 &T, float3 &L, float3 &no,
                                           float3 &nd) {
    if (rec < 0) {
        L = add3(L, emul3(T, miss_colour(sp, d)));
        return false;
    }
    if (level > sp.max_depth) return false;  // render.go:210-212: beyond MaxDepth the surface returns black
    const float4 *pr = recs + 3 * (size_t)rec;
    const uint32_t id = (uint32_t)__float_as_int(__ldg(pr).w);
    const uint32_t mi = __ldg(prim_mat + id);
    const float4 m = __ldg(mats + 2 * (size_t)mi);
    const float3 col = f3(m.x, m.y, m.z);
    const int type = __float_as_int(m.w);
    if (type == GBT_MAT_LIGHT) {
        L = add3(L, emul3(T, col));
        return false;
    }
    const float param = type >= GBT_MAT_REFLECTIVE ? __ldg(mats + 2 * (size_t)mi + 1).x : 0.f;
    float3 p, nrm, sd;
    bool front;
    surface_frame(recs, normals, rec, o, d, t, u, v, p, nrm, front);
    if (!scatter(type, param, d, nrm, front, philox2x32(g, (uint32_t)level, sp.seed_lo ^ sp.seed_hi), sd))
        return false;  // emitted light of a scattering material is black
    T = emul3(T, col);
    no = p;
    nd = sd;
    return true;
}

}  // namespace gbt_dev

// host: camera basis of camera.go:53-66 computed in float64 and rounded
gbt_dev::CamF gbt_make_cam(const gbt_camera *c);
gbt_dev::ShadeParams gbt_make_shade_params(const gbt_render_params *p, uint32_t n_tri);
