// Morton-code LBVH construction on the device.
//
// Restates pkg/pt/lbvh.go:13-25 (DefaultLBVH) as a chain of kernels on one
// stream, with no host synchronisation:
//   k_bounds     scene box, fp64 min/max fold            (bounding.go:19-25)
//   k_morton     fp64 quantisation + bit interleave       (lbvh.go:64-73, morton.go:6-20)
//   k_hist, k_sort_plan, k_onesweep x8
//                stable LSD radix sort of (code, index)   (lbvh.go:216-301 bucket sort)
//   k_rle_*      runs of equal codes -> leaves            (lbvh.go:134-145, 179-181)
//   k_emit       primitive records in leaf order, and the binary radix tree
//                over the distinct codes with the bottom-up box refit fused
//                in                                       (lbvh.go:76-203, bvh.go:104-126,201-222)
#include <cuda_runtime.h>

#include <algorithm>

#include "gbt_internal.cuh"
#include "morton_exact.cuh"

namespace {

// Keys per sort tile: 256 threads of 16 keys or 512 threads of 8 (the context's
// sort_threads); tiles of 2048 and 1024 keys were measured slower.
constexpr int SORT_TILE = 4096;
constexpr uint32_t ST_AGG = 1u << 30;
constexpr uint32_t ST_PREFIX = 2u << 30;
constexpr uint32_t ST_FLAGS = 3u << 30;
constexpr uint32_t ST_VALUE = (1u << 30) - 1;

// ---------------------------------------------------------------------------
// small device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t *p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Order-preserving map of a double onto uint64 (for atomicMin/atomicMax).
__device__ __forceinline__ unsigned long long dbl_to_ord(double d) {
    unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__device__ __forceinline__ double ord_to_dbl(unsigned long long o) {
    unsigned long long b = (o >> 63) ? (o & 0x7fffffffffffffffULL) : ~o;
    return __longlong_as_double((long long)b);
}

// Primitive box in float64: triangle min/max of three widened floats
// (primitive.go:102-114), sphere centre -/+ radius (primitive.go:31-40).
__device__ __forceinline__ void prim_box_f64(const float *__restrict__ verts, const float4 *__restrict__ sph,
                                             uint32_t n_tri, uint32_t i, double lo[3], double hi[3]) {
    if (i < n_tri) {
        const float *t = verts + (size_t)i * 9;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            float a = t[k], b = t[3 + k], c = t[6 + k];
            lo[k] = (double)fminf(fminf(a, b), c);
            hi[k] = (double)fmaxf(fmaxf(a, b), c);
        }
    } else {
        float4 s = sph[i - n_tri];
        double r = (double)s.w;
        lo[0] = __dsub_rn((double)s.x, r);
        lo[1] = __dsub_rn((double)s.y, r);
        lo[2] = __dsub_rn((double)s.z, r);
        hi[0] = __dadd_rn((double)s.x, r);
        hi[1] = __dadd_rn((double)s.y, r);
        hi[2] = __dadd_rn((double)s.z, r);
    }
}

// ---------------------------------------------------------------------------
// scene bounds
// ---------------------------------------------------------------------------
// Blocks per SM of the scene-box fold: each block ends with atomics on the same six words,
// which serialise (8 blocks per SM: 31 us for the 1M soup's 36 MB, 2: 0.367 against 0.381 ms
// for the whole build)
#ifndef GBT_BOUNDS_BLOCKS_PER_SM
#define GBT_BOUNDS_BLOCKS_PER_SM 2
#endif
// Triangle boxes are float32 values, so their fold is done in float32 (exact)
// over the vertex array read as float4 triples: 12 floats hold 4 vertices with
// the axis pattern x y z x | y z x y | z x y z.  Sphere boxes (c -+ r in
// float64) are folded in float64.
__global__ void __launch_bounds__(256) k_bounds(const float *__restrict__ verts, const float4 *__restrict__ sph,
                                                uint32_t n_tri, uint32_t n, unsigned long long *acc) {
    float flo[3] = {INFINITY, INFINITY, INFINITY}, fhi[3] = {-INFINITY, -INFINITY, -INFINITY};
    const size_t nf = (size_t)n_tri * 9, nchunk = nf / 12;
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x, stride = (size_t)gridDim.x * blockDim.x;
    const float4 *v4 = reinterpret_cast<const float4 *>(verts);
    auto fold = [&](const float4 &a, const float4 &b, const float4 &d) {
        flo[0] = fminf(fminf(fminf(flo[0], a.x), fminf(a.w, b.z)), d.y);
        fhi[0] = fmaxf(fmaxf(fmaxf(fhi[0], a.x), fmaxf(a.w, b.z)), d.y);
        flo[1] = fminf(fminf(fminf(flo[1], a.y), fminf(b.x, b.w)), d.z);
        fhi[1] = fmaxf(fmaxf(fmaxf(fhi[1], a.y), fmaxf(b.x, b.w)), d.z);
        flo[2] = fminf(fminf(fminf(flo[2], a.z), fminf(b.y, d.x)), d.w);
        fhi[2] = fmaxf(fmaxf(fmaxf(fhi[2], a.z), fmaxf(b.y, d.x)), d.w);
    };
    size_t c = tid;
    // four chunks' loads in flight per thread (the fold is order-free: min and max)
    for (; c + 3 * stride < nchunk; c += 4 * stride) {
        float4 a[4], b[4], d[4];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const float4 *q = v4 + 3 * (c + u * stride);
            a[u] = __ldg(q);
            b[u] = __ldg(q + 1);
            d[u] = __ldg(q + 2);
        }
#pragma unroll
        for (int u = 0; u < 4; u++) fold(a[u], b[u], d[u]);
    }
    for (; c < nchunk; c += stride) fold(__ldg(v4 + 3 * c), __ldg(v4 + 3 * c + 1), __ldg(v4 + 3 * c + 2));
    for (size_t f = nchunk * 12 + tid; f < nf; f += stride) {
        const float x = __ldg(verts + f);
        const int k = (int)(f % 3);
        flo[k] = fminf(flo[k], x);
        fhi[k] = fmaxf(fhi[k], x);
    }
    double lo[3], hi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        lo[k] = (double)flo[k];
        hi[k] = (double)fhi[k];
    }
    for (uint32_t i = n_tri + (uint32_t)tid; i < n; i += (uint32_t)stride) {
        double a[3], b[3];
        prim_box_f64(verts, sph, n_tri, i, a, b);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            lo[k] = fmin(lo[k], a[k]);
            hi[k] = fmax(hi[k], b[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fmin(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmax(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    __shared__ double s[8][6];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 3; k++) { s[w][k] = lo[k]; s[w][3 + k] = hi[k]; }
    __syncthreads();
    if (threadIdx.x < 6) {
        int k = threadIdx.x;
        double v = s[0][k];
        for (int j = 1; j < (int)(blockDim.x >> 5); j++) v = k < 3 ? fmin(v, s[j][k]) : fmax(v, s[j][k]);
        if (k < 3) atomicMin(&acc[k], dbl_to_ord(v));
        else atomicMax(&acc[k], dbl_to_ord(v));
    }
}

// ---------------------------------------------------------------------------
// Morton codes
// ---------------------------------------------------------------------------
// Interleave: bit k of a moves to bit 3k (the standard shift-and-mask spread
// of 21 bits over 63).
__device__ __forceinline__ uint64_t spread3(uint64_t a) {
    uint64_t x = a & 0x1fffffULL;
    x = (x | (x << 32)) & 0x001f00000000ffffULL;
    x = (x | (x << 16)) & 0x001f0000ff0000ffULL;
    x = (x | (x << 8)) & 0x100f00f00f00f00fULL;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ULL;
    x = (x | (x << 2)) & 0x1249249249249249ULL;
    return x;
}

// float32 -> float64 by moving the exponent and mantissa fields (exact; the
// fp64 pipe is the scarce unit here).  Zero, subnormal, Inf and NaN take the
// ordinary conversion.
__device__ __forceinline__ double widen(float x) {
    const uint32_t b = __float_as_uint(x), e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)x;
    const uint64_t d = ((uint64_t)(b & 0x80000000u) << 32) | ((uint64_t)(e + 896u) << 52) |
                       ((uint64_t)(b & 0x7fffffu) << 29);
    return __longlong_as_double((long long)d);
}

// x * 0.5 by decrementing the exponent field when the result stays normal (exact).
__device__ __forceinline__ double halve(double x) {
    const uint64_t b = (uint64_t)__double_as_longlong(x), e = (b >> 52) & 0x7ffu;
    if (e > 1u && e < 0x7ffu) return __longlong_as_double((long long)(b - (1ull << 52)));
    return __dmul_rn(x, 0.5);
}

// uint64(dx / step) exactly as the reference computes it: a correctly rounded
// float64 division, truncated.  The product with the rounded reciprocal is
// within a few ulp of the quotient, so its integer part is the answer unless
// the quotient lies within 2^-26 of an integer; only then is the division done.
// The integer and fractional parts of the product are read off its bits.
__device__ __forceinline__ uint64_t quantise(double dx, double step, double rstep) {
    const uint64_t b = (uint64_t)__double_as_longlong(__dmul_rn(dx, rstep));
    // 0 <= qa < 2^22 (dx >= 0, rstep > 0; NaN and larger values have larger bit patterns)
    if (b < 0x4150000000000000ull) {
        const int E = (int)(b >> 52) - 1023;  // qa in [2^E, 2^(E+1)), or qa < 1
        if (E < 0) {
            // integer part 0, fraction qa: 2^-26 < qa < 1 - 2^-26
            if (b > 0x3e50000000000000ull && b < 0x3feffffff8000000ull) return 0;
        } else {
            const uint64_t m = (b & 0xfffffffffffffull) | (1ull << 52);
            const int fb = 52 - E;  // fraction bits, 31..52
            const uint64_t frac = m & ((1ull << fb) - 1), lo = 1ull << (fb - 26);
            if (frac > lo && frac < (1ull << fb) - lo) return m >> fb;
        }
    }
    double q = __ddiv_rn(dx, step);
    if (!(q < 9223372036854775808.0) || q < 0.0) return 0;  // NaN (zero-extent axis) or out of domain
    return (uint64_t)__double2ull_rz(q);
}

// The 9 floats of triangle o: three 16-byte loads from the word boundary at or
// below its first float (9 o - (o mod 4); the vertex array is 16-byte aligned),
// so that a warp's gather of scattered triangles (the emission's, in Morton order)
// makes a third of the L1 requests of nine 4-byte loads.  The last triangles, whose
// words would reach past the array, load by float.  (The Morton kernel's loads of
// consecutive triangles measured faster as nine 4-byte loads.)
__device__ __forceinline__ void load_triangle(const float *__restrict__ verts, uint32_t n_tri, uint32_t o,
                                              float (&t)[9]) {
    const size_t f = (size_t)o * 9;
    const uint32_t off = o & 3u;  // 9 o mod 4
    if (f - off + 12 <= (size_t)n_tri * 9) {
        const float4 *w4 = reinterpret_cast<const float4 *>(verts + (f - off));
        const float4 a = __ldg(w4), b = __ldg(w4 + 1), c = __ldg(w4 + 2);
        const float w[12] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
#pragma unroll
        for (int j = 0; j < 9; j++) t[j] = off == 0 ? w[j] : off == 1 ? w[j + 1] : off == 2 ? w[j + 2] : w[j + 3];
    } else {
#pragma unroll
        for (int j = 0; j < 9; j++) t[j] = __ldg(verts + f + j);
    }
}

__global__ void __launch_bounds__(256) k_morton(const float *__restrict__ verts, const float4 *__restrict__ sph,
                                                uint32_t n_tri, uint32_t n, const unsigned long long *__restrict__ acc,
                                                uint64_t *__restrict__ codes) {
    gbt_pdl_wait();
    gbt_pdl_trigger();
    __shared__ double s_e[9];  // lo.xyz, step.xyz, 1/step.xyz
    __shared__ float s_f[15];  // lo.xyz and 1/step.xyz as float pairs, margin.xyz
    if (threadIdx.x < 3) {
        int k = threadIdx.x;
        double lo = ord_to_dbl(acc[k]), hi = ord_to_dbl(acc[3 + k]);
        double ext = __dsub_rn(hi, lo);                 // aabb.update width/height/depth
        double step = __ddiv_rn(ext, 2097151.0);        // extent / (MORTON_SIZE-1)
        double rstep = __drcp_rn(step);
        s_e[k] = lo;
        s_e[3 + k] = step;
        s_e[6 + k] = rstep;
        const gbt_morton::AxisF32x2 f = gbt_morton::axis_setup(lo, hi, rstep);
        s_f[k] = f.lo_h;
        s_f[3 + k] = f.lo_l;
        s_f[6 + k] = f.rs_h;
        s_f[9 + k] = f.rs_l;
        s_f[12 + k] = f.margin;
    }
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint64_t q[3];
        if (i < n_tri) {
            const float *t = verts + (size_t)i * 9;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const float a = __ldg(t + k), b = __ldg(t + 3 + k), c = __ldg(t + 6 + k);
                const float mn = fminf(fminf(a, b), c), mx = fmaxf(fmaxf(a, b), c);
                const int64_t f = gbt_morton::quantise_f32x2(mn, mx, s_f[k], s_f[3 + k], s_f[6 + k], s_f[9 + k], s_f[12 + k]);
                if (f >= 0) {
                    q[k] = (uint64_t)f;
                } else {  // the float64 path: the reference's operations
                    const double cb = halve(__dadd_rn(widen(mn), widen(mx)));  // aabb barycenter
                    const double dx = __longlong_as_double(__double_as_longlong(__dsub_rn(s_e[k], cb)) & 0x7fffffffffffffffll);
                    q[k] = quantise(dx, s_e[3 + k], s_e[6 + k]);
                }
            }
        } else {
            double lo[3], hi[3];
            prim_box_f64(verts, sph, n_tri, i, lo, hi);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const double cb = halve(__dadd_rn(lo[k], hi[k]));
                const double dx = __longlong_as_double(__double_as_longlong(__dsub_rn(s_e[k], cb)) & 0x7fffffffffffffffll);
                q[k] = quantise(dx, s_e[3 + k], s_e[6 + k]);
            }
        }
        codes[i] = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
    }
}

// ---------------------------------------------------------------------------
// LSD radix sort: 8 passes of 8 bits, one-sweep with decoupled look-back
// ---------------------------------------------------------------------------
struct SortPlan {
    const uint64_t *in_k[8];
    uint64_t *out_k[8];
    const uint32_t *in_v[8];
    uint32_t *out_v[8];
    uint32_t active[8];
    uint32_t identity[8];
    uint64_t *final_k;
    uint32_t *final_v;
    uint32_t final_sel;
    uint32_t pad;
    uint32_t digit_base[8][256];
};

struct SortScratch {  // byte offsets inside one scratch allocation
    size_t plan, hist, ctr, status, total;
    uint32_t n_tiles;
};

SortScratch sort_layout(uint32_t n, size_t base) {
    SortScratch s;
    s.n_tiles = (n + SORT_TILE - 1) / SORT_TILE;
    s.plan = gbt_align(base);
    s.hist = gbt_align(s.plan + sizeof(SortPlan));
    s.ctr = gbt_align(s.hist + 8 * 256 * sizeof(uint32_t));
    s.status = gbt_align(s.ctr + 8 * sizeof(uint32_t));
    s.total = gbt_align(s.status + (size_t)8 * s.n_tiles * 256 * sizeof(uint32_t));
    return s;
}

// One read of the keys builds the digit histograms of all eight passes.
__global__ void __launch_bounds__(256) k_hist(const uint64_t *__restrict__ keys, uint32_t n, uint32_t *__restrict__ ghist) {
    gbt_pdl_wait();
    gbt_pdl_trigger();
    __shared__ uint32_t h[8 * 256];
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // eight keys' loads in flight per thread
    for (; i + 7 * stride < n; i += 8 * stride) {
        uint64_t k[8];
#pragma unroll
        for (int u = 0; u < 8; u++) k[u] = __ldcs(keys + i + u * stride);
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
            for (int p = 0; p < 8; p++) atomicAdd(&h[p * 256 + (uint32_t)((k[u] >> (8 * p)) & 255u)], 1u);
    }
    for (; i < n; i += stride) {
        uint64_t k = keys[i];
#pragma unroll
        for (int p = 0; p < 8; p++) atomicAdd(&h[p * 256 + (uint32_t)((k >> (8 * p)) & 255u)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x)
        if (h[i]) atomicAdd(&ghist[i], h[i]);
}

// Exclusive scan of 256 values held one per thread (blockDim == 256).
// Threads past the first 256 of a larger block take part in the barriers only.
__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t v, uint32_t *s_tmp /*8*/, uint32_t *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31 && w < 8) s_tmp[w] = x;
    __syncthreads();
    uint32_t off = 0, tot = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        uint32_t c = s_tmp[j];
        off += (j < w) ? c : 0u;
        tot += c;
    }
    __syncthreads();
    if (total) *total = tot;
    return off + x - v;
}

// Decide which passes are needed (a pass whose digit is equal for every key
// leaves the order unchanged) and chain the ping-pong buffers through them.
__global__ void __launch_bounds__(256) k_sort_plan(SortPlan *plan, const uint32_t *__restrict__ ghist, uint32_t n,
                                                   uint64_t *kA, uint32_t *vA, uint64_t *kB, uint32_t *vB,
                                                   int identity_vals, BvhHeader *hdr) {
    gbt_pdl_wait();
    gbt_pdl_trigger();
    __shared__ uint32_t s_tmp[8];
    __shared__ uint32_t s_active[8];
    const int t = threadIdx.x;
    for (int p = 0; p < 8; p++) {
        uint32_t c = ghist[p * 256 + t];
        int full = __syncthreads_or(c == n);
        plan->digit_base[p][t] = block_excl_scan256(c, s_tmp, nullptr);
        if (t == 0) s_active[p] = full ? 0u : 1u;
    }
    __syncthreads();
    if (t == 0) {
        int any = 0;
        for (int p = 0; p < 8; p++) any |= s_active[p];
        if (!any) s_active[0] = 1;  // one pass still has to move the pairs (and write the values)
        uint64_t *ck = kA;
        uint32_t *cv = vA;
        int first = 1;
        for (int p = 0; p < 8; p++) {
            plan->active[p] = s_active[p];
            plan->identity[p] = 0;
            if (!s_active[p]) continue;
            uint64_t *ok = (ck == kA) ? kB : kA;
            uint32_t *ov = (cv == vA) ? vB : vA;
            plan->in_k[p] = ck;
            plan->in_v[p] = cv;
            plan->out_k[p] = ok;
            plan->out_v[p] = ov;
            plan->identity[p] = (first && identity_vals) ? 1u : 0u;
            first = 0;
            ck = ok;
            cv = ov;
        }
        plan->final_k = ck;
        plan->final_v = cv;
        plan->final_sel = (ck == kA) ? 0u : 1u;
        if (hdr) hdr->sorted_sel = plan->final_sel;
    }
}

__device__ __forceinline__ uint32_t lookback_wait(const uint32_t *p, unsigned int *err, uint32_t limit) {
    for (uint32_t it = 0;; ++it) {
        uint32_t s = ld_relaxed(p);
        if (s & ST_FLAGS) return s;
        if (it >= limit) {
            atomicOr(err, GBT_DEVERR_SPIN);
            return ST_PREFIX;  // give up: the result is wrong but the kernel ends; the host sees the flag
        }
        if (it > 64) __nanosleep(64);
    }
}

// True once a bounded wait of the sort has run out: the sorted order is then
// unusable, and every later kernel of the build returns at once instead of
// reading it.  The flag is only set by k_onesweep, so inside any later kernel
// every thread reads the same value.
__device__ __forceinline__ bool sort_failed(const unsigned int *err) {
    return (*reinterpret_cast<const volatile unsigned int *>(err) & GBT_DEVERR_SPIN) != 0u;
}

// One pass: rank each key within its warp by digit (match_any + ballot
// counts into warp-private shared histograms), publish the tile's digit
// counts, look back over earlier tiles for the global offsets, stage the tile
// in shared memory in digit order and write it out in runs.  Look-back waits
// give up after spin_limit polls.  withhold_tile (a testing aid, 0xffffffff
// when off) names a tile that never publishes its counts, so that the tiles
// after it wait for a status nothing sets and the limit is reached.
// T threads of I keys each (T * I = SORT_TILE); the register budget is sized for two
// resident blocks per SM.  Digit-wise steps take one thread per digit (the first 256).
// MINB: resident blocks per SM the registers are sized for.  3 (80 registers) is faster for
// sorts of many tiles (the 8.4M terrain: 1.622 against 1.642 ms a build) and slower for
// sorts of about one wave (the 1M soup: 0.376 against 0.367 ms).
template <int T, int I, int MINB = 2>
__global__ void __launch_bounds__(T, MINB) k_onesweep(const SortPlan *__restrict__ plan, int pass, uint32_t n,
                                                 uint32_t *__restrict__ status, uint32_t *__restrict__ tile_ctr,
                                                 unsigned int *err, uint32_t spin_limit, uint32_t withhold_tile) {
    static_assert(T * I == SORT_TILE && T >= 256 && T % 32 == 0, "tile shape");
    constexpr int NW = T / 32;
    gbt_pdl_wait();
    gbt_pdl_trigger();
    if (!plan->active[pass]) return;
    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t *s_wh = reinterpret_cast<uint32_t *>(smem);  // [NW][256]
    uint32_t *s_tstart = s_wh + NW * 256;                   // [256]
    uint32_t *s_gbase = s_tstart + 256;                      // [256]
    uint32_t *s_misc = s_gbase + 256;                        // [32]
    uint64_t *s_keys = reinterpret_cast<uint64_t *>(s_misc + 32);
    uint32_t *s_vals = reinterpret_cast<uint32_t *>(s_keys + SORT_TILE);
    uint32_t *s_mask = s_vals + SORT_TILE;  // [NW][257] lane masks per digit (digit 256: past the end)

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        s_misc[17] = sort_failed(err) ? 1u : 0u;  // an earlier pass or tile gave up: the input is unusable
        s_misc[16] = atomicAdd(&tile_ctr[pass], 1u);
    }
    for (int i = tid; i < NW * 256; i += T) s_wh[i] = 0;
    for (int i = tid; i < NW * 257; i += T) s_mask[i] = 0;
    __syncthreads();
    if (s_misc[17]) return;
    const uint32_t tile = s_misc[16];
    const bool publish = tile != withhold_tile;
    const uint32_t shift = 8u * pass;
    const uint64_t *__restrict__ kin = plan->in_k[pass];
    const uint32_t *__restrict__ vin = plan->in_v[pass];
    const bool ident = plan->identity[pass] != 0;
    const uint32_t wbase = tile * SORT_TILE + warp * 32 * I;

    uint64_t k[I];
    uint32_t v[I];
    uint32_t rk[I];
#pragma unroll
    for (int i = 0; i < I; i++) {
        uint32_t idx = wbase + i * 32 + lane;
        k[i] = idx < n ? __ldcs(kin + idx) : 0ull;
    }
    uint32_t *wh = s_wh + warp * 256;
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int i = 0; i < I; i++) {
        uint32_t idx = wbase + i * 32 + lane;
        bool ok = idx < n;
        uint32_t d = ok ? (uint32_t)((k[i] >> shift) & 255u) : 256u;
        // lanes with the same digit, from one vote per digit bit (valid lanes only; ranking by
        // __match_any_sync measured slower)
        // the lanes with the same digit: each lane ORs its bit into its digit's word of the
        // warp's masks and reads the word back (one ballot per digit bit measured 4% slower
        // for the whole build); the group's leader clears the word for the next round
        uint32_t *mk = s_mask + warp * 257;
        atomicOr(&mk[d], 1u << lane);
        __syncwarp();
        const uint32_t peers = mk[d];
        uint32_t base = ok ? wh[d] : 0u;
        __syncwarp();
        const bool leader = lane == (uint32_t)(__ffs(peers) - 1);
        if (ok && leader) wh[d] = base + __popc(peers);
        if (leader) mk[d] = 0;  // every lane of the group has read it
        __syncwarp();
        rk[i] = base + __popc(peers & lt);
    }
    // the values are needed only for the scatter: loaded now, they arrive during the
    // per-digit steps and the look-back, and take no registers during the ranking
#pragma unroll
    for (int i = 0; i < I; i++) {
        uint32_t idx = wbase + i * 32 + lane;
        v[i] = ident ? idx : (idx < n ? __ldcs(vin + idx) : 0u);
    }
    __syncthreads();

    const uint32_t t = (uint32_t)tid;  // one thread per digit (t < 256)
    uint32_t sum = 0;
    uint32_t *st = status + (size_t)tile * 256;
    if (t < 256) {
#pragma unroll
        for (int w = 0; w < NW; w++) {
            uint32_t c = s_wh[w * 256 + t];
            s_wh[w * 256 + t] = sum;
            sum += c;
        }
        if (publish) st_relaxed(&st[t], (tile == 0 ? ST_PREFIX : ST_AGG) | sum);
    }
    const uint32_t tstart = block_excl_scan256(sum, s_misc, nullptr);  // every thread takes part
    if (t < 256) {
        s_tstart[t] = tstart;
        uint32_t prefix = 0;
        if (tile > 0) {
            for (int j = (int)tile - 1; j >= 0; --j) {
                uint32_t s = lookback_wait(&status[(size_t)j * 256 + t], err, spin_limit);
                prefix += s & ST_VALUE;
                if ((s & ST_FLAGS) == ST_PREFIX) break;
            }
            if (publish) st_relaxed(&st[t], ST_PREFIX | (prefix + sum));
        }
        // output position of tile slot j of digit t: j + (global start - tile start), mod 2^32
        s_gbase[t] = plan->digit_base[pass][t] + prefix - tstart;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < I; i++) {
        uint32_t idx = wbase + i * 32 + lane;
        if (idx < n) {
            uint32_t d = (uint32_t)((k[i] >> shift) & 255u);
            uint32_t pos = s_tstart[d] + wh[d] + rk[i];
            s_keys[pos] = k[i];
            s_vals[pos] = v[i];
        }
    }
    __syncthreads();
    uint64_t *__restrict__ kout = plan->out_k[pass];
    uint32_t *__restrict__ vout = plan->out_v[pass];
    const uint32_t tile0 = tile * SORT_TILE;
    const uint32_t valid = (n - tile0) < (uint32_t)SORT_TILE ? (n - tile0) : (uint32_t)SORT_TILE;
    for (uint32_t j = tid; j < valid; j += T) {
        uint64_t kk = s_keys[j];
        uint32_t d = (uint32_t)((kk >> shift) & 255u);
        uint32_t g = s_gbase[d] + j;
        kout[g] = kk;
        vout[g] = s_vals[j];
    }
}

// Launches the eight passes (a pass whose plan entry is inactive returns at once) with tiles
// of 256 threads x 16 keys (threads 256) or 512 x 8 (threads 512, measured no faster).
// 256-thread tiles take the 3-blocks-per-SM register budget once there are more than four
// resident blocks' worth of tiles.
static cudaError_t onesweep_passes(int threads, int num_sms, const SortPlan *plan, uint32_t n, uint32_t n_tiles,
                                   uint32_t *status, uint32_t *ctr, unsigned int *err, uint32_t spin_limit,
                                   uint32_t withhold0, cudaStream_t st, bool pdl) {
    const int nw = threads / 32;
    const size_t smem = (size_t)(nw * 256 + 256 + 256 + 32) * sizeof(uint32_t) +
                        (size_t)SORT_TILE * (sizeof(uint64_t) + sizeof(uint32_t)) + (size_t)nw * 257 * sizeof(uint32_t);
    const bool many = threads == 256 && n_tiles > (uint32_t)num_sms * 8u;
    cudaError_t e;
    if (threads == 512) e = cudaFuncSetAttribute(k_onesweep<512, SORT_TILE / 512>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    else if (many) e = cudaFuncSetAttribute(k_onesweep<256, SORT_TILE / 256, 3>,
                                            cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    else e = cudaFuncSetAttribute(k_onesweep<256, SORT_TILE / 256>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem);
    if (e != cudaSuccess) return e;
    for (int p = 0; p < 8; p++) {
        uint32_t *sp = status + (size_t)p * n_tiles * 256;
        const uint32_t wh = p == 0 ? withhold0 : 0xffffffffu;
        if (threads == 512)
            e = gbt_launch_pdl(pdl, k_onesweep<512, SORT_TILE / 512>, n_tiles, 512, smem, st, plan, p, n, sp, ctr, err,
                               spin_limit, wh);
        else if (many)
            e = gbt_launch_pdl(pdl, k_onesweep<256, SORT_TILE / 256, 3>, n_tiles, 256, smem, st, plan, p, n, sp, ctr, err,
                               spin_limit, wh);
        else
            e = gbt_launch_pdl(pdl, k_onesweep<256, SORT_TILE / 256>, n_tiles, 256, smem, st, plan, p, n, sp, ctr, err,
                               spin_limit, wh);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// runs of equal codes
// ---------------------------------------------------------------------------
constexpr int RLE_THREADS = 256, RLE_ITEMS = 16, RLE_TILE = RLE_THREADS * RLE_ITEMS;

__device__ __forceinline__ bool run_start_at(const uint64_t *__restrict__ k, uint32_t i, uint32_t n) {
    return i < n && (i == 0 || k[i] != k[i - 1]);
}

__global__ void __launch_bounds__(RLE_THREADS) k_rle_count(const SortPlan *__restrict__ plan, uint32_t n,
                                                           uint32_t *__restrict__ tile_cnt, const unsigned int *err) {
    gbt_pdl_wait();
    gbt_pdl_trigger();
    if (sort_failed(err)) return;
    const uint64_t *k = plan->final_k;
    uint32_t base = blockIdx.x * RLE_TILE, c = 0;
#pragma unroll
    for (int i = 0; i < RLE_ITEMS; i++) c += run_start_at(k, base + i * RLE_THREADS + threadIdx.x, n);
    c = __reduce_add_sync(0xffffffffu, c);
    __shared__ uint32_t s[8];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int j = 0; j < 8; j++) t += s[j];
        tile_cnt[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(1024) k_rle_scan(uint32_t *tile_cnt, uint32_t n_tiles, BvhHeader *hdr,
                                                   const unsigned int *err) {
    gbt_pdl_wait();
    gbt_pdl_trigger();
    if (sort_failed(err)) return;
    __shared__ uint32_t s_w[32];
    __shared__ uint32_t s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t b = 0; b < n_tiles; b += 1024) {
        uint32_t i = b + threadIdx.x;
        uint32_t v = i < n_tiles ? tile_cnt[i] : 0u, x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_w[w] = x;
        __syncthreads();
        uint32_t off = s_carry, tot = 0;
        for (int j = 0; j < 32; j++) {
            off += (j < w) ? s_w[j] : 0u;
            tot += s_w[j];
        }
        if (i < n_tiles) tile_cnt[i] = off + x - v;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        hdr->n_unique = s_carry;
        hdr->n_nodes = s_carry > 0 ? s_carry - 1 : 0;
    }
}

__global__ void __launch_bounds__(RLE_THREADS) k_rle_write(const SortPlan *__restrict__ plan, uint32_t n,
                                                           const uint32_t *__restrict__ tile_off,
                                                           uint32_t *__restrict__ run, uint64_t *__restrict__ ukey,
                                                           const unsigned int *err) {
    gbt_pdl_wait();
    gbt_pdl_trigger();
    if (sort_failed(err)) return;
    const uint64_t *k = plan->final_k;
    __shared__ uint32_t s_w[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t lt = lanemask_lt();
    uint32_t base = blockIdx.x * RLE_TILE, carry = tile_off[blockIdx.x];
    for (int i = 0; i < RLE_ITEMS; i++) {
        uint32_t idx = base + i * RLE_THREADS + threadIdx.x;
        bool f = run_start_at(k, idx, n);
        uint32_t b = __ballot_sync(0xffffffffu, f);
        if (lane == 0) s_w[w] = __popc(b);
        __syncthreads();
        uint32_t off = carry, tot = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            off += (j < w) ? s_w[j] : 0u;
            tot += s_w[j];
        }
        if (f) {
            uint32_t u = off + __popc(b & lt);
            run[u] = idx;
            ukey[u] = k[idx];
        }
        if (idx == n - 1) run[off + __popc(b & lt) + (f ? 1u : 0u)] = n;
        carry += tot;
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// primitive records in sorted order: r0 = (v0, id), r1 = (v1 | centre r, kind), r2 = v2
// ---------------------------------------------------------------------------
// The record of primitive o: r0 = (v0, id), r1 = (v1 | radius, kind), r2 = v2.
__device__ __forceinline__ void make_record(const float *__restrict__ verts, const float4 *__restrict__ sph,
                                            uint32_t n_tri, uint32_t o, float4 &r0, float4 &r1, float4 &r2) {
    if (o < n_tri) {
        float t[9];
        load_triangle(verts, n_tri, o, t);
        r0 = make_float4(t[0], t[1], t[2], __int_as_float((int)o));
        r1 = make_float4(t[3], t[4], t[5], __int_as_float(0));
        r2 = make_float4(t[6], t[7], t[8], 0.f);
    } else {
        float4 c = sph[o - n_tri];
        r0 = make_float4(c.x, c.y, c.z, __int_as_float((int)o));
        r1 = make_float4(c.w, 0.f, 0.f, __int_as_float(1));
        r2 = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// ---------------------------------------------------------------------------
// hierarchy emission + refit
// ---------------------------------------------------------------------------
// Box of one stored primitive record, in float32.  Triangle boxes are exact;
// a sphere box (float64 centre -/+ radius in the reference) is rounded outward.
__device__ __forceinline__ void box_of_record(const float4 &r0, const float4 &r1, const float4 &r2, float3 &lo,
                                              float3 &hi) {
    if (__float_as_int(r1.w) == 0) {
        lo = make_float3(fminf(fminf(r0.x, r1.x), r2.x), fminf(fminf(r0.y, r1.y), r2.y), fminf(fminf(r0.z, r1.z), r2.z));
        hi = make_float3(fmaxf(fmaxf(r0.x, r1.x), r2.x), fmaxf(fmaxf(r0.y, r1.y), r2.y), fmaxf(fmaxf(r0.z, r1.z), r2.z));
    } else {
        double r = r1.x;
        lo = make_float3(__double2float_rd((double)r0.x - r), __double2float_rd((double)r0.y - r),
                         __double2float_rd((double)r0.z - r));
        hi = make_float3(__double2float_ru((double)r0.x + r), __double2float_ru((double)r0.y + r),
                         __double2float_ru((double)r0.z + r));
    }
}

__device__ __forceinline__ int prefix_len(const uint64_t *__restrict__ ukey, uint32_t i, uint32_t j) {
    return __clzll((long long)(ukey[i] ^ ukey[j]));
}

// One thread per leaf walks up the binary radix tree.  A node covering the
// distinct-code range [l, r] is the left child of the split r|r+1 or the right
// child of the split l-1|l, whichever boundary shares the longer common prefix
// (the reference splits a range at the highest differing bit, lbvh.go:147-176,
// so that boundary is its parent's split).  Inner node k is the split k|k+1.
// The second child to arrive at a node folds both boxes and carries on.
__device__ __forceinline__ int32_t exch_acq_rel(int32_t *p, int32_t v) {
    int32_t old;
    asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Emission block: the leaves of one block of threads and the inner nodes whose
// whole range lies inside them.  Such a node's two children both come from
// the block, so their hand-off goes through shared memory; the others go
// through the global hand-off word.
constexpr int EMIT_THREADS = 256;

// A node that k_emit hands to k_emit_top: its box, distinct-code range and index.
struct EmitState {
    float lo[3], hi[3];
    uint32_t l, r, ref, pad0;
    uint32_t pad[2];
};

// Second child at a node reached through the global hand-off word: fold in the
// sibling's slot (release by the sibling's exchange, acquire by this one's).
__device__ __forceinline__ void emit_merge_global(const float4 *nd, int slot, float3 &lo, float3 &hi) {
    const float4 sb = __ldcg(nd + (slot ^ 1));
    const float2 sz = __ldcg(reinterpret_cast<const float2 *>(nd + 2) + (slot ^ 1));
    lo = make_float3(fminf(lo.x, sb.x), fminf(lo.y, sb.z), fminf(lo.z, sz.x));
    hi = make_float3(fmaxf(hi.x, sb.y), fmaxf(hi.y, sb.w), fmaxf(hi.z, sz.y));
}

__device__ __forceinline__ void slot_write(float4 *nd, int slot, float3 lo, float3 hi, int32_t ref, int32_t cnt) {
    nd[slot] = make_float4(lo.x, hi.x, lo.y, hi.y);
    reinterpret_cast<float2 *>(nd + 2)[slot] = make_float2(lo.z, hi.z);
    reinterpret_cast<int2 *>(nd + 3)[slot] = make_int2(ref, cnt);
}

__device__ __forceinline__ float4 lds_f4(const float4 *p) {
    float4 v;
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a) : "memory");
    return v;
}

// Number of nodes (leaves included) under a node of distinct-code range [l, r].
__device__ __forceinline__ uint32_t range_size(uint32_t l, uint32_t r) { return 2u * (r - l) + 1u; }

// One leaf of k_emit: its records, then its climb while it is the second child to
// arrive.  The nodes inside the block keep both child slots, their subtree size and
// range in shared memory for k_emit's write-out; the others go as before.
__device__ __forceinline__ void emit_climb(BvhHeader *hdr, const uint32_t *__restrict__ run,
                                           const uint64_t *__restrict__ ukey, float4 *__restrict__ recs,
                                           float4 *nodes, int32_t *other, int32_t *parent_of, uint32_t *subtree,
                                           uint2 *range, EmitState *top, uint32_t *top_n, uint32_t top_cap,
                                           unsigned int *err, const SortPlan *__restrict__ plan,
                                           const float *__restrict__ verts, const float4 *__restrict__ sph,
                                           uint32_t n_tri, uint32_t U, uint32_t k0, uint32_t u, const int *s_d,
                                           int32_t *s_oth, float4 (*s_r0)[EMIT_THREADS],
                                           float4 (*s_r1)[EMIT_THREADS], uint32_t *s_sub, uint2 *s_rng,
                                           int32_t *s_par, const uint8_t *s_loc) {
    constexpr int B = EMIT_THREADS;
    uint32_t first = run[u], last = run[u + 1];
    float3 lo, hi;
    const uint32_t *__restrict__ idx = plan->final_v;
    for (uint32_t s = first; s < last; s++) {
        float4 r0, r1, r2;
        make_record(verts, sph, n_tri, idx[s], r0, r1, r2);
        recs[3 * (size_t)s + 0] = r0;
        recs[3 * (size_t)s + 1] = r1;
        recs[3 * (size_t)s + 2] = r2;
        float3 a, b;
        box_of_record(r0, r1, r2, a, b);
        if (s == first) {
            lo = a;
            hi = b;
        } else {
            lo = make_float3(fminf(lo.x, a.x), fminf(lo.y, a.y), fminf(lo.z, a.z));
            hi = make_float3(fmaxf(hi.x, b.x), fmaxf(hi.y, b.y), fmaxf(hi.z, b.z));
        }
    }
    int32_t ref = (int32_t)first, cnt = (int32_t)(last - first);
    uint32_t l = u, r = u;
    for (;;) {
        if (l == 0 && r == U - 1) {
            hdr->root_ref = ref;
            hdr->root_cnt = cnt;
            hdr->root_lo[0] = lo.x; hdr->root_lo[1] = lo.y; hdr->root_lo[2] = lo.z; hdr->root_lo[3] = 0.f;
            hdr->root_hi[0] = hi.x; hdr->root_hi[1] = hi.y; hdr->root_hi[2] = hi.z; hdr->root_hi[3] = 0.f;
            if (cnt == 0) parent_of[ref] = -1;
            return;
        }
        // prefix lengths at the splits r|r+1 and l-1|l (this block's from shared memory)
        const int dr = (r == U - 1) ? -1
                       : (r + 1 >= k0 && r + 1 <= k0 + B) ? s_d[r + 1 - k0] : prefix_len(ukey, r, r + 1);
        const int dl = (l == 0) ? -1 : (l >= k0 && l <= k0 + B) ? s_d[l - k0] : prefix_len(ukey, l - 1, l);
        const bool left = dr > dl;
        const uint32_t p = left ? r : l - 1;
        const int slot = left ? 0 : 1;
        float4 *nd = nodes + 4 * (size_t)p;
        const uint32_t q = p - k0;
        if (p >= k0 && q < (uint32_t)B && s_loc[q]) {
            // both children are this block's: each leaves its slot in shared memory (the
            // block writes the node out); the second to arrive carries on
            s_r0[slot][q] = make_float4(lo.x, lo.y, lo.z, hi.x);
            s_r1[slot][q] = make_float4(hi.y, hi.z, __int_as_float(ref), __int_as_float(cnt));
            __threadfence_block();
            const int32_t o = atomicExch(&s_oth[q], (int32_t)(left ? l : r));
            if (o < 0) return;  // first child here: the sibling finishes the node
            __threadfence_block();
            const float4 a = lds_f4(&s_r0[slot ^ 1][q]), b = lds_f4(&s_r1[slot ^ 1][q]);
            const float3 slo = make_float3(a.x, a.y, a.z), shi = make_float3(a.w, b.x, b.y);
            const int32_t sref = __float_as_int(b.z), scnt = __float_as_int(b.w);
            // inner children of a node inside the block are inside it too
            if (cnt == 0) s_par[ref - (int32_t)k0] = (int32_t)p;
            if (scnt == 0) s_par[sref - (int32_t)k0] = (int32_t)p;
            lo = make_float3(fminf(lo.x, slo.x), fminf(lo.y, slo.y), fminf(lo.z, slo.z));
            hi = make_float3(fmaxf(hi.x, shi.x), fmaxf(hi.y, shi.y), fmaxf(hi.z, shi.z));
            if (left) r = (uint32_t)o;
            else l = (uint32_t)o;
            s_sub[q] = range_size(l, r);
            s_rng[q] = make_uint2(l, r);  // distinct-code range of inner node p
            ref = (int32_t)p;
            cnt = 0;
            continue;
        }
        // Node p spans blocks.  Its second child arrives here only when both children
        // are this kernel's (p is the split at a block edge, one per edge); the node
        // then goes to k_emit_top, which climbs the rest of the tree.
        slot_write(nd, slot, lo, hi, ref, cnt);
        if (cnt == 0) parent_of[ref] = (int32_t)p;
        const int32_t o = exch_acq_rel(&other[p], (int32_t)(left ? l : r));
        if (o < 0) return;
        emit_merge_global(nd, slot, lo, hi);
        if (left) r = (uint32_t)o;
        else l = (uint32_t)o;
        subtree[p] = range_size(l, r);
        range[p] = make_uint2(l, r);
        const uint32_t k = atomicAdd(top_n, 1u);
        if (k >= top_cap) {
            atomicOr(err, GBT_DEVERR_CAPACITY);
            return;
        }
        top[k] = EmitState{{lo.x, lo.y, lo.z}, {hi.x, hi.y, hi.z}, l, r, p, 0u, {0u, 0u}};
        return;
    }
}

// Each leaf's primitive records are made here, from the sorted indices and the vertices,
// and its box is taken from the values in registers (one pass over the records instead of
// a gather launch that writes them and an emission that reads them back).
__global__ void __launch_bounds__(EMIT_THREADS, 8) k_emit(const BvhHeader *hdr_in, BvhHeader *hdr,
                                                       const uint32_t *__restrict__ run,
                                                       const uint64_t *__restrict__ ukey,
                                                       float4 *__restrict__ recs, float4 *nodes, int32_t *other,
                                                       uint32_t *subtree, int32_t *parent_of, uint2 *range,
                                                       uint32_t n, EmitState *top, uint32_t *top_n, uint32_t top_cap,
                                                       unsigned int *err, const SortPlan *__restrict__ plan,
                                                       const float *__restrict__ verts, const float4 *__restrict__ sph,
                                                       uint32_t n_tri) {
    gbt_pdl_wait();
    gbt_pdl_trigger();
    if (sort_failed(err)) return;
    constexpr int B = EMIT_THREADS, NW = B / 32;
    // s_d[i]: common prefix length at the split k0-1+i | k0+i (i = 0..B), -1 past
    // either end of the codes.  s_loc[t]: inner node k0+t has its whole range in
    // this block's leaves [k0, k0+B).  A node k covers the widest range around
    // split k whose splits all share at least its prefix length, so its range
    // stays inside iff a shorter prefix occurs among the block's splits on both
    // sides of k (the splits k0-1 and k0+B-1 at the block's edges included).
    __shared__ int s_d[B + 1];
    __shared__ int s_suf[B];
    __shared__ int s_wpre[NW], s_wsuf[NW];
    __shared__ int32_t s_oth[B];
    __shared__ float4 s_r0[2][B];  // per inner node, per child slot: lo.xyz, hi.x
    __shared__ float4 s_r1[2][B];  //                                 hi.yz, ref, count
    __shared__ uint32_t s_sub[B];  // per inner node: subtree size
    __shared__ uint2 s_rng[B];     //                 distinct-code range
    __shared__ int32_t s_par[B];   //                 parent when that is the block's too (-2: not)
    __shared__ uint8_t s_loc[B];
    const uint32_t U = hdr_in->n_unique;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const uint32_t k0 = blockIdx.x * B;
    for (int i = t; i <= B; i += B) {
        const long long j = (long long)k0 - 1 + i;  // split j | j+1
        s_d[i] = (j >= 0 && j + 1 < (long long)U) ? prefix_len(ukey, (uint32_t)j, (uint32_t)j + 1) : -1;
    }
    s_oth[t] = -1;
    s_par[t] = -2;
    __syncthreads();
    // pre = min s_d[0..t]; suf = min s_d[t+1..B-1+1] (inclusive scans, warp shuffles + warp totals)
    int pre = s_d[t], suf = s_d[t + 1];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int a = __shfl_up_sync(0xffffffffu, pre, o), b = __shfl_down_sync(0xffffffffu, suf, o);
        if (lane >= o) pre = min(pre, a);
        if (lane + o < 32) suf = min(suf, b);
    }
    if (lane == 31) s_wpre[w] = pre;
    if (lane == 0) s_wsuf[w] = suf;
    __syncthreads();
    for (int k = 0; k < NW; k++) {
        if (k < w) pre = min(pre, s_wpre[k]);
        if (k > w) suf = min(suf, s_wsuf[k]);
    }
    s_suf[t] = suf;  // min s_d[t+1..B]
    __syncthreads();
    {
        // node k0+t is split t+1: shorter prefixes needed in s_d[0..t] and s_d[t+2..B]
        const int dk = s_d[t + 1];
        const int right = t + 1 < B ? s_suf[t + 1] : 64;
        s_loc[t] = (dk >= 0 && pre < dk && right < dk) ? 1 : 0;
    }
    __syncthreads();

    const uint32_t u = k0 + t;
    if (u < U && u < n) emit_climb(hdr, run, ukey, recs, nodes, other, parent_of, subtree, range, top, top_n,
                                   top_cap, err, plan, verts, sph, n_tri, U, k0, u, s_d, s_oth, s_r0, s_r1, s_sub,
                                   s_rng, s_par, s_loc);
    // The block's inner nodes, whose two child slots the climb left in shared memory, are
    // written out with consecutive threads on consecutive 16-byte words.
    __syncthreads();
    for (int j = t; j < 4 * B; j += B) {
        const int q = j >> 2, part = j & 3;
        if (!s_loc[q]) continue;
        const float4 a0 = s_r0[0][q], a1 = s_r1[0][q], b0 = s_r0[1][q], b1 = s_r1[1][q];
        float4 v;
        if (part == 0) v = make_float4(a0.x, a0.w, a0.y, a1.x);       // left child: lo.x, hi.x, lo.y, hi.y
        else if (part == 1) v = make_float4(b0.x, b0.w, b0.y, b1.x);  // right child
        else if (part == 2) v = make_float4(a0.z, a1.y, b0.z, b1.y);  // lo.z, hi.z of both
        else v = make_float4(a1.z, a1.w, b1.z, b1.w);                 // ref, count of both
        nodes[4 * (size_t)(k0 + q) + part] = v;
    }
    if (s_loc[t]) {
        subtree[k0 + t] = s_sub[t];
        range[k0 + t] = s_rng[t];
    }
    if (s_par[t] != -2) parent_of[k0 + t] = s_par[t];
}

// The nodes that span blocks: one thread per node k_emit handed over, climbing
// with the global hand-off word (the same walk as k_emit, by split prefixes
// read from the codes).
__global__ void __launch_bounds__(128) k_emit_top(BvhHeader *hdr, const uint64_t *__restrict__ ukey, float4 *nodes,
                                                  int32_t *other, uint32_t *subtree, int32_t *parent_of,
                                                  uint2 *range, const EmitState *__restrict__ top,
                                                  const uint32_t *top_n, uint32_t top_cap, const unsigned int *err) {
    gbt_pdl_wait();
    gbt_pdl_trigger();
    if (sort_failed(err)) return;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= min(*top_n, top_cap)) return;
    const uint32_t U = hdr->n_unique;
    const EmitState e = top[i];
    float3 lo = make_float3(e.lo[0], e.lo[1], e.lo[2]), hi = make_float3(e.hi[0], e.hi[1], e.hi[2]);
    uint32_t l = e.l, r = e.r;
    int32_t ref = (int32_t)e.ref;
    // prefix lengths at the splits l-1|l and r|r+1 (-1 past either end of the codes); a
    // step changes one end, whose new prefix is read together with the sibling's box
    int dl = l == 0 ? -1 : prefix_len(ukey, l - 1, l);
    int dr = r == U - 1 ? -1 : prefix_len(ukey, r, r + 1);
    for (;;) {
        if (l == 0 && r == U - 1) {
            hdr->root_ref = ref;
            hdr->root_cnt = 0;
            hdr->root_lo[0] = lo.x; hdr->root_lo[1] = lo.y; hdr->root_lo[2] = lo.z; hdr->root_lo[3] = 0.f;
            hdr->root_hi[0] = hi.x; hdr->root_hi[1] = hi.y; hdr->root_hi[2] = hi.z; hdr->root_hi[3] = 0.f;
            parent_of[ref] = -1;
            return;
        }
        const bool left = dr > dl;  // l == 0 (dl = -1, r < U - 1) goes left, r == U - 1 right
        const uint32_t p = left ? r : l - 1;
        const int slot = left ? 0 : 1;
        float4 *nd = nodes + 4 * (size_t)p;
        slot_write(nd, slot, lo, hi, ref, 0);
        parent_of[ref] = (int32_t)p;
        const int32_t o = exch_acq_rel(&other[p], (int32_t)(left ? l : r));
        if (o < 0) return;
        if (left) {
            r = (uint32_t)o;
            dr = r == U - 1 ? -1 : prefix_len(ukey, r, r + 1);
        } else {
            l = (uint32_t)o;
            dl = l == 0 ? -1 : prefix_len(ukey, l - 1, l);
        }
        emit_merge_global(nd, slot, lo, hi);
        subtree[p] = range_size(l, r);
        range[p] = make_uint2(l, r);
        ref = (int32_t)p;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Programmatic dependent launches between a build's kernels: 0 never, 1 always, 2 for
// sorts of at most 8 tiles per SM, whose kernels are short enough for the launch
// latency between them to count.
#ifndef GBT_LBVH_PDL
#define GBT_LBVH_PDL 2
#endif
static bool lbvh_pdl(uint32_t n_tiles, int num_sms) {
    return GBT_LBVH_PDL == 1 || (GBT_LBVH_PDL == 2 && n_tiles <= (uint32_t)num_sms * 8u);
}

// Emission blocks: one per EMIT_THREADS distinct codes; at most one node per
// block edge goes to k_emit_top.
static uint32_t emit_blocks(uint32_t n) { return (n + EMIT_THREADS - 1) / EMIT_THREADS; }

static size_t lbvh_scratch_layout(uint32_t n, size_t *acc_off, SortScratch *ss, size_t *rle_off,
                                  size_t *top_off = nullptr) {
    *acc_off = 0;
    *ss = sort_layout(n, gbt_align(6 * sizeof(unsigned long long)));
    *rle_off = ss->total;
    uint32_t rt = (n + RLE_TILE - 1) / RLE_TILE;
    const size_t t = gbt_align(*rle_off + (size_t)(rt + 1) * sizeof(uint32_t));
    if (top_off) *top_off = t;
    // counter (16 bytes), then the hand-over list
    return gbt_align(t + 16 + (size_t)emit_blocks(n) * sizeof(EmitState));
}

size_t gbt_lbvh_scratch_bytes(uint32_t n) {
    size_t a, r;
    SortScratch s;
    return lbvh_scratch_layout(n, &a, &s, &r);
}

static int sort_enqueue(gbt_ctx *ctx, unsigned char *sbase, const SortScratch &ss, uint64_t *kA, uint32_t *vA,
                        uint64_t *kB, uint32_t *vB, uint32_t n, int identity_vals, BvhHeader *hdr, bool pdl) {
    cudaStream_t st = ctx->stream;
    SortPlan *plan = reinterpret_cast<SortPlan *>(sbase + ss.plan);
    uint32_t *hist = reinterpret_cast<uint32_t *>(sbase + ss.hist);
    uint32_t *ctr = reinterpret_cast<uint32_t *>(sbase + ss.ctr);
    uint32_t *status = reinterpret_cast<uint32_t *>(sbase + ss.status);
    // the histograms, tile counters and look-back words were zeroed before the build's first kernel
    GBT_CUDA(ctx, gbt_launch_pdl(pdl, k_hist, ctx->num_sms * 2, 256, 0, st, kA, n, hist));
    GBT_CUDA(ctx, gbt_launch_pdl(pdl, k_sort_plan, 1, 256, 0, st, plan, hist, n, kA, vA, kB, vB, identity_vals, hdr));
    GBT_CUDA(ctx, onesweep_passes(ctx->sort_threads, ctx->num_sms, plan, n, ss.n_tiles, status, ctr, ctx->d_error, ctx->spin_limit,
                                  ctx->withhold_tile, st, pdl));
    return GBT_OK;
}

int gbt_lbvh_enqueue(gbt_ctx *ctx, gbt_bvh *bvh) {
    gbt_scene *sc = bvh->scene;
    const uint32_t n_tri = sc->n_tri, n = sc->n_tri + sc->n_sph;
    if (n == 0) return gbt_fail(ctx, GBT_EINVAL, "empty scene");
    if (n >= (1u << 30)) return gbt_fail(ctx, GBT_EINVAL, "scene larger than 2^30 primitives");
    size_t acc_off, rle_off, top_off;
    SortScratch ss;
    size_t need = lbvh_scratch_layout(n, &acc_off, &ss, &rle_off, &top_off);
    void *scr = nullptr;
    int rc = gbt_scratch(ctx, need, &scr);
    if (rc) return rc;
    unsigned char *sb = static_cast<unsigned char *>(scr);
    cudaStream_t st = ctx->stream;
    unsigned long long *acc = reinterpret_cast<unsigned long long *>(sb + acc_off);
    uint32_t *top_n = reinterpret_cast<uint32_t *>(sb + top_off);
    EmitState *top = reinterpret_cast<EmitState *>(sb + top_off + 16);
    const bool pdl = lbvh_pdl(ss.n_tiles, ctx->num_sms);
    // Every buffer the build's kernels expect zeroed (or -1) is set before its first
    // kernel, so that the kernels follow one another as programmatic dependent launches.
    GBT_CUDA(ctx, cudaMemsetAsync(acc, 0xff, 3 * sizeof(unsigned long long), st));
    GBT_CUDA(ctx, cudaMemsetAsync(acc + 3, 0x00, 3 * sizeof(unsigned long long), st));
    GBT_CUDA(ctx, cudaMemsetAsync(sb + ss.hist, 0, ss.total - ss.hist, st));
    GBT_CUDA(ctx, cudaMemsetAsync(bvh->d_other, 0xff, (size_t)n * sizeof(int32_t), st));
    GBT_CUDA(ctx, cudaMemsetAsync(top_n, 0, sizeof(uint32_t), st));
    int grid = ctx->num_sms * 8;
    int g2 = (int)((n + 255) / 256);
    if (g2 < grid) grid = g2;
    // the scene box: each block ends with six atomics on the same six words
    const int gb = std::min(grid, ctx->num_sms * GBT_BOUNDS_BLOCKS_PER_SM);
    k_bounds<<<gb, 256, 0, st>>>(sc->d_verts, sc->d_sph, n_tri, n, acc);
    GBT_CUDA(ctx, gbt_launch_pdl(pdl, k_morton, grid, 256, 0, st, sc->d_verts, sc->d_sph, n_tri, n,
                                 (const unsigned long long *)acc, bvh->d_codes));
    rc = sort_enqueue(ctx, sb, ss, bvh->d_codes, bvh->d_idx, bvh->d_codes + n, bvh->d_idx + n, n, 1, bvh->d_hdr, pdl);
    if (rc) return rc;
    const SortPlan *plan = reinterpret_cast<const SortPlan *>(sb + ss.plan);
    uint32_t rt = (n + RLE_TILE - 1) / RLE_TILE;
    uint32_t *tcnt = reinterpret_cast<uint32_t *>(sb + rle_off);
    const unsigned int *cerr = ctx->d_error;
    GBT_CUDA(ctx, gbt_launch_pdl(pdl, k_rle_count, rt, RLE_THREADS, 0, st, plan, n, tcnt, cerr));
    GBT_CUDA(ctx, gbt_launch_pdl(pdl, k_rle_scan, 1, 1024, 0, st, tcnt, rt, bvh->d_hdr, cerr));
    GBT_CUDA(ctx, gbt_launch_pdl(pdl, k_rle_write, rt, RLE_THREADS, 0, st, plan, n, (const uint32_t *)tcnt, bvh->d_run,
                                 bvh->d_ukey, cerr));
    const uint32_t eb = emit_blocks(n);
    GBT_CUDA(ctx, gbt_launch_pdl(pdl, k_emit, eb, EMIT_THREADS, 0, st, (const BvhHeader *)bvh->d_hdr, bvh->d_hdr,
                                 (const uint32_t *)bvh->d_run, (const uint64_t *)bvh->d_ukey, bvh->d_prims,
                                 bvh->d_nodes, bvh->d_other, bvh->d_size, bvh->d_parent, bvh->d_range, n, top, top_n,
                                 eb, ctx->d_error, plan, (const float *)sc->d_verts, (const float4 *)sc->d_sph, n_tri));
    GBT_CUDA(ctx, gbt_launch_pdl(pdl, k_emit_top, (eb + 127) / 128, 128, 0, st, bvh->d_hdr, (const uint64_t *)bvh->d_ukey,
                                 bvh->d_nodes, bvh->d_other, bvh->d_size, bvh->d_parent, bvh->d_range,
                                 (const EmitState *)top, (const uint32_t *)top_n, eb, (const unsigned int *)ctx->d_error));
    GBT_CUDA(ctx, cudaGetLastError());
    return GBT_OK;
}

// ---------------------------------------------------------------------------
// pair sort into caller-given scratch (used by the entry point that allocates nothing)
// ---------------------------------------------------------------------------
namespace {

// All eight passes, reading the caller's codes first and ping-ponging
// out -> scratch -> out so that the sorted pairs land in the caller's output.
__global__ void __launch_bounds__(256) k_sort_plan_all(SortPlan *plan, const uint32_t *__restrict__ ghist,
                                                       const uint64_t *codes_in, uint64_t *kA, uint32_t *vA,
                                                       uint64_t *kB, uint32_t *vB) {
    __shared__ uint32_t s_tmp[8];
    const int t = threadIdx.x;
    for (int p = 0; p < 8; p++) plan->digit_base[p][t] = block_excl_scan256(ghist[p * 256 + t], s_tmp, nullptr);
    if (t == 0) {
        for (int p = 0; p < 8; p++) {
            plan->active[p] = 1;
            plan->identity[p] = p == 0 ? 1u : 0u;
            const bool to_b = (p & 1) == 0;  // pass 0: in -> B, 1: B -> A, 2: A -> B, ...
            plan->in_k[p] = p == 0 ? codes_in : (to_b ? kA : kB);
            plan->in_v[p] = to_b ? vA : vB;
            plan->out_k[p] = to_b ? kB : kA;
            plan->out_v[p] = to_b ? vB : vA;
        }
        plan->final_k = kA;
        plan->final_v = vA;
        plan->final_sel = 0;
    }
}

}  // namespace

size_t gbt_sort_static_bytes(uint32_t max_pairs) {
    SortScratch ss = sort_layout(max_pairs, 0);
    return gbt_align(ss.total + (size_t)max_pairs * (sizeof(uint64_t) + sizeof(uint32_t)) + 256);
}

int gbt_sort_pairs_static(cudaStream_t st, int num_sms, unsigned char *sbase, uint32_t max_pairs,
                          const uint64_t *codes_in, uint64_t *codes_out, uint32_t *idx_out, uint32_t n,
                          unsigned int **err_word) {
    SortScratch ss = sort_layout(n, 0);
    SortScratch smax = sort_layout(max_pairs, 0);
    uint64_t *kB = reinterpret_cast<uint64_t *>(sbase + smax.total);
    uint32_t *vB = reinterpret_cast<uint32_t *>(sbase + smax.total + (size_t)max_pairs * sizeof(uint64_t));
    unsigned int *err = reinterpret_cast<unsigned int *>(
        sbase + gbt_align(smax.total + (size_t)max_pairs * (sizeof(uint64_t) + sizeof(uint32_t))));
    *err_word = err;
    SortPlan *plan = reinterpret_cast<SortPlan *>(sbase + ss.plan);
    uint32_t *hist = reinterpret_cast<uint32_t *>(sbase + ss.hist);
    uint32_t *ctr = reinterpret_cast<uint32_t *>(sbase + ss.ctr);
    uint32_t *status = reinterpret_cast<uint32_t *>(sbase + ss.status);
    // state left by the previous call: histograms, tile counters, look-back words, error word
    if (cudaMemsetAsync(sbase + ss.hist, 0, ss.total - ss.hist, st) != cudaSuccess) return GBT_ECUDA;
    if (cudaMemsetAsync(err, 0, sizeof(unsigned int), st) != cudaSuccess) return GBT_ECUDA;
    k_hist<<<num_sms * 2, 256, 0, st>>>(codes_in, n, hist);
    k_sort_plan_all<<<1, 256, 0, st>>>(plan, hist, codes_in, codes_out, idx_out, kB, vB);
    return onesweep_passes(256, num_sms, plan, n, ss.n_tiles, status, ctr, err, GBT_SPIN_LIMIT, 0xffffffffu, st,
                           lbvh_pdl(ss.n_tiles, num_sms)) == cudaSuccess
               ? GBT_OK
               : GBT_ECUDA;
}
