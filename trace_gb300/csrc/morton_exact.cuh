// Morton quantisation in float32 pairs, shared by the device (lbvh.cu) and a
// host-side unit test.  The reference quantises in float64 (lbvh.go:64-73):
// q = uint64(|min - (lo + hi) * 0.5| / (extent / (2^21 - 1))).  GB300 issues
// float64 at a small fraction of its float32 rate, so a triangle axis is
// quantised in pairs of float32 values and only the rare values near an
// integer take the float64 path.
#pragma once

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define GBT_MHD __host__ __device__ __forceinline__
#else
#define GBT_MHD static inline
#endif

namespace gbt_morton {

// Single float32 operations, rounded to nearest, never contracted.
#ifdef __CUDA_ARCH__
GBT_MHD float fadd_rn(float a, float b) { return __fadd_rn(a, b); }
GBT_MHD float fsub_rn(float a, float b) { return __fsub_rn(a, b); }
GBT_MHD float fmul_rn(float a, float b) { return __fmul_rn(a, b); }
GBT_MHD float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
#else
GBT_MHD float fadd_rn(float a, float b) { volatile float r = a + b; return r; }
GBT_MHD float fsub_rn(float a, float b) { volatile float r = a - b; return r; }
GBT_MHD float fmul_rn(float a, float b) { volatile float r = a * b; return r; }
GBT_MHD float fma_rn(float a, float b, float c) { return fmaf(a, b, c); }
#endif

// Morton quantisation of one triangle axis in float32 pairs (double-float
// arithmetic): v = (c - lo) / step with c = (a + b) / 2 for the triangle's
// float32 bounds a <= b, lo and 1/step given as float pairs.  Returns the
// integer part when v lies more than `margin` from an integer, else -1 (then
// the float64 path decides).  The pair arithmetic is within about 2^-44 of v
// relative, the reference's float64 roundings within 2^-52; `margin` covers
// both, including the scene's offset from the origin (axis_setup).
GBT_MHD int64_t quantise_f32x2(float a, float b, float lo_h, float lo_l, float rs_h, float rs_l,
                                                  float margin) {
    // c = a + b exactly as a pair (two-sum), then halved (exact above the subnormal range)
    const float s = fadd_rn(a, b);
    const float bv = fsub_rn(s, a);
    const float e = fadd_rn(fsub_rn(a, fsub_rn(s, bv)), fsub_rn(b, bv));
    const float ch = fmul_rn(s, 0.5f), cl = fmul_rn(e, 0.5f);
    // d = c - lo (two-sum of the high parts, low parts added, renormalised)
    const float dh0 = fsub_rn(ch, lo_h);
    const float bv2 = fsub_rn(dh0, ch);
    const float de = fadd_rn(fsub_rn(ch, fsub_rn(dh0, bv2)), fsub_rn(-lo_h, bv2));
    const float dl0 = fadd_rn(de, fsub_rn(cl, lo_l));
    const float dh = fadd_rn(dh0, dl0), dl = fsub_rn(dl0, fsub_rn(dh, dh0));
    // v = d * (1/step): exact product of the high parts (fma), cross terms added
    const float ph = fmul_rn(dh, rs_h);
    const float pe = fma_rn(dh, rs_h, -ph);
    const float pl = fadd_rn(pe, fadd_rn(fmul_rn(dh, rs_l), fmul_rn(dl, rs_h)));
    const float vh = fadd_rn(ph, pl), vl = fsub_rn(pl, fsub_rn(vh, ph));
    if (!(vh >= 0.f && vh < 4194304.f)) return -1;  // NaN, negative or beyond 22 bits: float64 path
    float fi = floorf(vh);
    float r = fadd_rn(fsub_rn(vh, fi), vl);  // vh - fi is exact
    if (r < 0.f) {
        fi = fsub_rn(fi, 1.f);
        r = fadd_rn(r, 1.f);
    } else if (r >= 1.f) {
        fi = fadd_rn(fi, 1.f);
        r = fsub_rn(r, 1.f);
    }
    if (!(r > margin && r < fsub_rn(1.f, margin)) || fi < 0.f) return -1;
    return (int64_t)fi;
}

// Per-axis constants of the float32 path from the scene's float64 bounds and
// the float64 reciprocal of the quantisation step.  The margin is 2^-18 plus
// 2^-44 of the largest coordinate magnitude measured in steps; an axis whose
// margin would exceed 1/16 (a scene far from the origin relative to its
// extent, or a zero extent) always takes the float64 path.
struct AxisF32x2 {
    float lo_h, lo_l, rs_h, rs_l, margin;
};

GBT_MHD AxisF32x2 axis_setup(double lo, double hi, double rstep) {
    AxisF32x2 a;
    a.lo_h = (float)lo;
    a.lo_l = (float)(lo - (double)a.lo_h);
    a.rs_h = (float)rstep;
    a.rs_l = (float)(rstep - (double)a.rs_h);
    const double mag = fmax(fabs(lo), fabs(hi));
    const double m = 3.814697265625e-06 + mag * rstep * 5.684341886080802e-14;  // 2^-18 + 2^-44 * mag / step
    a.margin = (m < 0.0625 && a.lo_h == a.lo_h) ? (float)m : 2.f;            // 2: never decided in float32
    return a;
}

}  // namespace gbt_morton
