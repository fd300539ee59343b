// Host-side check of trace_gb300/csrc/morton_exact.cuh: the float32-pair
// Morton quantisation against the reference's float64 formula
// q = uint64(|min - (a + b) * 0.5| / (extent / (2^21 - 1))) on random scenes
// (unit, offset, tiny and wide extents, float64 minima as spheres give) and
// random and near-integer triangle bounds.  Every value the float32 path
// decides must equal the float64 one.  Prints "ok" and four counts, or the
// first mismatch; exit status 0 on success.  The counts are: decided, deferred
// to float64, random bounds in well-conditioned scenes, and those deferred.
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include "morton_exact.cuh"

using namespace gbt_morton;

static uint64_t state = 0x2545f4914f6cdd1dull;
static uint64_t next() {  // splitmix64
    uint64_t z = (state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static double uni() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }

static uint64_t ref_q(double lo, double step, float a, float b) {
    volatile double c = ((double)a + (double)b) * 0.5;
    volatile double dx = fabs(lo - c);
    volatile double q = dx / step;
    if (!(q < 9223372036854775808.0) || q < 0.0) return 0;
    return (uint64_t)q;
}

int main() {
    long decided = 0, deferred = 0;
    long plain = 0, plain_deferred = 0;  // random bounds in scenes the float32 path serves
    const double offsets[] = {0.0, 0.5, -3.0, 100.0, -1000.0, 12345.0};
    const double extents[] = {1.0, 1e-3, 2.0, 1000.0, 3e-5, 1e5};
    for (int sc = 0; sc < 36; sc++) {
        for (int sphere_lo = 0; sphere_lo < 2; sphere_lo++) {
            const double off = offsets[sc % 6], ext = extents[sc / 6];
            float flo = (float)off, fhi = (float)(off + ext);
            double lo = flo, hi = fhi;
            if (sphere_lo) lo = lo - ext * 1e-7 * 0.3183098861837907;  // a float64 minimum
            const double step = (hi - lo) / 2097151.0, rstep = 1.0 / step;
            const AxisF32x2 ax = axis_setup(lo, hi, rstep);
            for (int t = 0; t < 200000; t++) {
                float a, b;
                if (t % 4 == 3) {  // near an integer of the quantised axis
                    const double q = floor(uni() * 2097151.0);
                    const double c = lo + (q + (uni() - 0.5) * 1e-5) * step;
                    a = (float)(c - uni() * step * 3);
                    b = (float)(2 * c - (double)a);
                } else {
                    a = (float)(lo + uni() * (hi - lo));
                    b = (float)(lo + uni() * (hi - lo));
                }
                if (a > b) { float x = a; a = b; b = x; }
                if ((double)a < lo) a = (float)fhi;  // keep the box inside the scene
                if ((double)b > hi) b = fhi;
                if (a > b) a = b;
                const int64_t f = quantise_f32x2(a, b, ax.lo_h, ax.lo_l, ax.rs_h, ax.rs_l, ax.margin);
                const bool served = t % 4 != 3 && ax.margin < 1e-4f;
                plain += served;
                if (f < 0) {
                    deferred++;
                    plain_deferred += served;
                    continue;
                }
                decided++;
                const uint64_t r = ref_q(lo, step, a, b);
                if ((uint64_t)f != r) {
                    printf("mismatch scene %d sphere %d: a=%.9g b=%.9g fast=%lld ref=%llu margin=%g\n", sc, sphere_lo,
                           a, b, (long long)f, (unsigned long long)r, ax.margin);
                    return 1;
                }
            }
        }
    }
    printf("ok %ld %ld %ld %ld\n", decided, deferred, plain, plain_deferred);
    return 0;
}
