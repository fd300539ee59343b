// Host-side check of trace_gb300/csrc/phr_exact.cuh against float64 arithmetic:
// bary_bits over edge cases and random pairs, and the float32 screening bound
// of the SAH cost over random boxes in the screened coordinate range.
// Prints "ok <cases>" or the first mismatch; exit status 0 on success.
#include <math.h>
#include <stdio.h>
#include <stdint.h>
#include <string.h>

#include "phr_exact.cuh"

using namespace gbt_phr;

static uint64_t ref_bary(float a, float b) {
    volatile double s = (double)a + (double)b;
    volatile double h = s * 0.5;
    return f64_bits(h);
}

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next() {  // splitmix64
    uint64_t z = (state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static float bits_f(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}
static float rnd_float(int mode) {
    uint32_t u = (uint32_t)next();
    switch (mode) {
        case 0: return bits_f(u & 0x7f7fffffu | (u & 0x80000000u));           // any finite-ish
        case 1: return bits_f((u & 0x807fffffu) | ((120u + (u >> 23) % 16u) << 23));  // near 1
        case 2: return bits_f(u & 0x807fffffu);                                 // subnormal or zero
        default: return (float)((double)(int32_t)u / 65536.0);                   // grid values
    }
}

static double surface64(const float *lo, const float *hi) {
    double w = (double)hi[0] - (double)lo[0], h = (double)hi[1] - (double)lo[1], d = (double)hi[2] - (double)lo[2];
    double a = (2.0 * w) * h, b = (2.0 * w) * d, c = (2.0 * h) * d;
    return (a + b) + c;
}

int main() {
    long cases = 0;
    const float edge[] = {0.f, -0.f, 1.f, -1.f, 1e-45f, -1e-45f, 1.17549435e-38f, 3.4028235e38f, -3.4028235e38f,
                          INFINITY, -INFINITY, 0.5f, 1e30f, 1e-30f, 16777216.f, 16777217.f, 268435456.f, 3.f};
    const int ne = sizeof(edge) / sizeof(edge[0]);
    for (int i = 0; i < ne; i++)
        for (int j = 0; j < ne; j++) {
            uint64_t g = bary_bits(edge[i], edge[j]), r = ref_bary(edge[i], edge[j]);
            if (g != r) {
                printf("bary mismatch %a %a: %016llx vs %016llx\n", edge[i], edge[j], (unsigned long long)g,
                       (unsigned long long)r);
                return 1;
            }
            cases++;
        }
    for (long k = 0; k < 4000000; k++) {
        const int ma = (int)(next() % 4), mb = (int)(next() % 4);
        float a = rnd_float(ma), b = rnd_float(mb);
        if (k & 1) {  // nearby exponents, including differences of exactly 28 and 29
            uint32_t ua, ub;
            memcpy(&ua, &a, 4);
            ub = (ua & 0xff800000u) - ((uint32_t)(next() % 31) << 23);
            ub |= (uint32_t)next() & 0x807fffffu;
            if (((ub >> 23) & 0xffu) == 0xffu || ((ub >> 23) & 0xffu) > ((ua >> 23) & 0xffu)) ub = ua;
            b = bits_f(ub);
        }
        uint64_t g = bary_bits(a, b), r = ref_bary(a, b);
        if (g != r && !(isnan(a + b))) {
            printf("bary mismatch %a %a: %016llx vs %016llx\n", a, b, (unsigned long long)g, (unsigned long long)r);
            return 1;
        }
        cases++;
    }
    // screening: float32 and float64 costs of random boxes in [-2^30, 2^30] (values 0 or >= 2^-30)
    double worst = 0.0;
    for (long k = 0; k < 2000000; k++) {
        float lo[2][3], hi[2][3];
        for (int s = 0; s < 2; s++)
            for (int a = 0; a < 3; a++) {
                float x[2];
                for (int t = 0; t < 2; t++) {
                    int e = (int)(next() % 61) - 30;
                    float v = ldexpf(1.0f + (float)(next() % 8388608) / 8388608.0f, e - 1);
                    if (next() % 2) v = -v;
                    if (next() % 16 == 0) v = 0.f;
                    if (!phr_screen_ok(v)) v = 0.f;
                    x[t] = v;
                }
                if (next() % 8 == 0) x[1] = x[0];
                lo[s][a] = fminf(x[0], x[1]);
                hi[s][a] = fmaxf(x[0], x[1]);
            }
        uint32_t nl = 1 + (uint32_t)(next() % 1000000000u), nr = 1 + (uint32_t)(next() % 1000000000u);
        float c32 = surface32(lo[1], hi[1]) * count_f32(nr) + surface32(lo[0], hi[0]) * count_f32(nl);
        double c64 = surface64(lo[1], hi[1]) * (double)nr + surface64(lo[0], hi[0]) * (double)nl;
        if (!(c32 >= 0.f) || isinf(c32) || (c64 == 0.0) != (c32 == 0.f)) {
            printf("screen range violated: %a %a\n", c32, c64);
            return 1;
        }
        if (c64 > 0.0) {
            double rel = fabs((double)c32 - c64) / c64;
            if (rel > worst) worst = rel;
        }
        cases++;
    }
    const double bound = 16.1 * ldexp(1.0, -24);
    if (worst > bound / 2) {  // each side's own bound is half of the pair's
        printf("screen bound exceeded: %g > %g\n", worst, bound / 2);
        return 1;
    }
    // count_f32: within one rounding of the count
    for (long k = 0; k < 2000000; k++) {
        uint32_t c = (uint32_t)(k < 1000000 ? k : next());
        double f = (double)count_f32(c), e = (double)c;
        if (fabs(f - e) > e * ldexp(1.0, -24)) {
            printf("count_f32(%u) = %.9g\n", c, f);
            return 1;
        }
        cases++;
    }
    printf("ok %ld worst_rel %.3g\n", cases, worst);
    return 0;
}
