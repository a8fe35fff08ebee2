// Compares boidsgpu::add_f32_f64_rn with the double arithmetic it emulates,
// (float)((double)a +- F), on random and edge-case inputs.  Prints the number
// of mismatching results and exits non-zero if there is any.
#include "boids_softfp.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

static uint32_t bits(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u; }

int main(int argc, char **argv)
{
    const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
    const double fields[] = {1.0, 1.6, 4.0, 0.63, 0.5, 1.0 / 3.0, 0.1, 123.456789, 1e-3, 7.0000001, 2.52,
                             16.0, 0.7937005259840998, 3.9999999999999996};
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> u01(0.0, 1.0);
    long bad = 0, total = 0;
    for (double F : fields) {
        const boidsgpu::SoftDouble sd = boidsgpu::soft_double(F);
        const float Ff = (float)F;
        auto check = [&](float a) {
            for (int neg = 0; neg < 2; ++neg) {
                const float want = (float)((double)a + (neg ? -F : F));
                const float got = boidsgpu::add_f32_f64_rn(a, sd, neg);
                ++total;
                if (bits(want) != bits(got)) {
                    if (bad < 10) std::printf("F=%.17g a=%.9g neg=%d want %.9g got %.9g\n", F, a, neg, want, got);
                    ++bad;
                }
            }
        };
        for (long i = 0; i < n; ++i) {
            const int kind = (int)(i % 6);
            float a;
            if (kind == 0) a = (float)(F * u01(rng));                       // in the field
            else if (kind == 1) a = (float)std::pow(10.0, -40.0 * u01(rng)); // tiny positive
            else if (kind == 2) a = -(float)(0.01 * u01(rng));               // small negative
            else if (kind == 3) a = std::nextafter(Ff, (i & 8) ? 0.f : 10.f * Ff) + (float)((u01(rng) - 0.5) * 1e-6 * F);
            else if (kind == 4) a = (float)(F / 2 + (u01(rng) - 0.5) * 1e-6 * F);
            else a = (float)(F * (1.0 + 0.01 * u01(rng)));                   // just above F
            check(a);
        }
        // every float within 4096 ulps of F, F/2, 0
        for (float c : {Ff, (float)(F / 2), 0.0f}) {
            float x = c;
            for (int k = 0; k < 4096; ++k) x = std::nextafter(x, -INFINITY);
            for (int k = 0; k < 8192; ++k, x = std::nextafter(x, INFINITY)) check(x);
        }
        check(0.0f);
        check(-0.0f);
    }
    std::printf("%ld mismatches in %ld cases\n", bad, total);
    return bad != 0;
}
