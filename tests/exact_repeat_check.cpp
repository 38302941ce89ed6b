// Checks pbf::rep_add (novaphy_gb300/csrc/exact_repeat.h) against the plain
// loop of float additions on random and edge cases; prints the mismatch count
// and exits non-zero on any.  Built with -ffp-contract=off by
// tests/test_exact_repeat.py.
#include "exact_repeat.h"
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <random>
#include <cstring>
using namespace pbf;
static float loop_add(float s, float t, uint32_t m) { for (uint32_t i = 0; i < m; ++i) s = s + t; return s; }
static bool same(float a, float b) { uint32_t x, y; std::memcpy(&x,&a,4); std::memcpy(&y,&b,4); return x == y || (a != a && b != b); }
int main(int argc, char** argv) {
    std::mt19937_64 g(argc > 1 ? atoi(argv[1]) : 1);
    std::uniform_real_distribution<double> U(0, 1);
    long bad = 0, n = 0;
    auto check = [&](float s, float t, uint32_t m) {
        ++n; float a = rep_add(s, t, m), b = loop_add(s, t, m);
        if (!same(a, b)) { if (bad < 10) printf("MISMATCH s=%a t=%a m=%u got %a want %a\n", s, t, m, a, b); ++bad; }
    };
    for (int i = 0; i < 3000; ++i) {
        float s = (float)(std::pow(10.0, U(g) * 60 - 30) * (U(g) < 0.5 ? -1 : 1));
        float t = (float)(std::fabs(s) * std::pow(10.0, -U(g) * 9) * (U(g) < 0.5 ? -1 : 1));
        if (i % 7 == 0) s = 0.0f;
        uint32_t m = (uint32_t)(U(g) * 60000);
        check(s, t, m);
    }
    for (int i = 0; i < 3000; ++i) {  // ties at the current binade
        float s = (float)(std::pow(2.0, U(g) * 40 - 20) * (U(g) < 0.5 ? -1 : 1));
        int e; std::frexp(std::fabs(s), &e); double u = std::ldexp(1.0, e - 1 - 23);
        float t = (float)((std::floor(U(g) * 300) + 0.5) * u * (U(g) < 0.5 ? -1 : 1));
        check(s, t, (uint32_t)(U(g) * 40000));
        check(s, (float)(0.5 * u), 10);
        check(s, (float)(std::floor(U(g) * 2000) * u), (uint32_t)(U(g) * 40000));
    }
    for (int i = 0; i < 2000; ++i) {  // terms of all sizes from zero (density-like sums)
        float t = (float)(std::pow(10.0, U(g) * 50 - 35) * (U(g) < 0.3 ? -1 : 1));
        check(0.0f, t, (uint32_t)(U(g) * 100000));
        check(-0.0f, t, 3);
        float s = (float)(t * (U(g) * 200 - 100));
        check(s, t, (uint32_t)(U(g) * 100000));
    }
    for (int i = 0; i < 4000; ++i) {  // every exponent gap, both signs, long runs
        const int d = 1 + (int)(U(g) * 27);
        float s = (float)(std::ldexp(1.0 + U(g), (int)(U(g) * 80) - 40) * (U(g) < 0.5 ? -1 : 1));
        float t = (float)(std::ldexp(std::fabs((double)s) * (1.0 + U(g)), -d) * (U(g) < 0.5 ? -1 : 1));
        if (i % 5 == 0) t = (float)std::ldexp(std::floor(std::ldexp(std::fabs((double)t), 3)) + 0.5, -3);
        check(s, t, 17 + (uint32_t)(U(g) * 200000));
    }
    const float sp[] = {0.0f, -0.0f, 1.0f, -1.0f, 3.0e38f, -3.0e38f, INFINITY, -INFINITY, NAN, 1e-40f, -1e-44f, 1e-38f};
    for (float s : sp) for (float t : sp) for (uint32_t m : {0u, 1u, 2u, 3u, 17u, 1000u}) check(s, t, m);
    check(0.0f, 1e-3f, 54000); check(0.0f, 0.1f, 1u << 22); check(1.0f, 1e-8f, 100); check(16777215.0f, 0.5f, 10);
    printf("%ld cases, %ld mismatches\n", n, bad);
    return bad != 0;
}
