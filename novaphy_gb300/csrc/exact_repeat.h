// Exact repeated addition: the float that m additions s = s + t (each
// rounded to nearest, ties to even, as a single float add) leave, in a few
// dozen steps instead of m.
//
// Within one binade [2^e, 2^(e+1)) of |s| every float is a multiple of
// u = 2^(e-23), so |s| + t rounds to |s| + D u with D the nearest integer to
// t / u (for a tie, the choice that leaves |s| / u even).  D stays the same
// for every later sum while the exact sums stay in the binade (and, for a
// tie, while |s| / u stays even, which a tie's rounding makes it), so those
// additions collapse into one multiplication, counted and applied in double
// precision where every value involved is exact.  Each loop pass does one
// real float addition (which also settles zeros, signs, infinities and NaN
// exactly as the plain loop would) and then one such jump; the binade changes
// a few dozen times at most.  Subnormal sums, the top binade and steps of
// more than half of |s| are left to single additions.
//
// Used for runs of identical terms: particles with bit-identical state (the
// domain clamp piles fluid into a box corner) add identical terms to every
// sum that visits them in a row.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define PBF_HD __host__ __device__
#else
#define PBF_HD
#endif

namespace pbf {

PBF_HD inline double rep_floor(double x) {
    // floor of |x| < 2^52 without the math library (exact: the cast truncates).
    const double t = (double)(long long)x;
    return (t > x) ? t - 1.0 : t;
}

PBF_HD inline double rep_pow2(int e) {
    // 2^e for -1022 <= e <= 1023, from the bits.
    const unsigned long long b = (unsigned long long)(e + 1023) << 52;
    double d;
    std::memcpy(&d, &b, sizeof d);
    return d;
}

PBF_HD inline float rep_add(float s, float t, uint32_t m) {
    while (m > 0) {
        const float s1 = s + t;
        --m;
        if (m == 0 || s1 != s1 || s1 == s) return s1;  // done, NaN, or absorbed
        s = s1;
        uint32_t bits;
        std::memcpy(&bits, &s, sizeof bits);
        const int ex = (int)((bits >> 23) & 0xffu);  // biased exponent of |s|
        if (ex < 1 || ex > 253) continue;  // |s| subnormal, or in the top binade
        const double A = (double)(s < 0.0f ? -s : s);  // |s|
        const double T = (s < 0.0f) ? -(double)t : (double)t;  // t as |s| sees it
        if (!(T < A * 0.5 && T > -A * 0.5)) continue;  // large steps: a few single adds
        const int e = ex - 127;
        const double u = rep_pow2(e - 23), lo = rep_pow2(e), hi = rep_pow2(e + 1);
        const double a = A / u;  // an integer below 2^24
        const double x = a + T / u;
        const double fl = rep_floor(x);
        const double fr = x - fl;
        double r;
        if (fr > 0.5) r = fl + 1.0;
        else if (fr < 0.5) r = fl;
        else r = (rep_floor(fl * 0.5) * 2.0 == fl) ? fl : fl + 1.0;
        const double D = r - a;
        if (D == 0.0) return s;  // absorbed from here on
        if (fr == 0.5 && rep_floor(D * 0.5) * 2.0 != D) continue;  // parity flips: step singly
        // Additions j = 0, 1, ... whose exact sum A + j D u + T stays in [lo, hi).
        double k;
        if (D > 0.0) {
            k = rep_floor((hi - A - T) / (D * u)) + 1.0;
            while (k > 0.0 && !(A + (k - 1.0) * D * u + T < hi)) k -= 1.0;
        } else {
            k = rep_floor((A + T - lo) / (-D * u)) + 1.0;
            while (k > 0.0 && !(A + (k - 1.0) * D * u + T >= lo)) k -= 1.0;
        }
        if (k <= 0.0) continue;
        if (k > (double)m) k = (double)m;
        const float An = (float)(A + k * D * u);
        s = (s < 0.0f) ? -An : An;
        m -= (uint32_t)k;
    }
    return s;
}

}  // namespace pbf
