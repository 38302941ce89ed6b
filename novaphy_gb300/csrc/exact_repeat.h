// Exact repeated addition: the float that m additions s = s + t (each
// rounded to nearest, ties to even, as a single float add) leave, in a few
// dozen steps instead of m.
//
// Within one binade [2^e, 2^(e+1)) of |s| every float is a multiple of
// u = 2^(e-23), so |s| + t rounds to |s| + D u with D the nearest integer to
// t / u (for a tie, the choice that leaves |s| / u even).  D stays the same
// for every later sum while the exact sums stay in the binade (and, for a
// tie, while |s| / u stays even, which a tie's rounding makes it), so those
// additions collapse into one multiplication, counted in 64-bit integers in
// units of u / 2^25, where every value involved is exact.  Each loop pass
// does one real float addition (which also settles zeros, signs, infinities
// and NaN exactly as the plain loop would) and then one such jump; the binade
// changes a few dozen times at most.  Subnormal sums, the top binade, terms
// of more than a quarter of |s| and runs of up to 16 are left to single
// additions.
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

PBF_HD inline uint32_t rep_bits(float x) {
    uint32_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
}

PBF_HD inline float rep_float(uint32_t b) {
    float x;
    std::memcpy(&x, &b, sizeof x);
    return x;
}

PBF_HD inline float rep_add(float s, float t, uint32_t m) {
    if (m <= 16u) {  // short runs: the additions themselves are cheaper
        for (; m > 0u; --m) s = s + t;
        return s;
    }
    while (m > 0u) {
        const float s1 = s + t;
        --m;
        if (m == 0u || s1 != s1 || s1 == s) return s1;  // done, NaN, or absorbed
        s = s1;
        const uint32_t sb = rep_bits(s), tb = rep_bits(t);
        const int es = (int)((sb >> 23) & 0xffu), et = (int)((tb >> 23) & 0xffu);
        // Single additions for subnormal or top-binade sums, subnormal or
        // non-finite terms, and terms of more than a quarter of |s|.
        if (es < 1 || es > 253 || et < 1 || et == 255) continue;
        const int d = es - et;
        if (d < 2) continue;
        if (d > 24) return s;  // |t| < u / 2: absorbed from here on
        // In units of u / 2^25 (u = 2^(es - 150), the spacing of the binade):
        // |s| = S u exactly, and x = S + t' / u with t' = t as |s| sees it.
        const int64_t S = (int64_t)((sb & 0x7fffffu) | 0x800000u);
        const int64_t MT = (int64_t)((tb & 0x7fffffu) | 0x800000u);
        const int64_t one = (int64_t)1 << 25, half = one >> 1;
        const int64_t X = (S << 25) + (((sb ^ tb) >> 31) ? -(MT << (25 - d)) : (MT << (25 - d)));
        const int64_t fl = X >> 25, fr = X & (one - 1);
        const int64_t r = fr > half ? fl + 1 : (fr < half ? fl : ((fl & 1) ? fl + 1 : fl));
        const int64_t D = r - S;  // the rounded step, in units of u
        if (D == 0) return s;
        if (fr == half && (D & 1)) continue;  // a tie flips the parity: step singly
        // Additions j = 0, 1, ... whose exact sum stays in the binade [2^23, 2^24) u.
        const int64_t LO = (int64_t)1 << 48, HI = (int64_t)1 << 49;
        int64_t k;
        if (D > 0) k = X < HI ? (HI - 1 - X) / (D << 25) + 1 : 0;
        else k = X >= LO ? (X - LO) / ((-D) << 25) + 1 : 0;
        if (k <= 0) continue;
        if (k > (int64_t)m) k = (int64_t)m;
        const int64_t A = S + k * D;  // |s| / u after the k additions, in [2^23, 2^24]
        const uint32_t mag = A == ((int64_t)1 << 24) ? (uint32_t)(es + 1) << 23
                                                     : ((uint32_t)es << 23) | (uint32_t)(A - 0x800000);
        s = rep_float(mag | (sb & 0x80000000u));
        m -= (uint32_t)k;
    }
    return s;
}

}  // namespace pbf
