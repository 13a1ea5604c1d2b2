// crpow.cuh -- pow(x, 0.2) rounded to nearest from a double-double evaluation.
//
// The reference's step-size factor is (tol/(est + EPS))**(1/5)
// (oneka/capturezone.py:247), i.e. libm pow(x, 0.2) with 0.2 the double
// nearest 1/5.  This evaluates exp(0.2 * log(x)) in double-double arithmetic
// (Dekker 1971 error-free products and sums) to about 2^-75 relative error and
// rounds once, so the result is the correctly rounded power except when x^0.2
// lies within ~2^-75 of a rounding midpoint.
//
//   log x = e ln2 + log(c) + 2 atanh(s),  x = 2^e m, c = 1 + i/64 nearest m,
//           s = (m - c)/(m + c), |s| < 2^-7;
//   exp y = 2^(k/64) exp(r),  k = round(64 y / ln2), |r| <= ln2/128,
// with log(c) and 2^(j/64) from double-double tables (dd_tables.h).
//
// Compiled as device code under nvcc and as plain C++ elsewhere (the CPU
// tests check it against mpmath).  Needs round-to-nearest with no FMA
// contraction (--fmad=false / -ffp-contract=off).
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "dd_tables.h"

#ifdef __CUDACC__
#define ONEKA_HD __device__ __forceinline__
#define ONEKA_DDTAB __device__ const
#else
#define ONEKA_HD static inline
#define ONEKA_DDTAB static const
#endif

namespace oneka {
namespace crpow_detail {

ONEKA_DDTAB double kLogTable[130] = {ONEKA_DD_LOG_TABLE};
ONEKA_DDTAB double kExp2Table[128] = {ONEKA_DD_EXP2_TABLE};

ONEKA_HD void two_sum(double a, double b, double& s, double& e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

ONEKA_HD void fast_two_sum(double a, double b, double& s, double& e) {
    s = a + b;
    e = b - (s - a);
}

ONEKA_HD void two_prod(double a, double b, double& p, double& e) {
    p = a * b;
    e = fma(a, b, -p);
}

ONEKA_HD double scale2(double x, int n) {
    // x * 2^n for a normal result, by exponent arithmetic
    uint64_t b;
    memcpy(&b, &x, 8);
    b += (uint64_t)(int64_t)n << 52;
    memcpy(&x, &b, 8);
    return x;
}

}  // namespace crpow_detail

// x**0.2 for x >= 0 (NaN for NaN or negative x).
ONEKA_HD double cr_pow_fifth(double x) {
    using namespace crpow_detail;
    if (!(x > 0.0)) return (x == 0.0) ? 0.0 : (x - x) / (x - x);   // 0 -> 0, NaN/neg -> NaN
    if (x == (double)INFINITY) return x;
    // x = 2^e * m, m in [1, 2)
    uint64_t bits;
    memcpy(&bits, &x, 8);
    int e = (int)((bits >> 52) & 0x7ff);
    if (e == 0) {   // subnormal: scale by 2^54 first
        double xs = x * 18014398509481984.0;
        memcpy(&bits, &xs, 8);
        e = (int)((bits >> 52) & 0x7ff) - 54;
    }
    e -= 1023;
    uint64_t mb = (bits & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
    double m;
    memcpy(&m, &mb, 8);
    // c = 1 + i/64 nearest to m; d = m - c exact; t = m + c as a double-double
    const int i = (int)((m - 1.0) * 64.0 + 0.5);
    const double c = 1.0 + (double)i * 0.015625;
    const double d = m - c;
    double th, tl;
    two_sum(m, c, th, tl);
    // s = d / t to double-double accuracy
    const double sh = d / th;
    const double sl = (fma(-sh, th, d) - sh * tl) / th;
    // 2 atanh(s) = 2s + (2/3)s^3 + (2/5)s^5 + ...
    const double s2 = sh * sh;
    const double tail = sh * s2 * (2.0 / 3.0 + s2 * (2.0 / 5.0 + s2 * (2.0 / 7.0 + s2 * (2.0 / 9.0 + s2 * (2.0 / 11.0)))));
    // log x = e*ln2 + log(c) + 2s + tail, summed in double-double
    const double a_hi = (double)e * ONEKA_LN2_HI;   // exact: 42-bit constant, |e| < 2^11
    double s1, e1, s3, e3;
    two_sum(a_hi, kLogTable[2 * i], s1, e1);
    two_sum(s1, 2.0 * sh, s3, e3);
    double lo = e1 + e3 + ((double)e * ONEKA_LN2_LO + kLogTable[2 * i + 1] + 2.0 * sl + tail);
    double Lh, Ll;
    fast_two_sum(s3, lo, Lh, Ll);
    // y = 0.2 * log x
    double yh, yl;
    two_prod(0.2, Lh, yh, yl);
    yl += 0.2 * Ll;
    fast_two_sum(yh, yl, yh, yl);
    // y = k ln2/64 + r
    const double kd = nearbyint(yh * ONEKA_64_OVER_LN2);
    const int k = (int)kd;
    const double ra = yh - kd * ONEKA_LN2_64_HI;   // exact: 38-bit constant, |k| < 2^15
    double rh, re;
    two_sum(ra, -(kd * ONEKA_LN2_64_MID), rh, re);  // the product is exact, the sum is not
    double rl = re + (yl - kd * ONEKA_LN2_64_LO);
    fast_two_sum(rh, rl, rh, rl);
    // exp(rh) = 1 + rh + rh^2/2 + rh^3 p(rh), then * (1 + rl)
    double q2h, q2l;
    two_prod(rh, rh, q2h, q2l);
    const double p = rh * q2h *
        (1.0 / 6.0 + rh * (1.0 / 24.0 + rh * (1.0 / 120.0 + rh * (1.0 / 720.0 + rh * (1.0 / 5040.0 + rh * (1.0 / 40320.0 + rh * (1.0 / 362880.0)))))));
    double u1, f1, u2, f2;
    two_sum(1.0, rh, u1, f1);
    two_sum(u1, 0.5 * q2h, u2, f2);
    double Eh, El;
    fast_two_sum(u2, f1 + f2 + 0.5 * q2l + p, Eh, El);
    El += Eh * rl;
    // 2^(j/64) * E, then 2^(k div 64)
    const int j = k & 63;
    const int kq = (k - j) / 64;
    const double Th = kExp2Table[2 * j], Tl = kExp2Table[2 * j + 1];
    double Ph, Pl;
    two_prod(Th, Eh, Ph, Pl);
    Pl += Th * El + Tl * Eh;
    const double r = Ph + Pl;   // rounds the double-double to nearest
    return scale2(r, kq);
}

}  // namespace oneka
