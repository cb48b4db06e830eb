// FP64 exponential for the flux-statistics passes.
//
// The table-driven method of P. T. P. Tang ("Table-driven implementation of
// the exponential function in IEEE floating-point arithmetic", ACM Trans.
// Math. Softw. 15(2), 1989) with a table of 2^(j/256):
//     y = k ln2/256 + r,  k = 256 m + j (0 <= j < 256),  |r| <= ln2/512,
//     exp(y) = 2^m 2^(j/256) (1 + p(r)),  p(r) = r + r^2/2! + ... + r^5/5!
// (Taylor; the truncation r^6/6! is below 1e-20).  k is rounded with the
// 1.5 x 2^52 shift, r is formed by two FMAs with ln2/256 split into a head and
// a tail (Cody-Waite), and 2^m enters through the exponent field.  Ten FP64
// operations on the common path (|y| < 708); this GPU runs FP64 at 1/64 of the
// FP32 rate and the flux passes are bound by it.  Within about one ulp of
// exp (tested against CUDA's exp).
//
// tab: 2^(j/256), j < 256, rounded to double (fsg_exp_table fills it).
#pragma once

namespace fsg {

__device__ __forceinline__ double fexp(double y, const double *__restrict__ tab)
{
    constexpr double INV_L = 369.3299304675746;       // 256 / ln 2
    constexpr double L_HI = 0.0027076061740622863;    // ln 2 / 256, head
    constexpr double L_LO = 9.058776616587108e-20;    // ln 2 / 256 - L_HI
    constexpr double SHIFT = 6755399441055744.0;      // 1.5 x 2^52
    constexpr double C2 = 0.5, C3 = 0.16666666666666666, C4 = 0.041666666666666664,
                     C5 = 0.008333333333333333;
    const int ahi = __double2hiint(y) & 0x7fffffff;
    const bool wide = ahi >= 0x40862000;   // |y| >= 708, inf or NaN
    double yc = y;
    if (wide) {
        if (y != y)
            return y + y;
        yc = fmin(fmax(y, -800.0), 800.0);
    }
    const double t = fma(yc, INV_L, SHIFT);
    const int k = __double2loint(t);
    const double kd = t - SHIFT;
    double r = fma(kd, -L_HI, yc);
    r = fma(kd, -L_LO, r);
    double c = fma(r, C5, C4);
    c = fma(c, r, C3);
    c = fma(c, r, C2);
    const double p = fma(c, r * r, r);
    const double tj = __ldg(tab + (k & 255));
    const double res = fma(tj, p, tj);   // in [0.998, 2.003)
    const int m = k >> 8;
    if (!wide)
        return __longlong_as_double(__double_as_longlong(res) + ((long long)m << 52));
    // outside (-708, 708): two exact power-of-two factors, one rounding
    // (subnormal results, overflow to inf, underflow to 0)
    const int m1 = m / 2, m2 = m - m1;
    const double s1 = __longlong_as_double((long long)(m1 + 1023) << 52);
    const double s2 = __longlong_as_double((long long)(m2 + 1023) << 52);
    return res * s1 * s2;
}

}  // namespace fsg
