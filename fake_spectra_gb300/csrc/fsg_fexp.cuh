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
// operations on the common path (|y| < 708; y <= -746 gives 0 without any);
// this GPU runs FP64 at 1/64 of the FP32 rate and the flux passes are bound by
// it.  Within about one ulp of exp (tested against CUDA's exp and numpy's).
//
// tab: 2^(j/256), j < 256, rounded to double (exp_table_host computes it).
#pragma once

namespace fsg {

constexpr double FEXP_INV_L = 369.3299304675746;       // 256 / ln 2
constexpr double FEXP_L_HI = 0.0027076061740622863;    // ln 2 / 256, head
constexpr double FEXP_L_LO = 9.058776616587108e-20;    // ln 2 / 256 - FEXP_L_HI
constexpr double FEXP_SHIFT = 6755399441055744.0;      // 1.5 x 2^52

// 2^(j/256) (1 + p(r)) for y = k ln2/256 + r: returns it in [0.998, 2.003)
// and k.
__device__ __forceinline__ double fexp_core(double y, const double *__restrict__ tab, int &k)
{
    constexpr double C2 = 0.5, C3 = 0.16666666666666666, C4 = 0.041666666666666664,
                     C5 = 0.008333333333333333;
    const double t = fma(y, FEXP_INV_L, FEXP_SHIFT);
    k = __double2loint(t);
    const double kd = t - FEXP_SHIFT;
    double r = fma(kd, -FEXP_L_HI, y);
    r = fma(kd, -FEXP_L_LO, r);
    double c = fma(r, C5, C4);
    c = fma(c, r, C3);
    c = fma(c, r, C2);
    const double p = fma(c, r * r, r);
    const double tj = __ldg(tab + (k & 255));
    return fma(tj, p, tj);
}

// |y| >= 708, inf and NaN: 2^m applied as two exact power-of-two factors with
// one rounding (subnormal results, overflow to inf, underflow to 0).
static __device__ __noinline__ double fexp_wide(double y, const double *__restrict__ tab)
{
    if (y != y)
        return y + y;
    int k;
    const double res = fexp_core(fmin(fmax(y, -800.0), 800.0), tab, k);
    const int m = k >> 8;
    const int m1 = m / 2, m2 = m - m1;
    const double s1 = __longlong_as_double((long long)(m1 + 1023) << 52);
    const double s2 = __longlong_as_double((long long)(m2 + 1023) << 52);
    return res * s1 * s2;
}

__device__ __forceinline__ double fexp(double y, const double *__restrict__ tab)
{
    const int hi = __double2hiint(y);
    const int ahi = hi & 0x7fffffff;
    if (ahi >= 0x40862000) {                       // |y| >= 708, inf or NaN
        if (hi < 0 && ahi >= 0x40875000 && ahi < 0x7ff00000)
            return 0.0;                            // finite y <= -746: exp underflows
        return fexp_wide(y, tab);
    }
    int k;
    const double res = fexp_core(y, tab, k);
    // |y| < 708: the result and 2^m stay normal, so 2^m enters the exponent field
    return __longlong_as_double(__double_as_longlong(res) + ((long long)(k >> 8) << 52));
}

}  // namespace fsg
