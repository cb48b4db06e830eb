// Voigt function H(a, u) = Re w(u + i a), w(z) = exp(-z^2) erfc(-i z), on the
// device.  This replaces profile() (fake_spectra/singleabs.h:56-61), which
// the reference evaluates with the Faddeeva package; it is this project's own
// construction:
//
//  * |z| < 8, a <= 1: Taylor series of w about the nearest tabulated real
//    point x_j = j/10, with coefficients generated on the fly from the ODE
//    w'(z) = -2 z w(z) + 2i/sqrt(pi) (Abramowitz & Stegun 7.1.20):
//      c_0 = w(x_j),  c_1 = -2 x_j c_0 + 2i/sqrt(pi),
//      (n+1) c_{n+1} = -2 x_j c_n - 2 c_{n-1}.
//    The table (voigt_table.h) holds exp(-x_j^2) and the Dawson-integral
//    values 2/sqrt(pi) F(x_j), 2/sqrt(pi) F'(x_j) to full double precision.
//    12 terms reach ~3e-15 relative for a <= 0.1, 16 for a <= 0.25, 40 for a <= 1.
//  * |z| >= 8: the asymptotic series w(z) ~ i/(sqrt(pi) z) sum_k (2k-1)!!/(2 z^2)^k
//    (A&S 7.1.23), 18 terms, plus exp(-z^2) close to the real axis.
//  * a > 1, |z| < 8: the Laplace continued fraction (A&S 7.1.15), 160 levels.
//  * a < 0: w(z) = 2 exp(-z^2) - w(-z).
#pragma once

#include "voigt_table.h"

namespace fsg {

__device__ const double d_vtab[FSG_VTAB_N][4] = FSG_VTAB_INIT;

#define FSG_INV_SQRT_PI 0.56418958354775628695

// Re of the Taylor expansion about x0 = j/10 evaluated at x + i y, N terms.
template <int N>
__device__ __forceinline__ double voigt_taylor_f64(double x, double y)
{
    const int j = __double2int_rn(x * FSG_VTAB_INVH);
    const double2 ed = __ldg(reinterpret_cast<const double2 *>(&d_vtab[j][0]));
    const double gg = __ldg(&d_vtab[j][2]);
    const double x0 = (double)j * FSG_VTAB_H;
    const double dx = x - x0;
    const double m2x = -2.0 * x0;
    double cmr = ed.x, cmi = ed.y;          // c_{n-1}
    double cr = m2x * ed.x, ci = gg;        // c_n, n = 1
    double pr = dx, pi = y;                 // delta^n
    double sr = ed.x + (cr * pr - ci * pi);
#pragma unroll
    for (int n = 1; n < N; n++) {
        const double inv = 1.0 / (double)(n + 1);
        const double nr = fma(m2x, cr, -2.0 * cmr) * inv;
        const double ni = fma(m2x, ci, -2.0 * cmi) * inv;
        const double t = fma(pr, dx, -pi * y);
        pi = fma(pr, y, pi * dx);
        pr = t;
        sr = fma(nr, pr, fma(-ni, pi, sr));
        cmr = cr;
        cmi = ci;
        cr = nr;
        ci = ni;
    }
    return sr;
}

__device__ __forceinline__ double voigt_asym_f64(double x, double y)
{
    const double den = x * x + y * y;
    const double ir = x / den, ii = -y / den;        // 1/z
    const double w2r = ir * ir - ii * ii, w2i = 2.0 * ir * ii;   // 1/z^2
    // c_k = (2k-1)!!/2^k, k = 0..17, Horner from the top
    double sr = 0.0, si = 0.0;
    double c = 1.0;
    double coef[18];
#pragma unroll
    for (int k = 0; k < 18; k++) {
        coef[k] = c;
        c *= (2.0 * k + 1.0) * 0.5;
    }
#pragma unroll
    for (int k = 17; k >= 0; k--) {
        const double tr = fma(sr, w2r, fma(-si, w2i, coef[k]));
        si = fma(sr, w2i, si * w2r);
        sr = tr;
    }
    // Re[(i/sqrt(pi)) (1/z) s] = -(1/sqrt(pi)) Im[(1/z) s]
    double h = -FSG_INV_SQRT_PI * fma(ir, si, ii * sr);
    if (y < 1.0 && x < 9.0)
        h += exp(y * y - x * x) * cos(2.0 * x * y);
    return h;
}

__device__ __noinline__ double voigt_contfrac_f64(double x, double y)
{
    double rr = 0.0, ri = 0.0;
    for (int k = 160; k >= 1; k--) {
        const double dr = x - rr, di = y - ri;
        const double c = 0.5 * k / (dr * dr + di * di);
        rr = c * dr;
        ri = -c * di;
    }
    const double dr = x - rr, di = y - ri;
    return FSG_INV_SQRT_PI * di / (dr * dr + di * di);
}

// Inner region with a > 0.1 (cold gas or strong damping): kept out of line.
__device__ __noinline__ double voigt_wide_f64(double x, double y)
{
    if (y <= 0.25)
        return voigt_taylor_f64<16>(x, y);
    if (y <= 1.0)
        return voigt_taylor_f64<40>(x, y);
    return voigt_contfrac_f64(x, y);
}

// H for x >= 0, y >= 0
__device__ __forceinline__ double voigt_upper_f64(double x, double y)
{
    if (y == 0.0)
        return exp(-x * x);
    if (x * x + y * y >= 64.0)
        return voigt_asym_f64(x, y);
    if (y <= 0.1)
        return voigt_taylor_f64<12>(x, y);
    return voigt_wide_f64(x, y);
}

__device__ __noinline__ double voigt_lower_f64(double x, double y)
{
    // y < 0: Re w(x - iY) = 2 exp(Y^2 - x^2) cos(2 x Y) - Re w(x + iY)
    const double Y = -y;
    return 2.0 * exp(Y * Y - x * x) * cos(2.0 * x * Y) - voigt_upper_f64(x, Y);
}

__device__ __forceinline__ double voigt_f64(double u, double a)
{
    const double x = fabs(u);
    if (a < 0.0)
        return voigt_lower_f64(x, a);
    return voigt_upper_f64(x, a);
}

// ---------------------------------------------------------------------------
// FP32 Voigt for the tuned form, a <= 0.1 (wider profiles use voigt_f64).
//
// With z = x + i a, x = |u|, w(z) = exp(-z^2) + (2i/sqrt(pi)) F(z), F = Dawson's
// integral, so
//   H = exp(a^2 - x^2) cos(2 x a) - (2/sqrt(pi)) Im F(x + i a),
//   Im F(x + i a) = a F'(x) - a^3 F'''(x)/6 + a^5 F^(5)(x)/120 - ...
// (the Taylor series of F in the imaginary direction; the a^7 term is below
// 1e-7 relative for a <= 0.1).
//  * x < 6 (per node), x < 11.9 (a whole warp step in the core form): F and
//    G = F' are read at the nearest x_j = j/10 from a 121-entry table staged
//    in shared memory (the form keeps its accuracy out to x = 12: 5e-7
//    relative on [6, 12) in an emulation of these float operations against
//    scipy's wofz, so a warp step whose nodes straddle x = 6 stays in it
//    instead of running both forms); the higher derivatives follow from the
//    ODE F' = 1 - 2xF, i.e. F^(n+1) = -2x F^(n) - 2n F^(n-1), and G(x),
//    F'''(x), F^(5)(x) are Taylor series in d = x - x_j (|d| <= 0.05).
//  * x >= 6: the asymptotic series of w (A&S 7.1.23) expanded to order a^3:
//      H = (a/sqrt(pi)) t [P(t) - a^2 t Q(t)] (+ exp(-x^2) term for x < 6.5),
//    t = 1/x^2, P = sum c_k (2k+1) t^k, Q = sum c_k (2k+1)(2k+2)(2k+3)/6 t^k,
//    c_k = (2k-1)!!/2^k.
// Accuracy ~1e-6 relative against mpmath over a in [0, 0.1]; the residual is
// the float32 rounding of the argument (relative error of exp(-x^2) ~ 2 x^2 eps).
// ---------------------------------------------------------------------------
#define FSG_V32_N 121

struct Voigt32 {
    float a, a2, c3, c5, two_a_sqpi, a_sqpi;
};

__device__ __forceinline__ Voigt32 make_voigt32(float a)
{
    Voigt32 v;
    v.a = a;
    v.a2 = a * a;
    v.c3 = v.a2 * (1.0f / 6.0f);
    v.c5 = v.a2 * v.a2 * (1.0f / 120.0f);
    v.two_a_sqpi = a * 1.12837916709551257f;
    v.a_sqpi = a * 0.56418958354775628f;
    return v;
}

// Stage {F(x_j), F'(x_j)} for x_j = j/10 into shared memory (whole CTA).
__device__ __forceinline__ void stage_voigt32(float2 *tab)
{
    for (int j = threadIdx.x; j < FSG_V32_N; j += blockDim.x) {
        const double s = 0.88622692545275801365;   // sqrt(pi)/2
        tab[j] = make_float2((float)(d_vtab[j][1] * s), (float)(d_vtab[j][2] * s));
    }
}

// Wing form, valid for |u| >= 6.5 where exp(a^2 - x^2) < 1e-18 is negligible:
// branch-free, so several nodes interleave.
__device__ __forceinline__ float voigt_wing32(float u, const Voigt32 &c)
{
    const float t = __fdividef(1.0f, u * u);
    float p = 15836.1328125f;
    p = fmaf(p, t, 2111.484375f);
    p = fmaf(p, t, 324.84375f);
    p = fmaf(p, t, 59.0625f);
    p = fmaf(p, t, 13.125f);
    p = fmaf(p, t, 3.75f);
    p = fmaf(p, t, 1.5f);
    p = fmaf(p, t, 1.0f);
    float q = 1082.8125f;
    q = fmaf(q, t, 157.5f);
    q = fmaf(q, t, 26.25f);
    q = fmaf(q, t, 5.0f);
    q = fmaf(q, t, 1.0f);
    return c.a_sqpi * t * fmaf(-c.a2 * t, q, p);
}

// Core form, valid for |u| < 12 (table to x = 12.0).
// Nearest table index of x >= 0 (x < 6) without int<->float conversions, which
// run on the narrow FP64/conversion pipe of this GPU: adding 1.5 * 2^23 rounds
// x*10 to an integer held in the low mantissa bits.
__device__ __forceinline__ int vtab_index(float x, float &x0)
{
    const float m = fmaf(x, 10.0f, 12582912.0f);
    x0 = (m - 12582912.0f) * 0.1f;
    return __float_as_int(m) - 0x4B400000;
}

__device__ __forceinline__ float voigt_core32(float u, const Voigt32 &c, const float2 *tab)
{
    const float x = fabsf(u);
    float x0;
    const int j = vtab_index(x, x0);
    const float2 fg = tab[j];
    const float d = x - x0;
    const float m2x = -2.0f * x0;
    const float f0 = fg.x, f1 = fg.y;
    const float f2 = fmaf(m2x, f1, -2.0f * f0);
    const float f3 = fmaf(m2x, f2, -4.0f * f1);
    const float f4 = fmaf(m2x, f3, -6.0f * f2);
    const float f5 = fmaf(m2x, f4, -8.0f * f3);
    const float f6 = fmaf(m2x, f5, -10.0f * f4);
    const float f7 = fmaf(m2x, f6, -12.0f * f5);
    float g = f7 * (1.0f / 720.0f);
    g = fmaf(g, d, f6 * (1.0f / 120.0f));
    g = fmaf(g, d, f5 * (1.0f / 24.0f));
    g = fmaf(g, d, f4 * (1.0f / 6.0f));
    g = fmaf(g, d, f3 * 0.5f);
    g = fmaf(g, d, f2);
    g = fmaf(g, d, f1);
    const float f3x = fmaf(fmaf(fmaf(f6 * (1.0f / 6.0f), d, f5 * 0.5f), d, f4), d, f3);
    const float f5x = fmaf(f6, d, f5);
    const float br = fmaf(c.c5, f5x, fmaf(-c.c3, f3x, g));
    const float gauss = __expf(fmaf(-x, x, c.a2)) * __cosf(2.0f * x * c.a);
    return fmaf(-c.two_a_sqpi, br, gauss);
}

// Small-damping form (a <= VOIGT_SMALL_A, |u| < 15.9): to first order in a,
//   H = exp(-x^2) (1 + a^2 (1 - 2 x^2)) + a K(x),  K = -(2/sqrt(pi)) (1 - 2 x F(x)),
// from the expansion w(x + i a) = w(x) + i a w'(x) - a^2 w''(x)/2 + O(a^3) with
// w' = -2 z w + 2i/sqrt(pi); the dropped terms are below 6e-7 of H for
// a <= 2e-3 (checked against scipy's wofz).  K does not depend on a: one cubic
// per interval of 0.1 (voigt_table.h, read through L1) gives it within 2.3e-7
// of H.  About 17 instructions a node against about 47 for the core form.
constexpr float VOIGT_SMALL_A = 2e-3f;
constexpr float VOIGT_SMALL_X = 15.9f;   // the table covers [0, 16)

__device__ const float4 d_ktab[FSG_KTAB_N] = FSG_KTAB_INIT;

__device__ __forceinline__ float voigt_small32(float u, const Voigt32 &c)
{
    const float x = fabsf(u);
    const float x2 = x * x;
    // interval j = floor(10 x) (a tie at an integer may give j - 1 with t = 1,
    // the same value by continuity) without int<->float conversions
    const float m = fmaf(x, 10.0f, 12582912.0f - 0.5f);
    const int j = __float_as_int(m) - 0x4B400000;
    const float t = fmaf(x, 10.0f, -(m - 12582912.0f));
    const float4 k = __ldg(&d_ktab[j]);
    const float kx = fmaf(fmaf(fmaf(k.w, t, k.z), t, k.y), t, k.x);
    const float e = __expf(-x2);
    const float g = fmaf(c.a2, fmaf(-2.0f, x2, 1.0f), 1.0f);
    return fmaf(e, g, c.a * kx);
}

template <bool COUNT>
__device__ __forceinline__ float voigt_f32(float u, const Voigt32 &c, const float2 *tab,
                                           unsigned &n_near)
{
    const float x = fabsf(u);
    if (x < 6.0f) {
        if (COUNT)
            n_near++;
        float x0;
        const int j = vtab_index(x, x0);
        const float2 fg = tab[j];
        const float d = x - x0;
        const float m2x = -2.0f * x0;
        const float f0 = fg.x, f1 = fg.y;
        const float f2 = fmaf(m2x, f1, -2.0f * f0);
        const float f3 = fmaf(m2x, f2, -4.0f * f1);
        const float f4 = fmaf(m2x, f3, -6.0f * f2);
        const float f5 = fmaf(m2x, f4, -8.0f * f3);
        const float f6 = fmaf(m2x, f5, -10.0f * f4);
        const float f7 = fmaf(m2x, f6, -12.0f * f5);
        float g = f7 * (1.0f / 720.0f);
        g = fmaf(g, d, f6 * (1.0f / 120.0f));
        g = fmaf(g, d, f5 * (1.0f / 24.0f));
        g = fmaf(g, d, f4 * (1.0f / 6.0f));
        g = fmaf(g, d, f3 * 0.5f);
        g = fmaf(g, d, f2);
        g = fmaf(g, d, f1);
        const float f3x = fmaf(fmaf(fmaf(f6 * (1.0f / 6.0f), d, f5 * 0.5f), d, f4), d, f3);
        const float f5x = fmaf(f6, d, f5);
        const float br = fmaf(c.c5, f5x, fmaf(-c.c3, f3x, g));
        const float gauss = __expf(fmaf(-x, x, c.a2)) * __cosf(2.0f * x * c.a);
        return fmaf(-c.two_a_sqpi, br, gauss);
    }
    const float t = __frcp_rn(x * x);
    float p = 15836.1328125f;
    p = fmaf(p, t, 2111.484375f);
    p = fmaf(p, t, 324.84375f);
    p = fmaf(p, t, 59.0625f);
    p = fmaf(p, t, 13.125f);
    p = fmaf(p, t, 3.75f);
    p = fmaf(p, t, 1.5f);
    p = fmaf(p, t, 1.0f);
    float q = 1082.8125f;
    q = fmaf(q, t, 157.5f);
    q = fmaf(q, t, 26.25f);
    q = fmaf(q, t, 5.0f);
    q = fmaf(q, t, 1.0f);
    float h = c.a_sqpi * t * fmaf(-c.a2 * t, q, p);
    if (x < 6.5f)
        h += __expf(fmaf(-x, x, c.a2)) * __cosf(2.0f * x * c.a);
    return h;
}

}  // namespace fsg

namespace fsg {

// ---------------------------------------------------------------------------
// Voigt profile with its partial derivatives (backward pass, FP32, a <= 0.1):
// H(u, a), dH/du and dH/da, from the same two forms as voigt_f32.
//  wing (|u| >= 6): H = (a/sqrt(pi)) t [P(t) - a^2 t Q(t)], t = 1/u^2, so
//    dH/du = -(a/sqrt(pi)) (t/u) [P1(t) - a^2 t Q1(t)],
//      P1 = sum (2k+2) p_k t^k, Q1 = sum (2k+4) q_k t^k,
//    dH/da = (1/sqrt(pi)) t [P(t) - 3 a^2 t Q(t)];
//  core (|u| < 6): with E = exp(a^2-x^2), C = cos 2xa, S = sin 2xa,
//    H     = E C - (2a/sqrt(pi)) [G - a^2 F'''/6 + a^4 F^(5)/120],
//    dH/dx = E (-2x C - 2a S) - (2a/sqrt(pi)) [F'' - a^2 F^(4)/6 + a^4 F^(6)/120],
//    dH/da = E (2a C - 2x S) - (2/sqrt(pi)) [G - a^2 F'''/2 + a^4 F^(5)/24],
//    derivatives of Dawson's F as in voigt_core32; dH/du = sign(u) dH/dx.
//  (the exp(-x^2) term of the wing form is kept for 6 <= |u| < 6.5)
// ---------------------------------------------------------------------------
struct VoigtGrad {
    float h, hu, ha;
};

// The small-damping form (voigt_small32) with its derivatives:
//   dH/dx = -2 x exp(-x^2) (1 + a^2 (1 - 2 x^2) + 2 a^2) + a K'(x),
//   dH/da = 2 a (1 - 2 x^2) exp(-x^2) + K(x),
// K' from the derivative of the interval's cubic.
__device__ __forceinline__ VoigtGrad voigt_grad_small32(float u, const Voigt32 &c)
{
    VoigtGrad r;
    const float x = fabsf(u);
    const float x2 = x * x;
    const float m = fmaf(x, 10.0f, 12582912.0f - 0.5f);
    const int j = __float_as_int(m) - 0x4B400000;
    const float t = fmaf(x, 10.0f, -(m - 12582912.0f));
    const float4 k = __ldg(&d_ktab[j]);
    const float kx = fmaf(fmaf(fmaf(k.w, t, k.z), t, k.y), t, k.x);
    const float dk = 10.0f * fmaf(fmaf(3.0f * k.w, t, 2.0f * k.z), t, k.y);
    const float e = __expf(-x2);
    const float q = fmaf(-2.0f, x2, 1.0f);
    const float g = fmaf(c.a2, q, 1.0f);
    r.h = fmaf(e, g, c.a * kx);
    const float dhdx = fmaf(-2.0f * x * e, fmaf(2.0f, c.a2, g), c.a * dk);
    r.hu = u < 0.0f ? -dhdx : dhdx;
    r.ha = fmaf(2.0f * c.a * e, q, kx);
    return r;
}

__device__ __forceinline__ VoigtGrad voigt_grad32(float u, const Voigt32 &c, const float2 *tab)
{
    VoigtGrad r;
    const float x = fabsf(u);
    const float sgn = u < 0.0f ? -1.0f : 1.0f;
    if (x < 6.0f) {
        float x0;
        const int j = vtab_index(x, x0);
        const float2 fg = tab[j];
        const float d = x - x0;
        const float m2x = -2.0f * x0;
        const float f0 = fg.x, f1 = fg.y;
        const float f2 = fmaf(m2x, f1, -2.0f * f0);
        const float f3 = fmaf(m2x, f2, -4.0f * f1);
        const float f4 = fmaf(m2x, f3, -6.0f * f2);
        const float f5 = fmaf(m2x, f4, -8.0f * f3);
        const float f6 = fmaf(m2x, f5, -10.0f * f4);
        const float f7 = fmaf(m2x, f6, -12.0f * f5);
        const float f8 = fmaf(m2x, f7, -14.0f * f6);
        // F^(n)(x) = sum_m f_{n+m} d^m / m!
        float g = f7 * (1.0f / 720.0f);
        g = fmaf(g, d, f6 * (1.0f / 120.0f));
        g = fmaf(g, d, f5 * (1.0f / 24.0f));
        g = fmaf(g, d, f4 * (1.0f / 6.0f));
        g = fmaf(g, d, f3 * 0.5f);
        g = fmaf(g, d, f2);
        g = fmaf(g, d, f1);
        float F2 = f8 * (1.0f / 720.0f);
        F2 = fmaf(F2, d, f7 * (1.0f / 120.0f));
        F2 = fmaf(F2, d, f6 * (1.0f / 24.0f));
        F2 = fmaf(F2, d, f5 * (1.0f / 6.0f));
        F2 = fmaf(F2, d, f4 * 0.5f);
        F2 = fmaf(F2, d, f3);
        F2 = fmaf(F2, d, f2);
        const float F3 = fmaf(fmaf(fmaf(fmaf(f7 * (1.0f / 24.0f), d, f6 * (1.0f / 6.0f)), d,
                                        f5 * 0.5f), d, f4), d, f3);
        const float F4 = fmaf(fmaf(fmaf(f7 * (1.0f / 6.0f), d, f6 * 0.5f), d, f5), d, f4);
        const float F5 = fmaf(fmaf(f7 * 0.5f, d, f6), d, f5);
        const float F6 = fmaf(f7, d, f6);
        float S, C;
        __sincosf(2.0f * x * c.a, &S, &C);
        const float E = __expf(fmaf(-x, x, c.a2));
        const float a4_120 = c.c5;                 // a^4 / 120
        const float B = fmaf(a4_120, F5, fmaf(-c.c3, F3, g));
        const float Bx = fmaf(a4_120, F6, fmaf(-c.c3, F4, F2));
        const float Ba = fmaf(5.0f * a4_120, F5, fmaf(-3.0f * c.c3, F3, g));
        r.h = fmaf(-c.two_a_sqpi, B, E * C);
        const float dhdx = fmaf(-c.two_a_sqpi, Bx, E * fmaf(-2.0f * x, C, -2.0f * c.a * S));
        r.hu = sgn * dhdx;
        r.ha = fmaf(-1.12837916709551257f, Ba, E * fmaf(2.0f * c.a, C, -2.0f * x * S));
        return r;
    }
    const float t = __fdividef(1.0f, u * u);
    float p = 15836.1328125f, p1 = 253378.125f;
    p = fmaf(p, t, 2111.484375f);
    p1 = fmaf(p1, t, 29560.78125f);
    p = fmaf(p, t, 324.84375f);
    p1 = fmaf(p1, t, 3898.125f);
    p = fmaf(p, t, 59.0625f);
    p1 = fmaf(p1, t, 590.625f);
    p = fmaf(p, t, 13.125f);
    p1 = fmaf(p1, t, 105.0f);
    p = fmaf(p, t, 3.75f);
    p1 = fmaf(p1, t, 22.5f);
    p = fmaf(p, t, 1.5f);
    p1 = fmaf(p1, t, 6.0f);
    p = fmaf(p, t, 1.0f);
    p1 = fmaf(p1, t, 2.0f);
    float q = 1082.8125f, q1 = 12993.75f;
    q = fmaf(q, t, 157.5f);
    q1 = fmaf(q1, t, 1575.0f);
    q = fmaf(q, t, 26.25f);
    q1 = fmaf(q1, t, 210.0f);
    q = fmaf(q, t, 5.0f);
    q1 = fmaf(q1, t, 30.0f);
    q = fmaf(q, t, 1.0f);
    q1 = fmaf(q1, t, 4.0f);
    const float a2t = c.a2 * t;
    r.h = c.a_sqpi * t * fmaf(-a2t, q, p);
    r.hu = -c.a_sqpi * t * __fdividef(1.0f, u) * fmaf(-a2t, q1, p1);
    r.ha = 0.56418958354775628f * t * fmaf(-3.0f * a2t, q, p);
    if (x < 6.5f) {
        float S, C;
        __sincosf(2.0f * x * c.a, &S, &C);
        const float E = __expf(fmaf(-x, x, c.a2));
        r.h = fmaf(E, C, r.h);
        r.hu = fmaf(sgn * E, fmaf(-2.0f * x, C, -2.0f * c.a * S), r.hu);
        r.ha = fmaf(E, fmaf(2.0f * c.a, C, -2.0f * x * S), r.ha);
    }
    return r;
}

}  // namespace fsg
