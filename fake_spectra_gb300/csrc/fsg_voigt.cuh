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

}  // namespace fsg
