/*
 * TEST INFRASTRUCTURE ONLY -- CPU oracle (plain C restatement) of the
 * reference's `_Particle_Interpolate` path.  See fsg_oracle.h.
 *
 * Build: oracle/build_oracle.sh (gcc -O2 -fopenmp -ffp-contract=off).  FMA
 * contraction is disabled so the mixed float/double sightline predicate of
 * the reference IndexTable is reproduced bit for bit on x86-64 and aarch64.
 *
 * The Voigt function is this file's own: Dawson's integral from Rybicki's
 * sampling-theorem formula (G. B. Rybicki, Computers in Physics 3, 85, 1989),
 * a Taylor expansion of w(z) in Im z about the real axis driven by the ODE
 * w'(z) = -2 z w(z) + 2i/sqrt(pi) (Abramowitz & Stegun 7.1.20), and the
 * Laplace continued fraction of w(z) (A&S 7.1.15) for large |z|.
 */
#include "fsg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Physical constants, cgs -- same values as absorption.cpp:21-33 and absorption.h:4 */
#define O_PROTONMASS 1.67262178e-24
#define O_SIGMA_T 6.652458558e-25
#define O_BOLTZMANN 1.3806504e-16
#define O_LIGHT 2.99792458e10
#define O_NGRID 8 /* singleabs.h:8 */

static const double O_PI = 3.14159265358979323846;
static const double O_INV_SQRT_PI = 0.56418958354775628695;
static const double O_TWO_OVER_SQRT_PI = 1.12837916709551257390;

static int g_threads = 0;
void fsgo_set_threads(int n) { g_threads = n; }
int fsgo_get_threads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* Voigt function                                                      */
/* ------------------------------------------------------------------ */

/* Dawson's integral F(x) and its derivative G(x) = F'(x) = 1 - 2xF(x).
 * Rybicki: F(x) = lim_{h->0} pi^{-1/2} sum_{n odd} exp(-(x - n h)^2) / n.
 * With h = 0.2 the aliasing error is of order exp(-(pi/(2h))^2) ~ 1e-27.
 * Writing x = n0 h + xp (n0 even, |xp| <= h) and n = n0 + m (m odd):
 *   exp(-(xp - m h)^2) = exp(-xp^2) exp(2 xp m h) exp(-(m h)^2).
 * G is summed directly from the differentiated series to avoid the
 * cancellation in 1 - 2xF at large x. */
#define RYB_H 0.2
#define RYB_TERMS 24
static double ryb_g[RYB_TERMS]; /* exp(-((2k+1) h)^2) */
static int ryb_init = 0;

static void ryb_setup(void)
{
    if (ryb_init)
        return;
    for (int k = 0; k < RYB_TERMS; k++) {
        double mh = (2 * k + 1) * RYB_H;
        ryb_g[k] = exp(-mh * mh);
    }
    ryb_init = 1;
}

static void dawson_fg(double x, double *F, double *G)
{
    double ax = fabs(x);
    if (ax < 0.2) {
        /* F(x) = sum_k (-1)^k 2^k x^{2k+1} / (2k+1)!! */
        double x2 = ax * ax, term = ax, sum = ax;
        for (int k = 1; k < 16; k++) {
            term *= -2.0 * x2 / (2 * k + 1);
            sum += term;
        }
        *F = x < 0 ? -sum : sum;
        *G = 1.0 - 2.0 * ax * sum;
        return;
    }
    ryb_setup();
    long n0 = 2 * lround(0.5 * ax / RYB_H);
    double xp = ax - (double)n0 * RYB_H;
    double e1 = exp(2.0 * xp * RYB_H), e2 = e1 * e1;
    double ep = e1, em = 1.0 / e1;
    double sf = 0.0, sg = 0.0;
    for (int k = 0; k < RYB_TERMS; k++) {
        int m = 2 * k + 1;
        double dp = (double)(n0 + m), dm = (double)(n0 - m);
        double tp = ryb_g[k] * ep / dp; /* term for n = n0 + m */
        double tm = ryb_g[k] * em / dm; /* term for n = n0 - m */
        sf += tp + tm;
        sg += (xp - m * RYB_H) * tp + (xp + m * RYB_H) * tm;
        ep *= e2;
        em /= e2;
    }
    double ex = exp(-xp * xp);
    *F = (x < 0 ? -1.0 : 1.0) * O_INV_SQRT_PI * ex * sf;
    *G = -2.0 * O_INV_SQRT_PI * ex * sg;
}

double fsgo_dawson(double x)
{
    double F, G;
    dawson_fg(x, &F, &G);
    return F;
}

/* Laplace continued fraction, w(z) = (i/sqrt(pi)) / (z - (1/2)/(z - 1/(z - (3/2)/(z - ...)))) */
static void w_contfrac(double x, double y, int depth, double *re, double *im)
{
    double rr = 0.0, ri = 0.0;
    for (int k = depth; k >= 1; k--) {
        double dr = x - rr, di = y - ri;
        double den = dr * dr + di * di;
        double c = 0.5 * k / den;
        rr = c * dr;
        ri = -c * di;
    }
    double dr = x - rr, di = y - ri;
    double den = dr * dr + di * di;
    /* (i/sqrt(pi)) * conj(d)/|d|^2 */
    *re = O_INV_SQRT_PI * di / den;
    *im = O_INV_SQRT_PI * dr / den;
}

/* Taylor series of w about the real point x, evaluated at x + i y:
 * w(x+iy) = sum_n c_n (iy)^n with c_0 = w(x) = exp(-x^2) + i (2/sqrt(pi)) F(x),
 * c_1 = -2x c_0 + 2i/sqrt(pi), (n+1) c_{n+1} = -2x c_n - 2 c_{n-1}. */
static void w_taylor_axis(double x, double y, double *re, double *im)
{
    double F, G;
    dawson_fg(x, &F, &G);
    double ex = exp(-x * x);
    double c0r = ex, c0i = O_TWO_OVER_SQRT_PI * F;
    double c1r = -2.0 * x * ex, c1i = O_TWO_OVER_SQRT_PI * G;
    /* (iy)^n: n=0 -> 1, n=1 -> iy */
    double pr = 0.0, pi = y;
    double sr = c0r + (c1r * pr - c1i * pi);
    double si = c0i + (c1r * pi + c1i * pr);
    double cmr = c0r, cmi = c0i, cr = c1r, ci = c1i;
    int small = 0;
    for (int n = 1; n < 80; n++) {
        const double inv = 1.0 / (n + 1);
        double nr = (-2.0 * x * cr - 2.0 * cmr) * inv;
        double ni = (-2.0 * x * ci - 2.0 * cmi) * inv;
        /* multiply (pr + i pi) by iy */
        double t = pr;
        pr = -pi * y;
        pi = t * y;
        double tr = nr * pr - ni * pi;
        double ti = nr * pi + ni * pr;
        sr += tr;
        si += ti;
        cmr = cr;
        cmi = ci;
        cr = nr;
        ci = ni;
        double mag = (fabs(nr) + fabs(ni)) * (fabs(pr) + fabs(pi));
        if (mag <= 1e-18 * fabs(sr) && mag <= 1e-18 * (fabs(sr) + fabs(si))) {
            if (++small >= 3)
                break;
        } else {
            small = 0;
        }
    }
    *re = sr;
    *im = si;
}

/* Levels of the continued fraction for |z|^2 = r2 >= 49.  Its error falls
 * quickly with |z|: the levels needed for 2e-16 relative accuracy of both
 * parts (against 240 levels, over the whole quadrant including the real axis)
 * are 16, 13, 11, 10, 9, 7, 6, 5 at |z| = 8, 10, 12, 15, 20, 30, 50, 100;
 * each interval below uses its lower edge's count plus two.  Below |z| = 8
 * the 24 levels of the fixed form are kept. */
static int cf_levels(double r2)
{
    if (r2 < 64.0)
        return 24;
    if (r2 < 100.0)
        return 18;
    if (r2 < 144.0)
        return 15;
    if (r2 < 225.0)
        return 13;
    if (r2 < 400.0)
        return 12;
    if (r2 < 900.0)
        return 11;
    if (r2 < 2500.0)
        return 9;
    if (r2 < 10000.0)
        return 8;
    return 7;
}

/* w(x + iy) for y >= 0, x >= 0 */
static void w_upper(double x, double y, double *re, double *im)
{
    if (y == 0.0) {
        double F, G;
        dawson_fg(x, &F, &G);
        *re = exp(-x * x);
        *im = O_TWO_OVER_SQRT_PI * F;
        return;
    }
    double r2 = x * x + y * y;
    if (r2 >= 49.0) {
        w_contfrac(x, y, cf_levels(r2), re, im);
        if (y < 1.0 && x < 9.0) {
            /* exp(-z^2), exponentially small near the axis, beyond the reach of the fraction */
            double m = exp(y * y - x * x);
            *re += m * cos(2.0 * x * y);
            *im -= m * sin(2.0 * x * y);
        }
        return;
    }
    if (y < 1.0) {
        w_taylor_axis(x, y, re, im);
        return;
    }
    w_contfrac(x, y, 240, re, im);
}

void fsgo_faddeeva(double x, double y, double *re, double *im)
{
    double ax = fabs(x);
    if (y >= 0.0) {
        w_upper(ax, y, re, im);
        if (x < 0)
            *im = -*im; /* w(-x + iy) = conj(w(x + iy)) */
        return;
    }
    /* lower half plane: w(z) = 2 exp(-z^2) - w(-z), and -z is in the upper half plane */
    double r, i;
    w_upper(ax, -y, &r, &i);
    if (x < 0)
        i = -i;
    /* w(-z) with -z = -x - iy = -x + i|y| -> conj(w(x + i|y|)) */
    double wr = r, wi = -i;
    double m = exp(y * y - x * x);
    *re = 2.0 * m * cos(2.0 * x * y) - wr;
    *im = -2.0 * m * sin(2.0 * x * y) - wi;
}

/* profile(), singleabs.h:56-61: H(a, u) = Re w(u + i a) */
double fsgo_voigt(double u, double a)
{
    double re, im;
    fsgo_faddeeva(u, a, &re, &im);
    return re;
}

/* ------------------------------------------------------------------ */
/* SPH kernels and kernel integrals                                    */
/* ------------------------------------------------------------------ */

/* singleabs.h:17-26: cubic spline (Price 2011 eq. 6) with support q < 1 */
double fsgo_sph_cubic_kernel(double q)
{
    const double norm = 32. / 4 / O_PI;
    if (q >= 1)
        return 0;
    if (q < 0.5)
        return norm * (1 - 6 * q * q + 6 * q * q * q);
    double t = 1. - q;
    return norm * (2 * t * t * t);
}

/* singleabs.h:31-42: quintic spline (Price 2011 eq. 8) with support q < 1 */
double fsgo_sph_quintic_kernel(double q)
{
    const double norm = 9. / 40 / O_PI;
    if (q >= 1)
        return 0;
    if (q < (1. / 3))
        return norm * 6 * (11 - 90 * q * q + 405 * q * q * q * q - 405 * q * q * q * q * q);
    if (q < (2. / 3)) {
        double a = 3. - 3 * q, b = 2. - 3 * q;
        return norm * (a * a * a * a * a - 6 * b * b * b * b * b);
    }
    double t = 1. - q;
    return norm * (243 * t * t * t * t * t);
}

/* absorption.cpp:53-97: trapezoid (NGRID intervals) of the kernel along the
 * line of sight, clipped to the kernel support [-zrange, zrange]. */
static double spline_kern_frac(double (*kern)(double), double zlow, double zhigh, double smooth,
                               double dr2, double zrange)
{
    if (zlow < -zrange)
        zlow = -zrange;
    if (zhigh > zrange)
        zhigh = zrange;
    if (zlow > zhigh)
        return 0;
    double total = kern(sqrt(dr2 + zlow * zlow) / smooth) / 2.;
    const double deltaz = (zhigh - zlow) / O_NGRID;
    for (int i = 1; i < O_NGRID; ++i) {
        const double zz = i * deltaz + zlow;
        total += kern(sqrt(dr2 + zz * zz) / smooth);
    }
    total += kern(sqrt(dr2 + zhigh * zhigh) / smooth) / 2.;
    return deltaz * total;
}

/* absorption.cpp:109-115 */
static double tophat_kern_frac(double zlow, double zhigh, double zrange)
{
    if (zlow < -zrange)
        zlow = -zrange;
    if (zhigh > zrange)
        zhigh = zrange;
    double d = zhigh - zlow;
    return 3. / 4. / O_PI * (d > 0. ? d : 0.);
}

/* absorption.cpp:129-134: the Voronoi cell's share of the pixel is the length
 * of the overlap of the pixel with the cell's segment [-zrange, zrange]. */
static double arepo_kern_frac(double zlow, double zhigh, double zrange)
{
    if (zlow < -zrange)
        zlow = -zrange;
    if (zhigh > zrange)
        zhigh = zrange;
    return zhigh - zlow > 0. ? zhigh - zlow : 0.;
}

/* absorption.cpp:136-148 (dispatch; unknown ids use the top hat) */
double fsgo_kern_frac(int kernel, double zlow, double zhigh, double smooth, double dr2,
                      double zrange)
{
    if (kernel == FSGO_SPH_CUBIC)
        return spline_kern_frac(fsgo_sph_cubic_kernel, zlow, zhigh, smooth, dr2, zrange);
    if (kernel == FSGO_SPH_QUINTIC)
        return spline_kern_frac(fsgo_sph_quintic_kernel, zlow, zhigh, smooth, dr2, zrange);
    if (kernel == FSGO_VORONOI)
        return arepo_kern_frac(zlow, zhigh, zrange);
    return tophat_kern_frac(zlow, zhigh, zrange);
}

/* ------------------------------------------------------------------ */
/* SingleAbsorber, singleabs.h:63-175                                  */
/* ------------------------------------------------------------------ */
typedef struct {
    double btherm, vdr2, vsmooth, aa, vhigh;
    int kernel;
    long long evals;
} absorber_t;

static void absorber_init(absorber_t *s, double btherm, double vdr2, double vsmooth, double aa,
                          int kernel)
{
    s->btherm = btherm;
    s->vdr2 = vdr2;
    s->vsmooth = vsmooth;
    s->aa = aa;
    s->kernel = kernel;
    s->vhigh = (vsmooth * vsmooth > vdr2 ? sqrt(vsmooth * vsmooth - vdr2) : 0);
    /* singleabs.h:85-89: for the Voronoi mesh vdr2 and vsmooth are the cell's
     * segment ends (velocity units) and the half-length is the node range */
    if (kernel == FSGO_VORONOI)
        s->vhigh = (vdr2 > 0 && vsmooth > 0) ? (vsmooth - vdr2) / 2. : 0;
    s->evals = 0;
}

/* singleabs.h:143-167: 7 interior nodes of the LOS kernel integral, each a
 * Voigt profile evaluation weighted by the kernel. */
static double tau_kern_inner(absorber_t *s, double vouter)
{
    const double deltav = 2. * s->vhigh / O_NGRID;
    double total = 0;
    for (int i = 1; i < O_NGRID; ++i) {
        const double vv = i * deltav - s->vhigh;
        const double q = sqrt(s->vdr2 + vv * vv) / s->vsmooth;
        const double vdiff = vv - vouter;
        double tbin = fsgo_voigt(vdiff / s->btherm, s->aa);
        if (s->kernel == FSGO_SPH_CUBIC)
            tbin *= fsgo_sph_cubic_kernel(q);
        else if (s->kernel == FSGO_SPH_QUINTIC)
            tbin *= fsgo_sph_quintic_kernel(q);
        else if (s->kernel == FSGO_TOP_HAT)
            tbin *= 3. / 4. / O_PI;
        total += tbin;
    }
    s->evals += O_NGRID - 1;
    return deltav * total;
}

/* singleabs.h:104-126: pixel average, midpoint when the pixel is narrower
 * than b/2, else a trapezoid with 2*ceil(w/(b/2)/2)+1 points. */
static double tau_kern_outer(absorber_t *s, double vlow, double vhigh)
{
    if ((vhigh - vlow) < s->btherm / 2.)
        return tau_kern_inner(s, (vhigh + vlow) / 2.);
    const int npoints = (int)(2 * ceil((vhigh - vlow) / (s->btherm / 2.) / 2) + 1.);
    double total = tau_kern_inner(s, vlow) / 2.;
    const double deltav = (vhigh - vlow) / (npoints - 1);
    for (int i = 1; i < npoints - 1; ++i)
        total += tau_kern_inner(s, i * deltav + vlow);
    total += tau_kern_inner(s, vhigh) / 2.;
    return total / (npoints - 1);
}

double fsgo_tau_kern_outer(double btherm, double vdr2, double vsmooth, double aa, int kernel,
                           double vlow, double vhigh)
{
    absorber_t s;
    absorber_init(&s, btherm, vdr2, vsmooth, aa, kernel);
    return tau_kern_outer(&s, vlow, vhigh);
}

/* ------------------------------------------------------------------ */
/* LineAbsorption, absorption.cpp:152-279                              */
/* ------------------------------------------------------------------ */
typedef struct {
    double tautail, sigma_a, bfac, voigt_fac, velfac, vbox;
    int kernel;
} line_t;

/* absorption.cpp:152-161 */
static void line_init(line_t *l, double lambda, double gamma, double fosc, double amumass,
                      double velfac, double box, int kernel, double tautail)
{
    l->tautail = tautail;
    l->sigma_a = sqrt(3.0 * O_PI * O_SIGMA_T / 8.0) * lambda * fosc;
    l->bfac = sqrt(2.0 * O_BOLTZMANN / (amumass * O_PROTONMASS)) / 1e5;
    l->voigt_fac = gamma * lambda / (4. * O_PI) / 1e5;
    l->velfac = velfac;
    l->vbox = box * velfac;
    l->kernel = kernel;
}

static int wrap_bin(int z, int nbins)
{
    int j = z % nbins;
    if (j < 0)
        j += nbins;
    return j;
}

/* absorption.cpp:167-210.  For the Voronoi mesh dr2 and smooth are the lower
 * and upper ends of the cell's segment along the sightline. */
static void add_colden(const line_t *l, double *colden, int nbins, double dr2, float dens,
                       float ppos, float smooth)
{
    double pos1 = ppos;
    double zrange;
    if (l->kernel == FSGO_VORONOI) {
        if (dr2 > 2 * l->vbox / l->velfac || smooth > 2 * l->vbox / l->velfac)
            return;
        pos1 = (dr2 + smooth) / 2.;
        zrange = (smooth - dr2) / 2.;
    } else {
        const double hh2 = (double)(smooth * smooth); /* float product, as in the reference */
        if (hh2 - dr2 <= 0)
            return;
        zrange = sqrt(hh2 - dr2);
    }
    const double boxtokpc = l->vbox / nbins / l->velfac;
    const int zlow = (int)floor((pos1 - zrange) / boxtokpc);
    const int zhigh = (int)ceil((pos1 + zrange) / boxtokpc);
    for (int z = zlow; z <= zhigh; z++) {
        const double plow = (boxtokpc * z - pos1);
        colden[wrap_bin(z, nbins)] +=
            dens * fsgo_kern_frac(l->kernel, plow, plow + boxtokpc, smooth, dr2, zrange);
    }
}

/* absorption.cpp:212-279 */
static long long add_tau(const line_t *l, double *tau, int nbins, double dr2, float dens,
                         float ppos, float pvel, float temp, float smooth)
{
    double pos1 = ppos;
    const double btherm = l->bfac * sqrt((double)temp);
    if (l->kernel == FSGO_VORONOI) {
        if (dr2 > 2 * l->vbox / l->velfac || smooth > 2 * l->vbox / l->velfac)
            return 0;
        pos1 = (dr2 + smooth) / 2.;
    } else {
        const double hh2 = (double)(smooth * smooth);
        if (hh2 - dr2 <= 0)
            return 0;
    }
    const double vel = l->velfac * pos1 + pvel;
    double val1 = l->velfac * dr2;
    if (l->kernel != FSGO_VORONOI)
        val1 *= l->velfac;
    absorber_t s;
    absorber_init(&s, btherm, val1, l->velfac * smooth, l->voigt_fac / btherm, l->kernel);
    const double bintov = l->vbox / nbins;
    const double amp = l->sigma_a / sqrt(O_PI) * (O_LIGHT / 1e5 / btherm);
    const int zmax = (int)floor(vel / bintov);
    for (int z = zmax; z < zmax + nbins / 2; ++z) {
        double vlow = z * bintov - vel;
        const double taulast = amp * dens * tau_kern_outer(&s, vlow, vlow + bintov) / l->velfac;
        tau[wrap_bin(z, nbins)] += taulast;
        if (taulast < l->tautail)
            break;
    }
    for (int z = zmax - 1; z >= zmax - nbins / 2; --z) {
        double vlow = z * bintov - vel;
        const double taulast = amp * dens * tau_kern_outer(&s, vlow, vlow + bintov) / l->velfac;
        tau[wrap_bin(z, nbins)] += taulast;
        if (taulast < l->tautail)
            break;
    }
    return s.evals;
}

void fsgo_add_tau_particle(double lambda, double gamma, double fosc, double amumass,
                           double velfac, double box, double atime, int kernel, double tautail,
                           double *tau, int nbins, double dr2, float dens, float ppos, float pvel,
                           float temp, float smooth, long long *evals)
{
    (void)atime;
    line_t l;
    line_init(&l, lambda, gamma, fosc, amumass, velfac, box, kernel, tautail);
    long long e = add_tau(&l, tau, nbins, dr2, dens, ppos, pvel, temp, smooth);
    if (evals)
        *evals += e;
}

void fsgo_add_colden_particle(double lambda, double gamma, double fosc, double amumass,
                              double velfac, double box, double atime, int kernel, double tautail,
                              double *colden, int nbins, double dr2, float dens, float ppos,
                              float smooth)
{
    (void)atime;
    line_t l;
    line_init(&l, lambda, gamma, fosc, amumass, velfac, box, kernel, tautail);
    add_colden(&l, colden, nbins, dr2, dens, ppos, smooth);
}

/* ------------------------------------------------------------------ */
/* IndexTable, index_table.cpp:7-150                                   */
/* ------------------------------------------------------------------ */
typedef struct {
    double key;
    int line;
} tab_entry;

typedef struct {
    tab_entry *main_tab; /* axis 2/3 lines keyed by cofm[3i]   (index_table.cpp:14) */
    int n_main;
    tab_entry *xx_tab; /* axis 1 lines keyed by cofm[3i+1]     (index_table.cpp:12) */
    int n_xx;
    const double *cofm;
    const int32_t *axis;
    double box;
} index_t;

static int cmp_entry(const void *a, const void *b)
{
    const tab_entry *x = (const tab_entry *)a, *y = (const tab_entry *)b;
    if (x->key < y->key)
        return -1;
    if (x->key > y->key)
        return 1;
    /* equal keys keep insertion order, as std::multimap::insert does */
    return (x->line > y->line) - (x->line < y->line);
}

static void index_init(index_t *t, const double *cofm, const int32_t *axis, int nlos, double box)
{
    t->cofm = cofm;
    t->axis = axis;
    t->box = box;
    t->main_tab = (tab_entry *)malloc(sizeof(tab_entry) * (nlos > 0 ? nlos : 1));
    t->xx_tab = (tab_entry *)malloc(sizeof(tab_entry) * (nlos > 0 ? nlos : 1));
    t->n_main = t->n_xx = 0;
    for (int i = 0; i < nlos; i++) {
        if (axis[i] == 1) {
            t->xx_tab[t->n_xx].key = cofm[3 * i + 1];
            t->xx_tab[t->n_xx].line = i;
            t->n_xx++;
        } else {
            t->main_tab[t->n_main].key = cofm[3 * i];
            t->main_tab[t->n_main].line = i;
            t->n_main++;
        }
    }
    qsort(t->main_tab, t->n_main, sizeof(tab_entry), cmp_entry);
    qsort(t->xx_tab, t->n_xx, sizeof(tab_entry), cmp_entry);
}

static void index_free(index_t *t)
{
    free(t->main_tab);
    free(t->xx_tab);
}

/* std::multimap::lower_bound: first entry whose key is not less than x */
static int lower_bound(const tab_entry *tab, int n, double x)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = lo + (hi - lo) / 2;
        if (tab[mid].key < x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

/* index_table.cpp:52-68 */
static int second_close(float second, double lproj2, float hh, double box)
{
    float ffp = second + hh;
    if ((double)ffp > box)
        if (lproj2 < (double)ffp - box)
            return 1;
    float ffm = second - hh;
    if (ffm < 0)
        if (lproj2 > (double)ffm + box)
            return 1;
    return (lproj2 > (double)ffm && lproj2 < (double)ffp);
}

/* index_table.cpp:70-87 */
static double calc_dr2(double d1, double d2, double box)
{
    double dr = fabs(d1);
    if (dr > 0.5 * box)
        dr = box - dr;
    double dr2 = dr * dr;
    dr = fabs(d2);
    if (dr > 0.5 * box)
        dr = box - dr;
    dr2 += (dr * dr);
    return dr2;
}

typedef void (*emit_fn)(void *ctx, int line, double dr2);

/* index_table.cpp:22-50 */
static void nearby_from_range(const index_t *t, const tab_entry *tab, int lo, int hi,
                              const float *pos, float hh, float first, emit_fn emit, void *ctx)
{
    for (int e = lo; e < hi; e++) {
        const int iproc = tab[e].line;
        const int iaxis = t->axis[iproc];
        float second;
        double lproj2;
        if (iaxis == 3) {
            second = pos[1];
            lproj2 = t->cofm[3 * iproc + 1];
        } else {
            second = pos[2];
            lproj2 = t->cofm[3 * iproc + 2];
        }
        const double lproj = tab[e].key;
        if (second_close(second, lproj2, hh, t->box)) {
            double dr2 = calc_dr2((double)first - lproj, (double)second - lproj2, t->box);
            if (dr2 <= (double)(hh * hh))
                emit(ctx, iproc, dr2);
        }
    }
}

/* index_table.cpp:89-113 */
static void get_nearby(const index_t *t, const tab_entry *tab, int n, float first,
                       const float *pos, float hh, emit_fn emit, void *ctx)
{
    float ffp = first + hh;
    if ((double)ffp > t->box)
        ffp = (float)((double)ffp - t->box);
    float ffm = first - hh;
    if (ffm < 0)
        ffm = (float)((double)ffm + t->box);
    int low = lower_bound(tab, n, (double)ffm);
    int high = lower_bound(tab, n, (double)ffp);
    if (ffm <= ffp) {
        nearby_from_range(t, tab, low, high, pos, hh, first, emit, ctx);
    } else {
        nearby_from_range(t, tab, 0, high, pos, hh, first, emit, ctx);
        nearby_from_range(t, tab, low, n, pos, hh, first, emit, ctx);
    }
}

/* index_table.cpp:117-127 */
static void near_lines(const index_t *t, const float *pos, float hh, emit_fn emit, void *ctx)
{
    if (t->n_main > 0)
        get_nearby(t, t->main_tab, t->n_main, pos[0], pos, hh, emit, ctx);
    if (t->n_xx > 0)
        get_nearby(t, t->xx_tab, t->n_xx, pos[1], pos, hh, emit, ctx);
}

typedef struct {
    int32_t *lines;
    double *dr2;
    int n, cap;
} one_ctx;

static void emit_one(void *c, int line, double dr2)
{
    one_ctx *o = (one_ctx *)c;
    if (o->n < o->cap) {
        o->lines[o->n] = line;
        o->dr2[o->n] = dr2;
    }
    o->n++;
}

int fsgo_near_lines(const double *cofm, const int32_t *axis, int nlos, double box,
                    const float *pos3, float hh, int32_t *lines, double *dr2, int cap)
{
    index_t t;
    index_init(&t, cofm, axis, nlos, box);
    one_ctx o = {lines, dr2, 0, cap};
    near_lines(&t, pos3, hh, emit_one, &o);
    index_free(&t);
    /* std::map order: ascending sightline (insertion sort; lists are short) */
    int n = o.n < cap ? o.n : cap;
    for (int i = 1; i < n; i++) {
        int32_t l = lines[i];
        double d = dr2[i];
        int j = i - 1;
        while (j >= 0 && lines[j] > l) {
            lines[j + 1] = lines[j];
            dr2[j + 1] = dr2[j];
            j--;
        }
        lines[j + 1] = l;
        dr2[j + 1] = d;
    }
    return o.n;
}

/* growable per-thread pair buffer */
typedef struct {
    int32_t *line;
    int32_t *part;
    double *dr2;
    long long n, cap;
    int32_t cur_part;
} pair_buf;

static void emit_pair(void *c, int line, double dr2)
{
    pair_buf *b = (pair_buf *)c;
    if (b->n == b->cap) {
        long long nc = b->cap ? 2 * b->cap : 4096;
        b->line = (int32_t *)realloc(b->line, sizeof(int32_t) * nc);
        b->part = (int32_t *)realloc(b->part, sizeof(int32_t) * nc);
        b->dr2 = (double *)realloc(b->dr2, sizeof(double) * nc);
        b->cap = nc;
    }
    b->line[b->n] = line;
    b->part[b->n] = b->cur_part;
    b->dr2[b->n] = dr2;
    b->n++;
}

/* CSR pair lists.  Threads take contiguous particle chunks in order, so the
 * concatenation keeps ascending particle order within every sightline. */
typedef struct {
    long long *off; /* nlos + 1 */
    int32_t *part;
    double *dr2;
    long long total;
} csr_t;

static void build_csr(const float *pos, const float *h, long long npart, const int32_t *axis,
                      const double *cofm, int nlos, double box, csr_t *out)
{
    index_t t;
    index_init(&t, cofm, axis, nlos, box);
    int nth = fsgo_get_threads();
    pair_buf *bufs = (pair_buf *)calloc(nth, sizeof(pair_buf));
#pragma omp parallel num_threads(nth)
    {
        int tid = 0, nt = 1;
#ifdef _OPENMP
        tid = omp_get_thread_num();
        nt = omp_get_num_threads();
#endif
        long long chunk = (npart + nt - 1) / nt;
        long long p0 = tid * chunk, p1 = p0 + chunk < npart ? p0 + chunk : npart;
        pair_buf *b = &bufs[tid];
        for (long long i = p0; i < p1; i++) {
            b->cur_part = (int32_t)i;
            near_lines(&t, &pos[3 * i], h[i], emit_pair, b);
        }
    }
    out->off = (long long *)calloc((size_t)nlos + 1, sizeof(long long));
    long long total = 0;
    for (int k = 0; k < nth; k++)
        for (long long e = 0; e < bufs[k].n; e++)
            out->off[bufs[k].line[e] + 1]++;
    for (int i = 0; i < nlos; i++)
        out->off[i + 1] += out->off[i];
    total = out->off[nlos];
    out->total = total;
    out->part = (int32_t *)malloc(sizeof(int32_t) * (total > 0 ? total : 1));
    out->dr2 = (double *)malloc(sizeof(double) * (total > 0 ? total : 1));
    long long *cur = (long long *)malloc(sizeof(long long) * (nlos > 0 ? nlos : 1));
    for (int i = 0; i < nlos; i++)
        cur[i] = out->off[i];
    for (int k = 0; k < nth; k++) {
        for (long long e = 0; e < bufs[k].n; e++) {
            long long s = cur[bufs[k].line[e]]++;
            out->part[s] = bufs[k].part[e];
            out->dr2[s] = bufs[k].dr2[e];
        }
        free(bufs[k].line);
        free(bufs[k].part);
        free(bufs[k].dr2);
    }
    free(cur);
    free(bufs);
    index_free(&t);
}

long long fsgo_near_particles(const float *pos, const float *h, long long npart,
                              const int32_t *axis, const double *cofm, int nlos, double box,
                              long long *counts, int32_t *part, double *dr2, long long cap)
{
    csr_t c;
    build_csr(pos, h, npart, axis, cofm, nlos, box, &c);
    for (int i = 0; i < nlos; i++)
        counts[i] = c.off[i + 1] - c.off[i];
    if (c.total <= cap) {
        memcpy(part, c.part, sizeof(int32_t) * c.total);
        memcpy(dr2, c.dr2, sizeof(double) * c.total);
    }
    long long total = c.total;
    free(c.off);
    free(c.part);
    free(c.dr2);
    return total;
}

/* ------------------------------------------------------------------ */
/* Voronoi cells along a sightline, index_table.cpp:152-223            */
/* ------------------------------------------------------------------ */
#define O_RESO 0.1 /* index_table.h:8 */

/* The sightline is sampled at N = int(box/RESO) points; each belongs to the
 * nearest of the line's particles (periodic 3-D distance, the first in
 * ascending particle order on a tie).  Cell k of the list gets the segment
 * [seg[2k], seg[2k+1]] covered by its points (float, as the reference stores
 * it), 3 box for cells with no point.  Returns 0, or -3 where the reference
 * exits: a cell's points are not contiguous. */
int fsgo_assign_cells(const float *pos, const int32_t *part, int ncells, int axis,
                      const double *cofm3, double box, float *seg)
{
    for (int i = 0; i < 2 * ncells; ++i)
        seg[i] = (float)(3 * box);
    const int N = (int)(box / O_RESO);
    const double reso = box / N;
    const double yp = cofm3[axis % 3], zp = cofm3[(axis + 1) % 3];
    for (int i = 0; i < N; ++i) {
        const double xp = (i + 0.5) * reso;
        double min_dist = box;
        int min_ind = 0;
        for (int k = 0; k < ncells; k++) {
            const float *p3 = &pos[3 * (size_t)part[k]];
            double dx = fabs(p3[axis - 1] - xp);
            if (dx > box / 2.)
                dx = box - dx;
            double dy = fabs(p3[axis % 3] - yp);
            if (dy > box / 2.)
                dy = box - dy;
            double dz = fabs(p3[(axis + 1) % 3] - zp);
            if (dz > box / 2.)
                dz = box - dz;
            const double dist = sqrt(dx * dx + dy * dy + dz * dz);
            if (dist < min_dist) {
                min_dist = dist;
                min_ind = k;
            }
        }
        /* the first cell wraps around the box: the rest of the line is its */
        if (seg[2 * min_ind] < reso && xp > box / 2. + 0.5 * reso) {
            seg[2 * min_ind] = (float)xp;
            seg[2 * min_ind + 1] = (float)(seg[2 * min_ind + 1] + box);
            break;
        }
        if (xp > 1.5 * reso + seg[2 * min_ind + 1])
            return -3;
        if (seg[2 * min_ind] > 2 * box)
            seg[2 * min_ind] = (float)xp;
        seg[2 * min_ind + 1] = (float)xp;
    }
    for (int k = 0; k < ncells; ++k) {
        seg[2 * k] = (float)(seg[2 * k] - 0.5 * reso);
        seg[2 * k + 1] = (float)(seg[2 * k + 1] + 0.5 * reso);
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* ParticleInterp, part_int.cpp:20-84                                  */
/* ------------------------------------------------------------------ */
/* The interpolation, optionally timed: *t_search receives the wall seconds of
 * the pair search and line_sec[i] the seconds one thread spent depositing
 * sightline i (either may be NULL). */
static int interpolate_impl(int compute_tau, int nbins, int kernel, double box, double velfac,
                            double lambda, double gamma, double fosc, double amumass,
                            double tautail, const float *pos, const float *vel,
                            const float *dens, const float *temp, const float *h,
                            long long npart, const int32_t *axis, const double *cofm, int nlos,
                            double *out, long long *evals, double *t_search, double *line_sec)
{
    memset(out, 0, sizeof(double) * (size_t)nlos * (size_t)nbins);
    csr_t c;
    const double t0 = omp_get_wtime();
    build_csr(pos, h, npart, axis, cofm, nlos, box, &c);
    if (t_search)
        *t_search = omp_get_wtime() - t0;
    line_t l;
    line_init(&l, lambda, gamma, fosc, amumass, velfac, box, kernel, tautail);
    long long nev = 0;
    int failed = 0;
    int nth = fsgo_get_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth) reduction(+ : nev, failed)
    for (int i = 0; i < nlos; i++) {
        const double tl0 = line_sec ? omp_get_wtime() : 0.0;
        const int ax = axis[i];
        double *row = &out[(size_t)i * nbins];
        const long long m = c.off[i + 1] - c.off[i];
        float *seg = NULL;
        if (kernel == FSGO_VORONOI) {
            seg = (float *)malloc(sizeof(float) * 2 * (m > 0 ? m : 1));
            if (fsgo_assign_cells(pos, &c.part[c.off[i]], (int)m, ax, &cofm[3 * (size_t)i], box,
                                  seg) != 0) {
                failed++;
                free(seg);
                continue;
            }
        }
        for (long long e = c.off[i]; e < c.off[i + 1]; e++) {
            const int ip = c.part[e];
            const float ppos = pos[3 * (size_t)ip + ax - 1];
            /* the Voronoi mesh passes its segment ends for dr2 and smooth */
            const double d2 = seg ? (double)seg[2 * (e - c.off[i])] : c.dr2[e];
            const float sm = seg ? seg[2 * (e - c.off[i]) + 1] : h[ip];
            if (compute_tau)
                nev += add_tau(&l, row, nbins, d2, dens[ip], ppos, vel[3 * (size_t)ip + ax - 1],
                               temp[ip], sm);
            else
                add_colden(&l, row, nbins, d2, dens[ip], ppos, sm);
        }
        free(seg);
        if (line_sec)
            line_sec[i] = omp_get_wtime() - tl0;
    }
    if (evals)
        *evals = nev;
    free(c.off);
    free(c.part);
    free(c.dr2);
    return failed ? -3 : 0;
}

int fsgo_particle_interpolate(int compute_tau, int nbins, int kernel, double box, double velfac,
                              double atime, double lambda, double gamma, double fosc,
                              double amumass, double tautail, const float *pos, const float *vel,
                              const float *dens, const float *temp, const float *h,
                              long long npart, const int32_t *axis, const double *cofm, int nlos,
                              double *out, long long *evals)
{
    (void)atime;
    return interpolate_impl(compute_tau, nbins, kernel, box, velfac, lambda, gamma, fosc,
                            amumass, tautail, pos, vel, dens, temp, h, npart, axis, cofm, nlos,
                            out, evals, NULL, NULL);
}

int fsgo_particle_interpolate_timed(int compute_tau, int nbins, int kernel, double box,
                                    double velfac, double atime, double lambda, double gamma,
                                    double fosc, double amumass, double tautail,
                                    const float *pos, const float *vel, const float *dens,
                                    const float *temp, const float *h, long long npart,
                                    const int32_t *axis, const double *cofm, int nlos,
                                    double *out, double *t_search, double *line_sec)
{
    (void)atime;
    return interpolate_impl(compute_tau, nbins, kernel, box, velfac, lambda, gamma, fosc,
                            amumass, tautail, pos, vel, dens, temp, h, npart, axis, cofm, nlos,
                            out, NULL, t_search, line_sec);
}

/* Wall seconds of the pair search alone (IndexTable::get_near_particles,
 * index_table.cpp:130-150) for these sightlines; *npairs receives the pair count. */
double fsgo_search_seconds(const float *pos, const float *h, long long npart,
                           const int32_t *axis, const double *cofm, int nlos, double box,
                           long long *npairs)
{
    csr_t c;
    const double t0 = omp_get_wtime();
    build_csr(pos, h, npart, axis, cofm, nlos, box, &c);
    const double dt = omp_get_wtime() - t0;
    if (npairs)
        *npairs = c.total;
    free(c.off);
    free(c.part);
    free(c.dr2);
    return dt;
}
