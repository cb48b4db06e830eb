/* Test helper (compiled by tests/test_search_bounds.py): restates in C the
 * float decisions of the GPU sightline search (fake_spectra_gb300/csrc/
 * fsg_index.cu: accept(), cell_range()) and checks them against the
 * reference predicate (fake_spectra/index_table.cpp:45-113: the float window,
 * second_close, calc_dr2) on seeded adversarial cases:
 *   1. the float fast accept implies the exact predicate;
 *   2. the float cell range covers the double cell range of the previous form
 *      (which covers every sightline the predicate can accept).
 * Compiled with -ffp-contract=off so every operation rounds as written.
 * Prints "bad=<n>" per check; exit status 0 when both are 0. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

typedef struct { float ffm, ffp; int nowrap; } Window;

static uint64_t rng_state = 88172645463325252ull;
static double U(void)
{
    rng_state ^= rng_state << 13;
    rng_state ^= rng_state >> 7;
    rng_state ^= rng_state << 17;
    return (double)(rng_state >> 11) * (1.0 / 9007199254740992.0);
}

static Window make_window(float first, float hh, double box)
{
    Window w;
    float ffp = first + hh;
    if ((double)ffp > box)
        ffp = (float)((double)ffp - box);
    float ffm = first - hh;
    if (ffm < 0.0f)
        ffm = (float)((double)ffm + box);
    w.ffm = ffm;
    w.ffp = ffp;
    w.nowrap = (ffm <= ffp);
    return w;
}

static int in_window(Window w, double key)
{
    if (w.nowrap)
        return ((double)w.ffm <= key) && (key < (double)w.ffp);
    return (key < (double)w.ffp) || (key >= (double)w.ffm);
}

static int second_close(float second, double l2, float hh, double box)
{
    float ffp = second + hh;
    if ((double)ffp > box && l2 < (double)ffp - box)
        return 1;
    float ffm = second - hh;
    if (ffm < 0.0f && l2 > (double)ffm + box)
        return 1;
    return (l2 > (double)ffm) && (l2 < (double)ffp);
}

static double calc_dr2(double d1, double d2, double box)
{
    const double half = 0.5 * box;
    double dr = fabs(d1);
    if (dr > half)
        dr = box - dr;
    double dr2 = dr * dr;
    dr = fabs(d2);
    if (dr > half)
        dr = box - dr;
    return dr2 + dr * dr;
}

static int exact(float f, float s, double K, double L, float hh, double box)
{
    Window w = make_window(f, hh, box);
    if (!in_window(w, K) || !second_close(s, L, hh, box))
        return 0;
    return calc_dr2((double)f - K, (double)s - L, box) <= (double)(float)(hh * hh);
}

static float pre_eps_of(double box)
{
    const float b = (float)box;
    return 4.0f * (nextafterf(b, 2.0f * b + 1.0f) - b) + 1e-30f;
}

static int fast(float f, float s, double K, double L, float hh, double box)
{
    if (!(K >= 0 && K <= box && L >= 0 && L <= box && box >= 1e-12 && box <= 1e18))
        return 0;
    const float bf = (float)box, pe = pre_eps_of(box), kx = (float)K, ky = (float)L;
    const float d1 = fabsf(f - kx), d2 = fabsf(s - ky);
    if (!(d1 <= bf && d2 <= bf && hh > 0.0f))
        return 0;
    const float a = fmaf(d1, 1.0000005f, pe), b = fmaf(d2, 1.0000005f, pe);
    const float half_in = 0.49f * bf;
    const Window w = make_window(f, hh, box);
    const int wh = w.nowrap ? (kx > w.ffm && kx < w.ffp) : (kx < w.ffp || kx > w.ffm);
    const int sh = ky > s - hh && ky < s + hh;
    return a <= half_in && b <= half_in && fmaf(a, a, b * b) <= (hh * hh) * 0.999995f && wh && sh;
}

static int covers(int a0, int an, int nc, long long cell)
{
    const long long c = ((cell % nc) + nc) % nc;
    if (an >= nc)
        return 1;
    return (((c - a0) % nc) + nc) % nc < an;
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 2000000;
    const double boxes[] = {25000., 1.0, 75000., 3.7e-3, 1e6, 100.123456789};
    long bad1 = 0, nfast = 0, nexact = 0, bad2 = 0;
    for (int bi = 0; bi < 6; bi++) {
        const double box = boxes[bi];
        for (long it = 0; it < n; it++) {
            const float hh = (float)(box * pow(10.0, -4 + 3.5 * U()));
            double K = box * U(), L = box * U();
            if (it % 3 == 0)   /* near the periodic edges */
                K = (U() < 0.5) ? box * U() * 1e-3 : box * (1 - U() * 1e-3);
            const double ang = 2 * M_PI * U();
            double rr = hh * (1 + (U() - 0.5) * 2e-5 * pow(10.0, -3 * U()));   /* the shell */
            if (it % 5 == 0)
                rr = hh * U();
            float f = (float)(K + rr * cos(ang)), s = (float)(L + rr * sin(ang));
            if (it % 7 == 0) {
                f = (float)fmod(f + box, box);
                s = (float)fmod(s + box, box);
            }
            const int fa = fast(f, s, K, L, hh, box), ex = exact(f, s, K, L, hh, box);
            nfast += fa;
            nexact += ex;
            if (fa && !ex)
                bad1++;
        }
        /* cell ranges: the float form against the double form */
        for (long it = 0; it < n; it++) {
            int nc = 1 + (int)(U() * 1024);
            if (it % 4 == 0)
                nc = 1024;
            const double cw = box / nc, inv = nc / box;
            const float cwf = (float)cw, invf = (float)inv;
            const float hh = (float)(box * pow(10.0, -5 + 4.5 * U()));
            float c = (float)(box * (-0.2 + 1.4 * U()));
            if (it % 3 == 0)   /* on cell edges */
                c = (float)(floor(U() * nc) * cw);
            const double reach = (double)hh * (1 + 1e-6) + 1e-6 * cw;
            const double lo = floor((c - reach) * inv), hi = floor((c + reach) * inv);
            const float r = fmaf(0.02f, cwf, hh * 1.00001f);
            const float flo = floorf((c - r) * invf), fhi = floorf((c + r) * invf);
            const float fn = fhi - flo + 1.0f;
            int a0, an;
            if (!(fabsf(c) <= 4.0f * (float)box) || !(fn < (float)nc)) {
                a0 = 0;
                an = nc;
            } else {
                int l = (int)flo % nc;
                if (l < 0)
                    l += nc;
                a0 = l;
                an = (int)fn;
            }
            if (hi - lo + 1 >= nc)
                continue;
            for (long long q = (long long)lo; q <= (long long)hi; q++)
                if (!covers(a0, an, nc, q)) {
                    bad2++;
                    break;
                }
        }
    }
    printf("fast_accept bad=%ld fast=%ld exact=%ld\n", bad1, nfast, nexact);
    printf("cell_range bad=%ld\n", bad2);
    return (bad1 || bad2 || nfast == 0) ? 1 : 0;
}
