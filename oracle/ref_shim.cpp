/*
 * Test infrastructure only: a C-linkage shim over the UNMODIFIED reference
 * C++ sources of fake_spectra (part_int.cpp, absorption.cpp, index_table.cpp,
 * Faddeeva.cpp), compiled from where they lie by oracle/build_ref.sh into
 * oracle/_ref/libfsref.so.  Nothing in the product links or loads this file;
 * tests use it to pin the C restatement in oracle/fsg_oracle.c.
 *
 * Each entry mirrors one reference interface:
 *   fsr_particle_interpolate  -> py_module.cpp:103-233 (Py_Particle_Interpolation)
 *   fsr_near_particles        -> index_table.cpp:130-150 (IndexTable::get_near_particles)
 *   fsr_near_lines            -> index_table.cpp:117-127 (IndexTable::get_near_lines)
 *   fsr_profile               -> singleabs.h:56-61 (profile)
 *   fsr_tau_kern_outer        -> singleabs.h:104-126 (SingleAbsorber::tau_kern_outer)
 *   fsr_sph_cubic_kernel      -> singleabs.h:17-26
 *   fsr_sph_quintic_kernel    -> singleabs.h:31-42
 *   fsr_sph_cubic_kern_frac   -> absorption.cpp:53-74
 *   fsr_add_tau_particle      -> absorption.cpp:212-279
 *   fsr_add_colden_particle   -> absorption.cpp:167-210
 */
#include "part_int.h"
#include "singleabs.h"
#include "index_table.h"
#include <cstdint>
#include <cstring>
#include <map>
#include <valarray>

extern "C" {

int fsr_particle_interpolate(int compute_tau, int nbins, int kernel, double box, double velfac,
                             double atime, double lambda, double gamma, double fosc,
                             double amumass, double tautail, const float *pos, const float *vel,
                             const float *dens, const float *temp, const float *h, long long npart,
                             const int32_t *axis, const double *cofm, int nlos, double *out)
{
    ParticleInterp pint(nbins, lambda, gamma, fosc, amumass, box, velfac, atime, cofm,
                        (const int *)axis, nlos, kernel, tautail);
    std::memset(out, 0, sizeof(double) * (size_t)nlos * (size_t)nbins);
    if (compute_tau)
        pint.compute_tau(out, pos, vel, dens, temp, h, npart);
    else
        pint.compute_colden(out, pos, dens, h, npart);
    return 0;
}

/* Pair lists as CSR by sightline: counts[nlos]; part/dr2 filled in sightline
 * order and ascending particle order inside a sightline (the std::map order).
 * Returns the total number of pairs; fills part/dr2 only when cap suffices. */
long long fsr_near_particles(const float *pos, const float *h, long long npart,
                             const int32_t *axis, const double *cofm, int nlos, double box,
                             long long *counts, int32_t *part, double *dr2, long long cap)
{
    IndexTable tab(cofm, (const int *)axis, nlos, box);
    std::valarray<std::map<int, double>> near = tab.get_near_particles(pos, h, npart);
    long long total = 0;
    for (int i = 0; i < nlos; i++) {
        counts[i] = (long long)near[i].size();
        total += counts[i];
    }
    if (total > cap)
        return total;
    long long k = 0;
    for (int i = 0; i < nlos; i++)
        for (std::map<int, double>::const_iterator it = near[i].begin(); it != near[i].end(); ++it) {
            part[k] = it->first;
            dr2[k] = it->second;
            k++;
        }
    return total;
}

/* Lines near one particle: returns count, fills (line, dr2) in line order up to cap. */
int fsr_near_lines(const double *cofm, const int32_t *axis, int nlos, double box,
                   const float *pos3, float hh, int32_t *lines, double *dr2, int cap)
{
    IndexTable tab(cofm, (const int *)axis, nlos, box);
    std::map<int, double> near = tab.get_near_lines(pos3, hh);
    int k = 0;
    for (std::map<int, double>::const_iterator it = near.begin(); it != near.end(); ++it) {
        if (k < cap) {
            lines[k] = it->first;
            dr2[k] = it->second;
        }
        k++;
    }
    return k;
}

double fsr_profile(double u, double a) { return profile(u, a); }
double fsr_sph_cubic_kernel(double q) { return sph_cubic_kernel(q); }
double fsr_sph_quintic_kernel(double q) { return sph_quintic_kernel(q); }
double fsr_sph_cubic_kern_frac(double zlow, double zhigh, double smooth, double dr2, double zrange)
{
    return sph_cubic_kern_frac(zlow, zhigh, smooth, dr2, zrange);
}

double fsr_tau_kern_outer(double btherm, double vdr2, double vsmooth, double aa, int kernel,
                          double vlow, double vhigh)
{
    SingleAbsorber s(btherm, vdr2, vsmooth, aa, kernel);
    return s.tau_kern_outer(vlow, vhigh);
}

void fsr_add_tau_particle(double lambda, double gamma, double fosc, double amumass, double velfac,
                          double box, double atime, int kernel, double tautail, double *tau,
                          int nbins, double dr2, float dens, float ppos, float pvel, float temp,
                          float smooth)
{
    LineAbsorption la(lambda, gamma, fosc, amumass, velfac, box, atime, kernel, tautail);
    la.add_tau_particle(tau, nbins, dr2, dens, ppos, pvel, temp, smooth);
}

void fsr_add_colden_particle(double lambda, double gamma, double fosc, double amumass,
                             double velfac, double box, double atime, int kernel, double tautail,
                             double *colden, int nbins, double dr2, float dens, float ppos,
                             float smooth)
{
    LineAbsorption la(lambda, gamma, fosc, amumass, velfac, box, atime, kernel, tautail);
    la.add_colden_particle(colden, nbins, dr2, dens, ppos, smooth);
}

} /* extern "C" */
