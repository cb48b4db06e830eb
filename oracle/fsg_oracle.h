/*
 * TEST INFRASTRUCTURE ONLY -- the CPU oracle for the sightline-interpolation
 * path of fake_spectra (`_Particle_Interpolate`).  It is a restatement in
 * plain C of the reference algorithm, written for this project; it is used by
 * tests/, by __graft_entry__.smoke() as the checker, and by bench.py's CPU
 * baseline leg.  The product library (fake_spectra_gb300) never links it.
 *
 * Parity is pinned two ways: against the known-answer values of the
 * reference's own unit tests (fake_spectra/test.cpp) and, where the reference
 * sources are present, against the reference compiled unmodified
 * (oracle/build_ref.sh -> oracle/_ref/libfsref.so).
 */
#ifndef FSG_ORACLE_H
#define FSG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* kernel ids, fake_spectra/singleabs.h:9-12 */
#define FSGO_TOP_HAT 0
#define FSGO_SPH_CUBIC 1
#define FSGO_VORONOI 2
#define FSGO_SPH_QUINTIC 3

/* Full call, mirrors py_module.cpp:103-233 + part_int.cpp:20-84.
 * out: nlos*nbins doubles, zeroed here.  evals (may be NULL): receives the
 * number of Voigt-profile evaluations the reference's window rule performs
 * (compute_tau only).  Returns 0, or -2 for the unsupported Voronoi kernel. */
int fsgo_particle_interpolate(int compute_tau, int nbins, int kernel, double box, double velfac,
                              double atime, double lambda, double gamma, double fosc,
                              double amumass, double tautail, const float *pos, const float *vel,
                              const float *dens, const float *temp, const float *h,
                              long long npart, const int32_t *axis, const double *cofm, int nlos,
                              double *out, long long *evals);

/* Pair lists (index_table.cpp:130-150) as CSR by sightline, particles ascending.
 * Returns total pairs; part/dr2 are filled only if total <= cap. */
/* The same with timing: *t_search = wall seconds of the pair search,
 * line_sec[i] = one thread's seconds depositing sightline i (NULL = not wanted). */
int fsgo_particle_interpolate_timed(int compute_tau, int nbins, int kernel, double box,
                                    double velfac, double atime, double lambda, double gamma,
                                    double fosc, double amumass, double tautail,
                                    const float *pos, const float *vel, const float *dens,
                                    const float *temp, const float *h, long long npart,
                                    const int32_t *axis, const double *cofm, int nlos,
                                    double *out, double *t_search, double *line_sec);
/* Wall seconds of the pair search alone; *npairs receives the pair count. */
double fsgo_search_seconds(const float *pos, const float *h, long long npart,
                           const int32_t *axis, const double *cofm, int nlos, double box,
                           long long *npairs);

long long fsgo_near_particles(const float *pos, const float *h, long long npart,
                              const int32_t *axis, const double *cofm, int nlos, double box,
                              long long *counts, int32_t *part, double *dr2, long long cap);

/* Voronoi segments of one sightline's cells (index_table.cpp:152-223):
 * part[ncells] in ascending order, cofm3 the sightline position; seg[2*ncells].
 * Returns 0, or -3 where the reference exits (non-contiguous cell). */
int fsgo_assign_cells(const float *pos, const int32_t *part, int ncells, int axis,
                      const double *cofm3, double box, float *seg);

/* Lines near one particle (index_table.cpp:117-127); returns count. */
int fsgo_near_lines(const double *cofm, const int32_t *axis, int nlos, double box,
                    const float *pos3, float hh, int32_t *lines, double *dr2, int cap);

/* Voigt H(a,u) = Re w(u + i a) (singleabs.h:56-61 semantics) and w itself. */
double fsgo_voigt(double u, double a);
void fsgo_faddeeva(double x, double y, double *re, double *im);
double fsgo_dawson(double x);

double fsgo_sph_cubic_kernel(double q);
double fsgo_sph_quintic_kernel(double q);
double fsgo_kern_frac(int kernel, double zlow, double zhigh, double smooth, double dr2,
                      double zrange);
double fsgo_tau_kern_outer(double btherm, double vdr2, double vsmooth, double aa, int kernel,
                           double vlow, double vhigh);

void fsgo_add_tau_particle(double lambda, double gamma, double fosc, double amumass,
                           double velfac, double box, double atime, int kernel, double tautail,
                           double *tau, int nbins, double dr2, float dens, float ppos, float pvel,
                           float temp, float smooth, long long *evals);
void fsgo_add_colden_particle(double lambda, double gamma, double fosc, double amumass,
                              double velfac, double box, double atime, int kernel, double tautail,
                              double *colden, int nbins, double dr2, float dens, float ppos,
                              float smooth);

/* Threads the oracle's OpenMP regions use (0 = OpenMP default). */
void fsgo_set_threads(int n);
int fsgo_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
