/*
 * fsg.h -- C ABI of libfsg, the GB300 (sm_103a) implementation of
 * fake_spectra's sightline-interpolation path (`_Particle_Interpolate`).
 *
 * Plain C types only: pointers, sizes, doubles.  Every entry returns an
 * fsg_status; on failure a message is written to errbuf (if non-NULL).
 * Host-pointer entries behave like the reference call (synchronous, the
 * output is allocated by the caller and fully written).  Device-pointer
 * entries take CUDA device pointers for particle arrays and outputs, host
 * pointers for the (small) sightline tables, and run on the context's
 * stream; they return after the work has completed.
 */
#ifndef FSG_H
#define FSG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The Python layer maps them onto the exception classes the
 * reference raises (py_module.cpp:117-233). */
typedef enum {
    FSG_OK = 0,
    FSG_ERR_VALUE = 1,           /* bad size/shape/value      -> ValueError     */
    FSG_ERR_TYPE = 2,            /* wrong element type        -> TypeError      */
    FSG_ERR_MEMORY = 3,          /* allocation failed         -> MemoryError    */
    FSG_ERR_CUDA = 4,            /* CUDA runtime failure      -> RuntimeError   */
    FSG_ERR_NOT_IMPLEMENTED = 5, /* Voronoi kernel (kernel==2) -> NotImplementedError */
    FSG_ERR_DEVICE = 6           /* a kernel reported an internal limit        */
} fsg_status;

/* Arithmetic form of the deposit. */
typedef enum {
    FSG_PREC_FP64 = 0, /* plain form: FP64 everywhere (the drop-in default) */
    FSG_PREC_FP32 = 1  /* tuned form: FP32 profile/kernel arithmetic        */
} fsg_precision;

typedef struct {
    int precision;  /* fsg_precision                                         */
    int threads;    /* threads per deposit CTA; 0 = tuned (FP32 form) or the
                       library default                                        */
    int persistent; /* -1 = tuned (FP32) or default, 0 = one CTA per sightline,
                       1 = resident CTAs draining a sightline queue           */
    int count_work; /* 1 = run the counting variant of the deposit and report
                       the algorithmic work in fsg_stats (slower; for the
                       roofline only)                                         */
    int no_far_tiles; /* FP32 tau: 1 = deposit the far damping wing pixel by
                       pixel; 0 (default) = through per-tile Chebyshev nodes
                       where the node accumulators fit on chip               */
    int chunk;      /* FP32 form: sightline-particle pairs staged per warp
                       (1..32); 0 = tuned or default                          */
    int tune;       /* FP32 form, for the launch fields left at 0 / -1 above:
                       0 = the autotuner's choice for this class of workload,
                       timed on a sample of the call's sightlines the first
                       time the class is met, then cached; 1 = time again now;
                       -1 = library defaults, no tuning                       */
    int records;    /* FP32 optical depths: 1 = through 32-byte pair records
                       written by the deposit's bound pass and staged per warp
                       with bulk asynchronous copies; 0 = gather the particle
                       fields; -1 = tuned (FP32 form) or 0                    */
} fsg_options;

typedef struct {
    int64_t npairs;          /* sightline-particle pairs of the last search    */
    int64_t gpu_launches;    /* kernels this context has launched (cumulative) */
    int32_t fallback_lines;  /* sightlines re-run for non-finite contributions */
    int32_t reserved;
    double ms_search;        /* device time of the last pair search            */
    double ms_deposit;       /* device time of the last deposit                */
    /* Work of the last deposit when count_work was set: Voigt-profile
     * evaluations by branch and pixel contributions, for the pixels the
     * reference's tautail window rule evaluates (absorption.cpp:250-278). */
    int64_t evals_core;      /* FP64: Taylor branch; FP32: tabulated core form */
    int64_t evals_wing;      /* asymptotic branch                               */
    int64_t evals_other;     /* a == 0, a < 0 or a > 0.1 (FP32: FP64 profile)   */
    int64_t pixels;          /* pixel contributions                             */
    int64_t evals_wing_multipole; /* wing evaluations summed by the far-wing
                                     multipole form (FP32; subset of evals_wing) */
    /* FP32 node-sum samples (7 evaluations each) by warp-uniform path; the
     * multipole path has evals_wing_multipole / 7 */
    int64_t samples_wing_path;   /* every node asymptotic                  */
    int64_t samples_core_path;   /* every node in the tabulated core       */
    int64_t samples_mixed_path;  /* node by node                           */
    /* Launch of the last deposit and where it came from */
    int32_t launch_threads, launch_chunk, launch_persistent;
    int32_t launch_tuned;        /* 1: from the autotuner (cache or a run in this call) */
    int32_t tune_ran;            /* 1: the autotuner timed candidates in this call */
    int32_t tune_candidates;     /* candidates timed by that run */
    int32_t tune_sample_lines;   /* sightlines of its timing sample */
    int32_t launch_records;      /* 1: the deposit went through pair records */
    double tune_ms_default;      /* deposit of the sample with the library defaults */
    double tune_ms_best;         /* ... with the chosen launch */
    /* host-pointer entry points: the host->device copies of the inputs and the
     * device->host copy of the output of the last call, device time */
    double ms_h2d, ms_d2h;
    double ms_flux;              /* device time of the last flux-statistics call's kernels */
    int32_t search_reused;       /* 1: the last backward call reused the last search */
} fsg_stats;

typedef struct fsg_context fsg_context;

/* Library version string. */
const char *fsg_version(void);

/* Peak FMA throughput of the current GPU in TFLOP/s (2 flops per FMA) for
 * precision FSG_PREC_FP64 or FSG_PREC_FP32, from this library's own
 * microbenchmark; the roofline denominator of the compute-bound deposit. */
int fsg_measure_fma_peak(int precision, double *tflops, char *errbuf, size_t errlen);

/* Context: one device, one stream, a grow-only device workspace and the pair
 * lists of the last search. */
int fsg_context_create(int device, fsg_context **ctx, char *errbuf, size_t errlen);
void fsg_context_destroy(fsg_context *ctx);
/* Run the context's work on a caller's cudaStream_t; NULL is the CUDA default
 * stream (handle 0, torch's default).  Until the first call a context runs on
 * a non-blocking stream of its own, which is not ordered with the default
 * stream: a caller whose inputs are produced on another stream binds that
 * stream here first. */
int fsg_context_set_stream(fsg_context *ctx, void *cuda_stream);
int fsg_context_stats(const fsg_context *ctx, fsg_stats *out);
/* Statistics of the library-owned context of the current device, which the
 * host-pointer entry points (fsg_particle_interpolate, fsg_near_lines,
 * fsg_rescale_mean_flux) use; FSG_ERR_VALUE before its first use. */
int fsg_default_context_stats(fsg_stats *out);

/*
 * Drop-in for _spectra_priv._Particle_Interpolate
 * (fake_spectra/py_module.cpp:103-233, Py_Particle_Interpolation), with the
 * same positional arguments and units:
 *   compute_tau  1: optical depth (ParticleInterp::compute_tau, part_int.cpp:20-51)
 *                0: column density (ParticleInterp::compute_colden, part_int.cpp:53-84)
 *   pos, vel     [npart*3] float32; vel and temp are not read when compute_tau == 0
 *   dens, temp, h [npart] float32
 *   axis [nlos] int32 (1, 2 or 3), cofm [nlos*3] float64
 *   out  [nlos*nbins] float64, written completely (zero where nothing absorbs)
 * All pointers are HOST pointers.  opt may be NULL (plain FP64 form).
 * Uses a library-owned context for device 0 (or the current device).
 */
int fsg_particle_interpolate(int compute_tau, int nbins, int kernel, double box, double velfac,
                             double atime, double lambda, double gamma, double fosc,
                             double amumass, double tautail, const float *pos, const float *vel,
                             const float *dens, const float *temp, const float *h, int64_t npart,
                             const int32_t *axis, const double *cofm, int32_t nlos, double *out,
                             const fsg_options *opt, char *errbuf, size_t errlen);

/* Same computation with DEVICE pointers for pos/vel/dens/temp/h/out; axis and
 * cofm stay HOST pointers. */
int fsg_particle_interpolate_device(fsg_context *ctx, int compute_tau, int nbins, int kernel,
                                    double box, double velfac, double atime, double lambda,
                                    double gamma, double fosc, double amumass, double tautail,
                                    const float *pos, const float *vel, const float *dens,
                                    const float *temp, const float *h, int64_t npart,
                                    const int32_t *axis, const double *cofm, int32_t nlos,
                                    double *out, const fsg_options *opt, char *errbuf,
                                    size_t errlen);

/*
 * Sightline-particle search alone: replaces IndexTable::get_near_particles
 * (fake_spectra/index_table.cpp:130-150).  pos/h are DEVICE pointers; axis/cofm
 * HOST.  The pair lists stay in the context; *npairs receives their total.
 */
int fsg_build_pairs_device(fsg_context *ctx, double box, const float *pos, const float *h,
                           int64_t npart, const int32_t *axis, const double *cofm, int32_t nlos,
                           int64_t *npairs, char *errbuf, size_t errlen);

/*
 * Drop-in for _spectra_priv._near_lines (fake_spectra/py_module.cpp:25-99,
 * Py_near_lines): the indices of the particles that lie within their
 * smoothing length of at least one sightline (IndexTable::get_near_lines
 * non-empty, fake_spectra/index_table.cpp:117-127), in ascending order, as the
 * reference's std::set<int> returns them.  pos (npart x 3) and h are HOST
 * pointers; out (host) must hold npart entries; *nout receives the count.
 */
int fsg_near_lines(double box, const float *pos, const float *h, int64_t npart,
                   const int32_t *axis, const double *cofm, int32_t nlos, int32_t *out,
                   int64_t *nout, char *errbuf, size_t errlen);

/* The same with pos/h/out DEVICE pointers (axis/cofm HOST), on ctx's stream. */
int fsg_near_lines_device(fsg_context *ctx, double box, const float *pos, const float *h,
                          int64_t npart, const int32_t *axis, const double *cofm, int32_t nlos,
                          int32_t *out, int64_t *nout, char *errbuf, size_t errlen);

/*
 * Several weighted column densities in one pass: channel c is the
 * compute_tau=0 interpolation with density array dens[c] (DEVICE), written to
 * out[c] (DEVICE, nlos x nbins).  This replaces the weighted column-density
 * calls of Spectra.get_velocity, get_temp and get_dens_weighted_density
 * (fake_spectra/spectra.py:945-1043: one _Particle_Interpolate(0, ...) per
 * weight); every channel equals its single-channel result bit for bit.
 * 1 <= nch <= 8; pos/h DEVICE, axis/cofm HOST; opt->precision as for the
 * interpolation.
 */
int fsg_colden_channels_device(fsg_context *ctx, int nbins, int kernel, double box,
                               double velfac, const float *pos, const float *h, int64_t npart,
                               const int32_t *axis, const double *cofm, int32_t nlos, int nch,
                               const float *const *dens, double *const *out,
                               const fsg_options *opt, char *errbuf, size_t errlen);

/*
 * Flux statistics of optical depths (float64, row-major NumLos x npix).
 *
 * Drop-in for _spectra_priv._rescale_mean_flux (fake_spectra/py_module.cpp:
 * 235-282, get_mean_flux_scale / Py_mean_flux): the Newton-Raphson scale s
 * with mean(exp(-s tau)) = mean_flux_desired over the n pixels with
 * tau <= thresh, iterated until |s_new - s| <= tol s_new (s starts at 1 and is
 * kept above 0).  tau is a HOST pointer here and a DEVICE pointer in the
 * _device form; the sums run on the GPU in a fixed order.
 */
int fsg_rescale_mean_flux(const double *tau, int64_t n, double mean_flux_desired, double tol,
                          double thresh, double *scale, char *errbuf, size_t errlen);
int fsg_mean_flux_scale_device(fsg_context *ctx, const double *tau, int64_t n,
                               double mean_flux_desired, double tol, double thresh, double *scale,
                               char *errbuf, size_t errlen);

/* mean(exp(-scale tau)) over n device values (fluxstatistics.py:96, np.mean). */
int fsg_mean_flux_device(fsg_context *ctx, const double *tau, int64_t n, double scale,
                         double *mean, char *errbuf, size_t errlen);

/* out[i] = exp(y[i]) (y, out DEVICE, n doubles) with the FP64 exponential the
 * mean-flux and flux-power passes use (table-driven, within about one ulp of
 * exp); exposed so that its accuracy can be checked. */
int fsg_flux_exp_device(fsg_context *ctx, const double *y, int64_t n, double *out, char *errbuf,
                        size_t errlen);

/* The counts of np.histogram(exp(-scale tau), edges) for the flux PDF
 * (fake_spectra/fluxstatistics.py:42-51): bin j holds edges[j] <= F <
 * edges[j+1], the last bin also F == edges[nb]; F outside [edges[0], edges[nb]]
 * or NaN is not counted.  1 <= nb <= 8192.  tau DEVICE, edges (nb+1) and
 * counts (nb) HOST. */
int fsg_flux_histogram_device(fsg_context *ctx, const double *tau, int64_t n, double scale,
                              const double *edges, int nb, int64_t *counts, char *errbuf,
                              size_t errlen);

/* The 1-D flux power of fake_spectra/fluxstatistics.py:53-110 before its
 * window division: power[k] = vmax / nspec * sum over sightlines of
 * |rfft(exp(-scale tau) / mean_flux - 1)(k)|^2 / npix^2, k = 0 .. npix/2.
 * tau DEVICE (nspec x npix), power HOST (npix/2 + 1).  The transforms are
 * cuFFT double-precision real-to-complex, batched over sightlines. */
int fsg_flux_power_device(fsg_context *ctx, const double *tau, int64_t nspec, int64_t npix,
                          double scale, double mean_flux, double vmax, double *power,
                          char *errbuf, size_t errlen);

/*
 * Batched form: several absorption lines of one snapshot in one call.  The
 * reference needs one _Particle_Interpolate call per line and per quantity
 * (spectra.py:801-831 compute_spectra, once per line; colden via
 * compute_tau=0); here the sightline search runs once and every deposit of
 * the call is captured in one CUDA graph.  Per line: its constants, its
 * species density (DEVICE [npart], n_ion * rscale) and where to write tau
 * and/or colden (DEVICE [nlos*nbins], NULL = not wanted).
 */
typedef struct {
    double lambda, gamma, fosc, amumass;
    const float *dens;
    double *tau;
    double *colden;
} fsg_line;

int fsg_spectra_batch_device(fsg_context *ctx, int nbins, int kernel, double box, double velfac,
                             double atime, double tautail, const float *pos, const float *vel,
                             const float *temp, const float *h, int64_t npart,
                             const int32_t *axis, const double *cofm, int32_t nlos, int nlines,
                             const fsg_line *lines, const fsg_options *opt, char *errbuf,
                             size_t errlen);

/*
 * Backward of the tau deposit (tuned FP32 form), for gradient-based fitting of
 * particle fields; no counterpart call in the reference, whose tau is
 * ParticleInterp::compute_tau (part_int.cpp:20-51).  Given dL/dtau
 * (grad_tau, DEVICE [nlos*nbins] float64) it ADDS to grad_dens[npart],
 * grad_temp[npart] and grad_vel[3*npart] (DEVICE float32; the component along
 * each sightline's axis) the gradient of L with respect to dens, temp and the
 * line-of-sight velocity.  The sightline search and the profiles are
 * recomputed; the pixel windows and sub-sample counts are held fixed.
 */
int fsg_tau_backward_device(fsg_context *ctx, int nbins, int kernel, double box, double velfac,
                            double atime, double lambda, double gamma, double fosc,
                            double amumass, double tautail, const float *pos, const float *vel,
                            const float *dens, const float *temp, const float *h, int64_t npart,
                            const int32_t *axis, const double *cofm, int32_t nlos,
                            const double *grad_tau, float *grad_dens, float *grad_temp,
                            float *grad_vel, char *errbuf, size_t errlen);

/* fsg_tau_backward_device that reuses the sightline search of the forward call
 * it follows: when `generation` is the context's search generation
 * (fsg_context_search_generation right after that call) and pos, h, npart,
 * nlos, box and the axis/cofm contents are those the search used, the pair
 * lists are taken as they are (the caller must not have changed the contents
 * of pos and h in between); otherwise the search runs again.  Same arguments
 * and results as fsg_tau_backward_device. */
int fsg_tau_backward_reuse_device(fsg_context *ctx, uint64_t generation, int nbins, int kernel,
                                  double box, double velfac, double atime, double lambda,
                                  double gamma, double fosc, double amumass, double tautail,
                                  const float *pos, const float *vel, const float *dens,
                                  const float *temp, const float *h, int64_t npart,
                                  const int32_t *axis, const double *cofm, int32_t nlos,
                                  const double *grad_tau, float *grad_dens, float *grad_temp,
                                  float *grad_vel, char *errbuf, size_t errlen);

/* The context's sightline-search generation: it grows by one with every
 * search the context runs. */
int fsg_context_search_generation(const fsg_context *ctx, uint64_t *generation);

/* Copy the context's pair lists to HOST buffers as CSR by sightline:
 * offsets[nlos+1], part[npairs], dr2[npairs].  Within a sightline the pairs
 * are sorted by ascending particle index (the std::map order of the
 * reference) when sorted != 0, else in arrival order. */
int fsg_copy_pairs(fsg_context *ctx, int64_t *offsets, int32_t *part, double *dr2, int sorted,
                   char *errbuf, size_t errlen);

/*
 * Autotuner cache of the FP32 deposit's launch (no counterpart in the
 * reference, whose only schedule is OpenMP's default over sightlines,
 * part_int.cpp:25-27).  A workload class is described by fsg_tune_key; its
 * entry is the launch the tuner chose and the sample timings.  The cache lives
 * in the process; fsg_tune_cache_file names a text file that it is loaded from
 * and appended to (also taken from the FSG_TUNE_CACHE environment variable on
 * first use).  Host-only functions: no GPU is touched.
 */
typedef struct {
    int32_t sms;          /* multiprocessors of the device                       */
    int32_t precision;    /* fsg_precision                                       */
    int32_t compute_tau;
    int32_t kernel;
    int32_t nbins_b;      /* floor(2 log2 nbins)                                 */
    int32_t pairs_med_b;  /* floor(2 log2(1 + median pairs per sightline))      */
    int32_t pairs_p99_b;  /* floor(2 log2(1 + 99th-percentile pairs per line))  */
    int32_t lines_b;      /* floor(log2 sightlines)                              */
    int32_t damp_b;       /* floor(2 log2(Gamma lambda / 4 pi / b(T = 1 K)))    */
} fsg_tune_key;

typedef struct {
    int32_t threads, chunk, persistent, records;   /* the chosen launch (fsg_options) */
    int32_t candidates, sample_lines;
    double ms_default, ms_best;
} fsg_tune_entry;

int fsg_tune_cache_file(const char *path, char *errbuf, size_t errlen);
int fsg_tune_cache_lookup(const fsg_tune_key *key, fsg_tune_entry *entry); /* 1 found, 0 not */
int fsg_tune_cache_store(const fsg_tune_key *key, const fsg_tune_entry *entry, char *errbuf,
                         size_t errlen);
void fsg_tune_cache_clear(void);   /* empties the in-process cache (the file is kept) */

/*
 * The same interpolation with NO device memory allocation, for callers that
 * cannot call cudaMalloc (their host application's allocator owns the GPU
 * memory, or they run inside a loop that must not trigger the synchronisation
 * an allocation may imply).  This entry point has no counterpart in the
 * reference.  pos/vel/dens/temp/h/out are DEVICE pointers of the current
 * device (checked; another device's pointers return FSG_ERR_VALUE before any
 * work is queued), axis/cofm HOST pointers, stream a cudaStream_t of the
 * current device (NULL = the default stream); precision is an fsg_precision.
 * All scratch lives in one 64 MiB file-scope device array that every GPU
 * loading the library keeps until exit.  Limits, larger calls returning
 * FSG_ERR_VALUE:
 *   nlos <= 8192 sightlines;
 *   about 5.4 million sightline-particle pairs (the rest of the array, 12
 *   bytes per pair; checked after the pair count);
 *   nbins within the shared-memory capacity of one deposit block: 16 bytes
 *   per pixel beside the pair staging area, out of the device's opt-in
 *   maximum less 2 KiB.  With GB300's 227 KiB: 14400 pixels in the FP64 form,
 *   13760 for FP32 optical depths, 14016 for FP32 column densities.
 * The first call on a device looks up the array's address; the address is
 * kept for the life of the process, so a cudaDeviceReset between calls is not
 * supported.  Calls share the array:
 * they are serialised by a lock and complete before returning (error returns
 * included); GPU work overlapping a call on the same array would race.
 */
int fsg_particle_interpolate_noalloc(int compute_tau, int nbins, int kernel, double box,
                                     double velfac, double atime, double lambda, double gamma,
                                     double fosc, double amumass, double tautail,
                                     const float *pos, const float *vel, const float *dens,
                                     const float *temp, const float *h, int64_t npart,
                                     const int32_t *axis, const double *cofm, int32_t nlos,
                                     double *out, int precision, void *stream, char *errbuf,
                                     size_t errlen);

#ifdef __cplusplus
}
#endif

#endif /* FSG_H */
