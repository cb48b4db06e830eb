// Internal declarations shared by the CUDA translation units of libfsg.
//
// Data layout in HBM (one call):
//   particles   pos[3N] f32, vel[3N] f32, dens[N] f32, temp[N] f32, hh[N] f32
//               (the caller's arrays, structure-of-arrays except pos/vel)
//   sightlines  key[L] f64, second[L] f64, axis[L] i32  + one cell grid per axis
//   pairs       CSR by sightline: off[L+1] i64, part[P] i32, dr2[P] f64
//   spectra     out[L * nbins] f64 (row per sightline); per-sightline
//               128-bit fixed-point accumulators live in shared memory
#pragma once

#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>
#include <string>
#include <utility>
#include <vector>

namespace fsg {

inline float __int_as_float_host(int i)
{
    float f;
    static_assert(sizeof f == sizeof i, "int/float size");
    __builtin_memcpy(&f, &i, sizeof f);
    return f;
}

// Absolute slack of the float prefilter of the sightline search: the float
// minimum-image distance differs from the double one by at most ~2 ulp(box).
inline float prefilter_eps(double box)
{
    const float b = (float)box;
    return 4.0f * (__builtin_nextafterf(b, 2.0f * b + 1.0f) - b) + 1e-30f;
}

// kernel ids, fake_spectra/singleabs.h:9-12
enum KernelId { TOP_HAT = 0, SPH_CUBIC = 1, VORONOI = 2, SPH_QUINTIC = 3 };

// Device error bits (written by kernels, read by the host after a call)
enum DeviceError : unsigned {
    DEVERR_FIXED_OVERFLOW = 1u,   // a contribution exceeded its sightline's fixed-point range
    DEVERR_PAIR_SLOT = 2u,        // emit pass found more pairs than the count pass
    DEVERR_WINDOW_LIMIT = 4u,     // a pixel window or sub-sample count beyond the limits below
    DEVERR_PAIR_COUNT = 8u,       // emit pass wrote fewer pairs of a sightline than counted
    DEVERR_PAIR_INDEX = 16u,      // a pair names a particle outside [0, n) (pair skipped)
    DEVERR_VORONOI_CELL = 32u,    // a Voronoi cell's points along a sightline are not contiguous
    DEVERR_STAGE_WAIT = 64u,      // a staged copy of pair records did not complete in time
};

// Names of the set bits, for error messages ("fixed-point overflow, ...").
inline std::string deverr_text(unsigned bits)
{
    static const char *names[] = {"fixed-point overflow", "pair slot overflow",
                                  "window or sub-sample limit", "pair count mismatch",
                                  "pair particle index out of range",
                                  "non-contiguous Voronoi cell along a sightline",
                                  "staged pair-record copy timed out"};
    std::string r;
    for (int b = 0; b < 7; b++)
        if (bits & (1u << b))
            r += (r.empty() ? "" : ", ") + std::string(names[b]);
    return r.empty() ? "unknown" : r;
}

// Limits that turn inputs on which the reference loops for ever (or has
// undefined behaviour: T = 0, h = inf) into an error instead of a hang.
constexpr double MAX_SUBSAMPLES = 65536.0;       // tau_kern_outer points per pixel
constexpr long long MAX_COLDEN_WINDOW = 1ll << 26; // pixels of one colden pair

// One axis group of sightlines (all lines with axis a) on an nc x nc grid of
// transverse cells of width cw.  Lines sit in cells by their (first, second)
// transverse coordinates; the table key is the reference's multimap key.
struct LineGroup {
    int nlines;
    int nc;
    double cw, inv_cw;
    float cw_f, inv_cw_f;    // float copies for the cell-range superset
    const int *cell_start;   // nc*nc + 1
    const int *cell_line;    // global line ids, grouped by cell
};

struct LineTables {
    LineGroup g[3];          // axis 1, 2, 3
    const double *key;       // index_table.cpp:12-14: cofm[3i+1] (axis 1) or cofm[3i] (axes 2, 3)
    const double *second;    // index_table.cpp:33-39: cofm[3i+1] (axis 3) or cofm[3i+2]
    const int *axis;         // 1-based
    const float4 *pack;      // per line {key, second, axis bits, inside} in float (prefilter)
    int nlos;
    int n_main;              // lines with axis != 1 (the reference's index_table)
    int n_xx;                // lines with axis == 1 (the reference's index_table_xx)
    double box;
    float box_f;
    float box_up;            // smallest float f with (double)f > box
    float pre_eps;           // absolute slack of the float prefilter (4 ulp of the box)
};

// Float copy of the sightline tables for the search prefilter.  w = 1 when
// both coordinates lie in [0, box]: their float copies are then within half
// an ulp of the box of the double values, which the float accept test uses.
// Boxes outside [1e-12, 1e18] keep w = 0, so that the float squares of that
// test neither underflow nor overflow.
inline float4 pack_line(double key, double second, int axis, double box)
{
    float4 v;
    v.x = (float)key;
    v.y = (float)second;
    v.z = __int_as_float_host(axis);
    const bool inside = key >= 0.0 && key <= box && second >= 0.0 && second <= box;
    v.w = (inside && box >= 1e-12 && box <= 1e18) ? 1.f : 0.f;
    return v;
}

// The float constants of the tables derived from the box and the cell width.
inline void set_float_box(LineTables &t, double box)
{
    t.box_f = (float)box;
    float up = t.box_f;
    if (!((double)up > box))
        up = __builtin_nextafterf(up, __builtin_inff());
    t.box_up = up;
    t.pre_eps = prefilter_eps(box);
    for (LineGroup &G : t.g) {
        G.cw_f = (float)G.cw;
        G.inv_cw_f = (float)G.inv_cw;
    }
}

struct Particles {
    const float *pos;        // [3N]
    const float *vel;        // [3N] (tau only)
    const float *dens;       // [N]
    const float *temp;       // [N] (tau only)
    const float *hh;         // [N]
    long long n;
};

// LineAbsorption constants (absorption.cpp:152-161) plus the call geometry.
struct LineParams {
    int compute_tau;
    int nbins;
    int kernel;
    double tautail;
    double sigma_a;          // sqrt(3 pi sigma_T / 8) lambda f
    double bfac;             // sqrt(2 k_B / (m m_p)) / 1e5
    double voigt_fac;        // Gamma lambda / (4 pi) / 1e5
    double velfac;
    double vbox;             // box * velfac
    double box;
};

struct PairLists {
    const long long *off;    // [L+1]
    const int *part;         // [P]
    const double *dr2;       // [P]
    const float2 *seg = nullptr;   // [P] Voronoi cell segments (kernel 2), else null
    // [P] 32-byte pair records of the FP32 optical-depth deposit (written by
    // its bound pass, read by the deposit), or null: gather from the particles
    void *rec = nullptr;
};

// Host launchers (stream-ordered; no synchronisation inside).
// perm (may be null = identity): the order in which particles are visited.
void launch_count_pairs(const LineTables &t, const Particles &p, const int *perm,
                        unsigned long long *line_count, unsigned char *part_flag, cudaStream_t s);
// The emit pass writes part[]; dr2[] of every pair follows from it in a
// second, pair-parallel kernel inside the same launcher.
void launch_emit_pairs(const LineTables &t, const Particles &p, const int *perm,
                       const long long *off, unsigned long long *cursor, int *part, double *dr2,
                       unsigned *dev_err, cudaStream_t s);
// _near_lines: flag[i] = 1 when particle i is near any sightline (same
// predicate as the pair search); then an ordered compaction into ascending
// indices: tile counts (flag_tiles(n) of them), their exclusive scan
// (n <= 2048 * 2048 tiles) and the scatter.
void launch_flag_near(const LineTables &t, const Particles &p, const int *perm,
                      unsigned char *flag, cudaStream_t s);
long long flag_tiles(long long n);
void launch_flag_count(const unsigned char *flag, long long n, unsigned *tile_count,
                       cudaStream_t s);
void launch_exclusive_scan(const unsigned *in, unsigned *out, unsigned *sums, int n,
                           cudaStream_t s);
void launch_flag_scatter(const unsigned char *flag, long long n, const unsigned *tile_start,
                         int *out, cudaStream_t s);
// K weighted column densities in one pass (colden_channels_kernel): per
// channel a density array in and a (nlos x nbins) row block out; bad_lines
// [nch][nlos] and n_bad[nch] list the lines each channel leaves to the
// fallback.  Outside shared memory the accumulators take grid x
// acc_words_per_cta words of gacc.
constexpr int MAX_CHANNELS = 8;
struct ChannelPlan {
    int threads, smem_mode, per_sm;
    size_t smem, acc_words_per_cta;
};
ChannelPlan colden_channels_plan(int precision, int nch, int nbins);
void launch_colden_channels(const LineParams &lp, const LineTables &t, const Particles &p,
                            const PairLists &pl, const int *line_order, int nlos, int nch,
                            const float *const *dens, double *const *out, int *bad_lines,
                            int *n_bad, unsigned *ticket, unsigned *dev_err,
                            unsigned long long *gacc, int precision, const ChannelPlan &plan,
                            int grid, cudaStream_t s);

// Voronoi-mesh cells (fsg_voronoi.cu): seg[P] = the [left, right] segment
// of each pair's cell along its sightline (IndexTable::assign_cells); the
// pairs of a sightline must be in ascending particle order.  scratch holds
// voronoi_scratch_ints(P, L) ints; cofm is a device copy (3L doubles).
long long voronoi_scratch_ints(long long npairs, int nlos);
void launch_voronoi_cells(const float *pos, const int *part, const long long *off,
                          const int *axis, const double *cofm, int nlos, long long npairs,
                          double box, int *scratch, float2 *seg, unsigned *dev_err,
                          cudaStream_t s);

// Flux statistics (fsg_flux.cu): deterministic two-pass reductions over tau.
// part needs flux_partials(1) (resp. flux_partials(3)) doubles; etab is the
// table of exp_table_host on the device (the passes' exponential, fsg_fexp.cuh).
void launch_flux_sum(const double *tau, long long n, double scale, const double *etab,
                     double *part, double *out1, cudaStream_t s);
// `passes` Newton iterations of the mean-flux scale kept on the device:
// state[4] = {scale of the last pass, next scale (start: 1), converged, passes}.
// Passes after convergence do nothing.
void launch_newton_passes(const double *tau, long long n, double mfd, double tol, double thresh,
                          int passes, const double *etab, double *part, double *state,
                          cudaStream_t s);
// out[i] = exp(y[i]) with the passes' exponential
void launch_fexp(const double *y, long long n, const double *etab, double *out, cudaStream_t s);
// tab[256] = 2^(j/256) rounded to double
void exp_table_host(double *tab);
size_t flux_partials(int width);
// counts[nb] += np.histogram(exp(-scale tau), edges[nb+1]) (device edges)
void launch_flux_hist(const double *tau, long long n, double scale, const double *edges, int nb,
                      unsigned long long *counts, cudaStream_t s);

// Flux power (fsg_power.cu): own FP64 transforms of sightline pairs.
// Odd radices up to POWER_MAX_ODD_RADIX run as direct passes; a length with a
// larger prime factor goes through Bluestein's algorithm.
constexpr int POWER_MAX_ODD_RADIX = 63;
struct PowerPass {
    int radix = 0;
    long long ns = 1;        // product of the earlier passes' radices
    long long tw_off = 0;    // table offset of exp(-2 pi i k r / (ns R)), k < ns, r < R
    long long cs_off = -1;   // odd radix: table offset of (cos, sin)(2 pi t / R), t < R
};
struct PowerPlan {
    long long npix = -1;     // N
    long long len = 0;       // transform length: N, or Bluestein's M >= 2N - 1
    bool bluestein = false;
    std::vector<PowerPass> passes;
    long long table_len = 0;  // double2 entries of the pass tables
};
PowerPlan power_plan(long long npix);
// Fills the pass tables (table_len entries) and, for Bluestein, the chirp
// (npix entries) and the transform of the chirp filter (bhat, len entries;
// scratch: len entries).  Returns the kernel launches.
int power_plan_tables(const PowerPlan &pl, double2 *tables, double2 *chirp, double2 *bhat,
                      double2 *scratch, cudaStream_t s);
// Sightline pairs per chunk: a and b hold pairs x len complex values each.
long long power_pairs_per_chunk(const PowerPlan &pl, long long nspec);
// power[k] += vmax / npix^2 * sum over the rows of |rfft(exp(-scale tau) inv_mean - 1)(k)|^2,
// k = 0 .. npix/2, for `rows` sightlines of tau (DEVICE, rows x npix);
// partial needs power_partials(npix) doubles.  Returns the kernel launches.
int power_chunk(const PowerPlan &pl, const double2 *tables, const double2 *chirp,
                const double2 *bhat, const double *etab, const double *tau, long long rows,
                double scale, double inv_mean, double vmax, double2 *a, double2 *b,
                double *partial, double *power, cudaStream_t s);
size_t power_partials(long long npix);

// After emit: every sightline's cursor must equal its count (DEVERR_PAIR_COUNT
// otherwise), so no slot of the pair lists is left unwritten.
void launch_check_emit(const unsigned long long *line_count, const unsigned long long *cursor,
                       int nlos, unsigned *dev_err, cudaStream_t s);

// Counting sort of the particles by a G^3 spatial cell, so that the search
// visits neighbouring particles together.  Scratch: key[N], perm[N] (output),
// hist[G^3], start[G^3], sums[G^3/2048 + 1].
int sort_grid_side(long long n);
void launch_particle_order(const Particles &p, double box, int G, unsigned *key, unsigned *hist,
                           unsigned *start, unsigned *sums, int *perm, cudaStream_t s);

struct DepositLaunch {
    int precision;           // 0 = FP64 plain, 1 = FP32 tuned
    int threads;             // CTA size
    int persistent;          // 1: grid of resident CTAs draining a ticket queue
    int grid;                // persistent grid size (CTAs)
    int smem_mode;           // 1: per-sightline shared-memory accumulators
    int chunk;               // pairs staged per warp (FP32 form), else 0
    int tiles;               // in: allow far-field tiles (FP32 tau); out: planned
    int tiles_asked;         // what the caller allowed (tiles before planning)
    int rec;                 // FP32 tau: through pair records (PairLists::rec must be set)
};

// Deposits all pairs of all sightlines into out[L*nbins] (pre-zeroed).  Lines
// whose contributions are not all finite are appended to bad_lines (counter
// *n_bad) and left for deposit_fallback.
// counters (may be null): launches the counting variant, which adds {core-branch
// evals, wing-branch evals, other evals, pixels, multipole wing evals} into counters[0..4].
// Returns the number of kernels launched.
int launch_deposit(const LineParams &lp, const LineTables &t, const Particles &p,
                   const PairLists &pl, const int *line_order, int nlos, double *out,
                   unsigned *ticket, int *bad_lines, int *n_bad, unsigned *dev_err,
                   unsigned long long *gacc, unsigned long long *counters,
                   const DepositLaunch &cfg, cudaStream_t s);
// Chooses cfg.smem_mode and cfg.chunk (cfg.precision and cfg.threads set):
// shared-memory accumulators whenever they fit beside the pair staging area.
void deposit_plan(DepositLaunch &cfg, int compute_tau, int nbins);
// Dynamic shared memory of one deposit CTA.
size_t deposit_smem_bytes(const DepositLaunch &cfg, int compute_tau, int nbins);
// CTAs of the deposit kernel that fit on one SM for this configuration.
int deposit_resident_ctas(const DepositLaunch &cfg, int compute_tau, int nbins);
// Plain FP64 atomics into out for the listed lines (non-finite propagation).
void launch_deposit_fallback(const LineParams &lp, const LineTables &t, const Particles &p,
                             const PairLists &pl, const int *bad_lines, int n_bad, double *out,
                             unsigned *dev_err, cudaStream_t s);

// Same, with the count of listed sightlines read on the device (no host
// round trip, so it can be captured in a CUDA graph): grid of nlos blocks.
void launch_deposit_fallback_dev(const LineParams &lp, const LineTables &t, const Particles &p,
                                 const PairLists &pl, const int *bad_lines, const int *n_bad_dev,
                                 int nlos, double *out, unsigned *dev_err, cudaStream_t s);

// Largest nbins whose accumulators fit in shared memory (smallest staging area).
int deposit_max_smem_bins(int compute_tau, int precision, int threads);

// Backward of the FP32 tau deposit: accumulates (+=) dL/d(dens), dL/dT and
// dL/d(vel[3p+axis-1]) from dL/dtau (grad_tau, [L*nbins]).  Persistent grid.
void launch_tau_backward(const LineParams &lp, const LineTables &t, const Particles &p,
                         const PairLists &pl, const int *line_order, int nlos,
                         const double *grad_tau, float *g_dens, float *g_temp, float *g_vel,
                         unsigned *ticket, unsigned *dev_err, int grid, cudaStream_t s);
int tau_backward_resident_ctas();

// Peak FMA throughput of this GPU (TFLOP/s, 2 flops per FMA), own microbenchmark.
double measure_fma_peak(int precision, cudaStream_t s);

}  // namespace fsg
