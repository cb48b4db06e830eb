// fsg_particle_interpolate_noalloc: the interpolation with no device memory
// allocation at all.
//
// Some callers cannot call cudaMalloc: a host application whose own memory
// manager owns the GPU's memory (a caching allocator that has reserved most of
// HBM, or a simulation code running this as an in-situ plugin that may not
// allocate behind its back), and loops that cannot afford the device-wide
// synchronisation a cudaMalloc/cudaFree may imply.  This entry point serves
// them: the caller passes inputs and outputs, and every piece of scratch
// (sightline tables, per-sightline counters and offsets, pair lists, queue and
// error words) lives in one file-scope device array of NOALLOC_SCRATCH_BYTES
// (64 MiB), which every GPU that loads the library holds until the process
// exits.  Host-side staging uses fixed static arrays as well.
//
// Limits: at most NOALLOC_MAX_LINES sightlines, as many pairs as fit in the
// rest of the array (about 5.4 million), and nbins small enough for the
// per-sightline accumulators to sit in shared memory (the per-form figures
// are in include/fsg.h); larger calls are rejected with FSG_ERR_VALUE and a
// message naming the limit.
//
// The array's address is looked up with cudaGetSymbolAddress on the first call
// on each device, with that device current; that first call should therefore
// come before any stream capture.  The address is kept for the life of the
// process, so a cudaDeviceReset between calls is not supported.  The particle
// arrays and the output must be device memory of the current device (checked
// with cudaPointerGetAttributes before anything is queued).  All calls share
// the array and it keeps the previous call's contents (everything that must
// start at zero is cleared by each call).  Calls are serialised by a
// process-wide lock and return only after their GPU work has finished, on
// error paths as well; GPU work that overlapped a call using the same array
// (for example from another thread bypassing this entry point's lock) would
// race on it.
#include "fsg.h"
#include "fsg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

using namespace fsg;

namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = 64ull << 20;
constexpr int NOALLOC_MAX_LINES = 8192;
constexpr int NOALLOC_MAX_NC = 91;   // ceil(sqrt(NOALLOC_MAX_LINES))
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[NOALLOC_MAX_DEVICES] = {nullptr};

// host staging (static: no heap use)
double h_key[NOALLOC_MAX_LINES], h_second[NOALLOC_MAX_LINES];
float4 h_pack[NOALLOC_MAX_LINES];
int h_group[3][NOALLOC_MAX_LINES];
int h_cell_of[NOALLOC_MAX_LINES];
int h_cell_start[3][NOALLOC_MAX_NC * NOALLOC_MAX_NC + 1];
int h_cell_cur[NOALLOC_MAX_NC * NOALLOC_MAX_NC];
int h_cell_line[3][NOALLOC_MAX_LINES];
unsigned long long h_count[NOALLOC_MAX_LINES];
long long h_off[NOALLOC_MAX_LINES + 1];
int h_order[NOALLOC_MAX_LINES];

int set_error(char *errbuf, size_t errlen, int code, const char *fmt, ...)
{
    if (errbuf && errlen) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(errbuf, errlen, fmt, ap);
        va_end(ap);
    }
    return code;
}

#define NA_CUDA(call, what)                                                                    \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return set_error(errbuf, errlen, FSG_ERR_CUDA, "%s: %s", what,                     \
                             cudaGetErrorString(e_));                                          \
    } while (0)

// Bump allocator over the scratch array (256-byte aligned regions).
struct Carver {
    unsigned char *base;
    size_t used;
    void *take(size_t bytes)
    {
        used = (used + 255) & ~size_t(255);
        void *p = base + used;
        used += bytes;
        return used <= NOALLOC_SCRATCH_BYTES ? p : nullptr;
    }
};

// absorption.cpp:152-161 (constants absorption.cpp:21-33, absorption.h:4)
LineParams noalloc_line_params(int compute_tau, int nbins, int kernel, double box, double velfac,
                               double lambda, double gamma, double fosc, double amumass,
                               double tautail)
{
    const double PI_D = 3.14159265358979323846;
    LineParams lp;
    lp.compute_tau = compute_tau ? 1 : 0;
    lp.nbins = nbins;
    lp.kernel = kernel;
    lp.tautail = tautail;
    lp.sigma_a = std::sqrt(3.0 * PI_D * 6.652458558e-25 / 8.0) * lambda * fosc;
    lp.bfac = std::sqrt(2.0 * 1.3806504e-16 / (amumass * 1.67262178e-24)) / 1e5;
    lp.voigt_fac = gamma * lambda / (4. * PI_D) / 1e5;
    lp.velfac = velfac;
    lp.vbox = box * velfac;
    lp.box = box;
    return lp;
}

}  // namespace

namespace {

// The body of fsg_particle_interpolate_noalloc after its argument checks, run
// under the lock.  `enqueued` is set once GPU work has been queued on the
// stream, so that the caller can wait for it on every error return.
int noalloc_run(int compute_tau, int nbins, int kernel, double box, double velfac,
                double lambda, double gamma, double fosc, double amumass, double tautail,
                const float *pos, const float *vel, const float *dens, const float *temp,
                const float *h, int64_t npart, const int32_t *axis, const double *cofm,
                int32_t nlos, double *out, int precision, int threads, cudaStream_t stream_in,
                bool &enqueued, char *errbuf, size_t errlen)
{
    int dev = 0;
    NA_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return set_error(errbuf, errlen, FSG_ERR_VALUE, "device ordinal %d out of range", dev);
    // the arrays must be device memory of the current device: the scratch
    // address, the stream and every launch below belong to that device
    {
        const void *ptrs[] = {pos, h, dens, compute_tau ? vel : nullptr,
                              compute_tau ? temp : nullptr, out};
        const char *names[] = {"pos", "h", "dens", "vel", "temp", "out"};
        for (int k = 0; k < 6; k++) {
            if (!ptrs[k] || (k < 5 && npart == 0))
                continue;
            cudaPointerAttributes at{};
            NA_CUDA(cudaPointerGetAttributes(&at, ptrs[k]), "cudaPointerGetAttributes");
            if (at.type == cudaMemoryTypeManaged)
                continue;
            if (at.type != cudaMemoryTypeDevice)
                return set_error(errbuf, errlen, FSG_ERR_VALUE,
                                 "%s is not device memory (this entry point takes device "
                                 "pointers)", names[k]);
            if (at.device != dev)
                return set_error(errbuf, errlen, FSG_ERR_VALUE,
                                 "%s is on device %d but device %d is current", names[k],
                                 at.device, dev);
        }
    }
    if (!g_noalloc_addr[dev]) {
        // once per device, with that device current
        void *p = nullptr;
        NA_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress");
        g_noalloc_addr[dev] = p;
    }
    cudaStream_t s = stream_in;

    // ---- sightline tables on the host (static staging)
    LineTables t{};
    t.nlos = nlos;
    t.box = box;
    int ng[3] = {0, 0, 0};
    for (int i = 0; i < nlos; i++) {
        const int a = axis[i];
        h_key[i] = (a == 1) ? cofm[3 * (size_t)i + 1] : cofm[3 * (size_t)i];
        h_second[i] = (a == 3) ? cofm[3 * (size_t)i + 1] : cofm[3 * (size_t)i + 2];
        h_pack[i] = pack_line(h_key[i], h_second[i], a, box);
        h_group[a - 1][ng[a - 1]++] = i;
    }
    t.n_xx = ng[0];
    t.n_main = nlos - ng[0];
    Carver cv{(unsigned char *)g_noalloc_addr[dev], 0};
    double *d_key = (double *)cv.take(sizeof(double) * nlos);
    double *d_second = (double *)cv.take(sizeof(double) * nlos);
    int *d_axis = (int *)cv.take(sizeof(int) * nlos);
    float4 *d_pack = (float4 *)cv.take(sizeof(float4) * nlos);
    for (int g = 0; g < 3; g++) {
        LineGroup &G = t.g[g];
        const int n = ng[g];
        G.nlines = n;
        if (n == 0)
            continue;
        int nc = (int)std::ceil(std::sqrt((double)n));
        nc = std::max(1, std::min(nc, NOALLOC_MAX_NC));
        G.nc = nc;
        G.cw = box / nc;
        G.inv_cw = nc / box;
        const int ncell = nc * nc;
        for (int c = 0; c <= ncell; c++)
            h_cell_start[g][c] = 0;
        for (int k = 0; k < n; k++) {
            const int l = h_group[g][k];
            auto cell_of = [&](double v) {
                double m = v - box * std::floor(v / box);
                long long ci = (long long)std::floor(m * G.inv_cw);
                return (int)std::min<long long>(std::max<long long>(ci, 0), nc - 1);
            };
            h_cell_of[k] = cell_of(h_key[l]) * nc + cell_of(h_second[l]);
            h_cell_start[g][h_cell_of[k] + 1]++;
        }
        for (int c = 0; c < ncell; c++)
            h_cell_start[g][c + 1] += h_cell_start[g][c];
        for (int c = 0; c < ncell; c++)
            h_cell_cur[c] = h_cell_start[g][c];
        for (int k = 0; k < n; k++)
            h_cell_line[g][h_cell_cur[h_cell_of[k]]++] = h_group[g][k];
        int *cs = (int *)cv.take(sizeof(int) * (ncell + 1));
        int *cl = (int *)cv.take(sizeof(int) * n);
        if (!cl)
            return set_error(errbuf, errlen, FSG_ERR_VALUE, "no-allocation scratch exhausted");
        enqueued = true;
        NA_CUDA(cudaMemcpyAsync(cs, h_cell_start[g], sizeof(int) * (ncell + 1),
                                cudaMemcpyHostToDevice, s), "upload cells");
        NA_CUDA(cudaMemcpyAsync(cl, h_cell_line[g], sizeof(int) * n, cudaMemcpyHostToDevice, s),
                "upload cells");
        G.cell_start = cs;
        G.cell_line = cl;
    }
    unsigned long long *d_count = (unsigned long long *)cv.take(8ull * nlos);
    long long *d_off = (long long *)cv.take(8ull * (nlos + 1));
    unsigned long long *d_cursor = (unsigned long long *)cv.take(8ull * nlos);
    int *d_order = (int *)cv.take(4ull * nlos);
    int *d_bad = (int *)cv.take(4ull * nlos);
    unsigned *d_ticket = (unsigned *)cv.take(4);
    int *d_nbad = (int *)cv.take(4);
    unsigned *d_err = (unsigned *)cv.take(4);
    if (!d_err)
        return set_error(errbuf, errlen, FSG_ERR_VALUE, "no-allocation scratch exhausted");
    cv.used = (cv.used + 255) & ~size_t(255);
    const long long pair_cap = (long long)((NOALLOC_SCRATCH_BYTES - cv.used - 512) / 12);
    int *d_part = (int *)cv.take(4ull * pair_cap);
    double *d_dr2 = (double *)cv.take(8ull * pair_cap);
    if (!d_dr2)
        return set_error(errbuf, errlen, FSG_ERR_VALUE, "no-allocation scratch exhausted");
    enqueued = true;
    NA_CUDA(cudaMemcpyAsync(d_key, h_key, sizeof(double) * nlos, cudaMemcpyHostToDevice, s),
            "upload sightlines");
    NA_CUDA(cudaMemcpyAsync(d_second, h_second, sizeof(double) * nlos, cudaMemcpyHostToDevice,
                            s), "upload sightlines");
    NA_CUDA(cudaMemcpyAsync(d_axis, axis, sizeof(int) * nlos, cudaMemcpyHostToDevice, s),
            "upload sightlines");
    NA_CUDA(cudaMemcpyAsync(d_pack, h_pack, sizeof(float4) * nlos, cudaMemcpyHostToDevice, s),
            "upload sightlines");
    t.key = d_key;
    t.second = d_second;
    t.axis = d_axis;
    t.pack = d_pack;
    set_float_box(t, box);

    // ---- pair search: count, prefix sum, emit
    Particles p{pos, compute_tau ? vel : nullptr, dens, compute_tau ? temp : nullptr, h,
                (long long)npart};
    NA_CUDA(cudaMemsetAsync(d_count, 0, 8ull * nlos, s), "memset");
    launch_count_pairs(t, p, nullptr, d_count, nullptr, s);
    NA_CUDA(cudaGetLastError(), "count_pairs launch");
    NA_CUDA(cudaMemcpyAsync(h_count, d_count, 8ull * nlos, cudaMemcpyDeviceToHost, s),
            "read counts");
    NA_CUDA(cudaStreamSynchronize(s), "count_pairs");
    h_off[0] = 0;
    for (int i = 0; i < nlos; i++)
        h_off[i + 1] = h_off[i] + (long long)h_count[i];
    const long long total = h_off[nlos];
    if (total > pair_cap)
        return set_error(errbuf, errlen, FSG_ERR_VALUE,
                         "%lld sightline-particle pairs exceed the no-allocation limit of %lld",
                         total, pair_cap);
    NA_CUDA(cudaMemcpyAsync(d_off, h_off, 8ull * (nlos + 1), cudaMemcpyHostToDevice, s),
            "upload offsets");
    NA_CUDA(cudaMemsetAsync(d_cursor, 0, 8ull * nlos, s), "memset");
    NA_CUDA(cudaMemsetAsync(d_err, 0, 4, s), "memset");
    if (total > 0) {
        launch_emit_pairs(t, p, nullptr, d_off, d_cursor, d_part, d_dr2, d_err, s);
        launch_check_emit(d_count, d_cursor, nlos, d_err, s);
        NA_CUDA(cudaGetLastError(), "emit_pairs launch");
    }
    for (int i = 0; i < nlos; i++)
        h_order[i] = i;
    std::sort(h_order, h_order + nlos, [](int a, int b) {
        return h_count[a] != h_count[b] ? h_count[a] > h_count[b] : a < b;
    });
    NA_CUDA(cudaMemcpyAsync(d_order, h_order, 4ull * nlos, cudaMemcpyHostToDevice, s),
            "upload order");

    // ---- deposit
    NA_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * (size_t)nlos * nbins, s), "memset out");
    unsigned h_err = 0;
    if (total > 0) {
        LineParams lp = noalloc_line_params(compute_tau, nbins, kernel, box, velfac, lambda,
                                            gamma, fosc, amumass, tautail);
        DepositLaunch cfg{};
        cfg.precision = precision;
        cfg.threads = threads;
        cfg.tiles = 1;
        deposit_plan(cfg, compute_tau, nbins);   // smem_mode = 1 within max_bins
        cfg.persistent = precision == FSG_PREC_FP32 ? 1 : 0;
        int sms = 0;
        NA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attribute");
        const int per_sm = std::max(1, deposit_resident_ctas(cfg, compute_tau, nbins));
        cfg.grid = std::min(nlos, sms * per_sm);
        PairLists pl{d_off, d_part, d_dr2};
        NA_CUDA(cudaMemsetAsync(d_ticket, 0, 4, s), "memset");
        NA_CUDA(cudaMemsetAsync(d_nbad, 0, 4, s), "memset");
        launch_deposit(lp, t, p, pl, d_order, nlos, out, d_ticket, d_bad, d_nbad, d_err, nullptr,
                       nullptr, cfg, s);
        NA_CUDA(cudaGetLastError(), "deposit launch");
        int h_nbad = 0;
        NA_CUDA(cudaMemcpyAsync(&h_nbad, d_nbad, 4, cudaMemcpyDeviceToHost, s), "read");
        NA_CUDA(cudaStreamSynchronize(s), "deposit");
        if (h_nbad > 0) {
            launch_deposit_fallback(lp, t, p, pl, d_bad, h_nbad, out, d_err, s);
            NA_CUDA(cudaGetLastError(), "fallback launch");
        }
    }
    NA_CUDA(cudaMemcpyAsync(&h_err, d_err, 4, cudaMemcpyDeviceToHost, s), "read");
    NA_CUDA(cudaStreamSynchronize(s), "deposit");
    if (h_err)
        return set_error(errbuf, errlen, FSG_ERR_DEVICE,
                         "kernels reported device error bits 0x%x (%s)", h_err,
                         deverr_text(h_err).c_str());
    return FSG_OK;
}

}  // namespace

extern "C" int fsg_particle_interpolate_noalloc(
    int compute_tau, int nbins, int kernel, double box, double velfac, double atime,
    double lambda, double gamma, double fosc, double amumass, double tautail, const float *pos,
    const float *vel, const float *dens, const float *temp, const float *h, int64_t npart,
    const int32_t *axis, const double *cofm, int32_t nlos, double *out, int precision,
    void *stream, char *errbuf, size_t errlen)
{
    (void)atime;
    // ---- argument checks (same rules as the allocating entry points, plus the limits)
    if (nbins < 0 || npart < 0 || nlos < 0)
        return set_error(errbuf, errlen, FSG_ERR_VALUE, "negative size");
    if (kernel == VORONOI)
        return set_error(errbuf, errlen, FSG_ERR_NOT_IMPLEMENTED,
                         "the Voronoi-mesh kernel (kernel == 2) is not implemented");
    if (!(box > 0.0) || !std::isfinite(box))
        return set_error(errbuf, errlen, FSG_ERR_VALUE, "box size must be positive and finite");
    if (precision != FSG_PREC_FP64 && precision != FSG_PREC_FP32)
        return set_error(errbuf, errlen, FSG_ERR_VALUE, "unknown precision %d", precision);
    if (npart > 2147483647LL)
        return set_error(errbuf, errlen, FSG_ERR_VALUE, "at most 2^31-1 particles");
    if (nlos > NOALLOC_MAX_LINES)
        return set_error(errbuf, errlen, FSG_ERR_VALUE,
                         "%d sightlines exceed the no-allocation limit of %d", nlos,
                         NOALLOC_MAX_LINES);
    for (int i = 0; i < nlos; i++) {
        if (axis[i] < 1 || axis[i] > 3)
            return set_error(errbuf, errlen, FSG_ERR_VALUE,
                             "axis[%d] = %d: sightline axes must be 1, 2 or 3", i, axis[i]);
        for (int k = 0; k < 3; k++)
            if (!std::isfinite(cofm[3 * (size_t)i + k]))
                return set_error(errbuf, errlen, FSG_ERR_VALUE, "cofm[%d] is not finite", i);
    }
    if (nlos == 0 || nbins == 0)
        return FSG_OK;
    const int threads = precision == FSG_PREC_FP64 ? 256 : 512;
    const int max_bins = deposit_max_smem_bins(compute_tau, precision, threads);
    if (nbins > max_bins)
        return set_error(errbuf, errlen, FSG_ERR_VALUE,
                         "nbins = %d exceeds the no-allocation limit of %d pixels (accumulators "
                         "must fit in shared memory)", nbins, max_bins);

    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    bool enqueued = false;
    const int rc = noalloc_run(compute_tau, nbins, kernel, box, velfac, lambda, gamma, fosc,
                               amumass, tautail, pos, vel, dens, temp, h, npart, axis, cofm, nlos,
                               out, precision, threads, (cudaStream_t)stream, enqueued, errbuf,
                               errlen);
    // every return leaves no work of this call in flight on the shared array
    if (rc != FSG_OK && enqueued)
        (void)cudaStreamSynchronize((cudaStream_t)stream);
    return rc;
}
