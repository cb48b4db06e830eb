// Host side of libfsg: the C ABI declared in include/fsg.h.
//
// Call pipeline (all on the context's stream):
//   1. sightline tables: keys, second coordinates and one transverse cell grid
//      per axis group, built on the host from axis/cofm (tiny) and uploaded;
//   2. pair search: count kernel -> per-sightline totals -> host prefix sum
//      (one small device->host copy, which also sizes the pair buffers) ->
//      emit kernel writing CSR pair lists;
//   3. deposit: sightlines ordered by descending pair count; one kernel;
//      sightlines with non-finite contributions re-run by the fallback kernel.
#include "fsg.h"

#include "fsg_internal.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>

using namespace fsg;

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

// Pinned host memory owned by a context (grow-only).
struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
};

// Thrown internally and turned into a status at the API boundary.
struct FsgError {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw FsgError{code, buf};
}

void cuda_check(cudaError_t e, const char *what)
{
    if (e != cudaSuccess) {
        if (e == cudaErrorMemoryAllocation)
            fail(FSG_ERR_MEMORY, "%s: %s", what, cudaGetErrorString(e));
        fail(FSG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    }
}

int report(const FsgError &e, char *errbuf, size_t errlen)
{
    if (errbuf && errlen) {
        strncpy(errbuf, e.msg.c_str(), errlen - 1);
        errbuf[errlen - 1] = '\0';
    }
    return e.code;
}

}  // namespace

struct fsg_context {
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t stream = nullptr;
    // workspace
    DevBuf pos, vel, dens, temp, hh, out;                    // staging for host-pointer calls
    DevBuf key, second, axis, pack, cell_start[3], cell_line[3];   // sightline tables
    DevBuf line_count, cursor, off, part, dr2, line_order;   // pair lists
    DevBuf ticket, bad, nbad, err, gacc, counters;           // deposit bookkeeping
    DevBuf skey, sperm, shist, sstart, ssums;                // particle ordering
    DevBuf flag, tcount, tstart, tsums, idx;                 // _near_lines
    DevBuf fpart, fout, fedges, fcounts, ftau, fdflux, ffft, fpower;   // flux statistics
    DevBuf ptables, pchirp, pbhat, ppart;                    // flux power plan and partials
    DevBuf fexp;                                             // 2^(j/256) of the flux exponential
    bool fexp_ready = false;
    PowerPlan pplan;                                         // plan of the last flux power call
    DevBuf vseg, vscratch, vcofm;                            // Voronoi cells
    DevBuf tune_order;                                       // autotuner sample
    DevBuf prec;                                             // pair records (FP32 tau)
    HostBuf hstage;   // host-pointer entries: pinned staging of inputs and output
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t cp[2] = {nullptr, nullptr};   // copy timing of the host-pointer entries
    // host-pointer entries: the inputs the search does not read are uploaded on
    // `side` while the search runs; up[0] orders them after the search's
    // inputs, up[1] orders the deposit after them
    cudaStream_t side = nullptr;
    cudaEvent_t up[2] = {nullptr, nullptr};
    // host-pointer entry: row groups of the deposit (their order, the event
    // after each group's launch, the event after each group's output copy)
    static constexpr int ROW_GROUPS = 4;
    DevBuf gorder;
    cudaEvent_t gdone[ROW_GROUPS] = {}, gcopied[ROW_GROUPS] = {};
    std::vector<int> h_bad;   // sightlines the FP64 fallback redid in the last deposit
    // host mirrors
    std::vector<long long> h_off;
    std::vector<int> h_order;
    // batched form: instantiated graph of the deposits and the call it was built for
    cudaGraphExec_t graph = nullptr;
    std::vector<double> graph_key;
    int nlos = 0;
    long long npairs = 0;
    LineTables tables{};
    // The last sightline search: a generation count and its inputs.  A
    // backward call may reuse its pair lists only when all of them match
    // (build_tables clears the record; search_pairs writes it when it is done).
    unsigned long long search_gen = 0;
    struct SearchRecord {
        const void *pos = nullptr, *hh = nullptr;
        long long npart = -1;
        int nlos = -1;
        double box = 0.0;
        unsigned long long lines = 0;   // hash of the axis and cofm arrays
    } search_rec;
    unsigned long long lines_hash = 0;   // of the tables build_tables last built
    fsg_stats stats{};

    void *ensure(DevBuf &b, size_t bytes)
    {
        if (bytes == 0)
            bytes = 16;
        if (b.cap < bytes) {
            if (b.p)
                cuda_check(cudaFree(b.p), "cudaFree");
            b.p = nullptr;
            b.cap = 0;
            size_t want = bytes + bytes / 8;
            cuda_check(cudaMalloc(&b.p, want), "cudaMalloc");
            b.cap = want;
        }
        return b.p;
    }

    void *ensure_host(HostBuf &b, size_t bytes)
    {
        if (bytes == 0)
            bytes = 16;
        if (b.cap < bytes) {
            if (b.p)
                cuda_check(cudaFreeHost(b.p), "cudaFreeHost");
            b.p = nullptr;
            b.cap = 0;
            const size_t want = bytes + bytes / 8;
            cuda_check(cudaHostAlloc(&b.p, want, cudaHostAllocDefault), "cudaHostAlloc");
            b.cap = want;
        }
        return b.p;
    }

    void release_all()
    {
        if (hstage.p)
            cudaFreeHost(hstage.p);
        hstage.p = nullptr;
        hstage.cap = 0;
        DevBuf *bufs[] = {&pos, &vel, &dens, &temp, &hh, &out, &key, &second, &axis, &pack,
                          &cell_start[0], &cell_start[1], &cell_start[2], &cell_line[0],
                          &cell_line[1], &cell_line[2], &line_count, &cursor, &off, &part, &dr2,
                          &line_order, &ticket, &bad, &nbad, &err, &gacc, &counters,
                          &skey, &sperm, &shist, &sstart, &ssums, &flag, &tcount, &tstart,
                          &tsums, &idx, &fpart, &fout, &fedges, &fcounts, &ftau, &fdflux,
                          &ffft, &fpower, &ptables, &pchirp, &pbhat, &ppart, &fexp, &vseg,
                          &vscratch, &vcofm, &tune_order, &prec, &gorder};
        pplan = PowerPlan{};
        fexp_ready = false;
        for (DevBuf *b : bufs) {
            if (b->p)
                cudaFree(b->p);
            b->p = nullptr;
            b->cap = 0;
        }
    }
};

namespace {

void validate_common(int nbins, int kernel, double box, int64_t npart, int32_t nlos,
                     const int32_t *axis, const double *cofm, bool allow_voronoi = false)
{
    if (nbins < 0)
        fail(FSG_ERR_VALUE, "nbins must be non-negative (got %d)", nbins);
    if (npart < 0 || nlos < 0)
        fail(FSG_ERR_VALUE, "negative array length");
    if (npart > 2147483647LL)
        fail(FSG_ERR_VALUE, "at most 2^31-1 particles (particle indices are int, as in the "
                            "reference's std::map<int, double>)");
    if (kernel == VORONOI && !allow_voronoi)
        fail(FSG_ERR_NOT_IMPLEMENTED, "the Voronoi-mesh kernel (kernel == 2) is supported by "
                                      "the single-line interpolation entry points only");
    if (!(box > 0.0) || !std::isfinite(box))
        fail(FSG_ERR_VALUE, "box size must be positive and finite (got %g)", box);
    for (int i = 0; i < nlos; i++) {
        if (axis[i] < 1 || axis[i] > 3)
            fail(FSG_ERR_VALUE, "axis[%d] = %d: sightline axes must be 1, 2 or 3", i, axis[i]);
        for (int k = 0; k < 3; k++)
            if (!std::isfinite(cofm[3 * (size_t)i + k]))
                fail(FSG_ERR_VALUE, "cofm[%d] is not finite", i);
    }
}

// 1. sightline tables
// FNV-1a over the sightline arrays (identifies the tables a search used).
unsigned long long lines_hash_of(const int32_t *axis, const double *cofm, int nlos)
{
    unsigned long long h = 1469598103934665603ull;
    const auto mix = [&](const void *p, size_t n) {
        const unsigned char *b = (const unsigned char *)p;
        for (size_t i = 0; i < n; i++) {
            h ^= b[i];
            h *= 1099511628211ull;
        }
    };
    mix(axis, sizeof(int32_t) * (size_t)nlos);
    mix(cofm, sizeof(double) * 3 * (size_t)nlos);
    return h;
}

void build_tables(fsg_context *c, const int32_t *axis, const double *cofm, int nlos, double box)
{
    c->search_rec = fsg_context::SearchRecord{};
    c->lines_hash = lines_hash_of(axis, cofm, nlos);
    std::vector<double> key(nlos), second(nlos);
    std::vector<int> grp_lines[3];
    for (int i = 0; i < nlos; i++) {
        const int a = axis[i];
        key[i] = (a == 1) ? cofm[3 * (size_t)i + 1] : cofm[3 * (size_t)i];
        second[i] = (a == 3) ? cofm[3 * (size_t)i + 1] : cofm[3 * (size_t)i + 2];
        grp_lines[a - 1].push_back(i);
    }
    LineTables &t = c->tables;
    t = LineTables{};
    t.nlos = nlos;
    t.box = box;
    t.n_xx = (int)grp_lines[0].size();
    t.n_main = nlos - t.n_xx;
    cudaStream_t s = c->stream;
    for (int g = 0; g < 3; g++) {
        LineGroup &G = t.g[g];
        const int n = (int)grp_lines[g].size();
        G.nlines = n;
        if (n == 0)
            continue;
        int nc = (int)std::ceil(std::sqrt((double)n));
        nc = std::max(1, std::min(nc, 1024));
        G.nc = nc;
        G.cw = box / nc;
        G.inv_cw = nc / box;
        auto cell_of = [&](double v) {
            double m = v - box * std::floor(v / box);
            long long ci = (long long)std::floor(m * G.inv_cw);
            return (int)std::min<long long>(std::max<long long>(ci, 0), nc - 1);
        };
        std::vector<int> cnt((size_t)nc * nc + 1, 0), cell(n);
        for (int k = 0; k < n; k++) {
            const int l = grp_lines[g][k];
            cell[k] = cell_of(key[l]) * nc + cell_of(second[l]);
            cnt[cell[k] + 1]++;
        }
        for (size_t k = 0; k < (size_t)nc * nc; k++)
            cnt[k + 1] += cnt[k];
        std::vector<int> lines(n), cur(cnt.begin(), cnt.end() - 1);
        for (int k = 0; k < n; k++)
            lines[cur[cell[k]]++] = grp_lines[g][k];
        void *cs = c->ensure(c->cell_start[g], sizeof(int) * cnt.size());
        void *cl = c->ensure(c->cell_line[g], sizeof(int) * n);
        cuda_check(cudaMemcpyAsync(cs, cnt.data(), sizeof(int) * cnt.size(),
                                   cudaMemcpyHostToDevice, s), "upload cells");
        cuda_check(cudaMemcpyAsync(cl, lines.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s),
                   "upload cells");
        // the host vectors die at scope end: finish the copies first
        cuda_check(cudaStreamSynchronize(s), "upload cells");
        G.cell_start = (const int *)cs;
        G.cell_line = (const int *)cl;
    }
    std::vector<float4> pk(nlos);
    for (int i = 0; i < nlos; i++)
        pk[i] = pack_line(key[i], second[i], axis[i], box);
    void *dk = c->ensure(c->key, sizeof(double) * nlos);
    void *ds = c->ensure(c->second, sizeof(double) * nlos);
    void *da = c->ensure(c->axis, sizeof(int) * nlos);
    void *dp = c->ensure(c->pack, sizeof(float4) * nlos);
    cuda_check(cudaMemcpyAsync(dp, pk.data(), sizeof(float4) * nlos, cudaMemcpyHostToDevice, s),
               "upload sightlines");
    cuda_check(cudaMemcpyAsync(dk, key.data(), sizeof(double) * nlos, cudaMemcpyHostToDevice, s),
               "upload sightlines");
    cuda_check(cudaMemcpyAsync(ds, second.data(), sizeof(double) * nlos, cudaMemcpyHostToDevice,
                               s), "upload sightlines");
    cuda_check(cudaMemcpyAsync(da, axis, sizeof(int) * nlos, cudaMemcpyHostToDevice, s),
               "upload sightlines");
    cuda_check(cudaStreamSynchronize(s), "upload sightlines");
    t.key = (const double *)dk;
    t.second = (const double *)ds;
    t.axis = (const int *)da;
    t.pack = (const float4 *)dp;
    set_float_box(t, box);
    c->nlos = nlos;
}

// 2. pair search
// spatial order of the particles (counting sort by 3-D cell); null when n = 0
int *order_particles(fsg_context *c, const Particles &p)
{
    if (p.n <= 0)
        return nullptr;
    const int G = sort_grid_side(p.n);
    const size_t M = (size_t)G * G * G;
    auto *key = (unsigned *)c->ensure(c->skey, sizeof(unsigned) * p.n);
    int *perm = (int *)c->ensure(c->sperm, sizeof(int) * p.n);
    auto *hist = (unsigned *)c->ensure(c->shist, sizeof(unsigned) * M);
    auto *start = (unsigned *)c->ensure(c->sstart, sizeof(unsigned) * M);
    auto *sums = (unsigned *)c->ensure(c->ssums, sizeof(unsigned) * (M / 2048 + 2));
    launch_particle_order(p, c->tables.box, G, key, hist, start, sums, perm, c->stream);
    c->stats.gpu_launches += 5;
    cuda_check(cudaGetLastError(), "particle order launch");
    return perm;
}

void search_pairs(fsg_context *c, const Particles &p, int nlos)
{
    cudaStream_t s = c->stream;
    cuda_check(cudaEventRecord(c->ev[0], s), "event");
    int *perm = order_particles(c, p);
    auto *cnt = (unsigned long long *)c->ensure(c->line_count, sizeof(unsigned long long) * nlos);
    cuda_check(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * nlos, s), "memset");
    launch_count_pairs(c->tables, p, perm, cnt, nullptr, s);
    if (p.n > 0)
        c->stats.gpu_launches++;
    cuda_check(cudaGetLastError(), "count_pairs launch");
    std::vector<unsigned long long> h_cnt(nlos);
    cuda_check(cudaMemcpyAsync(h_cnt.data(), cnt, sizeof(unsigned long long) * nlos,
                               cudaMemcpyDeviceToHost, s), "read counts");
    cuda_check(cudaStreamSynchronize(s), "count_pairs");
    c->h_off.assign((size_t)nlos + 1, 0);
    for (int i = 0; i < nlos; i++)
        c->h_off[i + 1] = c->h_off[i] + (long long)h_cnt[i];
    const long long total = c->h_off[nlos];
    c->npairs = total;
    auto *off = (long long *)c->ensure(c->off, sizeof(long long) * (nlos + 1));
    cuda_check(cudaMemcpyAsync(off, c->h_off.data(), sizeof(long long) * (nlos + 1),
                               cudaMemcpyHostToDevice, s), "upload offsets");
    auto *cur = (unsigned long long *)c->ensure(c->cursor, sizeof(unsigned long long) * nlos);
    cuda_check(cudaMemsetAsync(cur, 0, sizeof(unsigned long long) * nlos, s), "memset");
    int *part = (int *)c->ensure(c->part, sizeof(int) * total);
    double *dr2 = (double *)c->ensure(c->dr2, sizeof(double) * total);
    auto *err = (unsigned *)c->ensure(c->err, sizeof(unsigned));
    cuda_check(cudaMemsetAsync(err, 0, sizeof(unsigned), s), "memset");
    if (total > 0) {
        launch_emit_pairs(c->tables, p, perm, off, cur, part, dr2, err, s);
        launch_check_emit(cnt, cur, nlos, err, s);
        c->stats.gpu_launches += 3;   // emit, pair dr2, check
        cuda_check(cudaGetLastError(), "emit_pairs launch");
    }
    // sightline work order: descending pair count (largest first)
    c->h_order.resize(nlos);
    std::iota(c->h_order.begin(), c->h_order.end(), 0);
    std::stable_sort(c->h_order.begin(), c->h_order.end(),
                     [&](int a, int b) { return h_cnt[a] > h_cnt[b]; });
    void *ord = c->ensure(c->line_order, sizeof(int) * nlos);
    cuda_check(cudaMemcpyAsync(ord, c->h_order.data(), sizeof(int) * nlos,
                               cudaMemcpyHostToDevice, s), "upload order");
    cuda_check(cudaEventRecord(c->ev[1], s), "event");
    unsigned h_err = 0;
    cuda_check(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaStreamSynchronize(s), "emit_pairs");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
    c->stats.ms_search = ms;
    c->stats.npairs = total;
    if (h_err)
        fail(FSG_ERR_DEVICE, "pair search reported device error bits 0x%x (%s)", h_err,
             deverr_text(h_err).c_str());
    c->search_gen++;
    c->search_rec = fsg_context::SearchRecord{p.pos, p.hh, p.n, nlos, c->tables.box,
                                              c->lines_hash};
}

// _near_lines (py_module.cpp:25-99): ascending indices of the particles within
// their smoothing length of any sightline, written to out (device, capacity
// p.n); returns their number.
long long near_lines(fsg_context *c, const Particles &p, int *out)
{
    cudaStream_t s = c->stream;
    if (p.n <= 0 || c->nlos <= 0)
        return 0;
    int *perm = order_particles(c, p);
    auto *flag = (unsigned char *)c->ensure(c->flag, (size_t)p.n);
    launch_flag_near(c->tables, p, perm, flag, s);
    const long long nt = flag_tiles(p.n);
    if (nt > 2048LL * 2048LL)
        fail(FSG_ERR_VALUE, "too many particles for the near-lines compaction");
    auto *tcount = (unsigned *)c->ensure(c->tcount, sizeof(unsigned) * nt);
    auto *tstart = (unsigned *)c->ensure(c->tstart, sizeof(unsigned) * nt);
    auto *tsums = (unsigned *)c->ensure(c->tsums, sizeof(unsigned) * (nt / 2048 + 2));
    launch_flag_count(flag, p.n, tcount, s);
    launch_exclusive_scan(tcount, tstart, tsums, (int)nt, s);
    launch_flag_scatter(flag, p.n, tstart, out, s);
    c->stats.gpu_launches += 6;
    cuda_check(cudaGetLastError(), "near-lines launch");
    unsigned last_start = 0, last_count = 0;
    cuda_check(cudaMemcpyAsync(&last_start, tstart + (nt - 1), sizeof(unsigned),
                               cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaMemcpyAsync(&last_count, tcount + (nt - 1), sizeof(unsigned),
                               cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaStreamSynchronize(s), "near lines");
    return (long long)last_start + last_count;
}

// The table of the flux passes' exponential on the device (uploaded once).
const double *exp_table(fsg_context *c)
{
    auto *t = (double *)c->ensure(c->fexp, sizeof(double) * 256);
    if (!c->fexp_ready) {
        double h[256];
        exp_table_host(h);
        cuda_check(cudaMemcpyAsync(t, h, sizeof h, cudaMemcpyHostToDevice, c->stream), "H2D");
        cuda_check(cudaStreamSynchronize(c->stream), "exp table");
        c->fexp_ready = true;
    }
    return t;
}

// get_mean_flux_scale (py_module.cpp:235-260): Newton-Raphson on the scale of
// tau until the mean of exp(-scale tau) over the pixels with tau <= thresh is
// mean_flux_desired; the same update and stopping rule.  The scale stays on
// the device between passes: the host queues NEWTON_BATCH passes, then reads
// whether they converged (passes queued after convergence return at once).
constexpr int NEWTON_BATCH = 8;

double mean_flux_scale(fsg_context *c, const double *tau, long long n, double mfd, double tol,
                       double thresh)
{
    cudaStream_t s = c->stream;
    const double *etab = exp_table(c);
    auto *part = (double *)c->ensure(c->fpart, sizeof(double) * flux_partials(3));
    auto *state = (double *)c->ensure(c->fout, sizeof(double) * 4);
    const double init[4] = {1.0, 1.0, 0.0, 0.0};
    cuda_check(cudaMemcpyAsync(state, init, sizeof init, cudaMemcpyHostToDevice, s), "H2D");
    double h[4] = {0, 0, 0, 0};
    float total = 0.f;
    for (;;) {
        cuda_check(cudaEventRecord(c->ev[2], s), "event");
        launch_newton_passes(tau, n, mfd, tol, thresh, NEWTON_BATCH, etab, part, state, s);
        c->stats.gpu_launches += 2 * NEWTON_BATCH;
        cuda_check(cudaGetLastError(), "flux moments launch");
        cuda_check(cudaEventRecord(c->ev[3], s), "event");
        cuda_check(cudaMemcpyAsync(h, state, sizeof h, cudaMemcpyDeviceToHost, s), "read");
        cuda_check(cudaStreamSynchronize(s), "flux moments");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
        total += ms;
        c->stats.ms_flux = total;
        if (h[2] != 0.0)
            return h[1];
        if (h[3] > 10000)
            fail(FSG_ERR_VALUE, "mean-flux rescaling did not converge in 10000 iterations");
    }
}

double mean_flux_of(fsg_context *c, const double *tau, long long n, double scale)
{
    cudaStream_t s = c->stream;
    const double *etab = exp_table(c);
    auto *part = (double *)c->ensure(c->fpart, sizeof(double) * flux_partials(3));
    auto *out = (double *)c->ensure(c->fout, sizeof(double) * 4);
    cuda_check(cudaEventRecord(c->ev[2], s), "event");
    launch_flux_sum(tau, n, scale, etab, part, out, s);
    c->stats.gpu_launches += 2;
    cuda_check(cudaEventRecord(c->ev[3], s), "event");
    cuda_check(cudaGetLastError(), "flux sum launch");
    double h = 0.0;
    cuda_check(cudaMemcpyAsync(&h, out, sizeof h, cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaStreamSynchronize(s), "flux sum");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
    c->stats.ms_flux = ms;
    return h / (double)n;
}

DepositLaunch deposit_config(fsg_context *c, const LineParams &lp, const fsg_options *opt);
void apply_tuning(fsg_context *c, const LineParams &lp, const fsg_options *opt, const Particles &p,
                  PairLists pl, double *out, DepositLaunch &cfg);

// 3. deposit into out (device, nlos*nbins)
// Row groups of a deposit: the sightlines in `groups` contiguous index
// ranges, launched one range after another (each range in the descending
// pair-count order); on_group(g, row0, row1) runs after range g is queued,
// with c->gdone[g] recorded behind it.  The output is the same: the
// fixed-point sums do not depend on the launch.
struct RowGroups {
    int groups = 1;
    std::function<void(int, long long, long long)> on_group;
};

void deposit(fsg_context *c, const LineParams &lp, const Particles &p, double *out,
             const fsg_options *opt, const float2 *seg = nullptr,
             const RowGroups *rows = nullptr)
{
    cudaStream_t s = c->stream;
    const int nlos = c->nlos;
    const size_t nout = (size_t)nlos * lp.nbins;
    c->stats.fallback_lines = 0;
    c->stats.tune_ran = 0;
    if (nout == 0 || c->npairs == 0) {
        if (nout)
            cuda_check(cudaMemsetAsync(out, 0, sizeof(double) * nout, s), "memset out");
        cuda_check(cudaStreamSynchronize(s), "deposit");
        c->stats.ms_deposit = 0;
        return;
    }
    PairLists pl{(const long long *)c->off.p, (const int *)c->part.p, (const double *)c->dr2.p,
                 seg};
    DepositLaunch cfg = deposit_config(c, lp, opt);
    // the tuner times candidates on sample rows of `out`, which is cleared below
    apply_tuning(c, lp, opt, p, pl, out, cfg);
    if (cfg.rec)
        pl.rec = c->ensure(c->prec, 32 * (size_t)c->npairs);
    cuda_check(cudaEventRecord(c->ev[2], s), "event");
    cuda_check(cudaMemsetAsync(out, 0, sizeof(double) * nout, s), "memset out");
    unsigned long long *gacc = nullptr;
    if (!cfg.smem_mode) {
        gacc = (unsigned long long *)c->ensure(c->gacc, sizeof(unsigned long long) * 2 * nout);
    }
    const bool count = opt && opt->count_work;
    unsigned long long *ctr = nullptr;
    if (count) {
        ctr = (unsigned long long *)c->ensure(c->counters, sizeof(unsigned long long) * 8);
        cuda_check(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long) * 8, s), "memset");
    }
    const int G = (rows && rows->groups > 1 && !count && nlos >= 64 * rows->groups)
                      ? std::min(rows->groups, (int)fsg_context::ROW_GROUPS)
                      : 1;
    auto *ticket = (unsigned *)c->ensure(c->ticket, sizeof(unsigned) * G);
    auto *bad = (int *)c->ensure(c->bad, sizeof(int) * nlos);
    auto *nbad = (int *)c->ensure(c->nbad, sizeof(int));
    auto *err = (unsigned *)c->ensure(c->err, sizeof(unsigned));
    cuda_check(cudaMemsetAsync(ticket, 0, sizeof(unsigned) * G, s), "memset");
    cuda_check(cudaMemsetAsync(nbad, 0, sizeof(int), s), "memset");
    cuda_check(cudaMemsetAsync(err, 0, sizeof(unsigned), s), "memset");
    if (G == 1) {
        c->stats.gpu_launches += launch_deposit(lp, c->tables, p, pl,
                                                (const int *)c->line_order.p, nlos, out, ticket,
                                                bad, nbad, err, gacc, ctr, cfg, s);
        cuda_check(cudaGetLastError(), "deposit launch");
    } else {
        // group g: rows [nlos g / G, nlos (g + 1) / G), in the global order
        std::vector<int> gord((size_t)nlos);
        std::vector<long long> start((size_t)G + 1, 0);
        const auto group_of = [&](int line) { return (int)((long long)line * G / nlos); };
        for (int line : c->h_order)
            start[group_of(line) + 1]++;
        for (int g = 0; g < G; g++)
            start[g + 1] += start[g];
        std::vector<long long> fill(start.begin(), start.end() - 1);
        for (int line : c->h_order)
            gord[(size_t)fill[group_of(line)]++] = line;
        auto *dord = (int *)c->ensure(c->gorder, sizeof(int) * (size_t)nlos);
        cuda_check(cudaMemcpyAsync(dord, gord.data(), sizeof(int) * (size_t)nlos,
                                   cudaMemcpyHostToDevice, s), "upload order");
        // the host vector must outlive the copy
        cuda_check(cudaStreamSynchronize(s), "upload order");
        for (int g = 0; g < G; g++) {
            c->stats.gpu_launches += launch_deposit(
                lp, c->tables, p, pl, dord + start[g], (int)(start[g + 1] - start[g]), out,
                ticket + g, bad, nbad, err, gacc, ctr, cfg, s);
            cuda_check(cudaGetLastError(), "deposit launch");
            cuda_check(cudaEventRecord(c->gdone[g], s), "event");
            if (rows->on_group)
                rows->on_group(g, (long long)nlos * g / G, (long long)nlos * (g + 1) / G);
        }
    }
    int h_nbad = 0;
    unsigned h_err = 0;
    cuda_check(cudaMemcpyAsync(&h_nbad, nbad, sizeof(int), cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaStreamSynchronize(s), "deposit");
    c->h_bad.clear();
    if (h_nbad > 0) {
        launch_deposit_fallback(lp, c->tables, p, pl, bad, h_nbad, out, err, s);
        c->stats.gpu_launches++;
        cuda_check(cudaGetLastError(), "fallback launch");
        c->h_bad.resize((size_t)h_nbad);
        cuda_check(cudaMemcpyAsync(c->h_bad.data(), bad, sizeof(int) * (size_t)h_nbad,
                                   cudaMemcpyDeviceToHost, s), "read");
    }
    c->stats.fallback_lines = h_nbad;
    cuda_check(cudaEventRecord(c->ev[3], s), "event");
    cuda_check(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaStreamSynchronize(s), "deposit");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
    c->stats.ms_deposit = ms;
    if (count) {
        unsigned long long h_ctr[8];
        cuda_check(cudaMemcpy(h_ctr, ctr, sizeof h_ctr, cudaMemcpyDeviceToHost), "read counters");
        c->stats.evals_core = (int64_t)h_ctr[0];
        c->stats.evals_wing = (int64_t)h_ctr[1];
        c->stats.evals_other = (int64_t)h_ctr[2];
        c->stats.pixels = (int64_t)h_ctr[3];
        c->stats.evals_wing_multipole = (int64_t)h_ctr[4];
        c->stats.samples_wing_path = (int64_t)h_ctr[5];
        c->stats.samples_core_path = (int64_t)h_ctr[6];
        c->stats.samples_mixed_path = (int64_t)h_ctr[7];
    }
    if (h_err)
        fail(FSG_ERR_DEVICE, "deposit kernel reported device error bits 0x%x (%s)", h_err,
             deverr_text(h_err).c_str());
}

LineParams make_line_params(int compute_tau, int nbins, int kernel, double box, double velfac,
                            double lambda, double gamma, double fosc, double amumass,
                            double tautail)
{
    // absorption.cpp:152-161 (constants absorption.cpp:21-33, absorption.h:4)
    const double PI_D = 3.14159265358979323846;
    const double SIGMA_T = 6.652458558e-25, BOLTZMANN = 1.3806504e-16;
    const double PROTONMASS = 1.67262178e-24;
    LineParams lp;
    lp.compute_tau = compute_tau ? 1 : 0;
    lp.nbins = nbins;
    lp.kernel = kernel;
    lp.tautail = tautail;
    lp.sigma_a = std::sqrt(3.0 * PI_D * SIGMA_T / 8.0) * lambda * fosc;
    lp.bfac = std::sqrt(2.0 * BOLTZMANN / (amumass * PROTONMASS)) / 1e5;
    lp.voigt_fac = gamma * lambda / (4. * PI_D) / 1e5;
    lp.velfac = velfac;
    lp.vbox = box * velfac;
    lp.box = box;
    return lp;
}

void finish_config(fsg_context *c, const LineParams &lp, DepositLaunch &cfg);

// Launch configuration of the deposit for this call.
DepositLaunch deposit_config(fsg_context *c, const LineParams &lp, const fsg_options *opt)
{
    DepositLaunch cfg{};
    cfg.precision = opt ? opt->precision : FSG_PREC_FP64;
    if (cfg.precision != FSG_PREC_FP64 && cfg.precision != FSG_PREC_FP32)
        fail(FSG_ERR_VALUE, "unknown precision %d", cfg.precision);
    // the Voronoi mesh (kernel 2) has no FP32 form: it deposits in FP64
    const bool vor = lp.kernel == VORONOI;
    if (vor)
        cfg.precision = FSG_PREC_FP64;
    // FP32 optical depths have 768- and 1024-thread kernel builds and may go
    // through pair records (the context's buffer); the counting variant has not
    const bool count = opt && opt->count_work;
    const bool tau32 = cfg.precision == FSG_PREC_FP32 && lp.compute_tau && !vor && !count;
    cfg.rec = tau32 && opt && opt->records == 1;
    if (opt && opt->records > 1)
        fail(FSG_ERR_VALUE, "records must be -1 (tuned), 0 or 1");
    const int tdef = cfg.precision == FSG_PREC_FP64 ? 256 : 512;
    const int tmax = cfg.precision == FSG_PREC_FP64 ? 256 : (tau32 ? 1024 : 512);
    cfg.threads = (opt && opt->threads > 0 && !vor) ? opt->threads : tdef;
    if (cfg.threads % 32 || cfg.threads > tmax)
        fail(FSG_ERR_VALUE, "threads must be a multiple of 32 and at most %d", tmax);
    cfg.tiles = cfg.tiles_asked = !(opt && opt->no_far_tiles);
    cfg.chunk = (opt && cfg.precision == FSG_PREC_FP32) ? opt->chunk : 0;
    if (cfg.chunk < 0 || cfg.chunk > 32)
        fail(FSG_ERR_VALUE, "chunk must be between 1 and 32 (0 = tuned or default)");
    deposit_plan(cfg, lp.compute_tau, lp.nbins);
    cfg.persistent = (opt && opt->persistent >= 0 && !vor)
                         ? opt->persistent : (cfg.precision == FSG_PREC_FP32 ? 1 : 0);
    finish_config(c, lp, cfg);
    c->stats.launch_tuned = 0;
    return cfg;
}

// ---------------------------------------------------------------- autotuner
// The FP32 deposit's launch (threads per block, pairs staged per warp, queue
// mode) is chosen by timing candidates on a sample of the call's own
// sightlines, once per workload class (fsg_tune_key), and cached: in the
// process, and in a text file when one is named (fsg_tune_cache_file or the
// FSG_TUNE_CACHE environment variable).  Every candidate gives the same output
// bits (integer accumulation with a scale that does not depend on the launch),
// so the choice changes the speed only.
struct TuneKeyLess {
    bool operator()(const fsg_tune_key &a, const fsg_tune_key &b) const
    {
        return std::tie(a.sms, a.precision, a.compute_tau, a.kernel, a.nbins_b, a.pairs_med_b,
                        a.pairs_p99_b, a.lines_b, a.damp_b) <
               std::tie(b.sms, b.precision, b.compute_tau, b.kernel, b.nbins_b, b.pairs_med_b,
                        b.pairs_p99_b, b.lines_b, b.damp_b);
    }
};

std::mutex g_tune_mu;
std::map<fsg_tune_key, fsg_tune_entry, TuneKeyLess> g_tune;
std::string g_tune_file;
bool g_tune_env_read = false;

constexpr const char *TUNE_FILE_TAG = "fsg-tune-v2";

bool tune_entry_valid(const fsg_tune_entry &e)
{
    return e.threads > 0 && e.threads % 32 == 0 && e.threads <= 1024 && e.chunk >= 1 &&
           e.chunk <= 32 && (e.persistent == 0 || e.persistent == 1) &&
           (e.records == 0 || e.records == 1);
}

// Reads the entries of a cache file (lines that do not parse are skipped);
// the caller holds g_tune_mu.
void tune_load_locked(const std::string &path)
{
    FILE *f = fopen(path.c_str(), "r");
    if (!f)
        return;
    char line[512];
    while (fgets(line, sizeof line, f)) {
        char tag[32];
        fsg_tune_key k{};
        fsg_tune_entry e{};
        const int n = sscanf(line, "%31s %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %lf %lf",
                             tag, &k.sms, &k.precision, &k.compute_tau, &k.kernel, &k.nbins_b,
                             &k.pairs_med_b, &k.pairs_p99_b, &k.lines_b, &k.damp_b, &e.threads,
                             &e.chunk, &e.persistent, &e.records, &e.candidates, &e.sample_lines,
                             &e.ms_default, &e.ms_best);
        if (n == 18 && strcmp(tag, TUNE_FILE_TAG) == 0 && tune_entry_valid(e))
            g_tune[k] = e;
    }
    fclose(f);
}

void tune_env_locked()
{
    if (g_tune_env_read)
        return;
    g_tune_env_read = true;
    const char *env = getenv("FSG_TUNE_CACHE");
    if (env && *env && g_tune_file.empty()) {
        g_tune_file = env;
        tune_load_locked(g_tune_file);
    }
}

bool tune_store_locked(const fsg_tune_key &k, const fsg_tune_entry &e)
{
    g_tune[k] = e;
    if (g_tune_file.empty())
        return true;
    FILE *f = fopen(g_tune_file.c_str(), "a");
    if (!f)
        return false;
    fprintf(f, "%s %d %d %d %d %d %d %d %d %d %d %d %d %d %d %d %.6f %.6f\n", TUNE_FILE_TAG,
            k.sms, k.precision, k.compute_tau, k.kernel, k.nbins_b, k.pairs_med_b, k.pairs_p99_b,
            k.lines_b, k.damp_b, e.threads, e.chunk, e.persistent, e.records, e.candidates,
            e.sample_lines, e.ms_default, e.ms_best);
    fclose(f);
    return true;
}

int floor_log2x2(double v) { return (int)std::floor(2.0 * std::log2(v)); }

fsg_tune_key tune_key(fsg_context *c, const LineParams &lp, int precision)
{
    fsg_tune_key k{};
    cudaDeviceGetAttribute(&k.sms, cudaDevAttrMultiProcessorCount, c->device);
    k.precision = precision;
    k.compute_tau = lp.compute_tau;
    k.kernel = lp.kernel;
    k.nbins_b = floor_log2x2(std::max(1, lp.nbins));
    std::vector<long long> cnt((size_t)c->nlos);
    for (int i = 0; i < c->nlos; i++)
        cnt[i] = c->h_off[i + 1] - c->h_off[i];
    std::sort(cnt.begin(), cnt.end());
    const auto q = [&](double f) { return cnt[(size_t)std::min<double>(f * cnt.size(),
                                                                       cnt.size() - 1)]; };
    k.pairs_med_b = floor_log2x2(1.0 + (double)q(0.5));
    k.pairs_p99_b = floor_log2x2(1.0 + (double)q(0.99));
    k.lines_b = (int)std::floor(std::log2((double)std::max(1, c->nlos)));
    k.damp_b = lp.compute_tau ? floor_log2x2(std::max(1e-300, lp.voigt_fac / lp.bfac)) : 0;
    return k;
}

// The grid of a configuration: resident CTAs on every SM, at most one per sightline.
void finish_config(fsg_context *c, const LineParams &lp, DepositLaunch &cfg)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const int per_sm = std::max(1, deposit_resident_ctas(cfg, lp.compute_tau, lp.nbins));
    cfg.grid = std::min(c->nlos, sms * per_sm);
}

// Times the candidate launches on a sample of the call's sightlines (every
// k-th of the descending pair-count order, about four sightlines per resident
// CTA so that the queue's balance resembles the full call's) and returns the
// fastest.  The sample rows of `out` are overwritten.
fsg_tune_entry tune_deposit(fsg_context *c, const LineParams &lp, const Particles &p,
                            PairLists pl, double *out, const DepositLaunch &base)
{
    cudaStream_t s = c->stream;
    const int nlos = c->nlos;
    const int want = std::max(64, 4 * base.grid);
    const int nsamp = std::min(nlos, want);
    std::vector<int> order((size_t)nsamp);
    for (int i = 0; i < nsamp; i++)
        order[i] = c->h_order[(size_t)((double)i * nlos / nsamp)];
    int *d_order = (int *)c->ensure(c->tune_order, sizeof(int) * (size_t)nsamp);
    cuda_check(cudaMemcpyAsync(d_order, order.data(), sizeof(int) * nsamp,
                               cudaMemcpyHostToDevice, s), "upload tuning sample");
    auto *ticket = (unsigned *)c->ensure(c->ticket, sizeof(unsigned));
    auto *bad = (int *)c->ensure(c->bad, sizeof(int) * nlos);
    auto *nbad = (int *)c->ensure(c->nbad, sizeof(int));
    auto *err = (unsigned *)c->ensure(c->err, sizeof(unsigned));
    unsigned long long *gacc = nullptr;
    if (!base.smem_mode)
        gacc = (unsigned long long *)c->ensure(c->gacc, sizeof(unsigned long long) * 2 *
                                                            (size_t)nlos * lp.nbins);
    struct Cand {
        int threads, chunk, persistent, rec;
    };
    std::vector<Cand> cands;
    if (lp.compute_tau)
        cands = {{512, 8, 1, 0},  {512, 4, 1, 0},  {512, 16, 1, 0},  {512, 8, 0, 0},
                 {256, 8, 1, 0},  {768, 8, 1, 0},  {768, 16, 1, 0},  {1024, 4, 1, 0},
                 {1024, 8, 1, 0}, {1024, 16, 1, 0}, {1024, 8, 1, 1}, {768, 8, 1, 1}};
    else
        cands = {{512, 32, 1, 0}, {512, 16, 1, 0}, {512, 8, 1, 0}, {512, 32, 0, 0},
                 {256, 32, 1, 0}, {256, 16, 1, 0}};
    fsg_tune_entry best{};
    best.ms_best = 1e300;
    best.sample_lines = nsamp;
    for (const Cand &cd : cands) {
        DepositLaunch cfg = base;
        cfg.threads = cd.threads;
        cfg.chunk = cd.chunk;
        cfg.persistent = cd.persistent;
        cfg.rec = cd.rec;
        cfg.tiles = base.tiles_asked;
        deposit_plan(cfg, lp.compute_tau, lp.nbins);
        if (cfg.smem_mode != base.smem_mode || cfg.tiles != base.tiles)
            continue;   // only launches that keep the default's on-chip layout
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
        const int per_sm = std::max(1, deposit_resident_ctas(cfg, lp.compute_tau, lp.nbins));
        cfg.grid = std::min(nsamp, sms * per_sm);
        pl.rec = cfg.rec ? c->ensure(c->prec, 32 * (size_t)c->npairs) : nullptr;
        float ms_min = 1e30f;
        for (int rep = 0; rep < 2; rep++) {
            cuda_check(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s), "memset");
            cuda_check(cudaMemsetAsync(nbad, 0, sizeof(int), s), "memset");
            cuda_check(cudaEventRecord(c->ev[2], s), "event");
            c->stats.gpu_launches += launch_deposit(lp, c->tables, p, pl, d_order, nsamp, out,
                                                    ticket, bad, nbad, err, gacc, nullptr, cfg,
                                                    s);
            cuda_check(cudaGetLastError(), "tuning launch");
            cuda_check(cudaEventRecord(c->ev[3], s), "event");
            cuda_check(cudaEventSynchronize(c->ev[3]), "tuning");
            float ms = 0.f;
            cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
            ms_min = std::min(ms_min, ms);
        }
        best.candidates++;
        if (cd.threads == base.threads && cd.chunk == base.chunk &&
            cd.persistent == base.persistent && cd.rec == base.rec)
            best.ms_default = ms_min;
        if (ms_min < best.ms_best) {
            best.ms_best = ms_min;
            best.threads = cd.threads;
            best.chunk = cd.chunk;
            best.persistent = cd.persistent;
            best.records = cd.rec;
        }
    }
    if (best.candidates == 0) {   // nothing kept the layout: the defaults
        best.threads = base.threads;
        best.chunk = base.chunk;
        best.persistent = base.persistent;
        best.records = base.rec;
        best.ms_best = best.ms_default = 0.0;
    }
    return best;
}

void apply_tuning(fsg_context *c, const LineParams &lp, const fsg_options *opt, const Particles &p,
                  PairLists pl, double *out, DepositLaunch &cfg)
{
    c->stats.launch_threads = cfg.threads;
    c->stats.launch_chunk = cfg.chunk;
    c->stats.launch_persistent = cfg.persistent;
    c->stats.launch_records = cfg.rec;
    c->stats.launch_tuned = 0;
    const int mode = opt ? opt->tune : 0;
    if (cfg.precision != FSG_PREC_FP32 || lp.kernel == VORONOI || mode < 0 || !opt ||
        opt->count_work || opt->threads > 0 || opt->chunk > 0 || opt->persistent >= 0 ||
        opt->records >= 0 || c->nlos <= 0 || pl.seg)
        return;
    const fsg_tune_key key = tune_key(c, lp, cfg.precision);
    fsg_tune_entry e{};
    bool have = false;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        tune_env_locked();
        auto it = g_tune.find(key);
        if (it != g_tune.end() && mode == 0) {
            e = it->second;
            have = true;
        }
    }
    if (!have) {
        e = tune_deposit(c, lp, p, pl, out, cfg);
        c->stats.tune_ran = 1;
        c->stats.tune_candidates = e.candidates;
        c->stats.tune_sample_lines = e.sample_lines;
        c->stats.tune_ms_default = e.ms_default;
        c->stats.tune_ms_best = e.ms_best;
        std::lock_guard<std::mutex> lock(g_tune_mu);
        tune_store_locked(key, e);
    }
    DepositLaunch t = cfg;
    t.threads = e.threads;
    t.chunk = e.chunk;
    t.persistent = e.persistent;
    t.rec = lp.compute_tau ? e.records : 0;
    t.tiles = cfg.tiles_asked;
    deposit_plan(t, lp.compute_tau, lp.nbins);
    if (t.smem_mode != cfg.smem_mode || t.tiles != cfg.tiles)
        return;   // a cached choice that does not fit this call's layout
    finish_config(c, lp, t);
    cfg = t;
    c->stats.launch_threads = cfg.threads;
    c->stats.launch_chunk = cfg.chunk;
    c->stats.launch_persistent = cfg.persistent;
    c->stats.launch_records = cfg.rec;
    c->stats.launch_tuned = 1;
}

// The batched form (fsg_spectra_batch_device): every deposit of the call in
// one CUDA graph, re-captured only when the call's shape or buffers change.
void run_batch(fsg_context *c, const std::vector<LineParams> &lps,
               const std::vector<const float *> &dens, const std::vector<double *> &outs,
               const Particles &p0, const fsg_options *opt)
{
    const int nlos = c->nlos;
    const int nb = lps.empty() ? 0 : lps[0].nbins;
    const size_t nout = (size_t)nlos * nb;
    if (nout == 0 || lps.empty())
        return;
    PairLists pl{(const long long *)c->off.p, (const int *)c->part.p, (const double *)c->dr2.p};
    std::vector<DepositLaunch> cfgs;
    for (size_t k = 0; k < lps.size(); k++) {
        cfgs.push_back(deposit_config(c, lps[k], opt));
        Particles p = p0;
        p.dens = dens[k];
        apply_tuning(c, lps[k], opt, p, pl, outs[k], cfgs.back());
    }
    for (const DepositLaunch &cf : cfgs)
        if (cf.rec)
            pl.rec = c->ensure(c->prec, 32 * (size_t)c->npairs);
    unsigned long long *gacc = nullptr;
    if (!cfgs[0].smem_mode)
        gacc = (unsigned long long *)c->ensure(c->gacc, sizeof(unsigned long long) * 2 * nout);
    auto *ticket = (unsigned *)c->ensure(c->ticket, sizeof(unsigned));
    auto *bad = (int *)c->ensure(c->bad, sizeof(int) * nlos);
    auto *nbad = (int *)c->ensure(c->nbad, sizeof(int));
    auto *err = (unsigned *)c->ensure(c->err, sizeof(unsigned));
    // graph key: everything the captured launches depend on
    std::vector<double> key;
    auto put = [&](double v) { key.push_back(v); };
    auto putp = [&](const void *q) { key.push_back((double)(uintptr_t)q); };
    put(nlos);
    put(c->npairs);
    putp(c->off.p);
    putp(c->part.p);
    putp(c->dr2.p);
    putp(c->line_order.p);
    putp(pl.rec);
    putp(c->key.p);
    putp(c->second.p);
    putp(c->axis.p);
    putp(c->pack.p);
    putp(gacc);
    putp(ticket);
    putp(bad);
    putp(nbad);
    putp(err);
    putp(p0.pos);
    putp(p0.vel);
    putp(p0.temp);
    putp(p0.hh);
    put((double)p0.n);
    for (size_t k = 0; k < lps.size(); k++) {
        const LineParams &lp = lps[k];
        for (double v : {(double)lp.compute_tau, (double)lp.nbins, (double)lp.kernel, lp.tautail,
                         lp.sigma_a, lp.bfac, lp.voigt_fac, lp.velfac, lp.vbox, lp.box})
            put(v);
        putp(dens[k]);
        putp(outs[k]);
        put(cfgs[k].precision);
        put(cfgs[k].threads);
        put(cfgs[k].persistent);
        put(cfgs[k].grid);
        put(cfgs[k].chunk);
        put(cfgs[k].tiles);
        put(cfgs[k].rec);
    }
    cudaStream_t s = c->own;
    cuda_check(cudaStreamSynchronize(c->stream), "sync caller stream");
    if (!c->graph || key != c->graph_key) {
        if (c->graph) {
            cudaGraphExecDestroy(c->graph);
            c->graph = nullptr;
        }
        cuda_check(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed), "begin capture");
        cudaMemsetAsync(err, 0, sizeof(unsigned), s);
        for (size_t k = 0; k < lps.size(); k++) {
            Particles p = p0;
            p.dens = dens[k];
            cudaMemsetAsync(outs[k], 0, sizeof(double) * nout, s);
            cudaMemsetAsync(ticket, 0, sizeof(unsigned), s);
            cudaMemsetAsync(nbad, 0, sizeof(int), s);
            launch_deposit(lps[k], c->tables, p, pl, (const int *)c->line_order.p, nlos, outs[k],
                           ticket, bad, nbad, err, gacc, nullptr, cfgs[k], s);
            launch_deposit_fallback_dev(lps[k], c->tables, p, pl, bad, nbad, nlos, outs[k], err,
                                        s);
        }
        cudaGraph_t g = nullptr;
        cuda_check(cudaStreamEndCapture(s, &g), "end capture");
        cudaError_t e = cudaGraphInstantiate(&c->graph, g, 0);
        cudaGraphDestroy(g);
        cuda_check(e, "graph instantiate");
        c->graph_key = key;
    }
    cuda_check(cudaEventRecord(c->ev[2], s), "event");
    cuda_check(cudaGraphLaunch(c->graph, s), "graph launch");
    for (const DepositLaunch &cf : cfgs)   // deposit, fallback (+ tile weights)
        c->stats.gpu_launches += 2 + (nlos > 0 && cf.tiles ? 1 : 0);
    cuda_check(cudaEventRecord(c->ev[3], s), "event");
    unsigned h_err = 0;
    cuda_check(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaStreamSynchronize(s), "batch");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
    c->stats.ms_deposit = ms;
    if (h_err)
        fail(FSG_ERR_DEVICE, "deposit kernels reported device error bits 0x%x (%s)", h_err,
             deverr_text(h_err).c_str());
}

fsg_context *g_default[64] = {nullptr};
std::mutex g_default_mu;

void ctx_init(fsg_context *c, int device)
{
    c->device = device;
    cuda_check(cudaSetDevice(device), "cudaSetDevice");
    cuda_check(cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking), "cudaStreamCreate");
    c->stream = c->own;
    for (auto &e : c->ev)
        cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    for (auto &e : c->cp)
        cuda_check(cudaEventCreate(&e), "cudaEventCreate");
    cuda_check(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking), "cudaStreamCreate");
    for (auto &e : c->up)
        cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    for (auto &e : c->gdone)
        cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    for (auto &e : c->gcopied)
        cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
}

// Copies n bytes between host buffers with up to `threads` threads (pieces
// of at least 8 MiB).  The host-pointer entry points move the caller's arrays
// through the context's pinned staging memory: the GPU's copy engines read
// and write only that warm, pinned memory, whose transfer rate does not
// depend on how the caller allocated its arrays (on the GPU machine, copies
// straight from or to callers' buffers ran at 11-60 GB/s instead of about
// 200 GB/s, and slowed down from call to call), and the caller's pages are
// only ever touched by these CPU threads.
void parallel_copy(void *dst, const void *src, size_t n, unsigned threads)
{
    if (n == 0)
        return;
    const size_t min_piece = 8u << 20;
    size_t k = std::max<size_t>(1, std::min<size_t>(threads, (n + min_piece - 1) / min_piece));
    if (k == 1) {
        memcpy(dst, src, n);
        return;
    }
    const size_t piece = ((n + k - 1) / k + 63) & ~(size_t)63;
    std::vector<std::thread> pool;
    for (size_t i = 1; i < k; i++) {
        const size_t off = i * piece;
        if (off >= n)
            break;
        const size_t len = std::min(piece, n - off);
        pool.emplace_back([dst, src, off, len] {
            memcpy((char *)dst + off, (const char *)src + off, len);
        });
    }
    memcpy(dst, src, std::min(piece, n));
    for (auto &t : pool)
        t.join();
}

unsigned copy_threads()
{
    return std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
}

// The per-device context of the host-pointer entry points (created on first
// use; the caller holds g_default_mu).
fsg_context *default_context()
{
    int dev = 0;
    cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= 64)
        fail(FSG_ERR_VALUE, "device ordinal %d out of range", dev);
    if (!g_default[dev]) {
        auto *c = new fsg_context();
        try {
            ctx_init(c, dev);
        } catch (...) {
            delete c;
            throw;
        }
        g_default[dev] = c;
    }
    return g_default[dev];
}

// Pairs of every sightline in ascending particle order (the reference's
// std::map order, which the Voronoi cell assignment depends on).
void sort_pairs_by_particle(fsg_context *c)
{
    const long long total = c->npairs;
    if (total <= 0)
        return;
    cudaStream_t s = c->stream;
    std::vector<int> part((size_t)total);
    std::vector<double> dr2((size_t)total);
    cuda_check(cudaMemcpyAsync(part.data(), c->part.p, sizeof(int) * total, cudaMemcpyDeviceToHost,
                               s), "D2H pairs");
    cuda_check(cudaMemcpyAsync(dr2.data(), c->dr2.p, sizeof(double) * total,
                               cudaMemcpyDeviceToHost, s), "D2H pairs");
    cuda_check(cudaStreamSynchronize(s), "D2H pairs");
    std::vector<std::pair<int, double>> tmp;
    for (int l = 0; l < c->nlos; l++) {
        const long long a = c->h_off[l], b = c->h_off[l + 1];
        tmp.resize((size_t)(b - a));
        for (long long e = a; e < b; e++)
            tmp[e - a] = {part[e], dr2[e]};
        std::sort(tmp.begin(), tmp.end(),
                  [](const std::pair<int, double> &x, const std::pair<int, double> &y) {
                      return x.first < y.first;
                  });
        for (long long e = a; e < b; e++) {
            part[e] = tmp[e - a].first;
            dr2[e] = tmp[e - a].second;
        }
    }
    cuda_check(cudaMemcpyAsync(c->part.p, part.data(), sizeof(int) * total, cudaMemcpyHostToDevice,
                               s), "H2D pairs");
    cuda_check(cudaMemcpyAsync(c->dr2.p, dr2.data(), sizeof(double) * total,
                               cudaMemcpyHostToDevice, s), "H2D pairs");
    cuda_check(cudaStreamSynchronize(s), "H2D pairs");
}

// IndexTable::assign_cells for every sightline: the segment of each pair's cell.
const float2 *voronoi_cells(fsg_context *c, const Particles &p, const double *cofm, double box)
{
    const long long total = c->npairs;
    const int nlos = c->nlos;
    if (total <= 0)
        return nullptr;
    if (!(box / 0.1 < 1e9))
        fail(FSG_ERR_VALUE, "box %g too large for the Voronoi sightline grid (0.1 kpc/h points)",
             box);
    cudaStream_t s = c->stream;
    sort_pairs_by_particle(c);
    auto *seg = (float2 *)c->ensure(c->vseg, sizeof(float2) * total);
    auto *scratch = (int *)c->ensure(c->vscratch,
                                     sizeof(int) * voronoi_scratch_ints(total, nlos));
    auto *dcofm = (double *)c->ensure(c->vcofm, sizeof(double) * 3 * nlos);
    auto *err = (unsigned *)c->ensure(c->err, sizeof(unsigned));
    cuda_check(cudaMemcpyAsync(dcofm, cofm, sizeof(double) * 3 * nlos, cudaMemcpyHostToDevice, s),
               "H2D cofm");
    cuda_check(cudaMemsetAsync(err, 0, sizeof(unsigned), s), "memset");
    launch_voronoi_cells(p.pos, (const int *)c->part.p, (const long long *)c->off.p,
                         c->tables.axis, dcofm, nlos, total, box, scratch, seg, err, s);
    c->stats.gpu_launches += 10;
    cuda_check(cudaGetLastError(), "Voronoi cells launch");
    unsigned h_err = 0;
    cuda_check(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaStreamSynchronize(s), "Voronoi cells");
    if (h_err & DEVERR_VORONOI_CELL)
        fail(FSG_ERR_VALUE, "a Voronoi cell's points along a sightline are not contiguous (the "
                            "reference stops the program here: index_table.cpp:199-204)");
    if (h_err)
        fail(FSG_ERR_DEVICE, "Voronoi cells reported device error bits 0x%x (%s)", h_err,
             deverr_text(h_err).c_str());
    return seg;
}

void run_interpolate(fsg_context *c, int compute_tau, int nbins, int kernel, double box,
                     double velfac, double lambda, double gamma, double fosc, double amumass,
                     double tautail, const Particles &p, const int32_t *axis, const double *cofm,
                     int32_t nlos, double *out, const fsg_options *opt,
                     const std::function<void()> &before_deposit = nullptr,
                     const RowGroups *rows = nullptr)
{
    cuda_check(cudaSetDevice(c->device), "cudaSetDevice");
    build_tables(c, axis, cofm, nlos, box);
    search_pairs(c, p, nlos);
    // the inputs only the deposit reads may still be on their way (host-pointer entry)
    if (before_deposit)
        before_deposit();
    LineParams lp = make_line_params(compute_tau, nbins, kernel, box, velfac, lambda, gamma, fosc,
                                     amumass, tautail);
    const float2 *seg = kernel == VORONOI ? voronoi_cells(c, p, cofm, box) : nullptr;
    deposit(c, lp, p, out, opt, seg, rows);
}

}  // namespace

extern "C" {

const char *fsg_version(void) { return "fsg 0.2 (sm_103a)"; }

int fsg_measure_fma_peak(int precision, double *tflops, char *errbuf, size_t errlen)
{
    try {
        if (!tflops)
            fail(FSG_ERR_VALUE, "tflops is NULL");
        if (precision != FSG_PREC_FP64 && precision != FSG_PREC_FP32)
            fail(FSG_ERR_VALUE, "unknown precision %d", precision);
        const double v = measure_fma_peak(precision, 0);
        cuda_check(cudaGetLastError(), "fma peak");
        cuda_check(cudaDeviceSynchronize(), "fma peak");
        if (!(v > 0))
            fail(FSG_ERR_CUDA, "fma peak measurement failed");
        *tflops = v;
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_context_create(int device, fsg_context **ctx, char *errbuf, size_t errlen)
{
    try {
        if (!ctx)
            fail(FSG_ERR_VALUE, "ctx is NULL");
        auto *c = new fsg_context();
        try {
            ctx_init(c, device);
        } catch (...) {
            delete c;
            throw;
        }
        *ctx = c;
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

void fsg_context_destroy(fsg_context *ctx)
{
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    if (ctx->stream)
        cudaStreamSynchronize(ctx->stream);
    ctx->release_all();
    for (auto &e : ctx->ev)
        if (e)
            cudaEventDestroy(e);
    for (auto &e : ctx->cp)
        if (e)
            cudaEventDestroy(e);
    for (auto &e : ctx->up)
        if (e)
            cudaEventDestroy(e);
    for (auto &e : ctx->gdone)
        if (e)
            cudaEventDestroy(e);
    for (auto &e : ctx->gcopied)
        if (e)
            cudaEventDestroy(e);
    if (ctx->side) {
        cudaStreamSynchronize(ctx->side);
        cudaStreamDestroy(ctx->side);
    }
    if (ctx->graph)
        cudaGraphExecDestroy(ctx->graph);
    if (ctx->own)
        cudaStreamDestroy(ctx->own);
    delete ctx;
}

int fsg_context_set_stream(fsg_context *ctx, void *cuda_stream)
{
    if (!ctx)
        return FSG_ERR_VALUE;
    // NULL is the CUDA default stream (handle 0), where torch runs unless told
    // otherwise: work on it is ordered after the caller's pending kernels.
    ctx->stream = (cudaStream_t)cuda_stream;
    return FSG_OK;
}

int fsg_context_stats(const fsg_context *ctx, fsg_stats *out)
{
    if (!ctx || !out)
        return FSG_ERR_VALUE;
    *out = ctx->stats;
    return FSG_OK;
}

int fsg_default_context_stats(fsg_stats *out)
{
    if (!out)
        return FSG_ERR_VALUE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return FSG_ERR_VALUE;
    std::lock_guard<std::mutex> lock(g_default_mu);
    if (!g_default[dev])
        return FSG_ERR_VALUE;
    *out = g_default[dev]->stats;
    return FSG_OK;
}

int fsg_particle_interpolate_device(fsg_context *ctx, int compute_tau, int nbins, int kernel,
                                    double box, double velfac, double atime, double lambda,
                                    double gamma, double fosc, double amumass, double tautail,
                                    const float *pos, const float *vel, const float *dens,
                                    const float *temp, const float *h, int64_t npart,
                                    const int32_t *axis, const double *cofm, int32_t nlos,
                                    double *out, const fsg_options *opt, char *errbuf,
                                    size_t errlen)
{
    (void)atime;   // stored but unused by the reference (absorption.cpp:157)
    try {
        if (!ctx)
            fail(FSG_ERR_VALUE, "ctx is NULL");
        validate_common(nbins, kernel, box, npart, nlos, axis, cofm, true);
        Particles p{pos, vel, dens, temp, h, (long long)npart};
        run_interpolate(ctx, compute_tau, nbins, kernel, box, velfac, lambda, gamma, fosc,
                        amumass, tautail, p, axis, cofm, nlos, out, opt);
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_particle_interpolate(int compute_tau, int nbins, int kernel, double box, double velfac,
                             double atime, double lambda, double gamma, double fosc,
                             double amumass, double tautail, const float *pos, const float *vel,
                             const float *dens, const float *temp, const float *h, int64_t npart,
                             const int32_t *axis, const double *cofm, int32_t nlos, double *out,
                             const fsg_options *opt, char *errbuf, size_t errlen)
{
    (void)atime;
    try {
        validate_common(nbins, kernel, box, npart, nlos, axis, cofm, true);
        std::lock_guard<std::mutex> lock(g_default_mu);
        fsg_context *c = default_context();
        cudaStream_t s = c->stream;
        const size_t n3 = sizeof(float) * 3 * (size_t)npart, n1 = sizeof(float) * (size_t)npart;
        const size_t nout = sizeof(double) * (size_t)nlos * (size_t)(nbins > 0 ? nbins : 0);
        // pinned staging: pos | h | dens | vel | temp | out (256-byte aligned parts)
        const auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
        const size_t o_h = al(n3), o_dens = o_h + al(n1), o_vel = o_dens + al(n1);
        const size_t o_temp = o_vel + (compute_tau ? al(n3) : 0);
        const size_t o_out = o_temp + (compute_tau ? al(n1) : 0);
        char *hs = (char *)c->ensure_host(c->hstage, o_out + al(nout));
        const unsigned nthr = copy_threads();
        // the helper thread stages what only the deposit reads while the search runs;
        // it is joined on every path, and no copy of the caller's arrays outlives
        // the call (error returns included)
        std::thread helper, drain;
        std::string helper_err;
        // output rows copied so far by row group (the drain thread copies group
        // g into the caller's array once its device-to-staging copy is done)
        std::mutex gmu;
        std::condition_variable gcv;
        int queued = 0;          // groups whose copies are queued
        bool abandon = false;    // error path: the drain thread stops
        struct Guard {
            fsg_context *c;
            std::thread &t, &d;
            std::mutex &mu;
            std::condition_variable &cv;
            bool &abandon;
            ~Guard()
            {
                {
                    std::lock_guard<std::mutex> l(mu);
                    abandon = true;
                }
                cv.notify_all();
                if (t.joinable())
                    t.join();
                if (d.joinable())
                    d.join();
                cudaStreamSynchronize(c->side);
                cudaStreamSynchronize(c->stream);
            }
        } guard{c, helper, drain, gmu, gcv, abandon};
        Particles p;
        p.n = npart;
        auto *dpos = (float *)c->ensure(c->pos, n3);
        auto *dh = (float *)c->ensure(c->hh, n1);
        auto *ddens = (float *)c->ensure(c->dens, n1);
        auto *dvel = compute_tau ? (float *)c->ensure(c->vel, n3) : nullptr;
        auto *dtemp = compute_tau ? (float *)c->ensure(c->temp, n1) : nullptr;
        p.pos = dpos;
        p.hh = dh;
        p.dens = ddens;
        p.vel = dvel;
        p.temp = dtemp;
        // the search reads pos and h: staged and sent first, in pieces, so
        // that each piece's upload overlaps the staging of the next
        cuda_check(cudaEventRecord(c->cp[0], s), "event");
        const auto stage_up = [&](void *dst, const void *src, size_t off, size_t n) {
            const size_t piece = (size_t)256 << 20;
            for (size_t b = 0; b < n; b += piece) {
                const size_t len = std::min(piece, n - b);
                parallel_copy(hs + off + b, (const char *)src + b, len, nthr);
                cuda_check(cudaMemcpyAsync((char *)dst + b, hs + off + b, len,
                                           cudaMemcpyHostToDevice, s), "H2D");
            }
        };
        if (npart > 0) {
            stage_up(dpos, pos, 0, n3);
            stage_up(dh, h, o_h, n1);
        }
        helper = std::thread([&] {
            const cudaError_t e0 = cudaSetDevice(c->device);
            if (e0 != cudaSuccess) {
                helper_err = cudaGetErrorString(e0);
                return;
            }
            parallel_copy(hs + o_dens, dens, n1, nthr);
            if (compute_tau) {
                parallel_copy(hs + o_vel, vel, n3, nthr);
                parallel_copy(hs + o_temp, temp, n1, nthr);
            }
            cudaError_t e = cudaSuccess;
            if (npart > 0) {
                e = cudaMemcpyAsync(ddens, hs + o_dens, n1, cudaMemcpyHostToDevice, c->side);
                if (e == cudaSuccess && compute_tau)
                    e = cudaMemcpyAsync(dvel, hs + o_vel, n3, cudaMemcpyHostToDevice, c->side);
                if (e == cudaSuccess && compute_tau)
                    e = cudaMemcpyAsync(dtemp, hs + o_temp, n1, cudaMemcpyHostToDevice,
                                        c->side);
            }
            if (e == cudaSuccess)
                e = cudaEventRecord(c->up[1], c->side);
            if (e == cudaSuccess)
                e = cudaEventRecord(c->cp[1], c->side);
            if (e != cudaSuccess)
                helper_err = cudaGetErrorString(e);
        });
        const auto inputs_ready = [&] {
            helper.join();
            if (!helper_err.empty())
                fail(FSG_ERR_CUDA, "staging the inputs: %s", helper_err.c_str());
            cuda_check(cudaStreamWaitEvent(s, c->up[1], 0), "wait for uploads");
        };
        double *dout = (double *)c->ensure(c->out, nout);
        // the output leaves in row groups: group g's rows go to the staging
        // area on the side stream once its deposit launch is done, and the
        // drain thread moves them into the caller's array while later groups
        // compute
        std::vector<long long> grow0(fsg_context::ROW_GROUPS), grow1(fsg_context::ROW_GROUPS);
        RowGroups rg;
        rg.groups = fsg_context::ROW_GROUPS;
        rg.on_group = [&](int g, long long r0, long long r1) {
            const size_t b0 = sizeof(double) * (size_t)r0 * nbins;
            const size_t nb = sizeof(double) * (size_t)(r1 - r0) * nbins;
            cuda_check(cudaStreamWaitEvent(c->side, c->gdone[g], 0), "wait for rows");
            if (nb)
                cuda_check(cudaMemcpyAsync(hs + o_out + b0, (char *)dout + b0, nb,
                                           cudaMemcpyDeviceToHost, c->side), "D2H");
            cuda_check(cudaEventRecord(c->gcopied[g], c->side), "event");
            grow0[g] = r0;
            grow1[g] = r1;
            {
                std::lock_guard<std::mutex> l(gmu);
                queued = g + 1;
            }
            gcv.notify_all();
        };
        std::string drain_err;
        drain = std::thread([&] {
            if (cudaSetDevice(c->device) != cudaSuccess)
                return;
            for (int g = 0; g < fsg_context::ROW_GROUPS; g++) {
                {
                    std::unique_lock<std::mutex> l(gmu);
                    gcv.wait(l, [&] { return queued > g || abandon; });
                    if (queued <= g)
                        return;
                }
                const cudaError_t e = cudaEventSynchronize(c->gcopied[g]);
                if (e != cudaSuccess) {
                    drain_err = cudaGetErrorString(e);
                    return;
                }
                const size_t b0 = sizeof(double) * (size_t)grow0[g] * nbins;
                parallel_copy((char *)out + b0, hs + o_out + b0,
                              sizeof(double) * (size_t)(grow1[g] - grow0[g]) * nbins, nthr);
            }
        });
        run_interpolate(c, compute_tau, nbins, kernel, box, velfac, lambda, gamma, fosc, amumass,
                        tautail, p, axis, cofm, nlos, dout, opt, inputs_ready, &rg);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->cp[0], c->cp[1]);
        c->stats.ms_h2d = ms;   // first staging copy to the last upload (search overlapped)
        const auto t0 = std::chrono::steady_clock::now();
        if (queued == 0) {
            // one launch (few sightlines, or nothing to deposit): copy it all
            {
                std::lock_guard<std::mutex> l(gmu);
                abandon = true;
            }
            gcv.notify_all();
            drain.join();
            if (nout)
                cuda_check(cudaMemcpyAsync(hs + o_out, dout, nout, cudaMemcpyDeviceToHost, s),
                           "D2H");
            cuda_check(cudaStreamSynchronize(s), "D2H");
            parallel_copy(out, hs + o_out, nout, nthr);
        } else {
            drain.join();
            if (!drain_err.empty())
                fail(FSG_ERR_CUDA, "output copy: %s", drain_err.c_str());
            // rows the FP64 fallback redid after their group was copied
            for (int line : c->h_bad) {
                const size_t b0 = sizeof(double) * (size_t)line * nbins;
                const size_t nb = sizeof(double) * (size_t)nbins;
                cuda_check(cudaMemcpyAsync(hs + o_out + b0, (char *)dout + b0, nb,
                                           cudaMemcpyDeviceToHost, s), "D2H");
                cuda_check(cudaStreamSynchronize(s), "D2H");
                memcpy((char *)out + b0, hs + o_out + b0, nb);
            }
        }
        c->stats.ms_d2h =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
                .count();   // device-to-staging copy and the copy into the caller's array
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_spectra_batch_device(fsg_context *ctx, int nbins, int kernel, double box, double velfac,
                             double atime, double tautail, const float *pos, const float *vel,
                             const float *temp, const float *h, int64_t npart,
                             const int32_t *axis, const double *cofm, int32_t nlos, int nlines,
                             const fsg_line *lines, const fsg_options *opt, char *errbuf,
                             size_t errlen)
{
    (void)atime;
    try {
        if (!ctx)
            fail(FSG_ERR_VALUE, "ctx is NULL");
        if (nlines < 0 || (nlines > 0 && !lines))
            fail(FSG_ERR_VALUE, "bad line list");
        validate_common(nbins, kernel, box, npart, nlos, axis, cofm);
        bool any_tau = false;
        for (int k = 0; k < nlines; k++) {
            if (!lines[k].dens)
                fail(FSG_ERR_VALUE, "line %d has no density array", k);
            any_tau |= lines[k].tau != nullptr;
        }
        if (any_tau && (!vel || !temp))
            fail(FSG_ERR_VALUE, "tau needs vel and temp");
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        build_tables(ctx, axis, cofm, nlos, box);
        Particles p{pos, vel, nullptr, temp, h, (long long)npart};
        search_pairs(ctx, p, nlos);
        std::vector<LineParams> lps;
        std::vector<const float *> dens;
        std::vector<double *> outs;
        for (int k = 0; k < nlines; k++) {
            const fsg_line &L = lines[k];
            if (L.tau) {
                lps.push_back(make_line_params(1, nbins, kernel, box, velfac, L.lambda, L.gamma,
                                               L.fosc, L.amumass, tautail));
                dens.push_back(L.dens);
                outs.push_back(L.tau);
            }
            if (L.colden) {
                lps.push_back(make_line_params(0, nbins, kernel, box, velfac, L.lambda, L.gamma,
                                               L.fosc, L.amumass, tautail));
                dens.push_back(L.dens);
                outs.push_back(L.colden);
            }
        }
        run_batch(ctx, lps, dens, outs, p, opt);
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

static int tau_backward(fsg_context *ctx, const unsigned long long *reuse_gen, int nbins,
                        int kernel, double box, double velfac, double lambda, double gamma,
                        double fosc, double amumass, double tautail, const float *pos,
                        const float *vel, const float *dens, const float *temp, const float *h,
                        int64_t npart, const int32_t *axis, const double *cofm, int32_t nlos,
                        const double *grad_tau, float *grad_dens, float *grad_temp,
                        float *grad_vel, char *errbuf, size_t errlen)
{
    try {
        if (!ctx)
            fail(FSG_ERR_VALUE, "ctx is NULL");
        validate_common(nbins, kernel, box, npart, nlos, axis, cofm);
        if (!grad_tau || !grad_dens || !grad_temp || !grad_vel)
            fail(FSG_ERR_VALUE, "gradient buffers must not be NULL");
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        Particles p{pos, vel, dens, temp, h, (long long)npart};
        const fsg_context::SearchRecord &r = ctx->search_rec;
        const bool reuse = reuse_gen && *reuse_gen == ctx->search_gen && r.pos == pos &&
                           r.hh == h && r.npart == (long long)npart && r.nlos == nlos &&
                           r.box == box && r.lines == lines_hash_of(axis, cofm, nlos);
        ctx->stats.search_reused = reuse ? 1 : 0;
        if (!reuse) {
            build_tables(ctx, axis, cofm, nlos, box);
            search_pairs(ctx, p, nlos);
        }
        if (nlos == 0 || nbins == 0 || ctx->npairs == 0)
            return FSG_OK;
        LineParams lp = make_line_params(1, nbins, kernel, box, velfac, lambda, gamma, fosc,
                                         amumass, tautail);
        PairLists pl{(const long long *)ctx->off.p, (const int *)ctx->part.p,
                     (const double *)ctx->dr2.p};
        cudaStream_t s = ctx->stream;
        auto *ticket = (unsigned *)ctx->ensure(ctx->ticket, sizeof(unsigned));
        auto *err = (unsigned *)ctx->ensure(ctx->err, sizeof(unsigned));
        cuda_check(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s), "memset");
        cuda_check(cudaMemsetAsync(err, 0, sizeof(unsigned), s), "memset");
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        const int grid = std::min(nlos, sms * std::max(1, tau_backward_resident_ctas()));
        cuda_check(cudaEventRecord(ctx->ev[2], s), "event");
        launch_tau_backward(lp, ctx->tables, p, pl, (const int *)ctx->line_order.p, nlos,
                            grad_tau, grad_dens, grad_temp, grad_vel, ticket, err, grid, s);
        ctx->stats.gpu_launches++;
        cuda_check(cudaGetLastError(), "backward launch");
        cuda_check(cudaEventRecord(ctx->ev[3], s), "event");
        unsigned h_err = 0;
        cuda_check(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s),
                   "read");
        cuda_check(cudaStreamSynchronize(s), "backward");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
        ctx->stats.ms_deposit = ms;
        if (h_err)
            fail(FSG_ERR_DEVICE, "backward kernel reported device error bits 0x%x (%s)", h_err,
                 deverr_text(h_err).c_str());
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_tau_backward_device(fsg_context *ctx, int nbins, int kernel, double box, double velfac,
                            double atime, double lambda, double gamma, double fosc,
                            double amumass, double tautail, const float *pos, const float *vel,
                            const float *dens, const float *temp, const float *h, int64_t npart,
                            const int32_t *axis, const double *cofm, int32_t nlos,
                            const double *grad_tau, float *grad_dens, float *grad_temp,
                            float *grad_vel, char *errbuf, size_t errlen)
{
    (void)atime;
    return tau_backward(ctx, nullptr, nbins, kernel, box, velfac, lambda, gamma, fosc, amumass,
                        tautail, pos, vel, dens, temp, h, npart, axis, cofm, nlos, grad_tau,
                        grad_dens, grad_temp, grad_vel, errbuf, errlen);
}

int fsg_tau_backward_reuse_device(fsg_context *ctx, uint64_t generation, int nbins, int kernel,
                                  double box, double velfac, double atime, double lambda,
                                  double gamma, double fosc, double amumass, double tautail,
                                  const float *pos, const float *vel, const float *dens,
                                  const float *temp, const float *h, int64_t npart,
                                  const int32_t *axis, const double *cofm, int32_t nlos,
                                  const double *grad_tau, float *grad_dens, float *grad_temp,
                                  float *grad_vel, char *errbuf, size_t errlen)
{
    (void)atime;
    const unsigned long long g = generation;
    return tau_backward(ctx, &g, nbins, kernel, box, velfac, lambda, gamma, fosc, amumass,
                        tautail, pos, vel, dens, temp, h, npart, axis, cofm, nlos, grad_tau,
                        grad_dens, grad_temp, grad_vel, errbuf, errlen);
}

int fsg_context_search_generation(const fsg_context *ctx, uint64_t *generation)
{
    if (!ctx || !generation)
        return FSG_ERR_VALUE;
    *generation = ctx->search_gen;
    return FSG_OK;
}

int fsg_build_pairs_device(fsg_context *ctx, double box, const float *pos, const float *h,
                           int64_t npart, const int32_t *axis, const double *cofm, int32_t nlos,
                           int64_t *npairs, char *errbuf, size_t errlen)
{
    try {
        if (!ctx)
            fail(FSG_ERR_VALUE, "ctx is NULL");
        validate_common(0, SPH_CUBIC, box, npart, nlos, axis, cofm);
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        build_tables(ctx, axis, cofm, nlos, box);
        Particles p{pos, nullptr, nullptr, nullptr, h, (long long)npart};
        search_pairs(ctx, p, nlos);
        if (npairs)
            *npairs = ctx->npairs;
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_near_lines_device(fsg_context *ctx, double box, const float *pos, const float *h,
                          int64_t npart, const int32_t *axis, const double *cofm, int32_t nlos,
                          int32_t *out, int64_t *nout, char *errbuf, size_t errlen)
{
    try {
        if (!ctx || !nout)
            fail(FSG_ERR_VALUE, "ctx and nout must not be NULL");
        validate_common(0, SPH_CUBIC, box, npart, nlos, axis, cofm);
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        build_tables(ctx, axis, cofm, nlos, box);
        Particles p{pos, nullptr, nullptr, nullptr, h, (long long)npart};
        *nout = near_lines(ctx, p, out);
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_near_lines(double box, const float *pos, const float *h, int64_t npart,
                   const int32_t *axis, const double *cofm, int32_t nlos, int32_t *out,
                   int64_t *nout, char *errbuf, size_t errlen)
{
    try {
        if (!nout)
            fail(FSG_ERR_VALUE, "nout must not be NULL");
        validate_common(0, SPH_CUBIC, box, npart, nlos, axis, cofm);
        std::lock_guard<std::mutex> lock(g_default_mu);
        fsg_context *c = default_context();
        cudaStream_t s = c->stream;
        const size_t n3 = sizeof(float) * 3 * (size_t)npart, n1 = sizeof(float) * (size_t)npart;
        auto *dpos = (float *)c->ensure(c->pos, n3);
        auto *dh = (float *)c->ensure(c->hh, n1);
        if (npart > 0) {
            cuda_check(cudaMemcpyAsync(dpos, pos, n3, cudaMemcpyHostToDevice, s), "H2D");
            cuda_check(cudaMemcpyAsync(dh, h, n1, cudaMemcpyHostToDevice, s), "H2D");
        }
        build_tables(c, axis, cofm, nlos, box);
        Particles p{dpos, nullptr, nullptr, nullptr, dh, (long long)npart};
        auto *didx = (int *)c->ensure(c->idx, sizeof(int) * (size_t)npart);
        const long long n = near_lines(c, p, didx);
        if (n > 0)
            cuda_check(cudaMemcpyAsync(out, didx, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost,
                                       s), "D2H");
        cuda_check(cudaStreamSynchronize(s), "D2H");
        *nout = n;
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_colden_channels_device(fsg_context *ctx, int nbins, int kernel, double box,
                               double velfac, const float *pos, const float *h, int64_t npart,
                               const int32_t *axis, const double *cofm, int32_t nlos, int nch,
                               const float *const *dens, double *const *out,
                               const fsg_options *opt, char *errbuf, size_t errlen)
{
    try {
        if (!ctx)
            fail(FSG_ERR_VALUE, "ctx is NULL");
        if (nch < 1 || nch > MAX_CHANNELS)
            fail(FSG_ERR_VALUE, "between 1 and %d channels (got %d)", MAX_CHANNELS, nch);
        for (int c = 0; c < nch; c++)
            if (!dens || !out || !dens[c] || !out[c])
                fail(FSG_ERR_VALUE, "channel %d has no density or output array", c);
        validate_common(nbins, kernel, box, npart, nlos, axis, cofm);
        const int precision = opt ? opt->precision : FSG_PREC_FP64;
        if (precision != FSG_PREC_FP64 && precision != FSG_PREC_FP32)
            fail(FSG_ERR_VALUE, "unknown precision %d", precision);
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        cudaStream_t s = ctx->stream;
        const size_t nout = (size_t)nlos * (size_t)(nbins > 0 ? nbins : 0);
        for (int c = 0; c < nch; c++)
            if (nout)
                cuda_check(cudaMemsetAsync(out[c], 0, sizeof(double) * nout, s), "memset out");
        if (nout == 0 || npart == 0) {
            cuda_check(cudaStreamSynchronize(s), "colden channels");
            return FSG_OK;
        }
        build_tables(ctx, axis, cofm, nlos, box);
        Particles p{pos, nullptr, nullptr, nullptr, h, (long long)npart};
        search_pairs(ctx, p, nlos);
        if (ctx->npairs == 0)
            return FSG_OK;
        const LineParams lp = make_line_params(0, nbins, kernel, box, velfac, 0.0, 0.0, 0.0, 1.0,
                                               0.0);
        const ChannelPlan plan = colden_channels_plan(precision, nch, nbins);
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
        const int grid = std::min(nlos, sms * plan.per_sm);
        unsigned long long *gacc = nullptr;
        if (!plan.smem_mode)
            gacc = (unsigned long long *)ctx->ensure(
                ctx->gacc, sizeof(unsigned long long) * plan.acc_words_per_cta * grid);
        auto *bad = (int *)ctx->ensure(ctx->bad, sizeof(int) * (size_t)nch * nlos);
        auto *nbad = (int *)ctx->ensure(ctx->nbad, sizeof(int) * MAX_CHANNELS);
        auto *ticket = (unsigned *)ctx->ensure(ctx->ticket, sizeof(unsigned));
        auto *err = (unsigned *)ctx->ensure(ctx->err, sizeof(unsigned));
        cuda_check(cudaMemsetAsync(nbad, 0, sizeof(int) * MAX_CHANNELS, s), "memset");
        cuda_check(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s), "memset");
        cuda_check(cudaMemsetAsync(err, 0, sizeof(unsigned), s), "memset");
        PairLists pl{(const long long *)ctx->off.p, (const int *)ctx->part.p,
                     (const double *)ctx->dr2.p};
        launch_colden_channels(lp, ctx->tables, p, pl, (const int *)ctx->line_order.p, nlos, nch,
                               dens, out, bad, nbad, ticket, err, gacc, precision, plan, grid, s);
        ctx->stats.gpu_launches++;
        cuda_check(cudaGetLastError(), "colden channels launch");
        int h_nbad[MAX_CHANNELS] = {0};
        cuda_check(cudaMemcpyAsync(h_nbad, nbad, sizeof(int) * MAX_CHANNELS,
                                   cudaMemcpyDeviceToHost, s), "read");
        cuda_check(cudaStreamSynchronize(s), "colden channels");
        int fallback = 0;
        for (int c = 0; c < nch; c++) {
            if (h_nbad[c] <= 0)
                continue;
            Particles pc = p;
            pc.dens = dens[c];
            launch_deposit_fallback(lp, ctx->tables, pc, pl, bad + (size_t)c * nlos, h_nbad[c],
                                    out[c], err, s);
            ctx->stats.gpu_launches++;
            fallback += h_nbad[c];
            cuda_check(cudaGetLastError(), "fallback launch");
        }
        ctx->stats.fallback_lines = fallback;
        unsigned h_err = 0;
        cuda_check(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s),
                   "read");
        cuda_check(cudaStreamSynchronize(s), "colden channels");
        if (h_err)
            fail(FSG_ERR_DEVICE, "column-density kernels reported device error bits 0x%x (%s)",
                 h_err, deverr_text(h_err).c_str());
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_mean_flux_scale_device(fsg_context *ctx, const double *tau, int64_t n,
                               double mean_flux_desired, double tol, double thresh, double *scale,
                               char *errbuf, size_t errlen)
{
    try {
        if (!ctx || !scale)
            fail(FSG_ERR_VALUE, "ctx and scale must not be NULL");
        if (n < 0)
            fail(FSG_ERR_VALUE, "negative array length");
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        *scale = mean_flux_scale(ctx, tau, n, mean_flux_desired, tol, thresh);
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_rescale_mean_flux(const double *tau, int64_t n, double mean_flux_desired, double tol,
                          double thresh, double *scale, char *errbuf, size_t errlen)
{
    try {
        if (!scale)
            fail(FSG_ERR_VALUE, "scale must not be NULL");
        if (n < 0)
            fail(FSG_ERR_VALUE, "negative array length");
        std::lock_guard<std::mutex> lock(g_default_mu);
        fsg_context *c = default_context();
        auto *d = (double *)c->ensure(c->ftau, sizeof(double) * (size_t)n);
        if (n > 0)
            cuda_check(cudaMemcpyAsync(d, tau, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice,
                                       c->stream), "H2D");
        *scale = mean_flux_scale(c, d, n, mean_flux_desired, tol, thresh);
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_mean_flux_device(fsg_context *ctx, const double *tau, int64_t n, double scale,
                         double *mean, char *errbuf, size_t errlen)
{
    try {
        if (!ctx || !mean)
            fail(FSG_ERR_VALUE, "ctx and mean must not be NULL");
        if (n <= 0)
            fail(FSG_ERR_VALUE, "the mean flux of an empty array is undefined");
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        *mean = mean_flux_of(ctx, tau, n, scale);
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_flux_exp_device(fsg_context *ctx, const double *y, int64_t n, double *out, char *errbuf,
                        size_t errlen)
{
    try {
        if (!ctx || (n > 0 && (!y || !out)))
            fail(FSG_ERR_VALUE, "ctx, y and out must not be NULL");
        if (n < 0)
            fail(FSG_ERR_VALUE, "n must be >= 0 (got %lld)", (long long)n);
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        const double *etab = exp_table(ctx);
        if (n > 0) {
            launch_fexp(y, n, etab, out, ctx->stream);
            ctx->stats.gpu_launches++;
            cuda_check(cudaGetLastError(), "exp launch");
        }
        cuda_check(cudaStreamSynchronize(ctx->stream), "exp");
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_flux_histogram_device(fsg_context *ctx, const double *tau, int64_t n, double scale,
                              const double *edges, int nb, int64_t *counts, char *errbuf,
                              size_t errlen)
{
    try {
        if (!ctx || !edges || !counts)
            fail(FSG_ERR_VALUE, "ctx, edges and counts must not be NULL");
        // the block histogram keeps 16 bytes of shared memory per bin
        if (n < 0 || nb < 1 || nb > 8192)
            fail(FSG_ERR_VALUE, "need n >= 0 and 1 <= nbins <= 8192 (got %lld, %d)",
                 (long long)n, nb);
        for (int j = 0; j < nb; j++)
            if (!(edges[j] < edges[j + 1]))
                fail(FSG_ERR_VALUE, "bin edges must increase monotonically");
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        cudaStream_t s = ctx->stream;
        auto *de = (double *)ctx->ensure(ctx->fedges, sizeof(double) * (nb + 1));
        auto *dc = (unsigned long long *)ctx->ensure(ctx->fcounts, sizeof(long long) * nb);
        cuda_check(cudaMemcpyAsync(de, edges, sizeof(double) * (nb + 1), cudaMemcpyHostToDevice,
                                   s), "H2D");
        cuda_check(cudaMemsetAsync(dc, 0, sizeof(long long) * nb, s), "memset");
        cuda_check(cudaEventRecord(ctx->ev[2], s), "event");
        if (n > 0) {
            launch_flux_hist(tau, n, scale, de, nb, dc, s);
            ctx->stats.gpu_launches++;
            cuda_check(cudaGetLastError(), "flux histogram launch");
        }
        cuda_check(cudaEventRecord(ctx->ev[3], s), "event");
        cuda_check(cudaMemcpyAsync(counts, dc, sizeof(long long) * nb, cudaMemcpyDeviceToHost, s),
                   "D2H");
        cuda_check(cudaStreamSynchronize(s), "flux histogram");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
        ctx->stats.ms_flux = ms;
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_flux_power_device(fsg_context *ctx, const double *tau, int64_t nspec, int64_t npix,
                          double scale, double mean_flux, double vmax, double *power,
                          char *errbuf, size_t errlen)
{
    try {
        if (!ctx || !power)
            fail(FSG_ERR_VALUE, "ctx and power must not be NULL");
        if (nspec <= 0 || npix <= 0 || npix > (1 << 28))
            fail(FSG_ERR_VALUE, "need nspec > 0 and 0 < npix <= 2^28 (got %lld, %lld)",
                 (long long)nspec, (long long)npix);
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        cudaStream_t s = ctx->stream;
        const long long nk = npix / 2 + 1;
        PowerPlan &pl = ctx->pplan;
        if (pl.npix != npix) {
            pl = PowerPlan{};
            PowerPlan fresh = power_plan(npix);
            auto *tables = (double2 *)ctx->ensure(ctx->ptables,
                                                  sizeof(double2) * (size_t)fresh.table_len);
            double2 *chirp = nullptr, *bhat = nullptr, *scratch = nullptr;
            if (fresh.bluestein) {
                chirp = (double2 *)ctx->ensure(ctx->pchirp, sizeof(double2) * (size_t)npix);
                bhat = (double2 *)ctx->ensure(ctx->pbhat, sizeof(double2) * (size_t)fresh.len);
                scratch = (double2 *)ctx->ensure(ctx->ffft, sizeof(double2) * (size_t)fresh.len);
            }
            ctx->stats.gpu_launches += power_plan_tables(fresh, tables, chirp, bhat, scratch, s);
            cuda_check(cudaGetLastError(), "flux power tables");
            // the scratch buffer is regrown below
            cuda_check(cudaStreamSynchronize(s), "flux power tables");
            pl = fresh;
        }
        const double *etab = exp_table(ctx);
        const long long chunk = power_pairs_per_chunk(pl, nspec);
        const size_t words = sizeof(double2) * (size_t)chunk * (size_t)pl.len;
        auto *a = (double2 *)ctx->ensure(ctx->fdflux, words);
        auto *b = (double2 *)ctx->ensure(ctx->ffft, words);
        auto *part = (double *)ctx->ensure(ctx->ppart, sizeof(double) * power_partials(npix));
        auto *dp = (double *)ctx->ensure(ctx->fpower, sizeof(double) * nk);
        cuda_check(cudaMemsetAsync(dp, 0, sizeof(double) * nk, s), "memset");
        cuda_check(cudaEventRecord(ctx->ev[2], s), "event");
        for (long long r0 = 0; r0 < nspec; r0 += 2 * chunk) {
            const long long r = (r0 + 2 * chunk <= nspec) ? 2 * chunk : nspec - r0;
            ctx->stats.gpu_launches += power_chunk(
                pl, (const double2 *)ctx->ptables.p, (const double2 *)ctx->pchirp.p,
                (const double2 *)ctx->pbhat.p, etab, tau + r0 * npix, r, scale, 1.0 / mean_flux,
                vmax, a, b, part, dp, s);
            cuda_check(cudaGetLastError(), "flux power launch");
        }
        cuda_check(cudaEventRecord(ctx->ev[3], s), "event");
        cuda_check(cudaMemcpyAsync(power, dp, sizeof(double) * nk, cudaMemcpyDeviceToHost, s),
                   "D2H");
        cuda_check(cudaStreamSynchronize(s), "flux power");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
        ctx->stats.ms_flux = ms;
        for (int k = 0; k < nk; k++)
            power[k] /= (double)nspec;
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_tune_cache_file(const char *path, char *errbuf, size_t errlen)
{
    try {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune_env_read = true;   // an explicit file replaces FSG_TUNE_CACHE
        g_tune_file = path ? path : "";
        if (!g_tune_file.empty()) {
            FILE *f = fopen(g_tune_file.c_str(), "a");
            if (!f)
                fail(FSG_ERR_VALUE, "cannot open the tuning cache file %s", g_tune_file.c_str());
            fclose(f);
            tune_load_locked(g_tune_file);
        }
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

int fsg_tune_cache_lookup(const fsg_tune_key *key, fsg_tune_entry *entry)
{
    if (!key || !entry)
        return 0;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    tune_env_locked();
    auto it = g_tune.find(*key);
    if (it == g_tune.end())
        return 0;
    *entry = it->second;
    return 1;
}

int fsg_tune_cache_store(const fsg_tune_key *key, const fsg_tune_entry *entry, char *errbuf,
                         size_t errlen)
{
    try {
        if (!key || !entry)
            fail(FSG_ERR_VALUE, "key and entry must not be NULL");
        if (!tune_entry_valid(*entry))
            fail(FSG_ERR_VALUE, "not a valid launch: threads a multiple of 32 up to 1024, "
                                "chunk 1..32, persistent and records 0 or 1");
        std::lock_guard<std::mutex> lock(g_tune_mu);
        tune_env_locked();
        if (!tune_store_locked(*key, *entry))
            fail(FSG_ERR_VALUE, "cannot append to the tuning cache file %s", g_tune_file.c_str());
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

void fsg_tune_cache_clear(void)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune.clear();
}

int fsg_copy_pairs(fsg_context *ctx, int64_t *offsets, int32_t *part, double *dr2, int sorted,
                   char *errbuf, size_t errlen)
{
    try {
        if (!ctx)
            fail(FSG_ERR_VALUE, "ctx is NULL");
        const int nlos = ctx->nlos;
        const long long total = ctx->npairs;
        for (int i = 0; i <= nlos; i++)
            offsets[i] = ctx->h_off[i];
        if (total > 0) {
            cuda_check(cudaMemcpyAsync(part, ctx->part.p, sizeof(int) * total,
                                       cudaMemcpyDeviceToHost, ctx->stream), "D2H pairs");
            cuda_check(cudaMemcpyAsync(dr2, ctx->dr2.p, sizeof(double) * total,
                                       cudaMemcpyDeviceToHost, ctx->stream), "D2H pairs");
            cuda_check(cudaStreamSynchronize(ctx->stream), "D2H pairs");
        }
        if (sorted) {
            std::vector<std::pair<int, double>> tmp;
            for (int i = 0; i < nlos; i++) {
                const long long a = offsets[i], b = offsets[i + 1];
                tmp.resize(b - a);
                for (long long k = a; k < b; k++)
                    tmp[k - a] = {part[k], dr2[k]};
                std::sort(tmp.begin(), tmp.end(),
                          [](const std::pair<int, double> &x, const std::pair<int, double> &y) {
                              return x.first < y.first;
                          });
                for (long long k = a; k < b; k++) {
                    part[k] = tmp[k - a].first;
                    dr2[k] = tmp[k - a].second;
                }
            }
        }
        return FSG_OK;
    } catch (const FsgError &e) {
        return report(e, errbuf, errlen);
    }
}

}  // extern "C"
