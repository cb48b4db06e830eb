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
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

using namespace fsg;

namespace {

struct DevBuf {
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
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    // host mirrors
    std::vector<long long> h_off;
    std::vector<int> h_order;
    // batched form: instantiated graph of the deposits and the call it was built for
    cudaGraphExec_t graph = nullptr;
    std::vector<double> graph_key;
    int nlos = 0;
    long long npairs = 0;
    LineTables tables{};
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

    void release_all()
    {
        DevBuf *bufs[] = {&pos, &vel, &dens, &temp, &hh, &out, &key, &second, &axis, &pack,
                          &cell_start[0], &cell_start[1], &cell_start[2], &cell_line[0],
                          &cell_line[1], &cell_line[2], &line_count, &cursor, &off, &part, &dr2,
                          &line_order, &ticket, &bad, &nbad, &err, &gacc, &counters,
                          &skey, &sperm, &shist, &sstart, &ssums};
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
                     const int32_t *axis, const double *cofm)
{
    if (nbins < 0)
        fail(FSG_ERR_VALUE, "nbins must be non-negative (got %d)", nbins);
    if (npart < 0 || nlos < 0)
        fail(FSG_ERR_VALUE, "negative array length");
    if (npart > 2147483647LL)
        fail(FSG_ERR_VALUE, "at most 2^31-1 particles (particle indices are int, as in the "
                            "reference's std::map<int, double>)");
    if (kernel == VORONOI)
        fail(FSG_ERR_NOT_IMPLEMENTED, "the Voronoi-mesh kernel (kernel == 2) is not implemented");
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
void build_tables(fsg_context *c, const int32_t *axis, const double *cofm, int nlos, double box)
{
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
        pk[i] = pack_line(key[i], second[i], axis[i]);
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
    t.box_f = (float)box;
    t.pre_eps = prefilter_eps(box);
    c->nlos = nlos;
}

// 2. pair search
void search_pairs(fsg_context *c, const Particles &p, int nlos)
{
    cudaStream_t s = c->stream;
    cuda_check(cudaEventRecord(c->ev[0], s), "event");
    // spatial order of the particles (counting sort by 3-D cell)
    int *perm = nullptr;
    if (p.n > 0) {
        const int G = sort_grid_side(p.n);
        const size_t M = (size_t)G * G * G;
        auto *key = (unsigned *)c->ensure(c->skey, sizeof(unsigned) * p.n);
        perm = (int *)c->ensure(c->sperm, sizeof(int) * p.n);
        auto *hist = (unsigned *)c->ensure(c->shist, sizeof(unsigned) * M);
        auto *start = (unsigned *)c->ensure(c->sstart, sizeof(unsigned) * M);
        auto *sums = (unsigned *)c->ensure(c->ssums, sizeof(unsigned) * (M / 2048 + 2));
        launch_particle_order(p, c->tables.box, G, key, hist, start, sums, perm, s);
        c->stats.gpu_launches += 5;
        cuda_check(cudaGetLastError(), "particle order launch");
    }
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
        c->stats.gpu_launches += 2;
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
}

DepositLaunch deposit_config(fsg_context *c, const LineParams &lp, const fsg_options *opt);

// 3. deposit into out (device, nlos*nbins)
void deposit(fsg_context *c, const LineParams &lp, const Particles &p, double *out,
             const fsg_options *opt)
{
    cudaStream_t s = c->stream;
    const int nlos = c->nlos;
    const size_t nout = (size_t)nlos * lp.nbins;
    cuda_check(cudaEventRecord(c->ev[2], s), "event");
    if (nout)
        cuda_check(cudaMemsetAsync(out, 0, sizeof(double) * nout, s), "memset out");
    c->stats.fallback_lines = 0;
    if (nout == 0 || c->npairs == 0) {
        cuda_check(cudaEventRecord(c->ev[3], s), "event");
        cuda_check(cudaStreamSynchronize(s), "deposit");
        c->stats.ms_deposit = 0;
        return;
    }
    PairLists pl{(const long long *)c->off.p, (const int *)c->part.p, (const double *)c->dr2.p};
    const DepositLaunch cfg = deposit_config(c, lp, opt);
    unsigned long long *gacc = nullptr;
    if (!cfg.smem_mode) {
        gacc = (unsigned long long *)c->ensure(c->gacc, sizeof(unsigned long long) * 2 * nout);
    }
    const bool count = opt && opt->count_work;
    unsigned long long *ctr = nullptr;
    if (count) {
        ctr = (unsigned long long *)c->ensure(c->counters, sizeof(unsigned long long) * 5);
        cuda_check(cudaMemsetAsync(ctr, 0, sizeof(unsigned long long) * 5, s), "memset");
    }
    auto *ticket = (unsigned *)c->ensure(c->ticket, sizeof(unsigned));
    auto *bad = (int *)c->ensure(c->bad, sizeof(int) * nlos);
    auto *nbad = (int *)c->ensure(c->nbad, sizeof(int));
    auto *err = (unsigned *)c->ensure(c->err, sizeof(unsigned));
    cuda_check(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s), "memset");
    cuda_check(cudaMemsetAsync(nbad, 0, sizeof(int), s), "memset");
    cuda_check(cudaMemsetAsync(err, 0, sizeof(unsigned), s), "memset");
    launch_deposit(lp, c->tables, p, pl, (const int *)c->line_order.p, nlos, out, ticket, bad,
                   nbad, err, gacc, ctr, cfg, s);
    c->stats.gpu_launches++;
    cuda_check(cudaGetLastError(), "deposit launch");
    int h_nbad = 0;
    unsigned h_err = 0;
    cuda_check(cudaMemcpyAsync(&h_nbad, nbad, sizeof(int), cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaStreamSynchronize(s), "deposit");
    if (h_nbad > 0) {
        launch_deposit_fallback(lp, c->tables, p, pl, bad, h_nbad, out, err, s);
        c->stats.gpu_launches++;
        cuda_check(cudaGetLastError(), "fallback launch");
    }
    c->stats.fallback_lines = h_nbad;
    cuda_check(cudaEventRecord(c->ev[3], s), "event");
    cuda_check(cudaMemcpyAsync(&h_err, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s), "read");
    cuda_check(cudaStreamSynchronize(s), "deposit");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
    c->stats.ms_deposit = ms;
    if (count) {
        unsigned long long h_ctr[5];
        cuda_check(cudaMemcpy(h_ctr, ctr, sizeof h_ctr, cudaMemcpyDeviceToHost), "read counters");
        c->stats.evals_core = (int64_t)h_ctr[0];
        c->stats.evals_wing = (int64_t)h_ctr[1];
        c->stats.evals_other = (int64_t)h_ctr[2];
        c->stats.pixels = (int64_t)h_ctr[3];
        c->stats.evals_wing_multipole = (int64_t)h_ctr[4];
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

// Launch configuration of the deposit for this call.
DepositLaunch deposit_config(fsg_context *c, const LineParams &lp, const fsg_options *opt)
{
    DepositLaunch cfg{};
    cfg.precision = opt ? opt->precision : FSG_PREC_FP64;
    if (cfg.precision != FSG_PREC_FP64 && cfg.precision != FSG_PREC_FP32)
        fail(FSG_ERR_VALUE, "unknown precision %d", cfg.precision);
    const int tmax = cfg.precision == FSG_PREC_FP64 ? 256 : 512;
    cfg.threads = (opt && opt->threads > 0) ? opt->threads : tmax;
    if (cfg.threads % 32 || cfg.threads > tmax)
        fail(FSG_ERR_VALUE, "threads must be a multiple of 32 and at most %d", tmax);
    deposit_plan(cfg, lp.compute_tau, lp.nbins);
    cfg.persistent = (opt && opt->persistent >= 0) ? opt->persistent
                                                    : (cfg.precision == FSG_PREC_FP32 ? 1 : 0);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const int per_sm = std::max(1, deposit_resident_ctas(cfg, lp.compute_tau, lp.nbins));
    cfg.grid = std::min(c->nlos, sms * per_sm);
    return cfg;
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
    for (const LineParams &lp : lps)
        cfgs.push_back(deposit_config(c, lp, opt));
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
    c->stats.gpu_launches += 2 * (int64_t)lps.size();
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
}

void run_interpolate(fsg_context *c, int compute_tau, int nbins, int kernel, double box,
                     double velfac, double lambda, double gamma, double fosc, double amumass,
                     double tautail, const Particles &p, const int32_t *axis, const double *cofm,
                     int32_t nlos, double *out, const fsg_options *opt)
{
    cuda_check(cudaSetDevice(c->device), "cudaSetDevice");
    build_tables(c, axis, cofm, nlos, box);
    search_pairs(c, p, nlos);
    LineParams lp = make_line_params(compute_tau, nbins, kernel, box, velfac, lambda, gamma, fosc,
                                     amumass, tautail);
    deposit(c, lp, p, out, opt);
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
        validate_common(nbins, kernel, box, npart, nlos, axis, cofm);
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
        validate_common(nbins, kernel, box, npart, nlos, axis, cofm);
        int dev = 0;
        cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
        if (dev < 0 || dev >= 64)
            fail(FSG_ERR_VALUE, "device ordinal %d out of range", dev);
        fsg_context *c;
        std::lock_guard<std::mutex> lock(g_default_mu);
        if (!g_default[dev]) {
            c = new fsg_context();
            try {
                ctx_init(c, dev);
            } catch (...) {
                delete c;
                throw;
            }
            g_default[dev] = c;
        }
        c = g_default[dev];
        cudaStream_t s = c->stream;
        const size_t n3 = sizeof(float) * 3 * (size_t)npart, n1 = sizeof(float) * (size_t)npart;
        auto up = [&](DevBuf &b, const void *src, size_t bytes) -> const float * {
            void *d = c->ensure(b, bytes);
            if (bytes)
                cuda_check(cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, s), "H2D");
            return (const float *)d;
        };
        Particles p;
        p.n = npart;
        p.pos = up(c->pos, pos, n3);
        p.dens = up(c->dens, dens, n1);
        p.hh = up(c->hh, h, n1);
        p.vel = compute_tau ? up(c->vel, vel, n3) : nullptr;
        p.temp = compute_tau ? up(c->temp, temp, n1) : nullptr;
        const size_t nout = sizeof(double) * (size_t)nlos * (size_t)(nbins > 0 ? nbins : 0);
        double *dout = (double *)c->ensure(c->out, nout);
        run_interpolate(c, compute_tau, nbins, kernel, box, velfac, lambda, gamma, fosc, amumass,
                        tautail, p, axis, cofm, nlos, dout, opt);
        if (nout)
            cuda_check(cudaMemcpyAsync(out, dout, nout, cudaMemcpyDeviceToHost, s), "D2H");
        cuda_check(cudaStreamSynchronize(s), "D2H");
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

int fsg_tau_backward_device(fsg_context *ctx, int nbins, int kernel, double box, double velfac,
                            double atime, double lambda, double gamma, double fosc,
                            double amumass, double tautail, const float *pos, const float *vel,
                            const float *dens, const float *temp, const float *h, int64_t npart,
                            const int32_t *axis, const double *cofm, int32_t nlos,
                            const double *grad_tau, float *grad_dens, float *grad_temp,
                            float *grad_vel, char *errbuf, size_t errlen)
{
    (void)atime;
    try {
        if (!ctx)
            fail(FSG_ERR_VALUE, "ctx is NULL");
        validate_common(nbins, kernel, box, npart, nlos, axis, cofm);
        if (!grad_tau || !grad_dens || !grad_temp || !grad_vel)
            fail(FSG_ERR_VALUE, "gradient buffers must not be NULL");
        cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
        build_tables(ctx, axis, cofm, nlos, box);
        Particles p{pos, vel, dens, temp, h, (long long)npart};
        search_pairs(ctx, p, nlos);
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
