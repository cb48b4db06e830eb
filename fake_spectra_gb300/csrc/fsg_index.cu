// Sightline-particle search on the GPU: the replacement for the reference
// IndexTable (fake_spectra/index_table.cpp:7-150).
//
// One thread per particle enumerates, for every axis group of sightlines, the
// transverse grid cells that can hold a sightline within its smoothing length
// (periodic, minimum image, plus a safety margin), and decides every
// candidate by the reference's accept predicate:
//   * the first-coordinate window [ffm, ffp) of index_table.cpp:89-113,
//     computed in float and compared against the double multimap key, with
//     the periodic wrap that splits the range in two;
//   * second_close, index_table.cpp:52-68 (float window, double compare);
//   * calc_dr2, index_table.cpp:70-87 (double minimum-image distance), and the
//     accept test dr2 <= hh*hh with hh*hh a float product (index_table.cpp:45).
// Most candidates are decided by float bounds that imply the predicate's
// answer (see accept()); the rest get the reference's float/double
// arithmetic operation by operation, with no FMA contraction (explicit
// __fadd_rn / __dmul_rn / __dadd_rn).  dr2 of every pair is then computed by
// pair_dr2_kernel with the same calc_dr2.  The cell walk is only a superset
// generator, so the accepted pair set and every dr2 bit equal the
// reference's.  Degenerate smoothing lengths are resolved exactly (see
// for_each_pair).
//
// Particles are first ordered by a 3-D spatial cell (counting sort), so that
// the 32 lanes of a warp are neighbours: they read the same cells and
// sightlines (broadcast loads, L1 hits) and share atomics on the same
// sightline counters.  Two passes: count (per-sightline totals) and emit (one
// slot per pair, consecutive within a warp's group).
#include "fsg_internal.cuh"

namespace fsg {

namespace {

struct Window {   // first-coordinate window of one table for one particle
    float ffm, ffp;
    bool nowrap;
};

__device__ __forceinline__ Window make_window(float first, float hh, const LineTables &t)
{
    Window w;
    const double box = t.box;
    float ffp = __fadd_rn(first, hh);
    if (ffp >= t.box_up)   // (double)ffp > box
        ffp = (float)__dsub_rn((double)ffp, box);
    float ffm = __fsub_rn(first, hh);
    if (ffm < 0.0f)
        ffm = (float)__dadd_rn((double)ffm, box);
    w.ffm = ffm;
    w.ffp = ffp;
    w.nowrap = (ffm <= ffp);
    return w;
}

__device__ __forceinline__ bool in_window(const Window &w, double key)
{
    // lower_bound(ffm) .. lower_bound(ffp) over the sorted keys (index_table.cpp:102-112)
    if (w.nowrap)
        return ((double)w.ffm <= key) && (key < (double)w.ffp);
    return (key < (double)w.ffp) || (key >= (double)w.ffm);
}

__device__ __forceinline__ bool second_close(float second, double lproj2, float hh, double box)
{
    float ffp = __fadd_rn(second, hh);
    if ((double)ffp > box)
        if (lproj2 < __dsub_rn((double)ffp, box))
            return true;
    float ffm = __fsub_rn(second, hh);
    if (ffm < 0.0f)
        if (lproj2 > __dadd_rn((double)ffm, box))
            return true;
    return (lproj2 > (double)ffm) && (lproj2 < (double)ffp);
}

__device__ __forceinline__ double calc_dr2(double d1, double d2, double box)
{
    const double half = 0.5 * box;
    double dr = fabs(d1);
    if (dr > half)
        dr = __dsub_rn(box, dr);
    double dr2 = __dmul_rn(dr, dr);
    dr = fabs(d2);
    if (dr > half)
        dr = __dsub_rn(box, dr);
    return __dadd_rn(dr2, __dmul_rn(dr, dr));
}

// Sufficient float conditions for the window tests.  Rounding to float is
// monotone, so for a float bound b and the float copy k = rn(key):
// k > b implies key > b and k < b implies key < b.
__device__ __forceinline__ bool window_holds(const Window &w, float k)
{
    return w.nowrap ? (k > w.ffm && k < w.ffp) : (k < w.ffp || k > w.ffm);
}

__device__ __forceinline__ bool second_holds(float second, float k, float hh)
{
    return k > __fsub_rn(second, hh) && k < __fadd_rn(second, hh);
}

// The reference predicate for (particle, line).  `first` is the particle's
// coordinate for the table the line is in; pos3 the particle position.
// Most candidates are decided in FP32 (FP64 runs at 1/64 of the FP32 rate on
// this GPU):
//   * reject: the float minimum-image distance exceeds hh by more than its
//     error bound (pre_eps, 4 ulp of the box), a strict superset test;
//   * accept: the line's float copies lie within half an ulp of the box of the
//     double values (pack.w), both distances stay below 0.49 box (no minimum
//     image in calc_dr2), the upper bound of dr2 with every rounding of the
//     float and double arithmetic (relative 2e-7, absolute pre_eps per
//     coordinate) is below hh*hh by a relative 5e-6, and both windows hold by
//     window_holds/second_holds, so the exact test below would return true.
// The rest (the thin shell |dr| ~ hh, sightlines near the periodic boundary,
// coordinates outside the box) takes the exact FP64 test.  The accepted set is
// the reference's; dr2 itself is computed by pair_dr2_kernel.
__device__ __forceinline__ bool accept(const LineTables &t, int line, const Window &w,
                                       float first, const float *pos3, float hh)
{
    const float4 pk = __ldg(&t.pack[line]);
    const int ax = __float_as_int(pk.z);
    const float second = (ax == 3) ? pos3[1] : pos3[2];
    {
        const float d1 = fabsf(first - pk.x), d2 = fabsf(second - pk.y);
        if (d1 <= t.box_f && d2 <= t.box_f && hh > 0.0f) {
            const float m1 = fminf(d1, t.box_f - d1), m2 = fminf(d2, t.box_f - d2);
            const float lim = hh + t.pre_eps;
            if (fmaf(m1, m1, m2 * m2) > lim * lim * 1.000001f)
                return false;
            if (pk.w != 0.0f) {
                const float a = fmaf(d1, 1.0000005f, t.pre_eps);
                const float b = fmaf(d2, 1.0000005f, t.pre_eps);
                const float half_in = 0.49f * t.box_f;
                if (a <= half_in && b <= half_in &&
                    fmaf(a, a, __fmul_rn(b, b)) <= __fmul_rn(__fmul_rn(hh, hh), 0.999995f) &&
                    window_holds(w, pk.x) && second_holds(second, pk.y, hh))
                    return true;
            }
        }
    }
    const double key = t.key[line];
    if (!in_window(w, key))
        return false;
    const double lproj2 = t.second[line];
    if (!second_close(second, lproj2, hh, t.box))
        return false;
    const double dr2 = calc_dr2(__dsub_rn((double)first, key), __dsub_rn((double)second, lproj2),
                                t.box);
    return dr2 <= (double)__fmul_rn(hh, hh);
}

// Coordinates of the particle in an axis group: (table first, cell second).
__device__ __forceinline__ void group_coords(int g, const float *pos3, float *first, float *second)
{
    if (g == 0) {          // axis 1: keyed by y, filtered on z
        *first = pos3[1];
        *second = pos3[2];
    } else if (g == 1) {   // axis 2: keyed by x, filtered on z
        *first = pos3[0];
        *second = pos3[2];
    } else {               // axis 3: keyed by x, filtered on y
        *first = pos3[0];
        *second = pos3[1];
    }
}

// Cell range [c0, c0+cn) (mod nc) covering coordinate c +- r, in float: the
// rounding of (c -+ r) * inv_cw is below 1e-3 of a cell for |c| <= 4 box and
// nc <= 1024, inside the margin the caller adds to r.  Coordinates further
// out (or a range as wide as the grid) take every cell.
__device__ __forceinline__ void cell_range(float c, float r, const LineGroup &G, float box_f,
                                           int *c0, int *cn)
{
    const float lo = floorf((c - r) * G.inv_cw_f);
    const float hi = floorf((c + r) * G.inv_cw_f);
    const float n = hi - lo + 1.0f;
    if (!(fabsf(c) <= 4.0f * box_f) || !(n < (float)G.nc)) {
        *c0 = 0;
        *cn = G.nc;
        return;
    }
    int l = (int)lo % G.nc;   // |lo| <= 4.5 nc + 1 here
    if (l < 0)
        l += G.nc;
    *c0 = l;
    *cn = (int)n;
}

__device__ __forceinline__ bool in_box(float c, double box)
{
    return c >= 0.0f && (double)c <= box;
}

template <class Visit>
__device__ __forceinline__ void for_each_pair(const LineTables &t, const float *pos3, float hh,
                                              Visit &&visit)
{
    if (isnan(hh))
        return;   // dr2 <= NaN is never true
    Window wmain, wxx;
    if (t.n_main)
        wmain = make_window(pos3[0], hh, t);
    if (t.n_xx)
        wxx = make_window(pos3[1], hh, t);
    if (!(hh > 0.0f) || isinf(hh)) {
        // hh <= 0 with every coordinate inside [0, box]: the first-coordinate
        // window is empty (hh == 0) or second_close needs ffm < lproj2 < ffp with
        // ffm > ffp (hh < 0), so no sightline is accepted.  hh = -inf empties the
        // window.  Anything else (coordinates outside the box, hh = +inf) tests
        // every sightline with the exact predicate.
        if (hh == -INFINITY)
            return;
        if (hh <= 0.0f && in_box(pos3[0], t.box) && in_box(pos3[1], t.box) &&
            in_box(pos3[2], t.box))
            return;
        for (int l = 0; l < t.nlos; l++) {
            const bool xx = (t.axis[l] == 1);
            if (accept(t, l, xx ? wxx : wmain, xx ? pos3[1] : pos3[0], pos3, hh))
                visit(l);
        }
        return;
    }
    // Safety margin: relative 1e-5 of hh plus 2e-2 of a cell covers every
    // rounding in the accept test, in the float cell range and in the cell
    // assignment of the lines.
    const float reach = hh * 1.00001f;
#pragma unroll 1
    for (int g = 0; g < 3; g++) {
        const LineGroup &G = t.g[g];
        if (G.nlines == 0)
            continue;
        float f, s;
        group_coords(g, pos3, &f, &s);
        if (!isfinite(f) || !isfinite(s))
            continue;   // with finite hh, a non-finite coordinate never passes dr2 <= hh^2
        const float r = fmaf(0.02f, G.cw_f, reach);
        int a0, an, b0, bn;
        cell_range(f, r, G, t.box_f, &a0, &an);
        cell_range(s, r, G, t.box_f, &b0, &bn);
        const Window &w = (g == 0) ? wxx : wmain;
        for (int ia = 0; ia < an; ia++) {
            int ca = a0 + ia;
            if (ca >= G.nc)
                ca -= G.nc;
            for (int ib = 0; ib < bn; ib++) {
                int cb = b0 + ib;
                if (cb >= G.nc)
                    cb -= G.nc;
                const int cell = ca * G.nc + cb;
                const int e1 = G.cell_start[cell + 1];
                for (int e = G.cell_start[cell]; e < e1; e++) {
                    const int l = G.cell_line[e];
                    if (accept(t, l, w, f, pos3, hh))
                        visit(l);
                }
            }
        }
    }
}

__device__ __forceinline__ void load_particle(const Particles &p, long long i, float *pos3,
                                              float *hh)
{
    pos3[0] = __ldg(&p.pos[3 * i]);
    pos3[1] = __ldg(&p.pos[3 * i + 1]);
    pos3[2] = __ldg(&p.pos[3 * i + 2]);
    *hh = __ldg(&p.hh[i]);
}

// Lanes that meet the same sightline together share one atomic (the particles
// of a warp are spatial neighbours once sorted, so they often do).
__global__ void count_pairs_kernel(LineTables t, Particles p, const int *perm,
                                   unsigned long long *line_count, unsigned char *part_flag)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < p.n; k += stride) {
        const long long i = perm ? (long long)perm[k] : k;
        float pos3[3], hh;
        load_particle(p, i, pos3, &hh);
        int found = 0;
        for_each_pair(t, pos3, hh, [&](int l) {
            const unsigned am = __activemask();
            const unsigned g = __match_any_sync(am, l);
            if (lane == __ffs(g) - 1)
                atomicAdd(&line_count[l], (unsigned long long)__popc(g));
            found = 1;
        });
        if (part_flag)
            part_flag[i] = (unsigned char)found;
    }
}

__global__ void emit_pairs_kernel(LineTables t, Particles p, const int *perm, const long long *off,
                                  unsigned long long *cursor, int *part, unsigned *dev_err)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < p.n; k += stride) {
        const long long i = perm ? (long long)perm[k] : k;
        float pos3[3], hh;
        load_particle(p, i, pos3, &hh);
        for_each_pair(t, pos3, hh, [&](int l) {
            const unsigned am = __activemask();
            const unsigned g = __match_any_sync(am, l);
            const int leader = __ffs(g) - 1;
            unsigned long long base = 0;
            if (lane == leader)
                base = atomicAdd(&cursor[l], (unsigned long long)__popc(g));
            base = __shfl_sync(g, base, leader);
            const long long slot = off[l] + (long long)base + __popc(g & below);
            if (slot < off[l + 1])
                part[slot] = (int)i;
            else
                atomicOr(dev_err, (unsigned)DEVERR_PAIR_SLOT);
        });
    }
}

// dr2 of every pair (calc_dr2, index_table.cpp:70-87): one CTA per sightline,
// its pairs across the threads, so the FP64 arithmetic runs with full warps.
// The emit pass accepted these pairs with the same function of the same
// values.  A slot the emit pass left unwritten (a count mismatch, flagged by
// check_emit_kernel) holds no particle index to trust: it is range-checked.
__global__ void __launch_bounds__(256) pair_dr2_kernel(LineTables t, const float *pos,
                                                       long long npart, const long long *off,
                                                       const int *part, double *dr2,
                                                       unsigned *dev_err)
{
    const int l = blockIdx.x;
    const int ax = t.axis[l];
    const double key = t.key[l], lproj2 = t.second[l];
    const int fi = (ax == 1) ? 1 : 0, si = (ax == 3) ? 1 : 2;
    const long long e1 = off[l + 1];
    for (long long e = off[l] + threadIdx.x; e < e1; e += blockDim.x) {
        const int i = part[e];
        if (i < 0 || (long long)i >= npart) {
            atomicOr(dev_err, (unsigned)DEVERR_PAIR_INDEX);
            dr2[e] = 0.0;
            continue;
        }
        const float f = __ldg(&pos[3 * (size_t)i + fi]), s = __ldg(&pos[3 * (size_t)i + si]);
        dr2[e] = calc_dr2(__dsub_rn((double)f, key), __dsub_rn((double)s, lproj2), t.box);
    }
}

// ------------------------------------------------------ particle ordering
__global__ void cell_hist_kernel(Particles p, float scale, int G, unsigned *key, unsigned *hist)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const float gmax = (float)(G - 1);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += stride) {
        // fmaxf/fminf map NaN to 0 and clamp out-of-box positions to the edge cells
        const float fx = fminf(fmaxf(floorf(__ldg(&p.pos[3 * i]) * scale), 0.f), gmax);
        const float fy = fminf(fmaxf(floorf(__ldg(&p.pos[3 * i + 1]) * scale), 0.f), gmax);
        const float fz = fminf(fmaxf(floorf(__ldg(&p.pos[3 * i + 2]) * scale), 0.f), gmax);
        const unsigned c = ((unsigned)fx * G + (unsigned)fy) * G + (unsigned)fz;
        key[i] = c;
        atomicAdd(&hist[c], 1u);
    }
}

// Exclusive scan, three kernels: per-1024-thread block (2048 elements) scans
// with block totals, a single-block scan of the totals, and the offsets added back.
constexpr int SCAN_T = 1024, SCAN_E = 2 * SCAN_T;

__device__ __forceinline__ unsigned block_exclusive_scan(unsigned *buf)
{
    // Blelloch scan of SCAN_E elements in shared memory; returns the total
    const int t = threadIdx.x;
    int off = 1;
    for (int d = SCAN_E >> 1; d > 0; d >>= 1) {
        __syncthreads();
        if (t < d) {
            const int ai = off * (2 * t + 1) - 1, bi = off * (2 * t + 2) - 1;
            buf[bi] += buf[ai];
        }
        off <<= 1;
    }
    __syncthreads();
    const unsigned total = buf[SCAN_E - 1];
    __syncthreads();
    if (t == 0)
        buf[SCAN_E - 1] = 0;
    for (int d = 1; d < SCAN_E; d <<= 1) {
        off >>= 1;
        __syncthreads();
        if (t < d) {
            const int ai = off * (2 * t + 1) - 1, bi = off * (2 * t + 2) - 1;
            const unsigned v = buf[ai];
            buf[ai] = buf[bi];
            buf[bi] += v;
        }
    }
    __syncthreads();
    return total;
}

__global__ void __launch_bounds__(SCAN_T) scan_blocks_kernel(const unsigned *in, unsigned *out,
                                                            unsigned *sums, int n)
{
    __shared__ unsigned buf[SCAN_E];
    const int base = blockIdx.x * SCAN_E;
    for (int k = threadIdx.x; k < SCAN_E; k += SCAN_T)
        buf[k] = (base + k < n) ? in[base + k] : 0u;
    const unsigned total = block_exclusive_scan(buf);
    for (int k = threadIdx.x; k < SCAN_E; k += SCAN_T)
        if (base + k < n)
            out[base + k] = buf[k];
    if (threadIdx.x == 0)
        sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_T) scan_sums_kernel(unsigned *sums, int nb)
{
    // nb <= SCAN_E (G <= 128)
    __shared__ unsigned buf[SCAN_E];
    for (int k = threadIdx.x; k < SCAN_E; k += SCAN_T)
        buf[k] = (k < nb) ? sums[k] : 0u;
    block_exclusive_scan(buf);
    for (int k = threadIdx.x; k < nb; k += SCAN_T)
        sums[k] = buf[k];
}

__global__ void add_sums_kernel(unsigned *out, const unsigned *sums, int n)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n)
        out[k] += sums[k / SCAN_E];
}

__global__ void cell_scatter_kernel(const unsigned *key, unsigned *cursor, int *perm, long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned slot = atomicAdd(&cursor[key[i]], 1u);
        perm[slot] = (int)i;
    }
}

// _near_lines (py_module.cpp:25-99): flag[i] = 1 when particle i is within
// its smoothing length of any sightline (IndexTable::get_near_lines non-empty,
// index_table.cpp:117-127), by the same predicate as the pair search.
__global__ void flag_near_kernel(LineTables t, Particles p, const int *perm, unsigned char *flag)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < p.n; k += stride) {
        const long long i = perm ? (long long)perm[k] : k;
        float pos3[3], hh;
        load_particle(p, i, pos3, &hh);
        int found = 0;
        for_each_pair(t, pos3, hh, [&](int) { found = 1; });
        flag[i] = (unsigned char)found;
    }
}

// Ordered compaction of the flags into ascending particle indices: each
// 256-thread block owns a tile of FLAG_TILE particles, 16 consecutive ones per
// thread; pass 1 counts the tile, the tile counts are scanned, pass 2 writes.
constexpr int FLAG_THREADS = 256, FLAG_PER_THREAD = 16, FLAG_TILE = FLAG_THREADS * FLAG_PER_THREAD;

__device__ __forceinline__ int thread_flag_count(const unsigned char *flag, long long n,
                                                 long long first)
{
    int c = 0;
#pragma unroll
    for (int q = 0; q < FLAG_PER_THREAD; q++)
        c += (first + q < n) ? (int)(flag[first + q] != 0) : 0;
    return c;
}

__global__ void __launch_bounds__(FLAG_THREADS) flag_count_kernel(const unsigned char *flag,
                                                                  long long n, unsigned *tile_count)
{
    __shared__ int red[FLAG_THREADS / 32];
    const long long first = (long long)blockIdx.x * FLAG_TILE + (long long)threadIdx.x * FLAG_PER_THREAD;
    int c = thread_flag_count(flag, n, first);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < FLAG_THREADS / 32; w++)
            t += red[w];
        tile_count[blockIdx.x] = (unsigned)t;
    }
}

__global__ void __launch_bounds__(FLAG_THREADS) flag_scatter_kernel(const unsigned char *flag,
                                                                    long long n,
                                                                    const unsigned *tile_start,
                                                                    int *out)
{
    __shared__ int wsum[FLAG_THREADS / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long first = (long long)blockIdx.x * FLAG_TILE + (long long)threadIdx.x * FLAG_PER_THREAD;
    const int c = thread_flag_count(flag, n, first);
    // exclusive scan of the per-thread counts across the block
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
            incl += v;
    }
    if (lane == 31)
        wsum[warp] = incl;
    __syncthreads();
    int base = 0;
    for (int w = 0; w < warp; w++)
        base += wsum[w];
    long long slot = (long long)tile_start[blockIdx.x] + base + (incl - c);
#pragma unroll
    for (int q = 0; q < FLAG_PER_THREAD; q++) {
        const long long i = first + q;
        if (i < n && flag[i])
            out[slot++] = (int)i;
    }
}

__global__ void check_emit_kernel(const unsigned long long *line_count,
                                  const unsigned long long *cursor, int nlos, unsigned *dev_err)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l < nlos && cursor[l] != line_count[l])
        atomicOr(dev_err, (unsigned)DEVERR_PAIR_COUNT);
}

int search_grid(long long n)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long want = (n + 255) / 256;
    long long cap = (long long)sms * 8;
    if (want > cap)
        want = cap;
    return (int)(want > 0 ? want : 1);
}

}  // namespace

void launch_count_pairs(const LineTables &t, const Particles &p, const int *perm,
                        unsigned long long *line_count, unsigned char *part_flag, cudaStream_t s)
{
    if (p.n == 0)
        return;
    count_pairs_kernel<<<search_grid(p.n), 256, 0, s>>>(t, p, perm, line_count, part_flag);
}

void launch_emit_pairs(const LineTables &t, const Particles &p, const int *perm,
                       const long long *off, unsigned long long *cursor, int *part, double *dr2,
                       unsigned *dev_err, cudaStream_t s)
{
    if (p.n == 0)
        return;
    emit_pairs_kernel<<<search_grid(p.n), 256, 0, s>>>(t, p, perm, off, cursor, part, dev_err);
    if (t.nlos > 0)
        pair_dr2_kernel<<<t.nlos, 256, 0, s>>>(t, p.pos, p.n, off, part, dr2, dev_err);
}

void launch_check_emit(const unsigned long long *line_count, const unsigned long long *cursor,
                       int nlos, unsigned *dev_err, cudaStream_t s)
{
    if (nlos <= 0)
        return;
    check_emit_kernel<<<(nlos + 255) / 256, 256, 0, s>>>(line_count, cursor, nlos, dev_err);
}

void launch_flag_near(const LineTables &t, const Particles &p, const int *perm,
                      unsigned char *flag, cudaStream_t s)
{
    if (p.n == 0)
        return;
    flag_near_kernel<<<search_grid(p.n), 256, 0, s>>>(t, p, perm, flag);
}

long long flag_tiles(long long n) { return (n + FLAG_TILE - 1) / FLAG_TILE; }

void launch_flag_count(const unsigned char *flag, long long n, unsigned *tile_count,
                       cudaStream_t s)
{
    const long long nt = flag_tiles(n);
    if (nt > 0)
        flag_count_kernel<<<(unsigned)nt, FLAG_THREADS, 0, s>>>(flag, n, tile_count);
}

void launch_exclusive_scan(const unsigned *in, unsigned *out, unsigned *sums, int n,
                           cudaStream_t s)
{
    if (n <= 0)
        return;
    const int nb = (n + SCAN_E - 1) / SCAN_E;
    scan_blocks_kernel<<<nb, SCAN_T, 0, s>>>(in, out, sums, n);
    scan_sums_kernel<<<1, SCAN_T, 0, s>>>(sums, nb);
    add_sums_kernel<<<(n + 255) / 256, 256, 0, s>>>(out, sums, n);
}

void launch_flag_scatter(const unsigned char *flag, long long n, const unsigned *tile_start,
                         int *out, cudaStream_t s)
{
    const long long nt = flag_tiles(n);
    if (nt > 0)
        flag_scatter_kernel<<<(unsigned)nt, FLAG_THREADS, 0, s>>>(flag, n, tile_start, out);
}

// ~64 particles per cell, at most 128^3 cells (the totals then fit one scan block)
int sort_grid_side(long long n)
{
    int G = (int)cbrt((double)n / 64.0);
    return G < 1 ? 1 : (G > 128 ? 128 : G);
}

void launch_particle_order(const Particles &p, double box, int G, unsigned *key, unsigned *hist,
                           unsigned *start, unsigned *sums, int *perm, cudaStream_t s)
{
    if (p.n == 0)
        return;
    const int M = G * G * G;
    cudaMemsetAsync(hist, 0, sizeof(unsigned) * M, s);
    cell_hist_kernel<<<search_grid(p.n), 256, 0, s>>>(p, (float)(G / box), G, key, hist);
    const int nb = (M + SCAN_E - 1) / SCAN_E;
    scan_blocks_kernel<<<nb, SCAN_T, 0, s>>>(hist, start, sums, M);
    scan_sums_kernel<<<1, SCAN_T, 0, s>>>(sums, nb);
    add_sums_kernel<<<(M + 255) / 256, 256, 0, s>>>(start, sums, M);
    // the scan output is consumed as the scatter cursor
    cell_scatter_kernel<<<search_grid(p.n), 256, 0, s>>>(key, start, perm, p.n);
}

}  // namespace fsg
