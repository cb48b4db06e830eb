// Flux statistics of optical depths still resident in HBM: the mean-flux
// rescaling (fake_spectra/py_module.cpp:235-282, get_mean_flux_scale /
// Py_mean_flux) and the flux PDF (fake_spectra/fluxstatistics.py:42-51); the
// 1-D flux power spectrum is in fsg_power.cu.
//
// Each pass reads tau once.  Sums are deterministic: every block reduces a
// fixed contiguous range in a fixed order and a second pass adds the block
// partials in order, so a result does not depend on scheduling.
#include <cmath>

#include "fsg_fexp.cuh"
#include "fsg_internal.cuh"

namespace fsg {

namespace {

constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 1024;   // fixed: the summation order does not depend on the GPU

// Fixed-order block sum of one double per thread (tree over warps).
__device__ __forceinline__ double block_sum_ordered(double v, double *scratch)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        scratch[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < RED_THREADS / 32; w++)
            t += scratch[w];
    __syncthreads();
    return t;   // valid in thread 0
}

// The block's contiguous range of [0, n)
__device__ __forceinline__ void block_range(long long n, long long &lo, long long &hi)
{
    const long long per = (n + gridDim.x - 1) / gridDim.x;
    lo = (long long)blockIdx.x * per;
    hi = lo + per < n ? lo + per : n;
}

// Newton-Raphson on the device (py_module.cpp:242-258): state[0] = the scale
// of the last pass, state[1] = the next scale, state[2] = 1 once converged,
// state[3] = passes.  A pass reads the scale from state[1]; once state[2] is
// set, queued passes and updates return at once, so the host can queue several
// iterations between reads.
__global__ void __launch_bounds__(RED_THREADS)
    flux_moments_dev_kernel(const double *tau, long long n, const double *state, double thresh,
                            const double *etab, double *part)
{
    __shared__ double scratch[RED_THREADS / 32];
    if (state[2] != 0.0)
        return;
    const double scale = state[1];
    long long lo, hi;
    block_range(n, lo, hi);
    double f = 0.0, tf = 0.0;
    long long cnt = 0;   // counted in integers: exact, and off the FP64 pipe
    // t > thresh on the bit patterns when thresh has its sign bit clear (the
    // patterns of non-negative doubles order like the values; NaN compares
    // false as in FP64), else in FP64
    const long long thr_bits = __double_as_longlong(thresh);
    const bool int_cmp = thr_bits >= 0;
    const double nscale = -scale;
    for (long long i = lo + threadIdx.x; i < hi; i += RED_THREADS) {
        const double t = tau[i];
        const long long tb = __double_as_longlong(t);
        const bool above = int_cmp ? (tb > thr_bits && (tb & 0x7fffffffffffffffll) <=
                                                           0x7ff0000000000000ll)
                                   : t > thresh;
        if (above)
            continue;
        const double e = fexp(nscale * t, etab);
        f += e;
        tf = fma(e, t, tf);
        cnt++;
    }
    f = block_sum_ordered(f, scratch);
    tf = block_sum_ordered(tf, scratch);
    const double cntd = block_sum_ordered((double)cnt, scratch);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = f;
        part[3 * blockIdx.x + 1] = tf;
        part[3 * blockIdx.x + 2] = cntd;
    }
}

// Fixed-order sum of the `width`-strided block partials' component c by one
// warp: lane l adds blocks l, l + 32, ... in order, then an xor butterfly
// (each level adds the same two values in every lane, so all lanes agree).
__device__ __forceinline__ double warp_partial_sum(const double *part, int nblocks, int width,
                                                  int c)
{
    double t = 0.0;
    for (int b = threadIdx.x & 31; b < nblocks; b += 32)
        t += part[(size_t)b * width + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// The fixed-order sums of a pass's block partials and the Newton update (one warp).
__global__ void newton_update_kernel(const double *part, int nblocks, double mfd, double tol,
                                     double *state)
{
    if (state[2] != 0.0)
        return;
    const double f = warp_partial_sum(part, nblocks, 3, 0);
    const double tf = warp_partial_sum(part, nblocks, 3, 1);
    const double cnt = warp_partial_sum(part, nblocks, 3, 2);
    if (threadIdx.x != 0)
        return;
    const double scale = state[1];
    double newscale = scale + (f - mfd * cnt) / tf;
    if (newscale <= 0)
        newscale = 1e-10;
    state[0] = scale;
    state[1] = newscale;
    state[3] += 1.0;
    if (!(fabs(newscale - scale) > tol * newscale))
        state[2] = 1.0;
}

// Sum of exp(-scale tau) over all pixels (np.mean(np.exp(-tau)) with scale 1).
__global__ void __launch_bounds__(RED_THREADS) flux_sum_kernel(const double *tau, long long n,
                                                               double scale, const double *etab,
                                                               double *part)
{
    __shared__ double scratch[RED_THREADS / 32];
    long long lo, hi;
    block_range(n, lo, hi);
    double f = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += RED_THREADS)
        f += fexp(-scale * tau[i], etab);
    f = block_sum_ordered(f, scratch);
    if (threadIdx.x == 0)
        part[blockIdx.x] = f;
}

// Fixed-order sums of `width`-strided block partials (one warp).
__global__ void partial_sum_kernel(const double *part, int nblocks, int width, double *out)
{
    for (int c = 0; c < width; c++) {
        const double t = warp_partial_sum(part, nblocks, width, c);
        if (threadIdx.x == 0)
            out[c] = t;
    }
}

// np.histogram with explicit edges (numpy's sorted-search rule): bin j holds
// e_j <= x < e_{j+1}, the last bin also x == e_last; values outside
// [e_0, e_last] and NaN are not counted.  x = exp(-scale tau).
//
// The exponential is taken in FP32 (this GPU runs FP64 at 1/64 of the FP32
// rate): y = scale tau from float copies of both, x32 = expf(-y).  Relative to
// the exact exp(-scale tau), x32 is off by at most |y| 2^-21 (the float copies
// and the product, each within one float ulp, carried through the exponent)
// plus 2^-21 (expf's 2-ulp bound, doubled for margin), and by at most 2^-148
// absolutely where it underflows.  A pixel whose x32 is farther than that from
// every edge lies in the same bin as the FP64 value; the rest (near an edge,
// outside the bins, NaN) are decided with the FP64 exponential and numpy's
// comparisons, so the counts equal numpy's.
//
// Bins are counted in 32-bit per-warp private histograms in shared memory
// (nb <= FLUX_WARP_BINS; a warp never counts 2^32 pixels: the grid-stride loop
// gives each warp at most n / (grid warps) pixels, checked on the host), merged
// into the 64-bit global counts once per block.  Larger nb: one per-block
// 64-bit histogram.
constexpr int FLUX_HIST_THREADS = 256;
constexpr int FLUX_WARP_BINS = 256;

// float copy of a double by truncating its mantissa (integer operations only;
// within one float ulp below |d|): 0 for |d| < 2^-126, inf beyond the float range.
__device__ __forceinline__ float trunc_to_float(double d)
{
    const long long b = __double_as_longlong(d);
    const unsigned sign = (unsigned)((unsigned long long)b >> 32) & 0x80000000u;
    const int e11 = (int)((b >> 52) & 0x7ff);
    if (e11 == 0x7ff)
        return __int_as_float((int)(sign | 0x7f800000u | (((unsigned)b | (unsigned)(b >> 32)) &
                                                          0x000fffffu ? 0x400000u : 0u)));
    const int e8 = e11 - 1023 + 127;
    if (e8 <= 0)
        return __int_as_float((int)sign);
    if (e8 >= 255)
        return __int_as_float((int)(sign | 0x7f800000u));
    const unsigned mant = (unsigned)((unsigned long long)b >> 29) & 0x7fffffu;
    return __int_as_float((int)(sign | ((unsigned)e8 << 23) | mant));
}

__device__ __forceinline__ int hist_bin64(double x, const double *edges, int nb, double e0,
                                          double el, double norm)
{
    if (!(x >= e0 && x <= el))
        return -1;
    int j = (int)((x - e0) * norm);
    j = j < 0 ? 0 : (j > nb - 1 ? nb - 1 : j);
    while (j > 0 && x < edges[j])
        j--;
    while (j < nb - 1 && x >= edges[j + 1])
        j++;
    return j;
}

// Adds one count to bin j (j < 0: none) of the warp's or the block's histogram;
// lanes of the warp that hit the same bin add together (saturated spectra put
// most pixels of a warp in the same bin).
template <bool WARP_PRIVATE>
__device__ __forceinline__ void hist_add(int j, unsigned *wh, unsigned long long *bh)
{
    const unsigned peers = __match_any_sync(0xffffffffu, j);
    const int lane = threadIdx.x & 31;
    if (j >= 0 && lane == __ffs(peers) - 1) {
        if (WARP_PRIVATE)
            atomicAdd(&wh[j], (unsigned)__popc(peers));
        else
            atomicAdd(&bh[j], (unsigned long long)__popc(peers));
    }
}

template <bool WARP_PRIVATE>
__global__ void __launch_bounds__(FLUX_HIST_THREADS)
    flux_hist_kernel(const double *tau, long long n, double scale, const double *edges, int nb,
                     unsigned long long *counts)
{
    // dynamic shared memory: float edges rounded up [nb + 1], rounded down
    // [nb + 1], per warp a queue of 64 pixel indices for the FP64 recheck,
    // then the histograms
    extern __shared__ __align__(16) unsigned char hraw[];
    constexpr int NW = FLUX_HIST_THREADS / 32;
    float *eu = reinterpret_cast<float *>(hraw);
    float *ed = eu + (nb + 1);
    const size_t eb = ((size_t)2 * (nb + 1) * sizeof(float) + 15) & ~(size_t)15;
    long long *queue_all = reinterpret_cast<long long *>(hraw + eb);
    unsigned char *hist_base = hraw + eb + sizeof(long long) * 64 * NW;
    unsigned *wh_all = reinterpret_cast<unsigned *>(hist_base);
    unsigned long long *bh = reinterpret_cast<unsigned long long *>(hist_base);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned *wh = wh_all + (size_t)warp * nb;
    long long *queue = queue_all + 64 * warp;
    for (int j = threadIdx.x; j <= nb; j += blockDim.x) {
        // float bounds of each edge (no FP64 work per pixel): eu >= e >= ed
        eu[j] = __double2float_ru(edges[j]);
        ed[j] = __double2float_rd(edges[j]);
    }
    if (WARP_PRIVATE) {
        for (int j = threadIdx.x; j < nb * NW; j += blockDim.x)
            wh_all[j] = 0u;
    } else {
        for (int j = threadIdx.x; j < nb; j += blockDim.x)
            bh[j] = 0ull;
    }
    __syncthreads();
    const double e0 = edges[0], el = edges[nb];
    const double norm = nb / (el - e0);
    const float e0f = (float)e0, normf = (float)norm, vmax = (float)(nb - 1);
    const float sf = trunc_to_float(scale);
    // exp(-scale tau) <= 1 for tau >= 0 and scale >= 0: such a pixel is in the
    // last bin as soon as it clears that bin's lower edge, when the bins reach 1
    const bool top_closed = scale >= 0.0 && el >= 1.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    int qn = 0;   // entries in this warp's recheck queue (warp-uniform)
    // whole-warp trips: every lane runs the same number of iterations
    const long long first = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31);
    for (long long base = first; base < n; base += stride) {
        const long long i = base + lane;
        const bool valid = i < n;
        const double t = valid ? tau[i] : 0.0;
        const float y = sf * trunc_to_float(t);
        const float x32 = expf(-y);
        const float rel = fmaf(fabsf(y), 4.8e-7f, 4.8e-7f);
        // exp is never negative: the lower end is clamped at 0
        const float lo = fmaxf(fmaf(-x32, rel, x32) - 1e-44f, 0.f);
        const float hi = fmaf(x32, rel, x32) + 1e-44f;
        // floor of the bin coordinate, clamped, without a float->int conversion
        // (ties at an integer may land one bin low; the test below then fails)
        const float v = fminf(fmaxf((x32 - e0f) * normf, 0.f), vmax);
        int j = __float_as_int(v + (12582912.0f - 0.5f)) - 0x4B400000;
        j = j < 0 ? 0 : j;
        // certain: [lo, hi] inside [e_j, e_{j+1}) (the last bin: inside [e_j, e_nb])
        const bool last_ok = j == nb - 1 && (hi <= ed[nb] || (top_closed && t >= 0.0));
        const bool sure = isfinite(y) && lo >= eu[j] && (hi < ed[j + 1] || last_ok);
        const bool need = valid && !sure;
        hist_add<WARP_PRIVATE>(valid && sure ? j : -1, wh, bh);
        // the rest go to the warp's queue, decided 32 at a time by whole warps
        const unsigned m = __ballot_sync(0xffffffffu, need);
        if (need)
            queue[qn + __popc(m & ((1u << lane) - 1u))] = i;
        qn += __popc(m);
        __syncwarp();
        if (qn >= 32) {
            const long long k = queue[lane];
            hist_add<WARP_PRIVATE>(hist_bin64(exp(-scale * tau[k]), edges, nb, e0, el, norm),
                                   wh, bh);
            __syncwarp();
            if (lane < qn - 32)
                queue[lane] = queue[32 + lane];
            qn -= 32;
            __syncwarp();
        }
    }
    if (qn > 0) {
        const int jj = lane < qn ? hist_bin64(exp(-scale * tau[queue[lane]]), edges, nb, e0, el,
                                              norm)
                                 : -1;
        hist_add<WARP_PRIVATE>(jj, wh, bh);
    }
    __syncthreads();
    if (WARP_PRIVATE) {
        for (int j = threadIdx.x; j < nb; j += blockDim.x) {
            unsigned long long c = 0;
            for (int w = 0; w < NW; w++)
                c += wh_all[(size_t)w * nb + j];
            if (c)
                atomicAdd(&counts[j], c);
        }
    } else {
        for (int j = threadIdx.x; j < nb; j += blockDim.x)
            if (bh[j])
                atomicAdd(&counts[j], bh[j]);
    }
}

}  // namespace

void launch_newton_passes(const double *tau, long long n, double mfd, double tol, double thresh,
                          int passes, const double *etab, double *part, double *state,
                          cudaStream_t s)
{
    for (int k = 0; k < passes; k++) {
        flux_moments_dev_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(tau, n, state, thresh, etab,
                                                                   part);
        newton_update_kernel<<<1, 32, 0, s>>>(part, RED_BLOCKS, mfd, tol, state);
    }
}

void launch_flux_sum(const double *tau, long long n, double scale, const double *etab,
                     double *part, double *out1, cudaStream_t s)
{
    flux_sum_kernel<<<RED_BLOCKS, RED_THREADS, 0, s>>>(tau, n, scale, etab, part);
    partial_sum_kernel<<<1, 32, 0, s>>>(part, RED_BLOCKS, 1, out1);
}

// out[i] = exp(y[i]) as the flux passes evaluate it
__global__ void fexp_kernel(const double *y, long long n, const double *etab, double *out)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = fexp(y[i], etab);
}

void launch_fexp(const double *y, long long n, const double *etab, double *out, cudaStream_t s)
{
    long long blocks = (n + 255) / 256;
    blocks = blocks < 1 ? 1 : (blocks > 4096 ? 4096 : blocks);
    fexp_kernel<<<(unsigned)blocks, 256, 0, s>>>(y, n, etab, out);
}

void exp_table_host(double *tab)
{
    // 2^(j/256) in extended precision, rounded once to double
    for (int j = 0; j < 256; j++)
        tab[j] = (double)std::exp2l((long double)j / 256.0L);
}

size_t flux_partials(int width) { return (size_t)RED_BLOCKS * width; }

size_t flux_hist_smem(int nb, bool warp_private)
{
    const size_t eb = ((size_t)2 * (nb + 1) * sizeof(float) + 15) & ~(size_t)15;
    const size_t queues = sizeof(long long) * 64 * (FLUX_HIST_THREADS / 32);
    return eb + queues +
           (warp_private ? sizeof(unsigned) * (size_t)nb * (FLUX_HIST_THREADS / 32)
                         : sizeof(unsigned long long) * (size_t)nb);
}

void launch_flux_hist(const double *tau, long long n, double scale, const double *edges, int nb,
                      unsigned long long *counts, cudaStream_t s)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int grid = sms * 4;
    // per-warp 32-bit counters: each warp sees at most ceil(n / (grid threads)) * 32 pixels
    const long long per_warp = ((n + (long long)grid * FLUX_HIST_THREADS - 1) /
                                ((long long)grid * FLUX_HIST_THREADS)) * 32;
    if (nb <= FLUX_WARP_BINS && per_warp < (1ll << 32)) {
        const size_t smem = flux_hist_smem(nb, true);
        cudaFuncSetAttribute(flux_hist_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        flux_hist_kernel<true><<<grid, FLUX_HIST_THREADS, smem, s>>>(tau, n, scale, edges, nb,
                                                                     counts);
    } else {
        const size_t smem = flux_hist_smem(nb, false);
        cudaFuncSetAttribute(flux_hist_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
        flux_hist_kernel<false><<<grid, FLUX_HIST_THREADS, smem, s>>>(tau, n, scale, edges, nb,
                                                                      counts);
    }
}

}  // namespace fsg
